"""CPU restatements of two decisions the kernels make, checked exhaustively on edge cases.

1. ddx_collide's keys (csrc/ddx_collide.cu, half_cell): floor(x * inv2) with the product
   rounded to FP64 is taken from FP32 arithmetic (x truncated to FP32, inv2 rounded to
   FP32, the product rounded) whenever pf +- (2^-21 |pf| + 2^-100) has one floor; otherwise
   the FP64 form decides.  The FP32 decision must never differ from the FP64 floor.
2. The mixed image's warp aggregation (csrc/ddx_flux.cu, image_mixed_kernel): runs of
   adjacent lanes on one pixel are summed by a segmented tree of five shuffle-down steps;
   each run's first lane must end with the run's sum, so every tracer's flux reaches its
   pixel exactly once.
3. The spatial order's Hilbert index (csrc/ddx_order.cu, hilbert_index): on a grid of
   2^bits cells per axis it must number every cell once, and consecutive indices must be
   face neighbours, so that a run of bodies in index order stays in a compact region.
"""
import numpy as np


def f32_trunc(x):
    b = x.view(np.uint64)
    sign = ((b >> np.uint64(32)) & np.uint64(0x80000000)).astype(np.uint32)
    e = ((b >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64) - 1023
    mant = ((b >> np.uint64(29)) & np.uint64(0x7FFFFF)).astype(np.uint32)
    out = sign | (((e + 127).clip(0, 255).astype(np.uint32)) << np.uint32(23)) | mant
    out = np.where(e < -126, sign, out)
    out = np.where(e > 127, sign | np.uint32(0x7F800000), out)
    return out.astype(np.uint32).view(np.float32)


def half_cell_fp32(x, inv2):
    """(decided, floor) of the FP32 path; m is formed in FP64 and rounded once, as the
    kernel's fmaf does (|pf| 2^-21 is exact, so only the 2^-100 term can round)."""
    inv2f = np.float32(inv2)
    with np.errstate(all="ignore"):
        pf = (f32_trunc(x) * inv2f).astype(np.float32)
        m = (np.abs(pf).astype(np.float64) * 2.0 ** -21 + 2.0 ** -100).astype(np.float32)
        lo = np.floor((pf - m).astype(np.float32))
        hi = np.floor((pf + m).astype(np.float32))
        return (lo == hi) & (np.abs(pf) < 2.0 ** 21), lo


def test_fp32_cell_floor_never_differs_from_fp64():
    rng = np.random.default_rng(1)
    decided_total = 0
    for h in (0.1, 1e-3, 0.37, 5.0, 1e-8):
        cell = 2.0 * h * (1.0 + 1e-9)
        inv2 = 2.0 * (1.0 / cell)
        for scale in (1.0, 130.0, 1e3, 1e-6, 1e5):
            x = rng.normal(size=400_000) * scale
            k = np.round(x * inv2)
            near = k / inv2
            x[:40_000] = near[:40_000]                                    # on half-cell edges
            x[40_000:80_000] = np.nextafter(near[40_000:80_000], np.inf)    # one ulp above
            x[80_000:120_000] = np.nextafter(near[80_000:120_000], -np.inf)  # one ulp below
            x[120_000:122_000] = rng.choice([0.0, -0.0, 1e-310, -1e-310, 1e-45, -1e-45,
                                             2.0 ** -127, -3 * 2.0 ** -128], 2_000)
            ref = np.floor(x * inv2)
            ok, lo = half_cell_fp32(x, inv2)
            assert not (ok & (lo != ref)).any(), (h, scale)
            decided_total += int(ok[122_000:].sum())
    assert decided_total > 0.5 * 25 * 278_000   # the FP32 path decides most random values


def segmented_run_sums(key, f):
    """The kernel's five shuffle-down steps over 32 lanes (shfl_down past the end returns
    the lane's own value, which the take bits exclude)."""
    head = np.ones(32, bool)
    head[1:] = key[1:] != key[:-1]
    heads = sum(1 << i for i in range(32) if head[i])
    seg = np.array([bin(heads & (0xFFFFFFFF >> (31 - l))).count("1") for l in range(32)])
    take = np.zeros(32, int)
    for b in range(5):
        o = 1 << b
        so = np.concatenate([seg[o:], seg[32 - o:]])
        take |= np.where((np.arange(32) + o < 32) & (so == seg), 1 << b, 0)
    v = f.copy()
    for b in range(5):
        o = 1 << b
        vo = np.concatenate([v[o:], v[32 - o:]])
        v = v + np.where((take >> b) & 1, vo, 0.0)
    return head, v


def test_segmented_warp_sum_gives_each_run_to_its_first_lane():
    rng = np.random.default_rng(3)
    for trial in range(3000):
        k = np.sort(rng.integers(0, rng.integers(1, 40), 32)) if trial % 2 else rng.integers(0, 6, 32)
        valid = rng.random(32) > 0.1
        key = np.where(valid, k, 10 ** 9 - np.arange(32))   # a lane without a pixel: a key of its own
        f = rng.random(32) * valid
        head, v = segmented_run_sums(key, f)
        for l in np.flatnonzero(valid & head):
            r = l
            while r + 1 < 32 and key[r + 1] == key[l]:
                r += 1
            assert abs(v[l] - f[l:r + 1].sum()) < 1e-12
        assert abs(v[valid & head].sum() - f.sum()) < 1e-9


def hilbert_index(c, bits):
    """hilbert_index of csrc/ddx_order.cu, step for step: Skilling's transform of the axes to
    the transposed index, the Gray code, then the bits interleaved (axis 0 first)."""
    X = list(c)
    M = 1 << (bits - 1)
    Q = M
    while Q > 1:
        P = Q - 1
        for i in range(3):
            if X[i] & Q:
                X[0] ^= P
            else:
                t = (X[0] ^ X[i]) & P
                X[0] ^= t
                X[i] ^= t
        Q >>= 1
    X[1] ^= X[0]
    X[2] ^= X[1]
    t, Q = 0, M
    while Q > 1:
        if X[2] & Q:
            t ^= Q - 1
        Q >>= 1
    X = [x ^ t for x in X]
    key = 0
    for b in range(bits - 1, -1, -1):
        for i in range(3):
            key = key << 1 | ((X[i] >> b) & 1)
    return key


def test_hilbert_index_numbers_every_cell_once_in_face_neighbour_steps():
    for bits in (1, 2, 3, 5):   # 5: the planetesimals' grid (the tracers' 6 bits follow the same steps)
        n = 1 << bits
        cells = [(x, y, z) for x in range(n) for y in range(n) for z in range(n)]
        keys = [hilbert_index(c, bits) for c in cells]
        assert sorted(keys) == list(range(n ** 3))
        walk = [c for _, c in sorted(zip(keys, cells))]
        assert walk[0] == (0, 0, 0)
        steps = np.abs(np.diff(np.array(walk), axis=0)).sum(axis=1)
        assert (steps == 1).all()
