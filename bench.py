"""Benchmark of the GB300 DiskDyn RK4 step: body-steps/s of the mixed-precision
integrator on the dusty-ring workload (1.5 Msun star, 2 planets, 4,096 gravitating
planetesimals, 1,048,576 dust grains with radiation pressure, PR and stellar-wind drag),
with the plain-FP64 form, the error of mixed against FP64, the dust kernel's roofline, an
end-to-end figure through the C ABI with host buffers, and a CPU baseline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One JSON line on rank 0.  Under torchrun every rank integrates its own dust shard of the
same size against a replica of the massive set (weak scaling, no data-path collective).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "RK4 body-steps/s (mixed precision, FP64-error stated)"
UNIT = "body-steps/s"
WORKLOAD = "dusty_ring"
# Flops per body-body interaction (Nyland, Harris & Prins, GPU Gems 3 ch. 31) and per
# star term (gravity reduced by beta + PR/stellar-wind drag), per tracer per stage.
FLOP_PAIR = 20
FLOP_STAR = 45
# Mixed dust kernel, bytes per grain and launch: DRAM traffic measured by ncu (20.65 MB read
# + 6.20 MB written for 262,144 grains: `ncu --set full -k regex:"dust_rk4_mixed_kernel"` on
# `bench.py --n-dust 262144`; writes still in L2 when the kernel ends are not counted), and
# the algorithmic bytes (the state read, 68 B, and the positions, velocities and grain
# number written, 56 B).
DUST_TRAFFIC_PER_GRAIN = (20.65e6 + 6.20e6) / 262144
ALG_BYTES_PER_GRAIN = 68 + 56


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=40)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--n-dust", type=int, default=1048576)
    p.add_argument("--n-plsml", type=int, default=4096)
    p.add_argument("--fp64-steps", type=int, default=2)
    p.add_argument("--comp-steps", type=int, default=5)
    p.add_argument("--err-steps", type=int, default=1000)
    p.add_argument("--err-dust", type=int, default=16384)
    p.add_argument("--err-seeds", type=int, default=4, help="shards drawn for the spread of the largest error")
    p.add_argument("--cpu-sample", type=int, default=262144)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-configs", action="store_true", help="leave out the brief legs of the other configurations")
    p.add_argument("--workload", choices=["dusty_ring", "imaging", "scale", "solar", "setup", "cadence", "accuracy"],
                   default="dusty_ring")
    p.add_argument("--solar-steps", type=int, default=1000)
    p.add_argument("--scale-err-steps", type=int, default=500)
    p.add_argument("--adjoint-steps", type=int, default=2000)
    p.add_argument("--adjoint-plsml-steps", type=int, default=20)
    p.add_argument("--adjoint-n-dust", type=int, default=262144, help="grains of the image-loss workload")
    return p.parse_args()


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: str):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", self.index, f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def smi_index(local_rank: int) -> str:
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    if vis:
        ids = [v.strip() for v in vis.split(",") if v.strip()]
        if local_rank < len(ids):
            return ids[local_rank]
    return str(local_rank)


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    return json.loads(p.read_text()) if p.exists() else {}


def run_ours(args, world, rank, local):
    import torch
    from diskdyn_gb300 import abi, shard, synth
    from diskdyn_gb300.engine import DeviceState, Engine, make_phys, probe_fma_peak

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    def barrier():
        if dist:
            dist.barrier()
    def allmax(v):
        if not dist:
            return v
        t = torch.tensor([v], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    def allsum(v):
        if not dist:
            return v
        t = torch.tensor([v], dtype=torch.float64, device="cuda")
        dist.all_reduce(t)
        return float(t.item())

    sysm = synth.dusty_ring(n_dust=args.n_dust, n_plsml=args.n_plsml, seed=synth.SEED + 7919 * rank)
    ng, nd = sysm.n_grav, sysm.n_dust
    eng = Engine(local)
    eng.set_size_table(**sysm.size_table)
    phys = make_phys(**sysm.phys)
    st0 = DeviceState.from_numpy(sysm.state, device=f"cuda:{local}")
    st = st0.clone()
    MIX, F64 = abi.DDX_PREC_MIXED, abi.DDX_PREC_FP64
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MiB > L2
    stream = torch.cuda.current_stream()

    # spatial-hash collisions over the grains, every step (the workload's collision pass):
    # pairs closer than h_coll into a buffer sized once, with room to spare
    h_coll = 0.1
    n_found = C.c_longlong(0)
    sh = C.c_void_p(stream.cuda_stream)

    def collide_call(buf):
        abi.check(eng.lib.ddx_collide(eng.ctx, C.byref(st._abi), ng, ng + nd, C.c_double(h_coll),
                                      C.c_void_p(buf.data_ptr()), buf.shape[0], C.byref(n_found), sh), "ddx_collide")
        return n_found.value

    def one_step(prec, ev=None, coll=None):
        if ev:
            ev[0].record(stream)
        eng.stage("massive_rk4", st, ng, sysm.dt, phys, prec)
        if ev:
            ev[1].record(stream)
        eng.stage("small_rk4", st, ng, sysm.dt, phys, prec)
        if ev:
            ev[2].record(stream)
        eng.stage("massive_final", st, ng, sysm.dt, phys, prec)
        if ev:
            ev[3].record(stream)
        if coll is not None:
            found = collide_call(coll)   # synchronises the stream: the count comes back to the host
            if ev:
                ev[4].record(stream)
            return found

    pair_buf = torch.empty((1, 2), dtype=torch.int32, device="cuda")
    pair_buf = torch.empty((4 * collide_call(pair_buf) + 65536, 2), dtype=torch.int32, device="cuda")
    for _ in range(args.warmup):
        found = one_step(MIX, coll=pair_buf)
        if found > pair_buf.shape[0]:
            pair_buf = torch.empty((4 * found + 65536, 2), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    alive0 = int((st.N[ng:] != 0).sum().item())
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(5)] for _ in range(args.steps)]
    pairs_per_step = []
    barrier()
    torch.cuda.synchronize()
    with Clocks(smi_index(local)) as clk:
        t0 = time.perf_counter()
        for k in range(args.steps):
            flush.zero_()
            pairs_per_step.append(one_step(MIX, evs[k], coll=pair_buf))
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    barrier()
    step_ms = [e[0].elapsed_time(e[4]) for e in evs]
    rk4_ms = [e[0].elapsed_time(e[3]) for e in evs]
    coll_ms = [e[3].elapsed_time(e[4]) for e in evs]
    dust_ms = [e[1].elapsed_time(e[2]) for e in evs]
    alive1 = int((st.N[ng:] != 0).sum().item())
    assert max(pairs_per_step) <= pair_buf.shape[0], "collision buffer too small"
    # whole job: units of all ranks over the slowest rank's time (diskdyn_gb300.shard)
    units, t_total, value = shard.job_rate((ng + 0.5 * (alive0 + alive1)) * args.steps, sum(step_ms) / 1e3,
                                           device="cuda")
    _, _, value_rk4 = shard.job_rate((ng + 0.5 * (alive0 + alive1)) * args.steps, sum(rk4_ms) / 1e3, device="cuda")
    collide = {"h_AU": h_coll, "pairs_per_step_median": statistics.median(pairs_per_step),
               "ms_per_call": statistics.mean(coll_ms),
               "bodies_per_s": nd / (statistics.mean(coll_ms) / 1e3),
               "what": "ddx_collide over the grains after every timed step, inside the timed region: hash keys "
                       "and bucket ranks on 2h cells, bucket scan, scatter to bucket order, octant count, scan, "
                       "write, count read back to the host (CUDA events around the call)"}

    # roofline of the dust kernel (FP32-pipe bound in the mixed path)
    fp32_peak, fp64_peak = probe_fma_peak(local)
    inter = 4.0 * 0.5 * (alive0 + alive1) * (ng - 1)
    flops = FLOP_PAIR * inter + FLOP_STAR * 4.0 * 0.5 * (alive0 + alive1)
    t_dust = statistics.mean(dust_ms) / 1e3
    achieved = flops / t_dust / 1e12

    def rel_err(a, b):
        live = (a["N"] != 0) & (b.N != 0)
        d = torch.sqrt((a["x"] - b.x) ** 2 + (a["y"] - b.y) ** 2 + (a["z"] - b.z) ** 2)
        r = torch.sqrt(a["x"] ** 2 + a["y"] ** 2 + a["z"] ** 2)
        return (d / r)[live].double().cpu().numpy()

    # plain FP64 from the same initial state, and the error of mixed against it
    fp64 = None
    err_short = None
    if args.fp64_steps > 0:
        st = st0.clone()
        one_step(F64)
        st = st0.clone()
        f64_evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.fp64_steps)]
        torch.cuda.synchronize()
        for k in range(args.fp64_steps):
            flush.zero_()
            one_step(F64, f64_evs[k])
        torch.cuda.synchronize()
        f64_ms = [e[0].elapsed_time(e[3]) for e in f64_evs]
        f64_dust_ms = [e[1].elapsed_time(e[2]) for e in f64_evs]
        ref64 = {k: getattr(st, k).clone() for k in ("x", "y", "z", "N")}
        f64_value = allsum((ng + alive0) * args.fp64_steps) / allmax(sum(f64_ms) / 1e3)
        fp64 = {"value": f64_value, "unit": UNIT, "ms_per_step": statistics.mean(f64_ms),
                "steps": args.fp64_steps, "dust_kernel_ms": statistics.mean(f64_dust_ms)}
        st = st0.clone()
        for _ in range(args.fp64_steps):
            one_step(MIX)
        torch.cuda.synchronize()
        e_short = rel_err(ref64, st)
        err_short = {"steps": args.fp64_steps, "dust_rel_pos_err_median": float(np.median(e_short)),
                     "dust_rel_pos_err_max": float(e_short.max())}

    # the compensated step (massive set FP64, float-float planetesimal pulls within half the
    # tracer's largest coordinate, FP64 within 1.6e-2 of it) on the full workload
    comp = None
    if args.comp_steps > 0:
        COMP = abi.DDX_PREC_COMPENSATED
        st = st0.clone()
        one_step(COMP)
        c_evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.comp_steps)]
        torch.cuda.synchronize()
        for k in range(args.comp_steps):
            flush.zero_()
            one_step(COMP, c_evs[k])
        torch.cuda.synchronize()
        c_ms = [e[0].elapsed_time(e[3]) for e in c_evs]
        c_value = allsum((ng + alive0) * args.comp_steps) / allmax(sum(c_ms) / 1e3)
        comp = {"value": c_value, "unit": UNIT, "ms_per_step": statistics.mean(c_ms), "steps": args.comp_steps,
                "dust_kernel_ms": statistics.mean(e[1].elapsed_time(e[2]) for e in c_evs),
                "massive_ms": statistics.mean(e[0].elapsed_time(e[1]) + e[2].elapsed_time(e[3]) for e in c_evs),
                "over_fp64": c_value / fp64["value"] if fp64 else None,
                "what": "DDX_PREC_COMPENSATED: FP64 massive set, float-float planetesimal pulls for spans within "
                        "0.5 x the tracer's largest coordinate, FP32 beyond, FP64 within 1.6e-2 of it; the RK4 "
                        "step only (no collisions)"}

    # long-horizon error: err_steps steps of a smaller shard, mixed vs FP64
    err_long = err_seeds = None
    if args.err_steps > 0 and rank == 0:
        err_long = long_error_leg(eng, phys, args)
        if args.err_seeds > 1:
            err_seeds = seed_spread(eng, phys, args, [synth.SEED + 17 + k for k in range(1, args.err_seeds)])

    # end to end through the C ABI with host buffers (ddx_step_host): per step, the state
    # from pinned host memory to the device, the step, the updated state back; the dust
    # streams through in chunks with the copies overlapping the compute
    # ... then the step's collision pairs: ddx_collide on the device state, and the pairs
    # found copied to pinned host memory
    host = {k: getattr(st0, k).cpu().pin_memory() for k in ("x", "y", "z", "vx", "vy", "vz", "m", "N", "id")}
    out = {k: torch.empty_like(host[k]).pin_memory() for k in host}
    pairs_host = torch.empty(pair_buf.shape, dtype=torch.int32).pin_memory()
    h2d = sum(t.numel() * t.element_size() for t in host.values())
    d2h = sum(out[k].numel() * out[k].element_size() for k in ("x", "y", "z", "vx", "vy", "vz", "N"))
    st = st0.clone()

    def e2e_step():
        eng.step_host(st, host, out, ng, sysm.dt, phys, MIX)
        found = collide_call(pair_buf)
        pairs_host[:found].copy_(pair_buf[:found], non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return found

    e2e_step()                                  # creates the copy streams
    torch.cuda.synchronize()
    barrier()
    e2e_ms, e2e_pairs = [], []
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        e2e_pairs.append(e2e_step())
        e2e_ms.append((time.perf_counter() - t1) * 1e3)
    e2e_value = allsum((ng + alive0) * args.steps) / allmax(sum(e2e_ms) / 1e3)
    d2h_pairs = 8.0 * statistics.mean(e2e_pairs)

    peaks = measured_peaks()
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_total * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 state + f32 perturbations (mixed)",
        "data": "synthetic (seeded Philox), dusty-ring configuration",
        "config": {"workload": WORKLOAD, "n_grav": ng, "n_dust_per_gpu": nd, "n_planetesimals": args.n_plsml,
                   "dt_yr": sysm.dt, "precision": "mixed", "physics": "radiation+PR+stellar-wind drag",
                   "step": "massive_rk4 + small_rk4 + massive_final + ddx_collide (h = %.2f AU)" % h_coll,
                   "near_radius_eta": 4e-3, "l2": "flushed between timed steps (256 MiB write)"},
        "wall_s_timed_region": wall,
        "rk4_only": {"value": value_rk4, "unit": UNIT, "ms_per_step": statistics.mean(rk4_ms),
                     "what": "the same timed steps without the collision call"},
        "fp64": fp64,
        "mixed_over_fp64": value_rk4 / fp64["value"] if fp64 else None,
        "compensated": comp,
        "error_vs_fp64": err_short,
        "error_vs_fp64_long": err_long,
        "error_vs_fp64_other_shards": err_seeds,
        "collide": collide,
        "roofline": {"kernel": "dust_rk4_mixed_kernel", "bound": "fp32_pipe", "achieved": achieved,
                     "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                     "peak_source": "ddx_probe_fma_peak (FMA chains, measured in this run); "
                                    "MEASURED_PEAKS.json has no FP32/FP64 pipe figure",
                     "sm_count": sms,
                     "fp32_nominal_tflops": sms * 128 * 2 * 2.070e9 / 1e12,
                     "fp32_nominal_at_median_clock_tflops": (sms * 128 * 2 * clocks["sm_mhz"] * 1e6 / 1e12
                                                             if clocks.get("sm_mhz") else None),
                     "frac_of_nominal": achieved / (sms * 128 * 2 * 2.070e9 / 1e12),
                     "nominal_definition": "SMs x 128 FP32 lanes x 2 flops (FMA) x 2,070 MHz",
                     "flops_per_launch": flops, "dust_kernel_ms": t_dust * 1e3,
                     "fp64_peak_tflops": fp64_peak,
                     # DRAM bytes per launch: ncu dram__bytes_read.sum + dram__bytes_write.sum of
                     # one 262,144-grain launch of this kernel (the same 4,099 massive bodies),
                     # scaled by the grains to a 1,048,576-grain launch
                     "traffic": DUST_TRAFFIC_PER_GRAIN * nd,
                     "traffic_source": "ncu capture of a 262,144-grain launch, scaled by the grains",
                     "algorithmic_bytes": ALG_BYTES_PER_GRAIN * nd,
                     "hbm_peak_gbs": peaks.get("hbm_gbs")},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h + d2h_pairs,
                "what": "ddx_step_host (state in from pinned host memory, step, state out) + ddx_collide + the "
                        "pairs found copied to pinned host memory, host wall time per step"},
        # per step: planetesimal order (one block up to 8,192 planetesimals, else 14 launches of
        # the radix sort), prepare, 2 x (slice sums + gather), tracer order (7), span boxes, dust;
        # collisions: keys, bucket scan (3), scatter, count, scan (3), write
        "gpu_launches": ((1 if args.n_plsml <= 8192 else 14) + 14 + 10) * args.steps,
        "clocks": clocks,
    }
    if rank == 0 and world == 1 and not args.no_configs:
        # the other configurations in brief, each with its own roofline
        line["configs"] = {"solar": solar_leg(local, fp64_peak), "imaging": imaging_leg(local),
                           "scale": scale_leg(local, fp32_peak)}
    if rank == 0 and args.adjoint_steps > 0:
        line["adjoint"] = adjoint_leg(local, n_dust=args.adjoint_n_dust, n_steps=args.adjoint_steps)
    if rank == 0 and args.adjoint_plsml_steps > 0:
        # the image-loss system with the dusty ring's 4,096 planetesimals in the massive set
        # (FP64 all-pairs, every grain feeling every planetesimal): fewer steps, since each FP64
        # step costs about 150 ms forward; forward, recompute and reverse all cost per step
        k = args.adjoint_plsml_steps
        leg = adjoint_leg(local, n_dust=args.adjoint_n_dust, n_steps=k, ckpt=max(1, k // 2), n_plsml=4096)
        leg["steps_note"] = ("%d of the workload's 2,000 steps, checkpoints every %d: the forward, the "
                             "recompute and the reverse all cost per step" % (k, max(1, k // 2)))
        line["adjoint_planetesimals"] = leg
    if rank == 0 and world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(sysm, args.cpu_sample)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def massive_energy(st, ng):
    """Total energy of the massive set, sum m v^2 / 2 - sum_{i<j} m_i m_j / r_ij, in the
    state's units (masses carry the 4 pi^2, so the pair potential needs no G)."""
    import torch
    x = torch.stack([st.x[:ng], st.y[:ng], st.z[:ng]], 1)
    v = torch.stack([st.vx[:ng], st.vy[:ng], st.vz[:ng]], 1)
    m = st.m[:ng]
    e = 0.5 * (m * (v * v).sum(1)).sum()
    j = torch.arange(ng, device=x.device)
    for i0 in range(0, ng, 512):
        i1 = min(ng, i0 + 512)
        d = torch.sqrt(((x[i0:i1, None, :] - x[None, :, :]) ** 2).sum(-1))
        upper = j[None, :] > torch.arange(i0, i1, device=x.device)[:, None]
        e = e - torch.where(upper, m[i0:i1, None] * m[None, :] / torch.where(upper, d, 1.0), 0.0).sum()
    return e.item()


def image_profiles(img, n_r=48, n_phi=36):
    """Radial profile (flux in annuli about the image centre, out to the frame's half
    width; beyond it the last annulus) and azimuthal profile (flux in n_phi sectors) of
    one image."""
    import torch
    X, Y = img.shape
    ii = torch.arange(X, device=img.device, dtype=torch.float64) - (X - 1) / 2.0
    jj = torch.arange(Y, device=img.device, dtype=torch.float64) - (Y - 1) / 2.0
    I, J = torch.meshgrid(ii, jj, indexing="ij")
    rb = (torch.sqrt(I * I + J * J) / (0.5 * X) * n_r).long().clamp(max=n_r - 1).flatten()
    pb = ((torch.atan2(J, I) + math.pi) / (2 * math.pi) * n_phi).long().clamp(max=n_phi - 1).flatten()
    f = img.flatten()
    radial = torch.zeros(n_r, dtype=torch.float64, device=img.device).index_add_(0, rb, f)
    azim = torch.zeros(n_phi, dtype=torch.float64, device=img.device).index_add_(0, pb, f)
    return radial, azim


def long_error_leg(eng, phys, args, n_plsml=None, seed=None, n_steps=None, floor=True):
    """Mixed precision against FP64 over err_steps steps of a dusty-ring shard (all massive
    bodies, err_dust grains): relative position error of grains and massive bodies, the
    massive set's energy drift, and the error of the radial and azimuthal profiles of the
    final images (1.25 um and 100 um, 512 x 512, 300 AU).  The same figures between two
    FP64 forms (rsqrt-based vs the reference's m/RR/sqrt(RR) expression) give the floor
    that FP64 rounding alone sets on this chaotic system."""
    import torch
    from diskdyn_gb300 import abi, synth
    from diskdyn_gb300.engine import DeviceState, Engine, make_view
    n_plsml = args.n_plsml if n_plsml is None else n_plsml
    seed = synth.SEED + 17 if seed is None else seed
    n_steps = args.err_steps if n_steps is None else n_steps
    small = synth.ring_imaging(synth.dusty_ring(n_dust=args.err_dust, n_plsml=n_plsml, seed=seed))
    ng = small.n_grav
    runs = {}
    forms = [("fp64", abi.DDX_PREC_FP64, abi.DDX_MODE_FIXED), ("mixed", abi.DDX_PREC_MIXED, abi.DDX_MODE_FIXED),
             ("compensated", abi.DDX_PREC_COMPENSATED, abi.DDX_MODE_FIXED)]
    if floor:
        forms.append(("fp64_ref_expr", abi.DDX_PREC_FP64, abi.DDX_MODE_REFERENCE))
    for name, prec, mode in forms:
        st = DeviceState.from_numpy(small.state)
        e0 = massive_energy(st, ng)
        eng.evolve(st, ng, small.dt, n_steps, phys, prec, mode)
        torch.cuda.synchronize()
        runs[name] = (st, (massive_energy(st, ng) - e0) / abs(e0))
    ie = Engine(torch.cuda.current_device())
    ie.set_size_table(**small.size_table)
    o = small.optics
    ie.set_optics(o["w"], o["in"], o["Qabs"], o["Qsca"], o["Qpfunc"], o["Td"], o["Rmin"], o["Rmax"])
    view = make_view(**small.view)
    imgs = {k: ie.image(st, ng, view, small.image_wj) for k, (st, _) in runs.items()}
    torch.cuda.synchronize()
    ie.close()

    def compare(name):
        a, b = runs["fp64"][0], runs[name][0]
        live = (a.N[ng:] != 0) & (b.N[ng:] != 0)
        d = torch.sqrt((a.x - b.x) ** 2 + (a.y - b.y) ** 2 + (a.z - b.z) ** 2)
        r = torch.sqrt(a.x ** 2 + a.y ** 2 + a.z ** 2)
        e = (d / r)[ng:][live].double().cpu().numpy()
        em = (d / r)[1:ng].double().cpu().numpy()
        out = {"dust_rel_pos_err_median": float(np.median(e)),
               "dust_rel_pos_err_p90": float(np.quantile(e, 0.9)),
               "dust_rel_pos_err_p99": float(np.quantile(e, 0.99)),
               "dust_rel_pos_err_max": float(e.max()),
               "massive_rel_pos_err_median": float(np.median(em)),
               "massive_rel_pos_err_max": float(em.max()),
               "massive_energy_drift": runs[name][1],
               "dust_removed_differently": int((a.N[ng:] != b.N[ng:]).sum().item())}
        prof = []
        for k in range(len(small.image_wj)):
            ra, pa = image_profiles(imgs["fp64"][k])
            rb, pb = image_profiles(imgs[name][k])
            prof.append({"wavelength_um": float(small.optics["w"][small.image_wj[k]] * 1e6),
                         "radial_profile_err": float(((rb - ra).abs().max() / ra.abs().max()).item()),
                         "azimuthal_profile_err": float(((pb - pa).abs().max() / pa.abs().max()).item()),
                         "total_flux_rel_err": float(((rb.sum() - ra.sum()) / ra.sum()).abs().item())})
        out["image"] = prof
        return out

    out = {"steps": n_steps, "n_dust": args.err_dust, "n_grav": ng, "n_planets": small.phys["n_planets"],
           "fp64_massive_energy_drift": runs["fp64"][1],
           "mixed_vs_fp64": compare("mixed"),
           "compensated_vs_fp64": compare("compensated"),
           "profile_error_definition": "max over bins of |profile - FP64 profile| / max FP64 profile; "
                                       "48 annuli to the frame half-width, 36 sectors"}
    if floor:
        out["fp64_floor_ref_expr_vs_fp64"] = compare("fp64_ref_expr")
    return out


def seed_spread(eng, phys, args, seeds):
    """The long-horizon comparison of long_error_leg on other draws of the shard (positions
    only): the largest grain error comes from the few grains in the closest encounters with
    planetesimals, which amplify any difference by 10^3 and more, so it varies from draw to
    draw far more than the median or the 99th percentile.  Per shard: mixed, compensated and
    the FP64 floor (the reference's m/RR/sqrt(RR) expression) against the FP64 step."""
    import torch
    from diskdyn_gb300 import abi, synth
    from diskdyn_gb300.engine import DeviceState
    forms = (("fp64", abi.DDX_PREC_FP64, abi.DDX_MODE_FIXED),
             ("fp64_ref_expr", abi.DDX_PREC_FP64, abi.DDX_MODE_REFERENCE),
             ("mixed", abi.DDX_PREC_MIXED, abi.DDX_MODE_FIXED),
             ("compensated", abi.DDX_PREC_COMPENSATED, abi.DDX_MODE_FIXED))
    out = []
    for seed in seeds:
        small = synth.dusty_ring(n_dust=args.err_dust, n_plsml=args.n_plsml, seed=seed)
        ng = small.n_grav
        runs = {}
        for name, prec, mode in forms:
            st = DeviceState.from_numpy(small.state)
            eng.evolve(st, ng, small.dt, args.err_steps, phys, prec, mode)
            runs[name] = st
        torch.cuda.synchronize()
        a = runs["fp64"]
        row = {"seed": seed, "steps": args.err_steps, "n_dust": args.err_dust}
        for name in ("mixed", "compensated", "fp64_ref_expr"):
            b = runs[name]
            live = (a.N[ng:] != 0) & (b.N[ng:] != 0)
            d = torch.sqrt((a.x - b.x) ** 2 + (a.y - b.y) ** 2 + (a.z - b.z) ** 2)
            r = torch.sqrt(a.x ** 2 + a.y ** 2 + a.z ** 2)
            e = (d / r)[ng:][live].double().cpu().numpy()
            em = (d / r)[1:ng].double().cpu().numpy()
            row[name] = {"dust_rel_pos_err_p99": float(np.quantile(e, 0.99)), "dust_rel_pos_err_max": float(e.max()),
                         "massive_rel_pos_err_max": float(em.max())}
        out.append(row)
    return out


def run_accuracy(args, world, rank, local):
    """Near radius of the mixed step (ddx_set_near_radius) against time and error on the
    dusty ring: for each radius eta, the full workload's step time (CUDA events, L2 flushed
    between steps) and the error of a 1,000-step run against the FP64 step on a shard of
    err_dust grains with all massive bodies.  Beside it, the FP64 CPU oracle runs the same
    1,000 steps of a 2,048-grain shard on the host cores (a thread; ctypes releases the
    interpreter lock), and the GPU's FP64 and mixed steps are compared with it."""
    import threading as th
    import torch
    import oracle.cpu as oc
    from diskdyn_gb300 import abi, synth
    from diskdyn_gb300.engine import DeviceState, Engine, make_phys

    torch.cuda.set_device(local)
    n_steps = args.err_steps
    osys = synth.dusty_ring(n_dust=2048, n_plsml=args.n_plsml, seed=synth.SEED + 29)
    oracle_out = {}

    def oracle_run():
        t0 = time.perf_counter()
        oracle_out["state"] = oc.step(osys.state, osys.n_grav, osys.dt, osys.size_table, osys.phys, n_steps)
        oracle_out["s"] = time.perf_counter() - t0
    worker = th.Thread(target=oracle_run, daemon=True)
    worker.start()

    full = synth.dusty_ring(n_dust=args.n_dust, n_plsml=args.n_plsml)
    ng = full.n_grav
    eng = Engine(local)
    eng.set_size_table(**full.size_table)
    phys = make_phys(**full.phys)
    st0 = DeviceState.from_numpy(full.state, device=f"cuda:{local}")
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    MIX, F64 = abi.DDX_PREC_MIXED, abi.DDX_PREC_FP64

    small = synth.dusty_ring(n_dust=args.err_dust, n_plsml=args.n_plsml, seed=synth.SEED + 17)
    sng = small.n_grav

    def evolve(sysm, prec, k, eta):
        st = DeviceState.from_numpy(sysm.state)
        eng.set_near_radius(eta)
        eng.set_size_table(**sysm.size_table)
        eng.evolve(st, sysm.n_grav, sysm.dt, k, make_phys(**sysm.phys), prec, abi.DDX_MODE_FIXED)
        torch.cuda.synchronize()
        return st

    def errs(a, b, n_grav):
        live = (a.N[n_grav:] != 0) & (b.N[n_grav:] != 0)
        d = torch.sqrt((a.x - b.x) ** 2 + (a.y - b.y) ** 2 + (a.z - b.z) ** 2)
        r = torch.sqrt(b.x ** 2 + b.y ** 2 + b.z ** 2)
        e = (d / r)[n_grav:][live].double().cpu().numpy()
        em = (d / r)[1:n_grav].double().cpu().numpy()
        return {"dust_median": float(np.median(e)), "dust_p99": float(np.quantile(e, 0.99)),
                "dust_max": float(e.max()), "massive_median": float(np.median(em)), "massive_max": float(em.max()),
                "removed_differently": int((a.N[n_grav:] != b.N[n_grav:]).sum().item())}

    ref = evolve(small, F64, n_steps, 0.0)
    sweep = []
    for eta in (0.0, 1e-3, 2e-3, 4e-3, 8e-3, 1.6e-2, 3.2e-2):
        eng.set_size_table(**full.size_table)
        eng.set_near_radius(eta)
        st = st0.clone()
        for _ in range(args.warmup):
            eng.step(st, ng, full.dt, phys, MIX)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        torch.cuda.synchronize()
        for e0, e1 in evs:
            flush.zero_()
            e0.record(stream)
            eng.step(st, ng, full.dt, phys, MIX)
            e1.record(stream)
        torch.cuda.synchronize()
        ms = statistics.mean(e0.elapsed_time(e1) for e0, e1 in evs)
        m = evolve(small, MIX, n_steps, eta)
        sweep.append({"eta": eta, "near_radius_at_130AU": eta * 130.0, "ms_per_step": ms,
                      "body_steps_per_s": (ng + full.n_dust) / (ms / 1e3), "error_vs_fp64": errs(m, ref, sng)})
    comp_sweep = []
    for ceta, neta in ((0.25, 4e-3), (0.25, 1.6e-2), (0.35, 1.6e-2), (0.5, 4e-3), (0.5, 1.6e-2), (0.5, 3.2e-2),
                       (1.0, 1.6e-2), (float("inf"), 1.6e-2)):
        eng.set_size_table(**full.size_table)
        eng.set_compensated_radius(ceta)
        eng.set_near_radius(neta)
        st = st0.clone()
        for _ in range(2):
            eng.step(st, ng, full.dt, phys, abi.DDX_PREC_COMPENSATED)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(3)]
        torch.cuda.synchronize()
        for e0, e1 in evs:
            flush.zero_()
            e0.record(stream)
            eng.step(st, ng, full.dt, phys, abi.DDX_PREC_COMPENSATED)
            e1.record(stream)
        torch.cuda.synchronize()
        ms = statistics.mean(e0.elapsed_time(e1) for e0, e1 in evs)
        eng.set_compensated_radius(ceta)
        c = evolve(small, abi.DDX_PREC_COMPENSATED, n_steps, neta)
        comp_sweep.append({"comp_eta": ceta if math.isfinite(ceta) else "inf", "near_eta": neta, "ms_per_step": ms,
                           "body_steps_per_s": (ng + full.n_dust) / (ms / 1e3), "error_vs_fp64": errs(c, ref, sng)})
    eng.set_compensated_radius(0.5)
    eng.set_near_radius(-1.0)
    worker.join()
    vs_oracle = None
    if "state" in oracle_out:
        o = oracle_out["state"]
        ost = DeviceState.from_numpy(o)
        f = evolve(osys, F64, n_steps, 4e-3)
        m = evolve(osys, MIX, n_steps, 4e-3)
        vs_oracle = {"steps": n_steps, "n_dust": 2048, "n_grav": osys.n_grav, "oracle_s": oracle_out["s"],
                     "oracle_cores": os.cpu_count(),
                     "fp64_gpu_vs_oracle": errs(f, ost, osys.n_grav),
                     "mixed_gpu_vs_oracle": errs(m, ost, osys.n_grav),
                     "compensated_gpu_vs_oracle": errs(evolve(osys, abi.DDX_PREC_COMPENSATED, n_steps, -1.0),
                                                       ost, osys.n_grav)}
    line = {"metric": "near radius vs step time and 1,000-step error (mixed precision)", "workload": "accuracy",
            "n_grav": ng, "n_dust": full.n_dust, "err_dust": args.err_dust, "err_steps": n_steps,
            "error_definition": "|x - x_ref| / |x_ref| per body after err_steps steps from the same state",
            "sweep": sweep, "compensated_sweep": comp_sweep, "vs_oracle": vs_oracle}
    eng.close()
    print(json.dumps(line), flush=True)


def run_scale(args, world, rank, local):
    """Mixed precision at scale: 16,777,216 grains + 65,536 gravitating planetesimals with
    the dusty ring's star and two planets.  Times `steps` full steps (L2 flushed between
    them) and reports the error against FP64 on a shard of err_dust grains with the same
    massive set over --scale-err-steps steps: grains are test particles given the massive
    trajectories, so a shard follows the dynamics of the full run."""
    import torch
    from diskdyn_gb300 import abi, synth
    from diskdyn_gb300.engine import DeviceState, Engine, make_phys, probe_fma_peak

    torch.cuda.set_device(local)
    n_dust = args.n_dust if args.n_dust != 1048576 else 16777216
    n_plsml = args.n_plsml if args.n_plsml != 4096 else 65536
    seed = synth.SEED + 4243 + 7919 * rank
    sysm = synth.dusty_ring(n_dust=n_dust, n_plsml=n_plsml, seed=seed, n_steps=500)
    ng = sysm.n_grav
    eng = Engine(local)
    eng.set_size_table(**sysm.size_table)
    phys = make_phys(**sysm.phys)
    st = DeviceState.from_numpy(sysm.state, device=f"cuda:{local}")
    del sysm.state
    MIX = abi.DDX_PREC_MIXED
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    def one_step(ev):
        ev[0].record(stream)
        eng.stage("massive_rk4", st, ng, sysm.dt, phys, MIX)
        ev[1].record(stream)
        eng.stage("small_rk4", st, ng, sysm.dt, phys, MIX)
        ev[2].record(stream)
        eng.stage("massive_final", st, ng, sysm.dt, phys, MIX)
        ev[3].record(stream)

    for _ in range(args.warmup):
        one_step([torch.cuda.Event(enable_timing=True) for _ in range(4)])
    torch.cuda.synchronize()
    alive0 = int((st.N[ng:] != 0).sum().item())
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
    with Clocks(smi_index(local)) as clk:
        for k in range(args.steps):
            flush.zero_()
            one_step(evs[k])
        torch.cuda.synchronize()
    alive1 = int((st.N[ng:] != 0).sum().item())
    step_ms = [e[0].elapsed_time(e[3]) for e in evs]
    massive_ms = [e[0].elapsed_time(e[1]) + e[2].elapsed_time(e[3]) for e in evs]
    dust_ms = [e[1].elapsed_time(e[2]) for e in evs]
    value = (ng + 0.5 * (alive0 + alive1)) * args.steps / (sum(step_ms) / 1e3)
    fp32_peak, _ = probe_fma_peak(local)
    inter = 4.0 * 0.5 * (alive0 + alive1) * (ng - 1)
    flops = FLOP_PAIR * inter + FLOP_STAR * 4.0 * 0.5 * (alive0 + alive1)
    achieved = flops / (statistics.mean(dust_ms) / 1e3) / 1e12
    line = {"metric": "RK4 body-steps/s (mixed precision, FP64-error stated)", "value": value,
            "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": statistics.mean(step_ms), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 state + f32 perturbations (mixed)",
            "data": "synthetic (seeded Philox), mixed precision at scale",
            "config": {"workload": "scale", "n_grav": ng, "n_dust": n_dust, "n_planetesimals": n_plsml,
                       "dt_yr": sysm.dt, "precision": "mixed", "l2": "flushed between timed steps (256 MiB write)"},
            "dust_kernel_ms": statistics.mean(dust_ms), "massive_ms": statistics.mean(massive_ms),
            "roofline": {"kernel": "dust_rk4_kernel<mixed>", "bound": "fp32_pipe", "achieved": achieved,
                         "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved / fp32_peak},
            "clocks": clk.summary()}
    del st
    torch.cuda.empty_cache()
    if args.scale_err_steps > 0:
        line["error_vs_fp64"] = long_error_leg(eng, phys, args, n_plsml=n_plsml, seed=seed,
                                               n_steps=args.scale_err_steps, floor=False)
    print(json.dumps(line), flush=True)


def solar_leg(local, fp64_peak, n_steps=1000, reps=3):
    """Configuration 1 in brief: 9 massive bodies + 16,384 planetesimals, the whole
    1,000-step FP64 run replayed as one CUDA graph, CUDA events; roofline of the FP64 pipe
    (20 flops per body-body interaction, 45 per star term)."""
    import torch
    from diskdyn_gb300 import abi, synth
    from diskdyn_gb300.engine import DeviceState, Engine, make_phys
    sysm = synth.solar_like(n_dust=16384)
    ng, nd = sysm.n_grav, sysm.n_dust
    eng = Engine(local)
    eng.set_size_table(**sysm.size_table)
    phys = make_phys(**sysm.phys)
    st0 = DeviceState.from_numpy(sysm.state, device=f"cuda:{local}")
    st = st0.clone()
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        eng.evolve(st, ng, sysm.dt, 10, phys, abi.DDX_PREC_FP64, stream=stream)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        eng.evolve(st, ng, sysm.dt, n_steps, phys, abi.DDX_PREC_FP64, stream=stream)
    ms = []
    for _ in range(reps + 1):
        st.copy_from_({f: getattr(st0, f) for f in ("x", "y", "z", "vx", "vy", "vz", "m", "N", "id")})
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            g.replay()
            e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    t = statistics.mean(ms[1:]) / 1e3
    flops = n_steps * (FLOP_PAIR * 4.0 * (nd * (ng - 1) + ng * (ng - 1)) + FLOP_STAR * 4.0 * nd)
    eng.close()
    return {"workload": "solar: 9 massive + 16,384 planetesimals, 1,000 FP64 steps (dt 0.05 yr) as one CUDA graph",
            "value": (ng + nd) * n_steps / t, "unit": UNIT, "ms_per_run": t * 1e3, "precision": "fp64",
            "gpu_launches_per_step": 4,
            "roofline": {"kernel": "whole step (dust_rk4_kernel<fp64> + massive passes)", "bound": "fp64_pipe",
                         "achieved": flops / t / 1e12, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": flops / t / 1e12 / fp64_peak,
                         "note": "16,384 tracers fill 64 blocks of 256 on 152 SMs: launch- and occupancy-bound"}}


def imaging_leg(local, reps=5):
    """Configuration 3 in brief: 4,194,304 tracers, 10 images of 1024 x 1024 and the
    200-wavelength SED in mixed precision, CUDA events with L2 flushed between calls;
    roofline of HBM with the algorithmic bytes (36 B per tracer read once plus 8 B per pixel
    and image written; the SED writes 200 doubles)."""
    import torch
    from diskdyn_gb300 import abi, synth
    from diskdyn_gb300.engine import DeviceState, Engine, make_view
    n = 4194304
    s = synth.imaging(n_dust=n)
    eng = Engine(local)
    eng.set_size_table(**s.size_table)
    o = s.optics
    eng.set_optics(o["w"], o["in"], o["Qabs"], o["Qsca"], o["Qpfunc"], o["Td"], o["Rmin"], o["Rmax"])
    st = DeviceState.from_numpy(s.state, device=f"cuda:{local}")
    view = make_view(**s.view)
    n_img = len(s.image_wj)
    F = torch.empty((n_img, s.view["xsize"], s.view["ysize"]), dtype=torch.float64, device="cuda")
    Fs = torch.empty(len(o["w"]), dtype=torch.float64, device="cuda")
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(2):
        eng.image(st, s.n_grav, view, s.image_wj, out=F, precision=abi.DDX_PREC_MIXED)
        eng.sed(st, s.n_grav, view, out=Fs, precision=abi.DDX_PREC_MIXED)
    ti, ts = [], []
    for _ in range(reps):
        flush.zero_()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        e[0].record(stream)
        eng.image(st, s.n_grav, view, s.image_wj, out=F, precision=abi.DDX_PREC_MIXED)
        e[1].record(stream)
        flush.zero_()
        e[2].record(stream)
        eng.sed(st, s.n_grav, view, out=Fs, precision=abi.DDX_PREC_MIXED)
        e[3].record(stream)
        torch.cuda.synchronize()
        ti.append(e[0].elapsed_time(e[1]))
        ts.append(e[2].elapsed_time(e[3]))
    t_img, t_sed = statistics.mean(ti) / 1e3, statistics.mean(ts) / 1e3
    # the same images with the tracers stored in pixel order: whole warps then land on one
    # pixel and the warp-aggregated scatter issues one atomic per pixel and warp
    pix, _ = eng.pixels(st, s.n_grav, view)
    order = torch.argsort(torch.where(pix < 0, torch.iinfo(torch.int32).max, pix).long(), stable=True)
    for f in ("x", "y", "z", "vx", "vy", "vz", "m", "N", "id"):
        a = getattr(st, f)
        a[s.n_grav:] = a[s.n_grav:][order]
    tp = []
    for _ in range(reps + 1):
        flush.zero_()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        e[0].record(stream)
        eng.image(st, s.n_grav, view, s.image_wj, out=F, precision=abi.DDX_PREC_MIXED)
        e[1].record(stream)
        torch.cuda.synchronize()
        tp.append(e[0].elapsed_time(e[1]))
    t_img_sorted = statistics.mean(tp[1:]) / 1e3
    npix = s.view["xsize"] * s.view["ysize"]
    b_img = n * 36 + n_img * npix * 8
    b_sed = n * 36 + len(o["w"]) * 8
    hbm = measured_peaks().get("hbm_gbs", 6800.0)
    eng.close()
    return {"workload": "imaging: 4,194,304 tracers, 10 images 1024x1024 + 200-wavelength SED, mixed precision",
            "value": n * n_img / t_img, "unit": "particle-wavelengths/s (images)", "image_ms": t_img * 1e3,
            "sed_ms": t_sed * 1e3, "sed_particle_wavelengths_per_s": n * len(o["w"]) / t_sed,
            "image_ms_tracers_in_pixel_order": t_img_sorted * 1e3,
            "roofline": {"kernel": "image_mixed_kernel (+ convert)", "bound": "hbm", "achieved": b_img / t_img / 1e9,
                         "peak": hbm, "unit": "GB/s", "frac": b_img / t_img / 1e9 / hbm,
                         "algorithmic_bytes": b_img},
            "sed_roofline": {"kernel": "sed_mixed_kernel", "bound": "hbm", "achieved": b_sed / t_sed / 1e9,
                             "peak": hbm, "unit": "GB/s", "frac": b_sed / t_sed / 1e9 / hbm,
                             "algorithmic_bytes": b_sed}}


def scale_leg(local, fp32_peak, steps=2, warmup=1):
    """Configuration 4 in brief: 16,777,216 grains + 65,536 gravitating planetesimals (with
    the dusty ring's star and planets), mixed precision, `steps` full steps after `warmup`,
    CUDA events with L2 flushed; roofline of the dust kernel on the FP32 pipe."""
    import torch
    from diskdyn_gb300 import abi, synth
    from diskdyn_gb300.engine import DeviceState, Engine, make_phys
    sysm = synth.dusty_ring(n_dust=16777216, n_plsml=65536, seed=synth.SEED + 4243, n_steps=500)
    ng, nd = sysm.n_grav, sysm.n_dust
    eng = Engine(local)
    eng.set_size_table(**sysm.size_table)
    phys = make_phys(**sysm.phys)
    st = DeviceState.from_numpy(sysm.state, device=f"cuda:{local}")
    del sysm.state
    MIX = abi.DDX_PREC_MIXED
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        eng.step(st, ng, sysm.dt, phys, MIX)
    torch.cuda.synchronize()
    alive0 = int((st.N[ng:] != 0).sum().item())
    rows = []
    for _ in range(steps):
        flush.zero_()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        ev[0].record(stream)
        eng.stage("massive_rk4", st, ng, sysm.dt, phys, MIX)
        ev[1].record(stream)
        eng.stage("small_rk4", st, ng, sysm.dt, phys, MIX)
        ev[2].record(stream)
        eng.stage("massive_final", st, ng, sysm.dt, phys, MIX)
        ev[3].record(stream)
        rows.append(ev)
    torch.cuda.synchronize()
    alive1 = int((st.N[ng:] != 0).sum().item())
    step_ms = statistics.mean(e[0].elapsed_time(e[3]) for e in rows)
    dust_ms = statistics.mean(e[1].elapsed_time(e[2]) for e in rows)
    alive = 0.5 * (alive0 + alive1)
    flops = FLOP_PAIR * 4.0 * alive * (ng - 1) + FLOP_STAR * 4.0 * alive
    del st
    eng.close()
    torch.cuda.empty_cache()
    return {"workload": "scale: 65,539 massive + 16,777,216 grains, mixed precision, %d steps" % steps,
            "value": (ng + alive) / (step_ms / 1e3), "unit": UNIT, "ms_per_step": step_ms,
            "dust_kernel_ms": dust_ms, "massive_ms": step_ms - dust_ms,
            "roofline": {"kernel": "dust_rk4_mixed_kernel", "bound": "fp32_pipe", "achieved": flops / (dust_ms / 1e3) / 1e12,
                         "peak": fp32_peak, "unit": "TFLOP/s", "frac": flops / (dust_ms / 1e3) / 1e12 / fp32_peak}}


def adjoint_leg(local, n_dust=262144, n_steps=2000, ckpt=100, n_plsml=0):
    """Adjoint/forward wall-time ratio on the image-loss workload: L2 loss between the
    image of the dusty-ring system (262,144 grains, 512x512, 2,000 steps; with n_plsml
    gravitating planetesimals in the massive set) and a target made by the same code with
    planet 1 at 1.2x the mass and a + 2 AU; gradients with respect to planet masses, a, e, i,
    the planetesimals' states and masses and every grain's initial state by
    checkpoint-and-recompute every ckpt steps.  Also a central finite-difference check of
    dL/dm of planet 1 (h = 1e-6 relative)."""
    import torch
    from diskdyn_gb300 import adjoint as adj
    from diskdyn_gb300.engine import Engine, make_phys, make_view

    s = adj.adjoint_system(n_dust=n_dust, xsize=512, ysize=512, n_steps=n_steps, n_plsml=n_plsml)
    eng = Engine(local)
    eng.set_size_table(**s.size_table)
    o = s.optics
    eng.set_optics(o["w"], o["in"], o["Qabs"], o["Qsca"], o["Qpfunc"], o["Td"], o["Rmin"], o["Rmax"])
    ng = s.n_grav
    dev = f"cuda:{local}"
    N = torch.tensor(s.state["N"][ng:], dtype=torch.float64, device=dev)
    ids = torch.tensor(s.state["id"][ng:], dtype=torch.int32, device=dev)
    dust0 = torch.tensor(np.stack([s.state[k][ng:] for k in ("x", "y", "z", "vx", "vy", "vz")], 1),
                         dtype=torch.float64, device=dev)
    phys, view = make_phys(**s.phys), make_view(**s.view)
    el = adj.planet_elements(s)
    plsml = torch.tensor(np.stack([s.state[k][3:ng] for k in ("x", "y", "z", "vx", "vy", "vz", "m")], 1),
                         dtype=torch.float64, device=dev).reshape(-1, 7)

    def elements(grad):
        t = {k: torch.tensor(np.asarray(v, dtype=np.float64), device=dev) for k, v in el.items()}
        if grad:
            for k in ("m", "a", "e", "i"):
                t[k].requires_grad_(True)
        return t

    def image(t, dust, pl=plsml):
        M = adj.planet_state(t["Mstar"], t["m"], t["a"], t["e"], t["i"], t["w"], t["o"], t["nu"])
        M = torch.cat([M, pl], dim=0)
        return adj.trajectory_image(eng, M, dust, N, ids, s.dt, n_steps, ckpt, phys, view, s.image_wj)

    with torch.no_grad():
        tt = elements(False)
        tt["m"][0] *= 1.2
        tt["a"][0] += 2.0
        target = image(tt, dust0)
        image(elements(False), dust0)          # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with torch.no_grad():
        img = image(elements(False), dust0)
        L0 = ((img - target) ** 2).sum().item()
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t0
    t = elements(True)
    d = dust0.clone().requires_grad_(True)
    pg = plsml.clone().requires_grad_(n_plsml > 0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    L = ((image(t, d, pg) - target) ** 2).sum()
    L.backward()
    torch.cuda.synchronize()
    t_grad = time.perf_counter() - t0
    g_m = t["m"].grad[0].item()
    base = el["m"][0]
    h = 1e-6 * base
    vals = []
    for sgn in (1.0, -1.0):
        with torch.no_grad():
            tp = elements(False)
            tp["m"][0] = base + sgn * h
            vals.append(((image(tp, dust0) - target) ** 2).sum().item())
    fd = (vals[0] - vals[1]) / (2 * h)
    eng.close()
    return {"workload": "image loss, %d massive + %d grains, %dx%d, %d steps, checkpoints every %d"
                        % (ng, n_dust, 512, 512, n_steps, ckpt),
            "forward_s": t_fwd, "forward_plus_gradient_s": t_grad, "adjoint_over_forward": t_grad / t_fwd,
            "loss": L0, "dL_dm_planet1_adjoint": g_m, "dL_dm_planet1_fd": fd,
            "fd_rel_err": abs(g_m - fd) / abs(fd) if fd != 0 else None,
            "grad_norm_a": t["a"].grad.norm().item(), "grad_norm_dust": d.grad.norm().item(),
            "grad_norm_planetesimals": pg.grad.norm().item() if n_plsml > 0 else None}


def cpu_baseline(sysm, n_sample):
    """The FP64 CPU oracle (OpenMP, every host core) on one step of a sample of the same
    workload: all massive bodies and the first n_sample grains."""
    import oracle.cpu as oc
    ng = sysm.n_grav
    n_sample = min(n_sample, sysm.n_dust)
    sub = {k: v[:ng + n_sample].copy() for k, v in sysm.state.items()}
    t0 = time.perf_counter()
    oc.step(sub, ng, sysm.dt, sysm.size_table, sysm.phys, 1)
    t = time.perf_counter() - t0
    return {"value": (ng + n_sample) / t, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": f"1 FP64 step of {ng} massive bodies + {n_sample} grains of the same workload"}


def run_reference(args, world, rank, local):
    """Reference arm: the reference's hot path on the host cores -- it has no CPU
    implementation of its own, so the oracle port (FP64, OpenMP over all cores) -- on the
    same workload, each step a bounded sample of it.  The reference's own CUDA kernels
    (compiled unmodified for sm_103a) are timed beside it on one full-size step."""
    if rank != 0:
        return
    import oracle.cpu as oc
    from diskdyn_gb300 import synth
    if args.workload == "solar":
        run_reference_solar(args, world)
        return
    sysm = synth.dusty_ring(n_dust=args.n_dust, n_plsml=args.n_plsml)
    ng = sysm.n_grav
    n_sample = min(65536, sysm.n_dust)
    sub = {k: v[:ng + n_sample].copy() for k, v in sysm.state.items()}
    for _ in range(args.warmup):
        oc.step(sub, ng, sysm.dt, sysm.size_table, sysm.phys, 1)
    t0 = time.perf_counter()
    cur = sub
    for _ in range(args.steps):
        cur = oc.step(cur, ng, sysm.dt, sysm.size_table, sysm.phys, 1)
    t = time.perf_counter() - t0
    value = (ng + n_sample) * args.steps / t
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Philox), dusty-ring configuration",
            "config": {"workload": WORKLOAD, "n_grav": ng, "n_dust_per_gpu": args.n_dust,
                       "n_planetesimals": args.n_plsml, "dt_yr": sysm.dt, "precision": "fp64"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                             "sample": f"each step: {ng} massive bodies + {n_sample} grains of the workload"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    line["sample_note"] = ("every counted body, massive or grain, takes n_grav - 1 = %d pair interactions per "
                           "stage in the sample and in the full workload alike, so the sample's rate stands for the "
                           "full workload's" % (ng - 1))
    try:
        import oracle.refk as rk
        if rk.available():
            _, ms = rk.step(sysm.state, ng, sysm.dt, sysm.size_table, sysm.phys, 1, return_ms=True)
            line["reference_cuda_gb300"] = {
                "value": (ng + sysm.n_dust) / (ms / 1e3), "unit": UNIT, "ms_per_step": ms,
                "what": "the reference's own kernels compiled unmodified for sm_103a, one full step, CUDA events"}
    except Exception as e:  # the GPU leg is informative only
        line["reference_cuda_gb300"] = {"unavailable": str(e)[:200]}
    print(json.dumps(line), flush=True)


def run_solar(args, world, rank, local):
    """Plain FP64 solar-system-like run: 1 Msun star, 8 planets (1.7e-7 to 9.5e-4 Msun,
    0.4-30 AU), 16,384 massless planetesimals at 30-50 AU, dt = 0.05 yr, 1,000 steps.  One
    timed repetition is the whole 1,000-step run through ddx_evolve (4 kernels per step),
    launched directly and replayed as a CUDA graph captured from the same call."""
    import torch
    from diskdyn_gb300 import abi, synth
    from diskdyn_gb300.engine import DeviceState, Engine, make_phys

    torch.cuda.set_device(local)
    n_dust = args.n_dust if args.n_dust != 1048576 else 16384
    sysm = synth.solar_like(n_dust=n_dust, seed=synth.SEED + 7919 * rank)
    ng, n_steps = sysm.n_grav, args.solar_steps
    eng = Engine(local)
    eng.set_size_table(**sysm.size_table)
    phys = make_phys(**sysm.phys)
    st0 = DeviceState.from_numpy(sysm.state, device=f"cuda:{local}")
    stream = torch.cuda.Stream()
    out = {}
    for prec, name in ((abi.DDX_PREC_FP64, "fp64"), (abi.DDX_PREC_MIXED, "mixed")):
        st = st0.clone()
        with torch.cuda.stream(stream):
            for _ in range(args.warmup):
                eng.evolve(st, ng, sysm.dt, 10, phys, prec, stream=stream)
        torch.cuda.synchronize()
        ms = []
        for _ in range(max(1, args.steps // 10)):
            st = st0.clone()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            eng.evolve(st, ng, sysm.dt, n_steps, phys, prec, stream=stream)
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        res = {"ms_per_run": statistics.mean(ms), "body_steps_per_s": (ng + n_dust) * n_steps / (statistics.mean(ms) / 1e3)}
        # the same 1,000 steps captured once into a CUDA graph and replayed
        try:
            st = st0.clone()
            g = torch.cuda.CUDAGraph()
            torch.cuda.synchronize()
            with torch.cuda.graph(g, stream=stream):
                eng.evolve(st, ng, sysm.dt, n_steps, phys, prec, stream=stream)
            gms = []
            for _ in range(max(1, args.steps // 10)):
                st.copy_from_({f: getattr(st0, f) for f in ("x", "y", "z", "vx", "vy", "vz", "m", "N", "id")})
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                with torch.cuda.stream(stream):
                    e0.record(stream)
                    g.replay()
                    e1.record(stream)
                torch.cuda.synchronize()
                gms.append(e0.elapsed_time(e1))
            res["graph_ms_per_run"] = statistics.mean(gms)
            res["graph_body_steps_per_s"] = (ng + n_dust) * n_steps / (statistics.mean(gms) / 1e3)
        except Exception as e:
            res["graph"] = {"unavailable": str(e)[:200]}
        out[name] = res
    best = max(out["fp64"].get("graph_body_steps_per_s", 0.0), out["fp64"]["body_steps_per_s"])
    line = {"metric": METRIC, "value": best, "unit": UNIT, "n_gpus": 1, "steps": n_steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded Philox), solar-system-like configuration",
            "config": {"workload": "solar", "n_grav": ng, "n_dust": n_dust, "dt_yr": sysm.dt, "precision": "fp64",
                       "kernels_per_step": 4, "l2": "inputs below L2; a whole 1,000-step run per timed repetition"},
            "results": out, "gpu_launches": 4 * n_steps}
    print(json.dumps(line), flush=True)


def run_reference_solar(args, world):
    """Reference arm of the solar-system run: the oracle port on all host cores over the
    whole 1,000-step run, and the reference's own CUDA kernels (sm_103a, its launch
    sequence: about 12 launches per step) over the same run."""
    import oracle.cpu as oc
    from diskdyn_gb300 import synth
    n_dust = args.n_dust if args.n_dust != 1048576 else 16384
    sysm = synth.solar_like(n_dust=n_dust)
    ng, n_steps = sysm.n_grav, args.solar_steps
    oc.step(sysm.state, ng, sysm.dt, sysm.size_table, sysm.phys, 10)
    t0 = time.perf_counter()
    oc.step(sysm.state, ng, sysm.dt, sysm.size_table, sysm.phys, n_steps)
    t = time.perf_counter() - t0
    value = (ng + n_dust) * n_steps / t
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": n_steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Philox), solar-system-like configuration",
            "config": {"workload": "solar", "n_grav": ng, "n_dust": n_dust, "dt_yr": sysm.dt, "precision": "fp64"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                             "sample": f"the whole run: {n_steps} steps of {ng} massive bodies + {n_dust} planetesimals"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    try:
        import oracle.refk as rk
        if rk.available():
            _, ms_step = rk.step(sysm.state, ng, sysm.dt, sysm.size_table, sysm.phys, n_steps, return_ms=True)
            ms = ms_step * n_steps
            line["reference_cuda_gb300"] = {
                "value": (ng + n_dust) * n_steps / (ms / 1e3), "unit": UNIT, "ms_per_run": ms,
                "what": "the reference's own kernels compiled unmodified for sm_103a, the whole run, CUDA events"}
    except Exception as e:
        line["reference_cuda_gb300"] = {"unavailable": str(e)[:200]}
    print(json.dumps(line), flush=True)


def run_imaging(args, world, rank, local):
    """Images (10 wavelengths, 1024x1024) and the 200-point SED of 4,194,304 tracers drawn
    from the solar-like dust distribution: particle-wavelengths/s and HBM GB/s."""
    import torch
    from diskdyn_gb300 import abi, synth
    from diskdyn_gb300.engine import DeviceState, Engine, make_view

    torch.cuda.set_device(local)
    n = args.n_dust if args.n_dust != 1048576 else 4194304
    s = synth.imaging(n_dust=n, seed=synth.SEED + rank)
    eng = Engine(local)
    eng.set_size_table(**s.size_table)
    o = s.optics
    eng.set_optics(o["w"], o["in"], o["Qabs"], o["Qsca"], o["Qpfunc"], o["Td"], o["Rmin"], o["Rmax"])
    st = DeviceState.from_numpy(s.state)
    view = make_view(**s.view)
    n_img = len(s.image_wj)
    F = torch.empty((n_img, s.view["xsize"], s.view["ysize"]), dtype=torch.float64, device="cuda")
    Fs = torch.empty(len(o["w"]), dtype=torch.float64, device="cuda")
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    out = {}
    results = {}
    for prec, name in ((abi.DDX_PREC_FP64, "fp64"), (abi.DDX_PREC_MIXED, "mixed")):
        for _ in range(args.warmup):
            eng.image(st, s.n_grav, view, s.image_wj, out=F, precision=prec)
            eng.sed(st, s.n_grav, view, out=Fs, precision=prec)
        ti, ts = [], []
        for _ in range(args.steps):
            flush.zero_()
            e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            e[0].record(stream)
            eng.image(st, s.n_grav, view, s.image_wj, out=F, precision=prec)
            e[1].record(stream)
            eng.sed(st, s.n_grav, view, out=Fs, precision=prec)
            e[2].record(stream)
            torch.cuda.synchronize()
            ti.append(e[0].elapsed_time(e[1]))
            ts.append(e[1].elapsed_time(e[2]))
        t_img = statistics.mean(ti) / 1e3
        t_sed = statistics.mean(ts) / 1e3
        npix = s.view["xsize"] * s.view["ysize"]
        bytes_img = n * 36 + n_img * npix * 8
        out[name] = {"image_ms": t_img * 1e3, "sed_ms": t_sed * 1e3,
                     "image_particle_wavelengths_per_s": n * n_img / t_img,
                     "sed_particle_wavelengths_per_s": n * len(o["w"]) / t_sed,
                     "image_algorithmic_GBps": bytes_img / t_img / 1e9,
                     "image_hbm_frac": bytes_img / t_img / 1e9 / measured_peaks().get("hbm_gbs", 6782.1)}
        results[name] = (F.clone(), Fs.clone())
    (F64, S64), (Fm, Sm) = results["fp64"], results["mixed"]
    # the mixed images again with the tracers stored in pixel order: adjacent lanes then share
    # pixels and the warp-aggregated scatter issues one atomic per run of lanes on a pixel
    pix, _ = eng.pixels(st, s.n_grav, view)
    order = torch.argsort(torch.where(pix < 0, torch.iinfo(torch.int32).max, pix).long(), stable=True)
    for f in ("x", "y", "z", "vx", "vy", "vz", "m", "N", "id"):
        a = getattr(st, f)
        a[s.n_grav:] = a[s.n_grav:][order]
    for _ in range(args.warmup):
        eng.image(st, s.n_grav, view, s.image_wj, out=F, precision=abi.DDX_PREC_MIXED)
    tp = []
    for _ in range(args.steps):
        flush.zero_()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        e[0].record(stream)
        eng.image(st, s.n_grav, view, s.image_wj, out=F, precision=abi.DDX_PREC_MIXED)
        e[1].record(stream)
        torch.cuda.synchronize()
        tp.append(e[0].elapsed_time(e[1]))
    out["mixed"]["image_ms_tracers_in_pixel_order"] = statistics.mean(tp)
    out["mixed"]["pixel_order_image_rel_diff_max"] = float(((F - Fm).abs()[F64 != 0] / Fm[F64 != 0].abs()).max().item())
    # and in a random order (seeded), where adjacent lanes almost never share a pixel
    perm = torch.randperm(n, generator=torch.Generator(device="cuda").manual_seed(11), device="cuda")
    for f in ("x", "y", "z", "vx", "vy", "vz", "m", "N", "id"):
        a = getattr(st, f)
        a[s.n_grav:] = a[s.n_grav:][perm]
    for _ in range(args.warmup):
        eng.image(st, s.n_grav, view, s.image_wj, out=F, precision=abi.DDX_PREC_MIXED)
    tr = []
    for _ in range(args.steps):
        flush.zero_()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        e[0].record(stream)
        eng.image(st, s.n_grav, view, s.image_wj, out=F, precision=abi.DDX_PREC_MIXED)
        e[1].record(stream)
        torch.cuda.synchronize()
        tr.append(e[0].elapsed_time(e[1]))
    out["mixed"]["image_ms_tracers_in_random_order"] = statistics.mean(tr)
    lit = F64 != 0
    out["mixed_vs_fp64"] = {
        "lit_pixels_identical": bool(torch.equal(lit, Fm != 0)),
        "image_pixel_rel_err_max": float(((Fm - F64).abs()[lit] / F64[lit].abs()).max().item()),
        "image_total_flux_rel_err_max": float(((Fm.sum((1, 2)) - F64.sum((1, 2))).abs() / F64.sum((1, 2))).max().item()),
        "sed_rel_err_max": float(((Sm - S64).abs() / S64.abs()).max().item()),
        "image_speedup": out["fp64"]["image_ms"] / out["mixed"]["image_ms"],
        "sed_speedup": out["fp64"]["sed_ms"] / out["mixed"]["sed_ms"]}
    # the dust-temperature table of the same optics (Grid::calculate_dust_temp): GPU vs the
    # oracle on all host cores
    import oracle.cpu as oc
    eng.dust_temp(o["w"], o["in"], o["Qabs"], s.view["dist"], 60.0)
    t0 = time.perf_counter()
    Td_g, rmin_g, _ = eng.dust_temp(o["w"], o["in"], o["Qabs"], s.view["dist"], 60.0)
    t_g = time.perf_counter() - t0
    t0 = time.perf_counter()
    Td_c, rmin_c, _ = oc.dust_temp(o["w"], o["in"], o["Qabs"], s.view["dist"], 60.0)
    t_c = time.perf_counter() - t0
    out["dust_temp"] = {"what": "Td table, %d bins x %d wavelengths x 1,999 temperatures" % o["Qabs"].shape,
                        "gpu_ms": t_g * 1e3, "cpu_oracle_ms": t_c * 1e3, "cpu_cores": os.cpu_count(),
                        "max_rel_diff": float(np.max(np.abs(Td_g / Td_c - 1.0))),
                        "rmin_rel_diff": abs(rmin_g / rmin_c - 1.0)}
    # the size grid and its tables (interpolate_dust_to_grid + calculate_beta) of a table
    # file of Mie size: 40 radii x 200 wavelengths x 181 angles onto 218 bins
    w_m, in_m, tab = synth.mie_table()
    grid = dict(n_grid=218, amin=1.3e-7, amax=float(tab["s"][-1]), dmax=float(tab["s"][-1]), kqe=3e-3, radQ=1,
                SWQ=1, rho=3300.0, dist=7.7 * synth.PC, mstar=2.1 * 4 * np.pi ** 2, mloss=1e-13, vsw=5e5)
    eng.dust_grid(w_m, in_m, tab, **grid)
    t0 = time.perf_counter()
    g_out = eng.dust_grid(w_m, in_m, tab, **grid)
    t_g = time.perf_counter() - t0
    t0 = time.perf_counter()
    c_out = oc.dust_grid(w_m, in_m, tab, **grid)
    t_c = time.perf_counter() - t0
    out["dust_grid"] = {"what": "218 bins from a 40 x 200 x 181 table, host arrays in and out",
                        "gpu_ms": t_g * 1e3, "cpu_oracle_ms": t_c * 1e3, "cpu_cores": 1,
                        "Qpfunc_max_rel_diff": float(np.max(np.abs(g_out["Qpfunc"] / c_out["Qpfunc"] - 1.0))),
                        "beta_identical": bool(np.array_equal(g_out["beta"], c_out["beta"]))}
    line = {"metric": "imaging particle-wavelengths/s", "workload": "imaging", "n_particles": n,
            "n_img": n_img, "n_wav": len(o["w"]), "image": [s.view["xsize"], s.view["ysize"]],
            "results": out, "l2": "flushed between timed calls"}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_setup(args, world, rank, local):
    """Start-of-run set-up of a 16.8M-tracer A-star debris system (synth.setup_param_text,
    the size of the largest single-GPU configuration): the size grid and its optical, beta
    and beta_sw tables from a 40 x 200 x 181 Mie table (ddx_dust_grid), the temperature
    table (ddx_dust_temp) and every body drawn into device memory (ddx_setup_device).
    Against the host path the reference runs: the oracle's restatement of its table
    set-up (one core; the temperature table on all cores) and its generator with ran3
    (ddx_setup_host, the reference's bodies to the bit) on a 1/16 sample, scaled."""
    import tempfile
    import torch
    import oracle.cpu as oc
    from diskdyn_gb300 import formats, synth
    from diskdyn_gb300.engine import Engine

    torch.cuda.set_device(local)
    eng = Engine(local)
    w, influx, tab = synth.mie_table()
    dmin, dmax = float(tab["s"][0]), float(tab["s"][-1])

    def param(n_grains, n_grav):
        with tempfile.TemporaryDirectory() as td:
            pf = Path(td) / "system.param"
            pf.write_text(synth.setup_param_text(n_grains=n_grains, n_gravitating=n_grav))
            p = formats.read_param_struct(pf)
        formats.param_grid(p, dmin, dmax)
        return p

    p = param(16777216, 4096)
    grid = dict(n_grid=p.n_grid, amin=p.amin, amax=p.amax, dmax=dmax, kqe=p.kqe, radQ=p.radQ, SWQ=p.SWQ,
                rho=p.rho, dist=p.dist, mstar=p.planets[0].m, mloss=p.mloss, vsw=p.vsw)

    def gpu_setup():
        g = eng.dust_grid(w, influx, tab, **grid)
        td = eng.dust_temp(w, influx, g["Qabs"], p.dist, 300.0)
        st, run = eng.setup_device(p, dmin, dmax, g["beta"], seed=20241203)
        torch.cuda.synchronize()
        return g, td, st, run

    for _ in range(max(1, args.warmup)):
        g, td, st, run = gpu_setup()
        del st
    reps = []
    for _ in range(3):
        t0 = time.perf_counter()
        g, td, st, run = gpu_setup()
        reps.append(time.perf_counter() - t0)
        del st
    # the generation alone, device-timed
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    st, run = eng.setup_device(p, dmin, dmax, g["beta"], seed=20241203)
    e1.record()
    torch.cuda.synchronize()
    gen_ms = e0.elapsed_time(e1)
    finite = bool(torch.isfinite(st.x).all().item() and torch.isfinite(st.vz).all().item())
    n_all = run.n_all
    del st
    # host path: table set-up (oracle, one core), temperature table (oracle, all cores),
    # generation with ran3 on a 1/16 sample
    t0 = time.perf_counter()
    c = oc.dust_grid(w, influx, tab, **grid)
    t_grid = time.perf_counter() - t0
    t0 = time.perf_counter()
    oc.dust_temp(w, influx, c["Qabs"], p.dist, 300.0)
    t_temp = time.perf_counter() - t0
    ps = param(16777216 // 16, 4096 // 16)
    t0 = time.perf_counter()
    hs, hrun = formats.setup_host(ps, dmin, dmax, c["beta"])
    t_gen = (time.perf_counter() - t0) * n_all / hrun.n_all
    line = {"metric": "set-up time (s)", "workload": "setup", "n_all": n_all, "n_mass": run.n_mass,
            "n_grid": p.n_grid, "table": "40 sizes x 200 wavelengths x 181 angles",
            "gpu_s": float(np.median(reps)), "gpu_generation_ms": gen_ms,
            "gpu_bodies_per_s": n_all / (gen_ms * 1e-3), "state_finite": finite,
            "host_s": t_grid + t_temp + t_gen,
            "host_parts_s": {"dust_grid_1core": t_grid, "dust_temp_all_cores": t_temp, "ran3_generation": t_gen},
            "host_sample": f"generation timed on {hrun.n_all} bodies and scaled to {n_all}",
            "cpu_cores": os.cpu_count(), "higher_is_better": False}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_cadence(args, world, rank, local):
    """A whole run with outputs (ddx_run): the dusty ring with 256 planetesimals and 262,144
    grains, mixed precision, 200 steps; SED (200 wavelengths) every 5 steps, two 512x512
    images every 10, the state every 50.  Against the same run made call by call with a
    host synchronisation and a host copy at every output, as the reference's evolve loop
    makes them (there per wavelength)."""
    import torch
    from diskdyn_gb300 import abi, synth
    from diskdyn_gb300.engine import DeviceState, Engine, make_phys, make_view

    torch.cuda.set_device(local)
    s = synth.dusty_ring(n_dust=262144, n_plsml=256, seed=synth.SEED + rank, n_steps=300)
    synth.ring_imaging(s, 512, 512)
    eng = Engine(local)
    eng.set_size_table(**s.size_table)
    o = s.optics
    eng.set_optics(o["w"], o["in"], o["Qabs"], o["Qsca"], o["Qpfunc"], o["Td"], o["Rmin"], o["Rmax"])
    phys, view, wj, ng, dt = make_phys(**s.phys), make_view(**s.view), s.image_wj, s.n_grav, s.dt
    n_steps = 200
    cad = dict(t_write=50 * dt, t_fits=10 * dt, t_sed=5 * dt, t_end=n_steps * dt)
    MIX = abi.DDX_PREC_MIXED
    counts = {}

    def on(out):
        counts[out["kind"]] = counts.get(out["kind"], 0) + 1
        return False

    def fused():
        st = DeviceState.from_numpy(s.state)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eng.run(st, ng, dt, phys, view, wj, cad, on, precision=MIX)
        return time.perf_counter() - t0

    def call_by_call():
        from diskdyn_gb300 import run as runmod
        st = DeviceState.from_numpy(s.state)
        h, m = runmod.schedule(cad, dt)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(len(h)):
            eng.step(st, ng, float(h[k]), phys, MIX)
            if m[k] & (1 << abi.DDX_OUT_SED):
                eng.sed(st, ng, view, precision=MIX).cpu()
            if m[k] & (1 << abi.DDX_OUT_IMAGES):
                eng.image(st, ng, view, wj, precision=MIX).cpu()
            if m[k] & (1 << abi.DDX_OUT_STATE):
                for f in ("x", "y", "z", "vx", "vy", "vz", "N", "m", "id"):
                    getattr(st, f).cpu()
        torch.cuda.synchronize()
        return time.perf_counter() - t0

    fused(), call_by_call()
    counts.clear()
    t_f = min(fused() for _ in range(3))
    per_run = {k: v // 3 for k, v in counts.items()}
    t_c = min(call_by_call() for _ in range(3))
    line = {"metric": "run time with outputs (s)", "workload": "cadence", "n_grav": ng, "n_dust": s.n_dust,
            "steps": n_steps, "precision": "mixed",
            "outputs_per_run": {"sed": per_run.get(abi.DDX_OUT_SED, 0), "images": per_run.get(abi.DDX_OUT_IMAGES, 0),
                                "state": per_run.get(abi.DDX_OUT_STATE, 0)},
            "ddx_run_s": t_f, "call_by_call_synchronous_s": t_c, "speedup": t_c / t_f, "higher_is_better": False}
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local = dist_setup(args)
    if args.workload == "setup":
        run_setup(args, world, rank, local)
        return
    if args.workload == "cadence":
        run_cadence(args, world, rank, local)
        return
    if args.workload == "imaging":
        run_imaging(args, world, rank, local)
        return
    if args.workload == "scale":
        run_scale(args, world, rank, local)
        return
    if args.workload == "accuracy":
        run_accuracy(args, world, rank, local)
        return
    if args.workload == "solar" and args.impl == "ours":
        run_solar(args, world, rank, local)
        return
    if args.impl == "reference":
        run_reference(args, world, rank, local)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
