"""The C ABI library: builds, loads, exports every symbol the header declares, and
rejects bad arguments with status codes before touching a GPU."""
import ctypes as C
import re

from conftest import ROOT


def header_functions():
    names = set()
    for h in ("diskdyn_gb300.h", "diskdyn_gb300_io.h", "diskdyn_gb300_setup.h", "diskdyn_gb300_run.h"):
        txt = (ROOT / "include" / h).read_text()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names |= set(re.findall(r"\b(ddx_\w+)\s*\(", txt))
    return sorted(names)


def test_header_declares_core_entry_points():
    fns = header_functions()
    for f in ("ddx_create", "ddx_destroy", "ddx_set_size_table", "ddx_set_optics", "ddx_step",
              "ddx_evolve", "ddx_image", "ddx_sed", "ddx_status_string", "ddx_abi_version"):
        assert f in fns


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(str(built_lib))
    missing = [f for f in header_functions() if not hasattr(lib, f)]
    assert not missing, missing


def test_python_binding_covers_header(built_lib):
    from diskdyn_gb300 import abi
    bound = {name for name, _, _ in abi.SIGNATURES}
    assert set(header_functions()) <= bound


def test_status_strings_and_version(built_lib):
    from diskdyn_gb300 import abi
    lib = abi.load()
    assert lib.ddx_abi_version() == 4
    assert lib.ddx_status_string(0) == b"ok"
    assert lib.ddx_status_string(5) == b"size beyond limit"
    assert lib.ddx_status_string(99) == b"unknown status"


def test_argument_errors_without_gpu(built_lib):
    from diskdyn_gb300 import abi
    lib = abi.load()
    st = abi.State()
    ph = abi.Phys()
    assert lib.ddx_create(None, 0) == abi.DDXError(1, "").status
    assert lib.ddx_destroy(None) == 1
    assert lib.ddx_step(None, C.byref(st), 1, 0, 0.1, C.byref(ph), 0, 0, None) == 1
    assert lib.ddx_set_size_table(None, 1, None, None, None, None) == 1
    assert lib.ddx_image(None, C.byref(st), 1, 0, None, None, 1, None, 0, None) == 1
    assert lib.ddx_sed(None, C.byref(st), 1, 0, None, None, 0, 0, None) == 1
    assert lib.ddx_set_near_radius(None, C.c_double(1e-3)) == 1
    assert lib.ddx_set_compensated_radius(None, C.c_double(0.5)) == 1
    assert lib.ddx_noalloc_sync_status(-1, None) == 1
    assert lib.ddx_debug_noalloc_lose_tile_copy(0, -1, 1000) == 1
    assert lib.ddx_debug_noalloc_lose_tile_copy(0, 0, 0) == 1


def test_argument_errors_of_the_setup_and_run_calls_without_gpu(built_lib):
    """The set-up, run and host-buffer calls check their arguments before any CUDA call."""
    from diskdyn_gb300 import abi, formats
    lib = abi.load()
    st = abi.State()
    ph = abi.Phys()
    vw = abi.View()
    cad = abi.Cadence(t_write=1.0, t_fits=1.0, t_sed=1.0, t_end=2.0)
    hs = formats.HostState()
    t = abi.OpticalTable()
    g = abi.GridSetup()
    lum, bsc = C.c_double(), C.c_double()
    assert lib.ddx_dust_grid(None, 2, None, None, C.byref(t), C.byref(g), C.byref(t), None, None, None,
                             C.byref(lum), C.byref(bsc), None) == 1
    assert lib.ddx_setup_device(None, None, 1e-7, 1e-4, None, 1, C.byref(st), 0, None, None) == 1
    assert lib.ddx_step_host(None, C.byref(hs), C.byref(hs), C.byref(st), 1, 0, 0.1, C.byref(ph), 1, 0, None) == 1
    assert lib.ddx_run(None, C.byref(st), 1, 0, 0.1, C.byref(ph), 1, 0, C.byref(vw), None, 0, C.byref(cad),
                       abi.OUTPUT_FN(lambda u, o: 0), None, None) == 1
    # host-only calls: bad sizes
    n = C.c_longlong()
    bad = abi.Cadence(t_write=0.0, t_fits=1.0, t_sed=1.0, t_end=2.0)
    assert lib.ddx_schedule(C.byref(bad), 0.1, 0, None, None, C.byref(n)) == 1
    assert lib.ddx_schedule(C.byref(cad), -1.0, 0, None, None, C.byref(n)) == 1
    assert lib.ddx_stellar_grid(1, None, 2, None, None, 0, None, None, None) == 1
    assert lib.ddx_param_grid(None, 1e-7, 1e-4) == 1


def test_oracle_builds_and_loads():
    import oracle.cpu as oc
    assert oc.lib() is not None
