"""ddx_dust_temp (Grid::calculate_dust_temp, src/grid.cu:754-834) on the GPU against the
oracle's restatement of the reference's host loop.  Tolerances: the Planck sums use the
CUDA math library's exp, log and pow instead of libm, so the tables agree to rounding:
1e-12 relative for the temperatures, 1e-13 for the grid limits."""
import numpy as np
import pytest

import oracle.cpu as oc
from diskdyn_gb300 import synth

pytestmark = pytest.mark.gpu


def nongrey(n_grid=24, n_wav=120):
    """Q_abs = 1 - exp(-2 pi s / lambda): grains absorb less at wavelengths beyond their size,
    so the bins have different equilibrium temperatures (and sublimation radii)."""
    opt = synth.hg_optics(n_grid=n_grid, n_theta=5, n_wav=n_wav, L=8.7, Teff=7500.0, Rstar=2.0 * synth.RSun)
    s, w = opt["size"], opt["w"]
    opt["Qabs"] = 1.0 - np.exp(-2 * np.pi * s[:, None] / w[None, :])
    return opt


@pytest.mark.parametrize("case", ["grey", "nongrey"])
def test_dust_temp_matches_oracle(engine, case):
    opt = synth.hg_optics(n_grid=16, n_wav=200) if case == "grey" else nongrey()
    dist = 10 * synth.PC
    for rmax in (50.0, 400.0):
        Td, rmin, rmax_out = engine.dust_temp(opt["w"], opt["in"], opt["Qabs"], dist, rmax)
        To, rmin_o, rmax_o = oc.dust_temp(opt["w"], opt["in"], opt["Qabs"], dist, rmax)
        assert rmax_out == rmax_o == 2 * rmax
        assert rmin == pytest.approx(rmin_o, rel=1e-13)
        assert np.isfinite(Td).all()
        np.testing.assert_allclose(Td, To, rtol=1e-12)
