"""1D lines above 8192 points (up to 16384, the long end of the served 1D sizes), held
by a cluster pair of CTAs: transforms against numpy, a full real-time run against the
oracle, and batch membership."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import cases as C

pytestmark = pytest.mark.gpu

LONG = [10240, 12288, 16384]


@pytest.mark.parametrize("n", LONG)
def test_long_line_fft_matches_numpy(n):
    import qsf_gb300 as Q
    rng = np.random.default_rng(n)
    psi = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    g = Q.Grid(1, n, 0.05)
    g.upload(psi)
    g.fourier(Q.REP_P)
    assert C.rel_l2(g.download(), np.fft.fft(psi)) < 1e-14 * np.log2(n)
    g.fourier(Q.REP_X)
    assert C.rel_l2(g.download(), psi) < 1e-14 * np.log2(n)
    g.close()


def _params(n):
    return dict(n=n, dx=0.05, nCAP=n // 10, Ncharge=1.0, Echarge=-1.0, Nsoft=1.0, Esoft=1.0, F0=0.05, omega=2.0,
                ncycles=1.0, phase=0.0, re_dt=0.05, box=n // 3)


@pytest.mark.parametrize("n,lg", [(16384, 0), (12288, 1)])
def test_long_line_real_time_run_matches_oracle(n, lg):
    import qsf_gb300 as Q
    p = _params(n)
    p["lg"] = lg
    C.set_borders(p)
    x = (np.arange(n) - (n - 1) / 2.0) * p["dx"]
    psi0 = np.exp(-0.5 * x * x).astype(np.complex128)
    psi0 /= np.sqrt(np.sum(np.abs(psi0) ** 2) * p["dx"])
    og, orows = C.oracle_re(p, 1, psi0)
    g, rows = C.gpu_re(p, 1, psi0)
    assert C.rel_l2(g.download(), og.psi) < 1e-10
    got = np.array([C.re_dat_row(r, 1) for r in rows])
    ref = np.array([C.re_dat_row(r, 1) for r in orows])
    assert got.shape == ref.shape
    np.testing.assert_allclose(got[:, 2:], ref[:, 2:], rtol=1e-9, atol=1e-12)
    g.close()
