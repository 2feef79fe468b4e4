"""Multi-region grids on the GPU (qsf_gb300.multigrid; the reference's multigrid.h).

Against the reference's own multi-region runs (tests/golden/mg{1,2,3}.npz: every
region's final wavefunction and the main region's .dat rows, written with one
process per region) and against the oracle on a larger seeded case.  Bar: relative
L2 <= 1e-10 per region, rows within 1e-9.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests import cases as C

pytestmark = pytest.mark.gpu

TOL_PSI = 1e-10
TOL_ROWS = 1e-9


def _coupling(p, dim):
    import qsf_gb300 as Q
    pulse = Q.Pulse(field=p["F0"], omega=p["omega"], ncycles=p["ncycles"],
                    phase_in_pi_units=p.get("phase", 0.0), delay_in_cycles=p.get("delay", 0.0))
    return Q.Coupling(Q.GAUGE_VELOCITY, [Q.Field(C.field_axis(dim), [pulse])])


def _gpu_run(p, dim, psi0):
    import qsf_gb300 as Q
    from qsf_gb300.multigrid import MultiGrid, MultiRegionPropagator
    mg = MultiGrid(dim, int(p["n"]), float(p["dx"]), int(p["nCAP"]), potential=Q.POT_EBERLY,
                   Ncharge=p["Ncharge"], Echarge=p["Echarge"], Nsoft=p["Nsoft"], Esoft=p["Esoft"],
                   gauge=Q.GAUGE_VELOCITY, n_fields=1)
    mg.main.upload(psi0)
    prop = MultiRegionPropagator(p["re_dt"], mg, _coupling(p, dim), C.MG_OUTPUTS)
    rows = prop.run()
    psis = [g.download() for g in mg.regions]
    mg.close()
    return psis, rows


# *_bs: axis lengths with a prime factor above 5 (130, 34, 14): Bluestein transforms
@pytest.mark.parametrize("name", ["mg1", "mg2", "mg3", "mg1_bs", "mg2_bs", "mg3_bs"])
def test_multigrid_matches_reference(name):
    z = C.load(name)
    p, dim = z["params"], int(z["dim"])
    psis, rows = _gpu_run(p, dim, z["psi_in"])
    got = np.array([C.mg_dat_row(r) for r in rows])
    assert got.shape == z["re_rows"].shape
    np.testing.assert_allclose(got, z["re_rows"], rtol=TOL_ROWS, atol=1e-12)
    for r in range(2 ** dim):
        assert C.rel_l2(psis[r], z["psi_r%d" % r]) < TOL_PSI, r


def test_multigrid_2d_matches_oracle_larger():
    p = dict(n=128, dx=0.3, nCAP=13, Ncharge=2.0, Echarge=-1.0, Nsoft=1.0, Esoft=1.0, F0=0.2, omega=1.2,
             ncycles=1, re_dt=0.05)
    rng = np.random.default_rng(11)
    x = (np.arange(128) - 63.5) * 0.3
    env = np.exp(-(x[:, None] ** 2 + x[None, :] ** 2) / 300.0)
    psi0 = env * (rng.standard_normal((128, 128)) + 1j * rng.standard_normal((128, 128)))
    gs, orows = C.oracle_mg(p, 2, psi0)
    psis, rows = _gpu_run(p, 2, psi0)
    np.testing.assert_allclose(np.array([C.mg_dat_row(r) for r in rows]),
                               np.array([C.mg_dat_row(r) for r in orows]), rtol=TOL_ROWS, atol=1e-12)
    for r in range(4):
        assert np.linalg.norm(gs[r].psi) > 0
        assert C.rel_l2(psis[r], gs[r].psi) < TOL_PSI, r


def test_multigrid_3d_128_matches_oracle():
    """The 3D multi-region grid at 128^3 (regions NO ... XYZ, three electrons, velocity
    gauge, transfers and masks every step) against the oracle over a short pulse."""
    n = 128
    p = dict(n=n, dx=0.4, nCAP=13, Ncharge=3.0, Echarge=-1.0, Nsoft=1.0, Esoft=1.0, F0=0.3, omega=20.0,
             ncycles=1, re_dt=0.05)
    rng = np.random.default_rng(13)
    x = (np.arange(n) - (n - 1) / 2.0) * p["dx"]
    r2 = x[:, None, None] ** 2 + x[None, :, None] ** 2 + x[None, None, :] ** 2
    env = np.exp(-r2 / (2 * (0.3 * n * p["dx"]) ** 2))
    psi0 = env * (rng.standard_normal((n,) * 3) + 1j * rng.standard_normal((n,) * 3))
    gs, orows = C.oracle_mg(p, 3, psi0)
    psis, rows = _gpu_run(p, 3, psi0)
    assert len(rows) == len(orows) > 5
    np.testing.assert_allclose(np.array([C.mg_dat_row(r) for r in rows]),
                               np.array([C.mg_dat_row(r) for r in orows]), rtol=TOL_ROWS, atol=1e-12)
    for r in range(8):
        assert np.linalg.norm(gs[r].psi) > 0, r
        assert C.rel_l2(psis[r], gs[r].psi) < TOL_PSI, r


def test_region_rules():
    import qsf_gb300 as Q
    from qsf_gb300.multigrid import MultiGrid
    mg = MultiGrid(2, 32, 0.4, 4)
    x, y, xy = mg.regions[1], mg.regions[2], mg.regions[3]
    with pytest.raises(Q.QsfError):   # XY receives along y from X, not from the main region
        xy.region_transfer(mg.main, 1, 2)
    with pytest.raises(Q.QsfError):   # wrong group
        xy.region_transfer(x, 1, 1)
    with pytest.raises(Q.QsfError):   # regions with free axes do not take fused steps
        x.step(Q.MODE_RE, 0.05, 1, np.zeros((1, 3)))
    with pytest.raises(Q.QsfError):   # the margins may not overlap
        Q.Grid(2, 32, 0.4, nCAP=17, multi_region=True)
    xy.region_transfer(x, 1, 2)
    xy.region_transfer(y, 0, 2)
    mg.synchronize()
    mg.close()
