"""The cos^(1/8) mask absorber on the GPU (QSF_ABS_COS8) against the oracle: the
factor of evolve<X>, fused multi-step calls in 1D (length gauge, BOX flux; the 1D
plain configuration's absorber on the outer 10% of each side) and 2D (velocity gauge,
ZOA_FLUX_2D), and the descriptor checks.  Bar: relative L2 <= 1e-10 for psi, 1e-9 for
the observables."""
import math

import numpy as np
import pytest

from tests import cases as C

pytestmark = pytest.mark.gpu

PSI_TOL = 1e-10
OBS_TOL = 1e-9


@pytest.fixture(scope="module")
def Q():
    import qsf_gb300
    return qsf_gb300


def test_cos8_factor_matches_oracle(Q):
    from oracle import oracle as O
    for dim, n, ncap in ((1, 256, 26), (2, 64, 7)):
        g = Q.Grid(dim, n, 0.3, nCAP=ncap, potential=Q.POT_NONE, absorber=Q.ABS_COS8, mask_dt=0.05)
        og = O.Grid(dim, n, 0.3, nCAP=ncap, pot=O.POT_NONE)
        og.set_absorber(O.ABS_COS8, 0.05)
        psi = np.ones((n,) * dim, dtype=np.complex128)
        g.upload(psi)
        og.psi[...] = psi
        for _ in range(2):
            g.evolve(Q.MODE_RE, Q.REP_X, 0.025)
            og.evolve(O.MODE_RE, O.REP_X, 0.025)
        got = g.download()
        np.testing.assert_allclose(got, og.psi, rtol=1e-14, atol=1e-16)
        edge = math.cos(0.5 * math.pi) ** 0.125
        assert abs(got.flat[0] - edge ** dim) < 1e-15


def _noise_psi(dim, n, dx, seed):
    rng = np.random.default_rng(seed)
    x = (np.arange(n) - (n - 1) / 2.0) * dx
    r2 = x ** 2
    for _ in range(dim - 1):
        r2 = np.add.outer(r2, x ** 2)
    env = np.exp(-r2 / (2 * (0.4 * n * dx) ** 2))  # reaches into the margins
    shape = (n,) * dim
    return env * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


@pytest.mark.parametrize("case", ["1d_lg", "2d_vg"])
def test_cos8_fused_steps_match_oracle(Q, case):
    from oracle import oracle as O
    from qsf_gb300.propagator import coupling_schedule
    if case == "1d_lg":
        dim, n, dx, dt, steps = 1, 1024, 0.2, 0.05, 40
        og_gauge, q_gauge, axis = O.GAUGE_LENGTH, Q.GAUGE_LENGTH, 1
        ob, qb, box = ["BOX"], ["BOX"], 400
        charge = 1.0
    else:
        dim, n, dx, dt, steps = 2, 256, 0.3, 0.05, 20
        og_gauge, q_gauge, axis = O.GAUGE_VELOCITY, Q.GAUGE_VELOCITY, 3
        ob, qb, box = O.ZOA_FLUX_2D, Q.ZOA_FLUX_2D, 0
        charge = 2.0
    ncap = n // 10
    psi0 = _noise_psi(dim, n, dx, 100 + dim)
    pulse = dict(field=0.08, omega=0.35, ncycles=2)
    O.set_border_nodes(25, 14, 10, 40)
    oc = O.Coupling(og_gauge, [O.Field(axis, [O.Pulse(**pulse)])])
    og = O.Grid(dim, n, dx, nCAP=ncap, pot=O.POT_EBERLY, Ncharge=charge, coupling=oc)
    og.set_absorber(O.ABS_COS8, dt)
    og.psi[...] = psi0
    prop = O.Propagator(O.MODE_RE, dt, 0, og, ["norm", "epot", ("flux", ob, box)])
    orows = []
    for _ in range(steps):
        prop.make_step()
        prop.compute_each()
        r = prop.rows[-1]
        orows.append([r["norm"], r["epot"]] + list(r["flux"]))
    g = Q.Grid(dim, n, dx, nCAP=ncap, potential=Q.POT_EBERLY, Ncharge=charge, gauge=q_gauge, n_fields=1,
               absorber=Q.ABS_COS8, mask_dt=dt)
    g.upload(psi0)
    c = Q.Coupling(q_gauge, [Q.Field(axis, [Q.Pulse(**pulse)])])
    rows, _ = coupling_schedule(c, dt, steps)
    out, done = g.step(Q.MODE_RE, dt, steps, rows, obs=Q.OBS_NORM | Q.OBS_EPOT, borders=qb, box_size=box)
    assert done == steps
    got = np.concatenate([out[:, :2], out[:, 3:]], axis=1)
    orows = np.array(orows)
    np.testing.assert_allclose(got, orows, rtol=OBS_TOL, atol=1e-12 * float(np.max(np.abs(orows))))
    assert C.rel_l2(g.download(), og.psi) < PSI_TOL
    # the mask did act: the norm fell
    assert orows[-1, 0] < orows[0, 0] * (1 - 1e-6)


def test_cos8_descriptor_checks(Q):
    with pytest.raises(Q.QsfError):
        Q.Grid(1, 256, 0.2, nCAP=26, absorber=Q.ABS_COS8, mask_dt=0.0)
    with pytest.raises(Q.QsfError):
        Q.Grid(1, 256, 0.2, nCAP=0, absorber=Q.ABS_COS8, mask_dt=0.05)
    with pytest.raises(Q.QsfError):
        Q.Grid(2, 64, 0.3, nCAP=6, absorber=Q.ABS_COS8, mask_dt=0.05, multi_region=True)
    with pytest.raises(Q.QsfError):
        Q.Grid(1, 256, 0.2, nCAP=26, absorber=7, mask_dt=0.05)
