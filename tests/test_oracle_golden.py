"""Pin the CPU oracle (oracle/qsf_oracle.c + oracle/oracle.py) to the reference.

The fixtures in tests/golden/ were written by the reference's own implementation
(tests/golden/make_golden.py runs oracle/_ref/qsf_ref).  Every primitive and every
full IM/RE run of the oracle must agree with them to near machine precision.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests import cases as C

TIGHT = 1e-12  # relative; both sides are FP64 on the same CPU


def _prim_grid(p, dim, gauge):
    c = O.Coupling(gauge, [O.Field(7, [O.Pulse(field=p["F0"], omega=1.0, ncycles=100.0, shape=O.PULSE_CONST)])])
    return C.oracle_grid(p, dim, c)


@pytest.mark.parametrize("name", ["prim2d", "prim3d", "prim2d_bs", "prim3d_bs"])
def test_primitives_match_reference(name):
    z = C.load(name)
    p, dim = z["params"], int(z["dim"])
    C.set_borders(p)
    lg = _prim_grid(p, dim, O.GAUGE_LENGTH)
    vg = _prim_grid(p, dim, O.GAUGE_VELOCITY)
    lg.psi[...] = z["psi_in"]
    vg.psi[...] = z["psi_in"]
    s = z["scalars"]
    assert lg.average(O.REP_X, O.OP_IDENTITY) == pytest.approx(s[0], rel=TIGHT)
    assert lg.average(O.REP_X, O.OP_POTENTIAL) == pytest.approx(s[1], rel=TIGHT)
    curr = lg.current_map(None)
    names = ["S2CAP", "D2CAP", "N2S", "N2D", "S2D"]
    names += ["N2D_SYM", "N2D_ASYM", "S2D_SYM", "S2D_ASYM"] if dim == 2 else ["N2T", "S2T", "D2T", "T2CAP"]
    fl = [lg.flux(curr, "BOX", 3)] + [lg.flux(curr, b) for b in names]
    np.testing.assert_allclose(fl, s[2:2 + len(fl)], rtol=1e-12, atol=1e-14)
    # length gauge: E = F0 on every axis at t = 0.5
    lg.coupling.precalc(0.5)
    E = lg.coupling.vector(dim)
    lg.evolve(O.MODE_RE, O.REP_X, p["delta"], E)
    assert C.rel_l2(lg.psi, z["psi_xre"]) < TIGHT
    lg.evolve(O.MODE_IM, O.REP_X, p["delta"], E)
    assert C.rel_l2(lg.psi, z["psi_xim"]) < TIGHT
    lg.fourier(O.REP_P)
    # the reference stores P space with axes 0 and 1 transposed
    assert C.rel_l2(np.swapaxes(lg.psi, 0, 1), z["psi_p"]) < TIGHT
    assert lg.average(O.REP_P, O.OP_KINETIC) == pytest.approx(s[-1], rel=TIGHT)
    lg.fourier(O.REP_X)
    assert C.rel_l2(lg.psi, z["psi_back"]) < TIGHT
    # velocity gauge P evolution, A = -F0 after precalc(0), precalc(1)
    vg.fourier(O.REP_P)
    vg.coupling.precalc(0.0)
    vg.coupling.precalc(1.0)
    A = vg.coupling.vector(dim)
    vg.evolve(O.MODE_RE, O.REP_P, p["delta"], A)
    vg.evolve(O.MODE_IM, O.REP_P, p["delta"] * 0.25, A)
    vg.fourier(O.REP_X)
    assert C.rel_l2(vg.psi, z["psi_pvg"]) < TIGHT
    vg.normalize()
    assert C.rel_l2(vg.psi, z["psi_norm"]) < TIGHT


# *_bs: axis lengths with a prime factor above 5 (the reference's FFTW plans take any n)
@pytest.mark.parametrize("name", ["c1_vg", "c1_lg", "c2_vg", "c3_lg", "c1_bs", "c2_bs", "c3_bs"])
def test_runs_match_reference(name):
    z = C.load(name)
    p, dim = z["params"], int(z["dim"])
    C.set_borders(p)
    g0 = C.oracle_grid(p, dim, O.Coupling(O.GAUGE_VELOCITY))
    g0.add_gaussian(0.0, 1.0)
    assert C.rel_l2(g0.psi, z["im_psi0"]) < 1e-15  # the IM run's start state
    g, rows = C.oracle_im(p, dim)
    np.testing.assert_allclose(np.array([C.im_dat_row(r) for r in rows]), z["im_rows"], rtol=1e-11, atol=1e-13)
    assert C.rel_l2(g.psi, z["im_psi"]) < 1e-12
    g2, rows2 = C.oracle_re(p, dim, z["re_psi0"])
    nb = len(C.re_borders(dim))
    got = np.array([C.re_dat_row(r, nb) for r in rows2])
    assert got.shape == z["re_rows"].shape
    np.testing.assert_allclose(got, z["re_rows"], rtol=1e-10, atol=1e-13)
    assert C.rel_l2(g2.psi, z["re_psi"]) < 1e-12


def test_gaussian_initial_state_matches_reference():
    z = C.load("c2_vg")
    g = C.oracle_grid(z["params"], 2, O.Coupling(O.GAUGE_VELOCITY))
    g.add_gaussian(0.0, 1.0)
    assert C.rel_l2(g.psi, z["im_psi0"]) < 1e-15
