"""The 1D plain configuration at its full size and run length against the oracle:
soft-core hydrogen V = -1/sqrt(x^2 + 1) on 4096 points (dx 0.2); imaginary-time ground
state (dt 0.01, 2000 steps, Normalize every step); then real time (dt 0.05) under a
2-cycle sin^2 800 nm pulse of 1e14 W/cm^2 in the length gauge, 4418 steps, with the
cos^(1/8) mask on the outer 10% of each side; outputs norm, E_pot, the BOX flux at the
inner mask edge every step, and the yields 1 - |<psi_0|psi(T)>|^2 and 1 - norm(T).
Bar: psi(T) within relative L2 1e-10 of the oracle, every observable and yield within
1e-9."""
import math

import numpy as np
import pytest

from tests import cases as C

pytestmark = pytest.mark.gpu

N, DX, NCAP, BOX = 4096, 0.2, 410, 1638
IM_DT, IM_STEPS, RE_DT = 0.01, 2000, 0.05
F0 = math.sqrt(1e14 / 3.50944e16)    # constants.h:35
OMEGA = 45.563352529 / 800.0          # constants.h:47-51
RE_OUT = ["step", "time", "norm", "epot", ("flux", ["BOX"], BOX)]


def _gpu(Q):
    common = dict(nCAP=NCAP, potential=Q.POT_EBERLY, Ncharge=1.0, Echarge=-1.0, Nsoft=1.0,
                  absorber=Q.ABS_COS8, mask_dt=RE_DT)
    gi = Q.Grid(1, N, DX, gauge=Q.GAUGE_VELOCITY, n_fields=0, **common)
    gi.add_gaussian(0.0, 1.0)
    im_rows = Q.SplitPropagator(Q.MODE_IM, IM_DT, IM_STEPS, gi, Q.Coupling(Q.GAUGE_VELOCITY), C.IM_OUTPUTS).run()
    psi0 = gi.download()
    gr = Q.Grid(1, N, DX, gauge=Q.GAUGE_LENGTH, n_fields=1, **common)
    gr.upload(psi0)
    c = Q.Coupling(Q.GAUGE_LENGTH, [Q.Field(1, [Q.Pulse(field=F0, omega=OMEGA, ncycles=2)])])
    re_rows = Q.SplitPropagator(Q.MODE_RE, RE_DT, 0, gr, c, RE_OUT).run()
    return psi0, im_rows, gr.download(), re_rows


def _oracle():
    from oracle import oracle as O
    O.set_border_nodes(25, 14, 10, 40)
    gi = O.Grid(1, N, DX, nCAP=NCAP, pot=O.POT_EBERLY, Ncharge=1.0, coupling=O.Coupling(O.GAUGE_VELOCITY))
    gi.set_absorber(O.ABS_COS8, RE_DT)
    gi.add_gaussian(0.0, 1.0)
    im_rows = O.Propagator(O.MODE_IM, IM_DT, IM_STEPS, gi, C.IM_OUTPUTS).run()
    psi0 = gi.psi.copy()
    c = O.Coupling(O.GAUGE_LENGTH, [O.Field(1, [O.Pulse(field=F0, omega=OMEGA, ncycles=2)])])
    gr = O.Grid(1, N, DX, nCAP=NCAP, pot=O.POT_EBERLY, Ncharge=1.0, coupling=c)
    gr.set_absorber(O.ABS_COS8, RE_DT)
    gr.psi[...] = psi0
    re_rows = O.Propagator(O.MODE_RE, RE_DT, 0, gr, RE_OUT).run()
    return psi0, im_rows, gr.psi.copy(), re_rows


def _yields(psi0, psiT):
    ov = np.vdot(psi0, psiT) * DX
    return 1.0 - abs(ov) ** 2, 1.0 - float(np.sum(np.abs(psiT) ** 2) * DX)


def test_c1_full_run_matches_oracle():
    import qsf_gb300 as Q
    g0, gim, gT, gre = _gpu(Q)
    o0, oim, oT, ore = _oracle()
    got = np.array([C.im_dat_row(r) for r in gim])
    ref = np.array([C.im_dat_row(r) for r in oim])
    assert got.shape == ref.shape
    np.testing.assert_allclose(got, ref, rtol=1e-9, atol=1e-9)
    assert C.rel_l2(g0, o0) < 1e-10
    assert abs(ref[-1][5] - (-0.66977)) < 2e-4   # E_tot of the soft-core ground state
    row = lambda r: [r["step"], r["time"], r["norm"], r["epot"], r["flux"][0]]  # noqa: E731
    got = np.array([row(r) for r in gre])
    ref = np.array([row(r) for r in ore])
    assert got.shape == ref.shape and len(ref) > 4413  # max_steps = T / dt + 1 (propagator.h:118-127)
    np.testing.assert_allclose(got[:, :2], ref[:, :2], rtol=1e-14, atol=0)
    np.testing.assert_allclose(got[:, 2:4], ref[:, 2:4], rtol=1e-9, atol=1e-12)
    fl = np.max(np.abs(ref[:, 4]))
    assert fl > 0.0
    np.testing.assert_allclose(got[:, 4], ref[:, 4], rtol=1e-9, atol=1e-9 * fl)
    # the flux integrated over the run (the border-flux integral)
    np.testing.assert_allclose(np.sum(got[:, 4]) * RE_DT, np.sum(ref[:, 4]) * RE_DT, rtol=1e-9)
    assert C.rel_l2(gT, oT) < 1e-10
    yg, yo = _yields(g0, gT), _yields(o0, oT)
    np.testing.assert_allclose(yg, yo, rtol=1e-9, atol=1e-12)
    assert yo[0] > 0.0 and yo[1] >= 0.0
