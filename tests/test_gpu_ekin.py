"""E_kin on every k-th step (qsf_step_desc.ekin_interval) keeps the steps between fused.

The reference evaluates AVG<KineticEnergy> with an extra transform pair after every
step (propagator.h:284-291) and records rows every comp_interval steps
(wf/buffer.h:6, 391).  With ekin_interval = k the GPU computes E_kin on steps k-1,
2k-1, ... and on the call's last step only; those steps end with psi_n in memory, the
others stay in fixed point.  Checked against the same run with E_kin every step (which
the golden IM fixtures pin to the reference): every norm / E_pot value and every E_kin
value that is computed agree to 1e-9, the final wavefunction to 1e-10, and the rows
in between carry E_kin = 0.
"""
import numpy as np
import pytest

from tests import cases as C

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,dim", [("c2_vg", 2), ("c3_lg", 3)])
@pytest.mark.parametrize("k", [3, 8])
def test_ekin_interval_matches_every_step(name, dim, k):
    import qsf_gb300 as Q
    z = C.load(name)
    p = z["params"]
    steps = 40
    out = {}
    for kk in (1, k):
        g = C.gpu_grid(p, dim, Q.GAUGE_VELOCITY, 0)
        g.add_gaussian(0.0, 1.0)
        g.normalize()
        rows, done = g.step(Q.MODE_IM, p["im_dt"], steps, None, obs=Q.OBS_NORM | Q.OBS_EPOT | Q.OBS_EKIN,
                            normalize=True, ekin_interval=kk)
        assert done == steps
        out[kk] = (rows.copy(), g.download())
        g.close()
    (r1, psi1), (rk, psik) = out[1], out[k]
    np.testing.assert_allclose(rk[:, :2], r1[:, :2], rtol=1e-9, atol=0)
    have = np.array([(s + 1) % k == 0 or s == steps - 1 for s in range(steps)])
    np.testing.assert_allclose(rk[have, 2], r1[have, 2], rtol=1e-9, atol=0)
    assert np.all(rk[~have, 2] == 0.0)
    assert np.all(r1[:, 2] > 0.0)
    assert C.rel_l2(psik, psi1) < 1e-10


def test_ekin_interval_propagator_run():
    """SplitPropagator(ekin_interval=k) over an imaginary-time run with etot outputs."""
    import qsf_gb300 as Q
    z = C.load("c2_vg")
    p = z["params"]
    res = {}
    for k in (1, 5):
        g = C.gpu_grid(p, 2, Q.GAUGE_VELOCITY, 0)
        g.add_gaussian(0.0, 1.0)
        prop = Q.SplitPropagator(Q.MODE_IM, p["im_dt"], 30, g, Q.Coupling(Q.GAUGE_VELOCITY), C.IM_OUTPUTS,
                                 ekin_interval=k)
        rows = prop.run()
        res[k] = (rows, g.download())
    rows1, psi1 = res[1]
    rows5, psi5 = res[5]
    assert len(rows1) == len(rows5)
    assert C.rel_l2(psi5, psi1) < 1e-10
    for a, b in zip(rows1, rows5):
        assert a["norm"] == pytest.approx(b["norm"], rel=1e-9)
        assert a["epot"] == pytest.approx(b["epot"], rel=1e-9)
        if b["ekin"] != 0.0:
            assert a["ekin"] == pytest.approx(b["ekin"], rel=1e-9)
