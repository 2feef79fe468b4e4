"""MultiProductSplit<Split3Base<X,P,X>, K> (splitting.h:63-91, propagator.h:331-413).

The fixtures tests/golden/mp.npz and mp_bs.npz hold real-time 1D runs of the reference's
own propagator with K = 2 and 3 in both gauges.  The oracle restates the chains literally
(including the completion test `chain == ChainCount - 1`, which leaves a step's result
equal to its last chain); the GPU path runs that last chain as K fused sub-steps."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import cases as C

TAGS = [("MP2VG", 2, 0), ("MP3VG", 3, 0), ("MP2LG", 2, 1), ("MP3LG", 3, 1)]
# mp: 256 points; mp_bs: 258 = 2 * 3 * 43 (Bluestein transforms on the GPU)
FIXTURES = ["mp", "mp_bs"]
MP_OUTPUTS = ["step", "time", "norm", "epot"]


def _rows(rows):
    return np.array([[r["step"], r["time"], r["norm"], r["epot"]] for r in rows])


@pytest.mark.parametrize("name", FIXTURES)
@pytest.mark.parametrize("tag,K,lg", TAGS)
def test_oracle_chains_match_reference(tag, K, lg, name):
    z = C.load(name)
    p = z["params"]
    gauge = O.GAUGE_LENGTH if lg else O.GAUGE_VELOCITY
    c = O.Coupling(gauge, [O.Field(1, [C.pulse(p)])])
    g = C.oracle_grid(p, 1, c)
    g.psi[...] = z[tag + "_psi0"]
    prop = O.Propagator(O.MODE_RE, p["re_dt"], 0, g, MP_OUTPUTS, order=K)
    rows = prop.run()
    assert np.array_equal(g.psi, z[tag + "_psi"])
    np.testing.assert_array_equal(_rows(rows), z[tag + "_rows"])


def test_chain_coefficients():
    # Chain<I>::value = prod_{J != I} I^2 / (I^2 - J^2): 2nd order -1/3, 4/3
    assert O.Propagator.chain_value(1, 2) == pytest.approx(-1.0 / 3.0)
    assert O.Propagator.chain_value(2, 2) == pytest.approx(4.0 / 3.0)
    assert O.Propagator.chain_mults(3) == pytest.approx([1 / 6, 1 / 3, 1 / 3, 1 / 3, 1 / 3, 1 / 3, 1 / 6])


@pytest.mark.gpu
@pytest.mark.parametrize("name", FIXTURES)
@pytest.mark.parametrize("tag,K,lg", TAGS)
def test_gpu_multiproduct_matches_reference(tag, K, lg, name):
    import qsf_gb300 as Q
    z = C.load(name)
    p = z["params"]
    gauge = Q.GAUGE_LENGTH if lg else Q.GAUGE_VELOCITY
    c = Q.Coupling(gauge, [Q.Field(1, [C.gpu_pulse(p)])])
    g = C.gpu_grid(p, 1, gauge, 1)
    g.upload(z[tag + "_psi0"])
    prop = Q.SplitPropagator(Q.MODE_RE, p["re_dt"], 0, g, c, MP_OUTPUTS, order=K)
    rows = prop.run()
    psi = g.download()
    assert C.rel_l2(psi, z[tag + "_psi"]) < 1e-10
    ref = z[tag + "_rows"]
    got = _rows(rows)
    assert got.shape == ref.shape
    np.testing.assert_array_equal(got[:, 0], ref[:, 0])          # step
    np.testing.assert_allclose(got[:, 1], ref[:, 1], rtol=1e-15)  # time
    np.testing.assert_allclose(got[:, 2:], ref[:, 2:], rtol=1e-9, atol=1e-12)
    g.close()
