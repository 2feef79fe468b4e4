"""average_der (grid.h:443-465) and AntiSymmetrize<2|3> (grid.h:611-723): the oracle is
pinned to the reference's own results (tests/golden/as2.npz, as3.npz, written by
oracle/_ref/qsf_ref), the GPU library is compared with both."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import cases as C


def _oracle(name):
    z = C.load(name)
    p, dim = z["params"], int(z["dim"])
    g = C.oracle_grid(p, dim, O.Coupling(O.GAUGE_VELOCITY))
    g.psi[...] = z["psi_in"]
    return z, p, dim, g


@pytest.mark.parametrize("name", ["as2", "as3"])
def test_oracle_average_der_matches_reference(name):
    z, p, dim, g = _oracle(name)
    got = [g.average_der(d) for d in range(dim)]
    np.testing.assert_allclose(got, z["der"], rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("name,particles", [("as2", 2), ("as3", 2), ("as3", 3)])
def test_oracle_antisymmetrize_matches_reference(name, particles):
    z, p, dim, g = _oracle(name)
    g.antisymmetrize(particles)
    assert np.array_equal(g.psi, z[f"psi_as{particles}"])


def test_antisymmetric_results_are_antisymmetric():
    z = C.load("as3")
    a3 = z["psi_as3"]
    for perm, sign in (((1, 0, 2), -1), ((0, 2, 1), -1), ((2, 1, 0), -1), ((1, 2, 0), 1), ((2, 0, 1), 1)):
        np.testing.assert_array_equal(np.transpose(a3, perm), sign * a3)
    a2 = C.load("as2")["psi_as2"]
    np.testing.assert_array_equal(a2.T, -a2)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["as2", "as3"])
def test_gpu_average_der(name):
    import qsf_gb300 as Q
    z = C.load(name)
    p, dim = z["params"], int(z["dim"])
    g = C.gpu_grid(p, dim, Q.GAUGE_VELOCITY, 0)
    g.upload(z["psi_in"])
    got = [g.average_der(d) for d in range(dim)]
    np.testing.assert_allclose(got, z["der"], rtol=1e-12, atol=1e-14)
    with pytest.raises(Q.QsfError):
        g.average_der(dim)
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name,particles", [("as2", 2), ("as3", 2), ("as3", 3)])
def test_gpu_antisymmetrize_bitwise(name, particles):
    import qsf_gb300 as Q
    z = C.load(name)
    p, dim = z["params"], int(z["dim"])
    g = C.gpu_grid(p, dim, Q.GAUGE_VELOCITY, 0)
    g.upload(z["psi_in"])
    g.antisymmetrize(particles)
    assert np.array_equal(g.download(), z[f"psi_as{particles}"])
    g.close()
