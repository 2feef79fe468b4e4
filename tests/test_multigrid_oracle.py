"""The oracle's multi-region grid against the reference's own multigrid.h.

The fixtures were written by the reference's LocalGrid<..., Slices, true>
(multigrid.h) running with one process per region (MultiRegionsReduced<dim>): every
region's final wavefunction and the main region's .dat rows.  1D and 2D agree to the
last bit; 3D to rounding (the order of the partial transforms differs).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests import cases as C


def test_region_order_and_sources():
    assert O.region_axes(2) == [0, 1, 2, 3]
    assert O.region_sources(2) == [[], [(0, 0)], [(0, 1)], [(1, 1), (2, 0)]]
    src3 = O.region_sources(3)
    assert src3[7] == [(4, 2), (5, 1), (6, 0)]  # XYZ from XY, XZ, YZ
    assert src3[4] == [(1, 1), (2, 0)]          # XY from X (via Y), Y (via X)


# *_bs: axis lengths with a prime factor above 5 (130, 34, 14)
@pytest.mark.parametrize("name", ["mg1", "mg2", "mg3", "mg1_bs", "mg2_bs", "mg3_bs"])
def test_multigrid_matches_reference(name):
    z = C.load(name)
    p, dim = z["params"], int(z["dim"])
    gs, rows = C.oracle_mg(p, dim, z["psi_in"])
    got = np.array([C.mg_dat_row(r) for r in rows])
    assert got.shape == z["re_rows"].shape
    np.testing.assert_allclose(got, z["re_rows"], rtol=1e-12, atol=1e-14)
    for r in range(2 ** dim):
        ref = z["psi_r%d" % r]
        assert np.linalg.norm(ref) > 0.0
        assert C.rel_l2(gs[r].psi, ref) < 1e-13, r


def test_transfer_moves_only_margins_in_2d():
    """A state zero in the margins transfers nothing; group-1 regions receive the
    masked margin of the main region along their free axis."""
    g = O.Grid(2, 16, 0.5, nCAP=3)
    g.set_region(1, True)
    src = O.Grid(2, 16, 0.5, nCAP=3)
    src.set_region(0, True)
    src.psi[3:13, :] = 1.0
    g.mg_transfer_from(src, 0, 1)
    assert np.all(g.psi == 0)
    src.psi[0, 5] = 2.0
    g.mg_transfer_from(src, 0, 1)
    assert np.count_nonzero(np.abs(g.psi) > 0) == 16  # one column, transformed along x
