"""The cos^(1/8) mask absorber in the oracle (the reference has only the quartic CAP
of absorbers.h; the mask is the 1D plain configuration's absorber, defined over the
same nCAP-node margins): the factor of evolve<X>(delta) on a field-free, potential-free
grid against the closed form, two X halves of a step applying the mask once, and the
quartic CAP left as it was."""
import math

import numpy as np

from oracle import oracle as O


def _mask_1d(n, ncap):
    """M_d per node: cos(pi/2 * nodes / nCAP)^(1/8) over the margins, 1 inside;
    nodes = nCAP + neg_dist_from_edge (grid.h:181-185)."""
    i = np.arange(n)
    n2 = n // 2
    nd = np.where(i < n2, -i, i - n + 1)
    nodes = ncap + nd
    m = np.ones(n)
    band = nodes > 0
    m[band] = np.cos(0.5 * math.pi * nodes[band] / ncap) ** 0.125
    return m


def _flat_grid(dim, n, ncap, kind, mask_dt=0.05):
    g = O.Grid(dim, n, 0.3, nCAP=ncap, pot=O.POT_NONE)
    g.set_absorber(kind, mask_dt)
    g.psi[...] = 1.0
    return g


def test_cos8_factor_matches_closed_form():
    for dim, n, ncap in ((1, 200, 20), (2, 48, 5), (3, 16, 3)):
        g = _flat_grid(dim, n, ncap, O.ABS_COS8)
        g.evolve(O.MODE_RE, O.REP_X, 0.025)   # half of mask_dt
        g.evolve(O.MODE_RE, O.REP_X, 0.025)
        m1 = _mask_1d(n, ncap)
        M = m1
        for _ in range(dim - 1):
            M = np.multiply.outer(M, m1)
        np.testing.assert_allclose(g.psi.real, M, rtol=1e-13, atol=1e-15)
        assert np.max(np.abs(g.psi.imag)) == 0.0
        # the outermost node is nearly cleared, the interior untouched
        assert abs(g.psi.flat[0]) < 0.01 ** dim
        assert g.psi[(n // 2,) * dim] == 1.0


def test_cos8_half_step_is_the_square_root():
    g = _flat_grid(1, 100, 10, O.ABS_COS8, mask_dt=0.1)
    g.evolve(O.MODE_RE, O.REP_X, 0.05)
    np.testing.assert_allclose(g.psi.real, np.sqrt(_mask_1d(100, 10)), rtol=1e-13)


def test_quartic_cap_is_unchanged():
    n, ncap, delta = 120, 12, 0.025
    g = _flat_grid(1, n, ncap, O.ABS_CAP)
    g.evolve(O.MODE_RE, O.REP_X, delta)
    i = np.arange(n)
    nd = np.where(i < n // 2, -i, i - n + 1)
    nodes = np.maximum(ncap + nd, 0).astype(np.float64)
    eta = (3.0 / ncap) ** 4
    np.testing.assert_allclose(g.psi.real, np.exp(-delta * nodes ** 4 * eta), rtol=1e-14)
