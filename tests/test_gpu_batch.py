"""Batched solves (qsf_batch) give the same bits as each solve run alone (qsf_step).

Solves of different sizes (2D edges 48, 64 and 96, a 1D line, a 3D cube), gauges
and pulses share one batch; every solve's rows and final wavefunction must be
identical to the solve run by itself, since per-solve work and reduction order do
not depend on the batch.
"""
import numpy as np
import pytest

import tests.cases as C

pytestmark = pytest.mark.gpu


def _solve(Q, dim, n, gauge, F0, omega, seed):
    nodes = (6, 4, 3, 12) if dim > 1 else (25, 14, 10, 40)
    g = Q.Grid(dim, n, 0.3, nCAP=max(2, n // 10), Ncharge=float(dim), gauge=gauge, n_fields=1, border_nodes=nodes)
    rng = np.random.default_rng(seed)
    shape = (n,) * dim
    psi = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    g.upload(psi)
    g.normalize()
    c = Q.Coupling(gauge, [Q.Field({1: 1, 2: 3, 3: 7}[dim], [Q.Pulse(field=F0, omega=omega, ncycles=1.0)])])
    prop = Q.SplitPropagator(Q.MODE_RE, 0.05, 0, g, c, ["norm", "epot"])
    sched = prop._schedule(prop.max_steps + 2)
    borders = ([] if dim == 1 else (Q.ZOA_FLUX_2D if dim == 2 else Q.ZOA_FLUX_3D))
    kw = dict(obs=Q.OBS_NORM | Q.OBS_EPOT | Q.OBS_EKIN, borders=borders, box_size=0)
    return g, g.download(), sched, kw


def test_batch_matches_alone():
    import qsf_gb300 as Q
    specs = [(2, 48, Q.GAUGE_VELOCITY, 0.1, 1.3, 1), (2, 64, Q.GAUGE_LENGTH, 0.08, 1.1, 2),
             (2, 96, Q.GAUGE_VELOCITY, 0.12, 0.9, 3), (2, 48, Q.GAUGE_LENGTH, 0.05, 1.7, 4),
             (1, 256, Q.GAUGE_VELOCITY, 0.05, 0.6, 5), (3, 16, Q.GAUGE_LENGTH, 0.1, 1.5, 6)]
    alone = []
    made = []
    for sp in specs:
        g, psi0, sched, kw = _solve(Q, *sp)
        made.append((g, psi0, sched, kw))
        rows, done = g.step(Q.MODE_RE, 0.05, len(sched), sched, **kw)
        alone.append((rows.copy(), g.download()))
    b = Q.Batch()
    slots = []
    for g, psi0, sched, kw in made:
        g.upload(psi0)
        slots.append(b.add(g, Q.MODE_RE, 0.05, len(sched), sched, **kw))
    active = len(slots)
    while active:
        active = b.run(37)
    for (g, _, sched, _), slot, (rows_a, psi_a) in zip(made, slots, alone):
        rows_b, done = b.result(slot)
        assert done == len(sched)
        assert np.array_equal(rows_a, rows_b)
        assert np.array_equal(psi_a, g.download())


def test_destroying_a_member_takes_it_out_of_its_batch():
    """qsf_grid_destroy of a batch member removes it from the batch first: the batch's
    next run leaves its memory alone, the other members finish as they would alone, and
    the destroyed member's slot is gone.  A grid is in one batch at a time; destroying
    a batch leaves its grids free to join another."""
    import qsf_gb300 as Q
    (g1, p1, s1, kw1), (g2, p2, s2, kw2) = [_solve(Q, *sp) for sp in
                                            [(2, 48, Q.GAUGE_VELOCITY, 0.1, 1.3, 1), (2, 64, Q.GAUGE_LENGTH, 0.08, 1.1, 2)]]
    rows_a, _ = g2.step(Q.MODE_RE, 0.05, len(s2), s2, **kw2)
    rows_a, psi_a = rows_a.copy(), g2.download()
    g2.upload(p2)
    b = Q.Batch()
    slot1 = b.add(g1, Q.MODE_RE, 0.05, len(s1), s1, **kw1)
    slot2 = b.add(g2, Q.MODE_RE, 0.05, len(s2), s2, **kw2)
    assert b.run(5) == 2
    g1.close()
    with pytest.raises(Q.QsfError):
        b.result(slot1)
    active = 1
    while active:
        active = b.run(37)
    rows_b, done = b.result(slot2)
    assert done == len(s2)
    assert np.array_equal(rows_a, rows_b)
    assert np.array_equal(psi_a, g2.download())
    b2 = Q.Batch()
    with pytest.raises(Q.QsfError):
        b2.add(g2, Q.MODE_RE, 0.05, len(s2), s2, **kw2)
    b.close()
    g2.upload(p2)
    slot = b2.add(g2, Q.MODE_RE, 0.05, len(s2), s2, **kw2)
    while b2.run(64):
        pass
    rows_c, done = b2.result(slot)
    assert done == len(s2) and np.array_equal(rows_a, rows_c)
    b2.close()
    g2.close()
