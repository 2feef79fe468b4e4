"""Failure detection, all triggered on the host (no GPU fault involved).

The reference aborts the process on a failed check (basics/logging.h:12,114); here
every failure comes back as a status code and leaves the device usable:
* a wavefunction holding a NaN (uploaded from the host) makes qsf_step return
  QSF_ENUMERIC, in the fused 2D path and in the 1D line kernel;
* in a batch the flagged member reports QSF_ENUMERIC while the other members'
  rows and wavefunctions stay bit-identical to their solo runs;
* the server finishes a NaN request with QSF_ENUMERIC and the rest of the mix
  normally; a request larger than the device can ever hold finishes at once with
  QSF_ENOMEM; a request that fits the device but not the free HBM left above the
  reserve stays queued (bounded waits time out cleanly) until it is cancelled
  (QSF_ECANCELED); a result is handed out once.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ENOMEM, ETIMEDOUT, ENUMERIC, ECANCELED = 2, 4, 5, 8


def _state(dim, n, seed):
    rng = np.random.default_rng(seed)
    psi = rng.standard_normal((n,) * dim) + 1j * rng.standard_normal((n,) * dim)
    return psi / np.sqrt(np.sum(np.abs(psi) ** 2) * 0.3 ** dim)


def _sched(Q, dim, nsteps, gauge=0):
    from qsf_gb300.propagator import coupling_schedule
    c = Q.Coupling(gauge, [Q.Field({1: 1, 2: 3, 3: 7}[dim], [Q.Pulse(field=0.1, omega=1.0, ncycles=1.0)])])
    return coupling_schedule(c, 0.05, nsteps)[0]


@pytest.mark.parametrize("dim,n", [(2, 64), (1, 1024)])
def test_nan_in_psi_is_enumeric(dim, n):
    import qsf_gb300 as Q
    g = Q.Grid(dim, n, 0.3, nCAP=n // 10, Ncharge=float(dim), gauge=Q.GAUGE_VELOCITY, n_fields=1)
    psi = _state(dim, n, 1)
    psi.reshape(-1)[n // 2] = complex(np.nan, 0.0)
    g.upload(psi)
    with pytest.raises(Q.QsfError) as e:
        g.step(Q.MODE_RE, 0.05, 20, _sched(Q, dim, 20), obs=Q.OBS_NORM | Q.OBS_EPOT)
    assert e.value.code == ENUMERIC
    # the grid (and the device) stay usable
    g.upload(_state(dim, n, 2))
    rows, done = g.step(Q.MODE_RE, 0.05, 20, _sched(Q, dim, 20), obs=Q.OBS_NORM | Q.OBS_EPOT)
    assert done == 20 and np.all(np.isfinite(rows))


def test_nan_member_of_a_batch():
    import qsf_gb300 as Q
    specs = [(2, 64, 3), (2, 96, 4), (2, 64, 5)]
    grids, starts, alone = [], [], []
    for dim, n, seed in specs:
        g = Q.Grid(dim, n, 0.3, nCAP=n // 10, Ncharge=2.0, gauge=Q.GAUGE_VELOCITY, n_fields=1)
        psi = _state(dim, n, seed)
        g.upload(psi)
        rows, _ = g.step(Q.MODE_RE, 0.05, 24, _sched(Q, dim, 24), obs=Q.OBS_NORM | Q.OBS_EPOT)
        alone.append((rows.copy(), g.download()))
        grids.append(g)
        starts.append(psi)
    bad = starts[2].copy()
    bad[10, 10] = complex(0.0, np.inf)
    b = Q.Batch()
    slots = []
    for i, (g, psi) in enumerate(zip(grids, starts)):
        g.upload(bad if i == 2 else psi)
        slots.append(b.add(g, Q.MODE_RE, 0.05, 24, _sched(Q, 2, 24), obs=Q.OBS_NORM | Q.OBS_EPOT))
    with pytest.raises(Q.QsfError) as e:
        b.run(24)
    assert e.value.code == ENUMERIC
    for i in range(2):
        rows, done = b.result(slots[i])
        assert done == 24
        assert np.array_equal(rows, alone[i][0])
        assert np.array_equal(grids[i].download(), alone[i][1])
    with pytest.raises(Q.QsfError) as e:
        b.result(slots[2])
    assert e.value.code == ENUMERIC
    b.close()


def _request(Q, S, n=64, psi0=None):
    d = S.grid_desc(2, n, 0.3, nCAP=n // 10, Ncharge=2.0, gauge=Q.GAUGE_VELOCITY, n_fields=1)
    return dict(gdesc=d, mode=Q.MODE_RE, dt=0.05, nsteps=40, coupling=_sched(Q, 2, 40), psi0=psi0,
                obs=Q.OBS_NORM | Q.OBS_EPOT, borders=Q.ZOA_FLUX_2D)


def test_server_isolates_a_nan_request():
    import qsf_gb300 as Q
    from qsf_gb300 import serve as S
    srv = S.Server(max_slots=8, steps_per_round=8)
    try:
        good = _request(Q, S, psi0=_state(2, 64, 7))
        ref = srv.wait(srv.submit(**good), 300)
        assert ref["status"] == 0
        bad_psi = _state(2, 64, 8)
        bad_psi[3, 4] = complex(np.nan, np.nan)
        tb = srv.submit(**_request(Q, S, psi0=bad_psi))
        tg = srv.submit(**good)
        t96 = srv.submit(**_request(Q, S, n=96, psi0=_state(2, 96, 9)))
        assert srv.wait(tb, 300)["status"] == ENUMERIC
        r = srv.wait(tg, 300)
        assert r["status"] == 0
        for k in ("final_norm", "final_epot", "flux_integral", "steps"):
            assert r[k] == ref[k], k
        assert srv.wait(t96, 300)["status"] == 0
    finally:
        srv.stop()


def test_server_rejects_a_request_larger_than_the_device():
    import qsf_gb300 as Q
    from qsf_gb300 import serve as S
    srv = S.Server(max_slots=4, hbm_reserve_gb=1e6, steps_per_round=8)  # reserve above any device
    try:
        r = srv.wait(srv.submit(**_request(Q, S)), 30)
        assert r["status"] == ENOMEM
        assert srv.stats()["queued"] == 0
    finally:
        srv.stop()


def test_server_queues_while_hbm_is_short_then_cancel():
    import torch
    import qsf_gb300 as Q
    from qsf_gb300 import serve as S
    torch.cuda.init()
    hold = torch.empty(2 * 1024 ** 3, dtype=torch.uint8, device="cuda")  # 2 GiB in use on the device
    free_b, total_b = torch.cuda.mem_get_info()
    assert total_b - free_b > 1.5e9
    # the request fits the device minus the reserve, but not the free HBM minus the reserve
    reserve_gb = (free_b - 1e5) / 1e9  # 100 kB left: below any solve's device bytes
    srv = S.Server(max_slots=4, hbm_reserve_gb=reserve_gb, steps_per_round=8)
    try:
        t = srv.submit(**_request(Q, S))
        with pytest.raises(Q.QsfError) as e:
            srv.wait(t, 0.5)
        assert e.value.code == ETIMEDOUT
        st = srv.stats()
        assert st["queued"] == 1 and st["in_flight"] == 0
        srv.cancel(t)
        r = srv.wait(t, 30)
        assert r["status"] == ECANCELED
        with pytest.raises(Q.QsfError) as e:  # handed out once
            srv.wait(t, 0.05)
        assert e.value.code == ETIMEDOUT
        with pytest.raises(Q.QsfError):
            srv.cancel(t)  # no longer known
    finally:
        srv.stop()
        del hold


def test_server_cancels_a_running_solve():
    import qsf_gb300 as Q
    from qsf_gb300 import serve as S
    srv = S.Server(max_slots=4, steps_per_round=2)
    try:
        req = _request(Q, S, n=256)
        req["nsteps"] = 4000
        req["coupling"] = _sched(Q, 2, 4000)
        t = srv.submit(**req)
        import time
        for _ in range(200):
            if srv.stats()["in_flight"] == 1:
                break
            time.sleep(0.01)
        srv.cancel(t)
        r = srv.wait(t, 60)
        assert r["status"] == ECANCELED
        assert 0 < r["steps"] < 4000
    finally:
        srv.stop()
