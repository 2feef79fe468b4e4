"""Native serving loop: continuous batching returns the same result alone and in a mix.

A reference solve is served on an idle server, then again while other solves of
different sizes and dimensions arrive before, with and after it; its result must be
bit-identical.  Also checks admission limits (slots) and the bounded wait.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _req(Q, S, dim, n, F0, omega, gauge=0):
    d = S.grid_desc(dim, n, 0.3, nCAP=max(2, n // 10), Ncharge=float(dim), gauge=gauge, n_fields=1,
                    border_nodes=(6, 4, 3, 12))
    c = Q.Coupling(gauge, [Q.Field({1: 1, 2: 3, 3: 7}[dim], [Q.Pulse(field=F0, omega=omega, ncycles=1.0)])])
    steps = int(c.max_pulse_duration() / 0.05 + 1) + 2
    from qsf_gb300.propagator import coupling_schedule
    sched, _ = coupling_schedule(c, 0.05, steps)
    borders = [] if dim == 1 else (Q.ZOA_FLUX_2D if dim == 2 else Q.ZOA_FLUX_3D)
    return dict(gdesc=d, mode=Q.MODE_RE, dt=0.05, nsteps=steps, coupling=sched, obs=Q.OBS_NORM | Q.OBS_EPOT,
                borders=borders)


def test_served_result_is_the_same_alone_and_in_the_mix():
    import qsf_gb300 as Q
    from qsf_gb300 import serve as S
    ref = _req(Q, S, 2, 64, 0.1, 1.2)
    srv = S.Server(max_slots=8, steps_per_round=16)
    try:
        alone = srv.wait(srv.submit(**ref), 300)
        assert alone["status"] == 0
        others = [_req(Q, S, 2, 48, 0.05, 1.5), _req(Q, S, 1, 512, 0.07, 0.8), _req(Q, S, 3, 16, 0.1, 1.4, 1),
                  _req(Q, S, 2, 96, 0.12, 1.0), _req(Q, S, 2, 64, 0.09, 1.1, 1)]
        tickets = [srv.submit(**o) for o in others[:3]]
        t_ref = srv.submit(**ref)
        tickets += [srv.submit(**o) for o in others[3:]]
        mixed = srv.wait(t_ref, 300)
        for t in tickets:
            assert srv.wait(t, 300)["status"] == 0
        for k in ("final_norm", "yield", "final_epot", "flux_integral", "steps"):
            assert alone[k] == mixed[k], k
        st = srv.stats()
        assert st["completed"] == 7 and st["in_flight"] == 0 and st["queued"] == 0
    finally:
        srv.stop()


def test_wait_times_out_and_slots_bound_residency():
    import qsf_gb300 as Q
    from qsf_gb300 import serve as S
    srv = S.Server(max_slots=1, steps_per_round=4)
    try:
        r = _req(Q, S, 2, 96, 0.1, 0.5)
        t1 = srv.submit(**r)
        t2 = srv.submit(**r)
        with pytest.raises(Q.QsfError) as e:
            srv.wait(t2, 0.001)
        assert e.value.code == 4
        time.sleep(0.05)
        assert srv.stats()["in_flight"] <= 1
        a, b = srv.wait(t1, 300), srv.wait(t2, 300)
        assert a["status"] == 0 and b["status"] == 0
        assert a["final_norm"] == b["final_norm"]
    finally:
        srv.stop()
