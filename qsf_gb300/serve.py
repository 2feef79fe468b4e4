"""Python handle on the native serving loop (qsf_server_* in include/qsf_gpu.h).

The loop itself -- queue, admission by slots and free HBM, continuous batching,
completion -- runs in C++ inside libqsfgpu.so on its own thread; this module only
submits requests and collects results.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np

from ._lib import MAX_BORDERS, GridDesc, Request, Result, ServerConfig, ServerStats, check, lib
from .grid import BORDERS, OBS_FLUX, OBS_NORM, POT_EBERLY


def grid_desc(dim: int, n, dx, nCAP: int = 0, potential: int = POT_EBERLY, Ncharge: float = 1.0,
              Echarge: float = -1.0, Nsoft: float = 1.0, Esoft: float = 1.0, gauge: int = 0, n_fields: int = 0,
              p_axis_swap: Optional[bool] = None, border_nodes=(25, 14, 10, 40), absorber: int = 0,
              mask_dt: float = 0.0) -> GridDesc:
    n = [int(n)] * dim if np.isscalar(n) else [int(v) for v in n]
    dx = [float(dx)] * dim if np.isscalar(dx) else [float(v) for v in dx]
    d = GridDesc()
    d.dim = dim
    for k in range(dim):
        d.n[k] = n[k]
        d.dx[k] = dx[k]
    d.nCAP = int(nCAP)
    d.potential = potential
    d.Ncharge, d.Echarge, d.Nsoft, d.Esoft = Ncharge, Echarge, Nsoft, Esoft
    d.gauge = gauge
    d.n_fields = n_fields
    d.p_axis_swap = int(dim >= 2 if p_axis_swap is None else p_axis_swap)
    for k in range(4):
        d.border_nodes[k] = int(border_nodes[k])
    d.absorber = int(absorber)
    d.mask_dt = float(mask_dt)
    return d


class Server:
    def __init__(self, max_slots: int = 64, hbm_reserve_gb: float = 8.0, steps_per_round: int = 32,
                 queue_capacity: int = 100000):
        cfg = ServerConfig(max_slots, hbm_reserve_gb, steps_per_round, queue_capacity)
        h = ctypes.c_void_p()
        check(lib().qsf_server_start(ctypes.byref(cfg), ctypes.byref(h)), "qsf_server_start")
        self._h = h

    def submit(self, gdesc: GridDesc, mode: int, dt: float, nsteps: int, coupling: Optional[np.ndarray] = None,
               psi0: Optional[np.ndarray] = None, obs: int = OBS_NORM, borders: Sequence[str] = (),
               box_size: int = 0) -> int:
        r = Request()
        r.grid = gdesc
        r.mode = mode
        r.dt = dt
        r.nsteps = int(nsteps)
        keep = []
        if coupling is not None:
            c = np.ascontiguousarray(coupling, dtype=np.float64)
            keep.append(c)
            r.coupling = c.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        if psi0 is not None:
            p = np.ascontiguousarray(psi0, dtype=np.complex128).reshape(-1)
            keep.append(p)
            r.psi0 = p.view(np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        r.obs = obs | (OBS_FLUX if borders else 0)
        r.nborders = len(borders)
        assert len(borders) <= MAX_BORDERS
        for i, b in enumerate(borders):
            r.border_types[i] = BORDERS[b]
        r.box_size = int(box_size)
        t = ctypes.c_int64()
        check(lib().qsf_server_submit(self._h, ctypes.byref(r), ctypes.byref(t)), "qsf_server_submit")
        return int(t.value)

    @staticmethod
    def _to_dict(res: Result, nb: int = MAX_BORDERS):
        return {"status": res.status, "steps": res.steps, "final_norm": res.final_norm, "yield": res.yield_,
                "final_epot": res.final_epot, "flux_integral": list(res.flux_integral)[:nb],
                "queue_s": res.queue_s, "latency_s": res.latency_s}

    def poll(self, ticket: int):
        res = Result()
        done = ctypes.c_int()
        check(lib().qsf_server_poll(self._h, int(ticket), ctypes.byref(res), ctypes.byref(done)), "qsf_server_poll")
        return self._to_dict(res) if done.value else None

    def wait(self, ticket: int, timeout_s: float = 600.0):
        res = Result()
        check(lib().qsf_server_wait(self._h, int(ticket), float(timeout_s), ctypes.byref(res)), "qsf_server_wait")
        return self._to_dict(res)

    def cancel(self, ticket: int) -> None:
        """Cancel a queued or running solve; its result then carries QSF_ECANCELED."""
        check(lib().qsf_server_cancel(self._h, int(ticket)), "qsf_server_cancel")

    def stats(self):
        st = ServerStats()
        check(lib().qsf_server_stats_get(self._h, ctypes.byref(st)), "qsf_server_stats_get")
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def stop(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().qsf_server_stop(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.stop()
        except Exception:
            pass


class ShardedServer:
    """One rank's part of a request stream served by several GPUs (one process per GPU):
    every rank sees the same ordered stream and submits to its own Server only the
    requests that shard.StreamAssigner gives it (cost: grid points x steps), so the
    ranks split the work without a collective.  submit() returns the local ticket, or
    None for a request another rank serves."""

    def __init__(self, rank: int, world_size: int, **server_kwargs):
        from .shard import StreamAssigner
        if not 0 <= rank < world_size:
            raise ValueError("rank must be in [0, world_size)")
        self.rank, self.world_size = rank, world_size
        self._assign = StreamAssigner(world_size)
        self.server = Server(**server_kwargs)

    def submit(self, gdesc: GridDesc, mode: int, dt: float, nsteps: int, **kw) -> Optional[int]:
        m = 1
        for k in range(gdesc.dim):
            m *= int(gdesc.n[k])
        if self._assign.assign(float(m) * float(nsteps)) != self.rank:
            return None
        return self.server.submit(gdesc, mode, dt, nsteps, **kw)

    def wait(self, ticket: int, timeout_s: float = 600.0):
        return self.server.wait(ticket, timeout_s)

    def stats(self):
        return self.server.stats()

    def stop(self):
        self.server.stop()

