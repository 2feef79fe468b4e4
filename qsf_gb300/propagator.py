"""SplitPropagator over the GPU grid, mirroring include/propagator.h.

``SplitPropagator.run()`` follows SplitPropagator::run (propagator.h:420-462): the
AT_START observables, the time loop of Strang steps (makeStep / chainEvolve,
propagator.h:311-346) with computeEach after each step (propagator.h:275-300), and
the final step.  The per-step coupling values are evaluated on the host exactly as
chainEvolve does (precalc at the running timer, timer advancing only in the coupling
representation) and the steps themselves run fused on the GPU through qsf_step.

Outputs mirror BufferedOutputs<..., Ts...> entries:
  "norm"  AVG<Identity>        "epot" AVG<PotentialEnergy>   "ekin" AVG<KineticEnergy>
  "normalize" OPERATION<Normalize>                             ("flux", [borders], box)
  "etot"  ENERGY_TOTAL          "ediff" ENERGY_DIFFERENCE      "time" / "step" VALUE<...>
X-space entries are evaluated in declaration order; entries after "normalize" see
the normalised wavefunction, as in computeEach.
"""
from __future__ import annotations

import os
import struct
from typing import List, Optional

import numpy as np

from .grid import (Grid, MODE_IM, MODE_RE, OBS_EKIN, OBS_EPOT, OBS_NORM, OP_IDENTITY, OP_KINETIC, OP_POTENTIAL,
                   REP_P, REP_X)
from .physics import Coupling


def _is_flux(o) -> bool:
    return isinstance(o, tuple) and o[0] == "flux"


def chain_mults(chain: int) -> List[float]:
    """_SplitChain::pack for Split3Base with `chain` coefficients 1/chain (splitting.h:43-58):
    X, then (P, X) `chain` times, the inner X halves joined."""
    c = 1.0 / chain
    arr = [0.0] * (2 * chain + 1)
    for j in range(chain):
        for k, mult in enumerate((0.5, 1.0, 0.5)):
            arr[2 * j + k] += mult * c
    return arr


def coupling_schedule(coupling: Coupling, dt: float, nsteps: int, timer: float = 0.0, order: int = 1):
    """Coupling rows of nsteps makeStep()s from `timer` on, as qsf_step takes them, and the
    timer afterwards; advances the coupling's state (propagator.h:311-346, 369-413).

    One row per sub-step (order rows per step).  Velocity gauge: A at each P sub-step;
    length gauge: E at the sub-step's opening and closing X half.  Every chain of a
    multi-product step evaluates the coupling at its sub-steps with the timer restored
    to the step's start but the coupling state (the PromoteFieldToA integral) carried
    over; only the last chain's values are kept, as only the last chain's wavefunction
    survives the step."""
    lg = coupling.couples_in_x
    K = int(order)
    rows = np.zeros((nsteps * K, 6 if lg else 3))
    for s in range(nsteps):
        t_start = timer
        t = t_start
        for chain in range(1, K + 1):
            t = t_start
            vals = []
            for si, mult in enumerate(chain_mults(chain)):
                if (si % 2 == 0) == lg:
                    coupling.precalc(t)
                    vals.append(list(coupling.vector()))
                    t += dt * (mult * 1.0)
            if chain == K:
                for k in range(K):
                    if lg:
                        rows[s * K + k, 0:3] = vals[k]
                        rows[s * K + k, 3:6] = vals[k + 1]
                    else:
                        rows[s * K + k, 0:3] = vals[k]
        timer = t
    return rows, timer


# BufferedOutputs column classes (computations.h:58-111): VALUE and CHANGE fill the
# plain buffer, AVG, FLUX and SUM of AVGs the reduced one; OPERATION stores nothing.
_PLAIN_OUTPUTS = ("time", "step", "ediff")
_REDUCED_OUTPUTS = ("norm", "epot", "ekin", "etot")
DAT_FORMAT = "|%13.5g "  # FMT_DOUBLE (constants.h:15); a row ends with FMT_END "\n"


def dat_columns(outputs: list) -> List[tuple]:
    """Column order of a .dat row (buffer.h:296-338): the plain-buffer entries in
    declaration order, then the reduced-buffer entries in declaration order.  Each item
    is (output name, index within a flux entry or None)."""
    plain = [(o, None) for o in outputs if isinstance(o, str) and o in _PLAIN_OUTPUTS]
    reduced = []
    for o in outputs:
        if _is_flux(o):
            reduced += [("flux", i) for i in range(len(o[1]))]
        elif isinstance(o, str) and o in _REDUCED_OUTPUTS:
            reduced.append((o, None))
    return plain + reduced


def dat_values(rows: List[dict], outputs: list) -> np.ndarray:
    """The rows as the (n_rows, n_columns) matrix a .dat file holds."""
    cols = dat_columns(outputs)
    out = np.empty((len(rows), len(cols)), dtype=np.float64)
    for r, row in enumerate(rows):
        for c, (name, i) in enumerate(cols):
            v = row.get(name, 0.0)
            out[r, c] = v[i] if i is not None else v
    return out


def write_dat(path: str, rows: List[dict], outputs: list, binary: bool = False) -> None:
    """Write rows in the reference's .dat layout (BufferedOutputs::logOrPass,
    buffer.h:296-338): text rows of FMT_DOUBLE fields, or raw doubles row after row."""
    vals = dat_values(rows, outputs)
    if binary:
        with open(path, "wb") as f:
            f.write(np.ascontiguousarray(vals, dtype="<f8").tobytes())
        return
    with open(path, "w") as f:
        for row in vals:
            f.write("".join(DAT_FORMAT % v for v in row) + "\n")


def read_dat(path: str, outputs: list, binary: bool = False) -> np.ndarray:
    """Inverse of write_dat (the reader side of flx.wl / wf.wl): (n_rows, n_columns)."""
    ncol = len(dat_columns(outputs))
    if binary:
        return np.fromfile(path, dtype="<f8").reshape(-1, ncol)
    rows = []
    with open(path) as f:
        for line in f:
            fields = [t.strip() for t in line.rstrip("\n").split("|")[1:]]
            rows.append([float(t) for t in fields])
    return np.array(rows, dtype=np.float64).reshape(-1, ncol)


class SplitPropagator:
    def __init__(self, mode: int, dt: float, max_steps: int, grid: Grid, coupling: Coupling, outputs: list,
                 state_accuracy: float = 0.0, order: int = 1, ekin_interval: int = 1):
        """SplitPropagator<M, MultiProductSplit<Split3Base<X,P,X>, order>, Spin0<...>>.

        ekin_interval = k > 1: the "ekin" / "etot" outputs are evaluated on every k-th
        step of each fused call and on its last step (rows in between carry E_kin = 0),
        so the steps between stay fused; 1 (the default) evaluates them every step as
        the reference's computeEach does."""
        self.order = int(order)
        self.ekin_interval = max(1, int(ekin_interval))
        if not 1 <= self.order <= 64:
            raise ValueError("order must be in [1, 64]")
        self.mode = mode
        self.dt = dt
        self.grid = grid
        self.coupling = coupling
        self.outputs = list(outputs)
        self.state_accuracy = state_accuracy
        self.step = 0
        self.timer = 0.0
        self.rows: List[dict] = []
        self._last_change = 0.0
        self.dif_energy = float("inf")
        if mode == MODE_RE:
            # propagator.h:118-127
            self.max_steps = int(coupling.max_pulse_duration() / dt + 1)
            self.state_accuracy = 0.0
        else:
            self.max_steps = int(max_steps)
        self.flux_spec = next((o for o in self.outputs if _is_flux(o)), None)

    # ------------------------------------------------------------ schedule
    chain_mults = staticmethod(chain_mults)

    def _schedule(self, nsteps: int) -> np.ndarray:
        """Coupling rows for the next nsteps steps; advances timer and coupling state."""
        rows, self.timer = coupling_schedule(self.coupling, self.dt, nsteps, self.timer, self.order)
        return rows

    # ------------------------------------------------------------ outputs
    def _x_order(self):
        return [o for o in self.outputs if o in ("norm", "epot", "normalize", "time", "step") or _is_flux(o)]

    def _finish_row(self, raw: dict, step: int, time: float) -> dict:
        """Apply computeEach's declaration-order semantics to raw (pre-Normalize) values."""
        row = {}
        scaled = False
        nrm = raw["norm"]
        for o in self._x_order():
            f = 1.0 / nrm if scaled else 1.0
            if o == "normalize":
                scaled = True
            elif o == "norm":
                row["norm"] = raw["norm"] * f
            elif o == "epot":
                row["epot"] = raw["epot"] * f
            elif o == "time":
                row["time"] = time
            elif o == "step":
                row["step"] = float(step)
            elif _is_flux(o):
                row["flux"] = [v * f for v in raw["flux"]]
        if "ekin" in self.outputs:
            row["ekin"] = raw["ekin"] * (1.0 / nrm if "normalize" in self.outputs else 1.0)
        for o in self.outputs:
            if o == "etot":
                row["etot"] = row["epot"] + row["ekin"]
            elif o == "ediff":
                cur = row["epot"] + row["ekin"]
                row["ediff"] = cur - self._last_change
                self.dif_energy = cur - self._last_change
                self._last_change = cur
        return row

    def _energy_after_normalize(self) -> int:
        if "normalize" not in self.outputs:
            return 0
        order = self._x_order()
        bits = 1 if ("epot" in order and order.index("epot") > order.index("normalize")) else 0
        return bits | (2 if "ekin" in self.outputs else 0)

    def compute_at_start(self) -> dict:
        """computeEach<AT_START> with the granular members (no step has run yet)."""
        g = self.grid
        raw = {"norm": g.average(REP_X, OP_IDENTITY), "epot": 0.0, "ekin": 0.0, "flux": []}
        if "epot" in self.outputs:
            raw["epot"] = g.average(REP_X, OP_POTENTIAL)
        if self.flux_spec:
            A = None if self.coupling.couples_in_x else self.coupling.vector()
            raw["flux"] = g.flux(self.flux_spec[1], self.flux_spec[2], A)
        if "ekin" in self.outputs:
            g.fourier(REP_P)
            raw["ekin"] = g.average(REP_P, OP_KINETIC)
            g.fourier(REP_X)
        if "normalize" in self.outputs:
            g.normalize()
        return self._finish_row(raw, self.step, self.timer)

    # ------------------------------------------------------------ run
    def _obs_mask(self) -> int:
        m = OBS_NORM
        if "epot" in self.outputs or "etot" in self.outputs or "ediff" in self.outputs:
            m |= OBS_EPOT
        if "ekin" in self.outputs:
            m |= OBS_EKIN
        return m

    def run_steps(self, nsteps: int, stop_on_convergence: bool = False):
        """Run up to nsteps fused steps; returns the number of steps that ran."""
        if nsteps <= 0:
            return 0
        timer0 = self.timer
        coup_state = (list(self.coupling.last), list(self.coupling.prev_time))
        sched = self._schedule(nsteps)
        borders = self.flux_spec[1] if self.flux_spec else ()
        box = self.flux_spec[2] if self.flux_spec else 0
        acc = self.state_accuracy if (stop_on_convergence and self.mode == MODE_IM) else 0.0
        rows, done = self.grid.step(self.mode, self.dt, nsteps, sched if self.coupling.size else None,
                                    obs=self._obs_mask(), normalize="normalize" in self.outputs, borders=borders,
                                    box_size=box, state_accuracy=acc, last_energy=self._last_change,
                                    energy_after_normalize=self._energy_after_normalize(), substeps=self.order,
                                    ekin_interval=self.ekin_interval)
        if done < nsteps:
            # the schedule ran ahead of the device: replay the host state to `done` steps
            self.timer = timer0
            self.coupling.last, self.coupling.prev_time = coup_state
            self._schedule(done)
        times = self._times(timer0, done)
        for s in range(done):
            nb = len(borders)
            raw = {"norm": rows[s, 0], "epot": rows[s, 1], "ekin": rows[s, 2], "flux": list(rows[s, 3:3 + nb])}
            self.step += 1
            self.rows.append(self._finish_row(raw, self.step, times[s]))
        return done

    def write_dat(self, name: str, binary: bool = False) -> str:
        """<name>.dat with one row per computed step (comp_interval 1), as
        BufferedOutputs writes it (buffer.h:89-91, 296-338); returns the path."""
        path = name + ".dat"
        write_dat(path, self.rows, self.outputs, binary)
        return path

    def _times(self, t0: float, n: int) -> List[float]:
        """Timer after each of n steps: the last chain's increments (incrementBy,
        propagator.h:327-330) over the sub-steps of the coupling's representation."""
        lg = self.coupling.couples_in_x
        incs = [m for si, m in enumerate(chain_mults(self.order)) if (si % 2 == 0) == lg]
        out = []
        t = t0
        for _ in range(n):
            for m in incs:
                t += self.dt * (m * 1.0)
            out.append(t)
        return out

    def run(self, restore: bool = False) -> List[dict]:
        """SplitPropagator::run (propagator.h:420-462).  With restore, the step stored in
        backup.info is read, the timer and coupling are fast-forwarded to it without
        evolving (makeFakeStep, propagator.h:362-366) and the backed-up psi is loaded;
        the AT_START outputs are then skipped.  At the end backup.info and the backup
        file are removed, as the reference does."""
        if restore:
            with open("backup.info", "rb") as f:
                atstep = struct.unpack("<q", f.read(8))[0]
            if atstep > self.step:
                self._schedule(atstep - self.step)
                self.step = atstep
            self.grid.restore()
        else:
            self.rows.append(self.compute_at_start())
        if self.mode == MODE_RE:
            # loop while step <= max_steps, then the final step (propagator.h:443-451)
            self.run_steps(max(0, self.max_steps + 1 - self.step) + 1)
        else:
            if not (abs(self.dif_energy) > self.state_accuracy) or self.step == self.max_steps:
                self.run_steps(1)
            else:
                self.run_steps(self.max_steps + 1 - self.step, stop_on_convergence=self.state_accuracy > 0.0)
        if os.path.exists("backup.info"):
            os.remove("backup.info")
        self.grid.remove_backups()
        return self.rows
