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

from typing import List, Optional

import numpy as np

from .grid import (Grid, MODE_IM, MODE_RE, OBS_EKIN, OBS_EPOT, OBS_NORM, OP_IDENTITY, OP_KINETIC, OP_POTENTIAL,
                   REP_P, REP_X)
from .physics import Coupling


def _is_flux(o) -> bool:
    return isinstance(o, tuple) and o[0] == "flux"


class SplitPropagator:
    def __init__(self, mode: int, dt: float, max_steps: int, grid: Grid, coupling: Coupling, outputs: list,
                 state_accuracy: float = 0.0):
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
    def _schedule(self, nsteps: int) -> np.ndarray:
        """Coupling rows for the next nsteps steps; advances timer and coupling state.

        Velocity gauge: A at the P sub-step (precalc at the step's start time, then the
        timer advances by dt).  Length gauge: E at the first X half, timer += dt/2,
        E at the second X half, timer += dt/2 (propagator.h:319-329)."""
        c = self.coupling
        lg = c.couples_in_x
        rows = np.zeros((nsteps, 6 if lg else 3))
        for s in range(nsteps):
            if lg:
                c.precalc(self.timer)
                rows[s, 0:3] = c.vector()
                self.timer += self.dt * (0.5 * 1.0)
                c.precalc(self.timer)
                rows[s, 3:6] = c.vector()
                self.timer += self.dt * (0.5 * 1.0)
            else:
                c.precalc(self.timer)
                rows[s, 0:3] = c.vector()
                self.timer += self.dt * (1.0 * 1.0)
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
                                    energy_after_normalize=self._energy_after_normalize())
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

    def _times(self, t0: float, n: int) -> List[float]:
        out = []
        t = t0
        for _ in range(n):
            if self.coupling.couples_in_x:
                t += self.dt * (0.5 * 1.0)
                t += self.dt * (0.5 * 1.0)
            else:
                t += self.dt * (1.0 * 1.0)
            out.append(t)
        return out

    def run(self) -> List[dict]:
        self.rows.append(self.compute_at_start())
        if self.mode == MODE_RE:
            # loop while step <= max_steps, then the final step (propagator.h:443-451)
            self.run_steps(self.max_steps + 2)
        else:
            if not (abs(self.dif_energy) > self.state_accuracy):
                self.run_steps(1)
            else:
                self.run_steps(self.max_steps + 1, stop_on_convergence=self.state_accuracy > 0.0)
        return self.rows
