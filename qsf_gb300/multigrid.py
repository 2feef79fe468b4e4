"""Multi-region grids on one GPU: the reference's CAP<MultiCartesianGrid<D>> (multigrid.h).

The reference runs a multi-region grid as one MPI job whose processes are split into
regions (MultiRegionsReduced<D>, mpi_logic.h:262-278): NO, X for D = 1; NO, X, Y, XY for
D = 2; NO, X, Y, Z, XY, XZ, YZ, XYZ for D = 3.  Region r holds a whole wavefunction
whose free axes (the letters) stay in momentum space; its group is the number of free
axes.  Every process makes the same Strang step on its own region (partial potential,
potential.h:144-178; Fourier transforms along the bounded axes only, multigrid.h:660-674;
no absorber in evolve, grid.h:408), the main region (group 0) alone computes the
outputs (calcsEnabled, mpi_logic.h:247), and postCompute (multigrid.h:617-625) moves
what the absorber margins hold into the regions with one more free axis (transfer,
multigrid.h:627-657: mask, one-axis DFT, coherent addition) and then masks every region
outside the last group (maskRegion, grid.h:582-597).

Here all regions live on the device of one process, each a Grid created with
multi_region=True and its free-axis mask, each on its own stream so that their steps
overlap; qsf_region_transfer orders the streams of the two regions it joins.  Every
region sees the same coupling values (the reference's processes advance identical
coupling states), computed once per sub-step.
"""
from __future__ import annotations

from typing import List, Optional, Sequence

from .grid import Grid, MODE_RE, OP_IDENTITY, OP_KINETIC, OP_POTENTIAL, REP_P, REP_X
from .physics import Coupling
from .propagator import chain_mults

REGIONS = {1: [0, 1], 2: [0, 1, 2, 3], 3: [0, 1, 2, 4, 3, 5, 6, 7]}


def region_sources(dim: int) -> List[List[tuple]]:
    """Per region, its sources (region index, transferred axis) in the order
    LocalGrid::init builds them (multigrid.h:127-146): the regions with one free axis
    fewer whose free set differs by exactly one axis."""
    regs = REGIONS[dim]
    out = []
    for fr in regs:
        src = []
        for i, fi in enumerate(regs):
            if bin(fr).count("1") - bin(fi).count("1") == 1 and (fr ^ fi) in (1, 2, 4):
                src.append((i, (fr ^ fi).bit_length() - 1))
        out.append(src)
    return out


class MultiGrid:
    """The regions of one multi-region grid; arguments as Grid's (nCAP >= 1 required)."""

    def __init__(self, dim: int, n, dx, nCAP: int, **grid_kwargs):
        self.dim = dim
        self.free = REGIONS[dim]
        self.groups = [bin(f).count("1") for f in self.free]
        self.sources = region_sources(dim)
        self.regions = [Grid(dim, n, dx, nCAP=nCAP, free_axes=f, multi_region=True, **grid_kwargs)
                        for f in self.free]

    @property
    def main(self) -> Grid:
        return self.regions[0]

    def close(self):
        for g in self.regions:
            g.close()

    def post_compute(self) -> None:
        """transfer() then maskRegion() (multigrid.h:617-657): group by group, each region
        adds its sources in order; then every region outside the last group is masked."""
        last = max(self.groups)
        for gi in range(1, last + 1):
            for si in range(gi):
                for r, g in enumerate(self.regions):
                    if self.groups[r] == gi:
                        src, axis = self.sources[r][si]
                        g.region_transfer(self.regions[src], axis, gi)
        for r, g in enumerate(self.regions):
            if self.groups[r] != last:
                g.mask_region([0 if (self.free[r] >> d) & 1 else 1 for d in range(self.dim)])

    def synchronize(self) -> None:
        for g in self.regions:
            g.synchronize()


class MultiRegionPropagator:
    """SplitPropagator<MODE::RE, Split3Base<X,P,X>, Spin0<CAP<MultiCartesianGrid<D>>>>
    (propagator.h:420-462 with the multi-region postCompute).  Outputs of the main
    region: "step", "time", "norm", "epot", "ekin"."""

    OUTPUTS = ("step", "time", "norm", "epot", "ekin")

    def __init__(self, dt: float, mg: MultiGrid, coupling: Coupling, outputs: Sequence[str]):
        for o in outputs:
            if o not in self.OUTPUTS:
                raise ValueError(f"output {o!r} is not available on multi-region grids")
        self.dt = dt
        self.mg = mg
        self.coupling = coupling
        self.outputs = list(outputs)
        self.timer = 0.0
        self.step = 0
        self.rows: List[dict] = []
        self._slots: List[dict] = []  # per row: output -> slot of the device log
        # propagator.h:118-127
        self.max_steps = int(coupling.max_pulse_duration() / dt + 1)

    def _make_step(self) -> None:
        """chainEvolve (propagator.h:311-328) on every region with shared coupling values."""
        c = self.coupling
        couples = REP_X if c.couples_in_x else REP_P
        for si, mult in enumerate(chain_mults(1)):
            rep = REP_X if si % 2 == 0 else REP_P
            cv: Optional[List[float]] = None
            if rep == couples:
                c.precalc(self.timer)
                if c.size:
                    cv = c.vector()[: self.mg.dim]
            for g in self.mg.regions:
                if si > 0:
                    g.fourier(rep)
                g.evolve(MODE_RE, rep, self.dt * mult, cv)
            if rep == couples:
                self.timer += self.dt * (mult * 1.0)
        self.step += 1

    def _compute_each(self) -> None:
        """The main region's outputs; the averages go into the grid's device log (no
        host wait, so the loop runs ahead of the GPU) and fill the rows at the end."""
        g = self.mg.main
        row, slots = {}, {}
        base = 3 * len(self.rows)
        for o in self.outputs:
            if o == "step":
                row["step"] = float(self.step)
            elif o == "time":
                row["time"] = self.timer
            elif o == "norm":
                g.average_log(REP_X, OP_IDENTITY, base)
                slots["norm"] = base
            elif o == "epot":
                g.average_log(REP_X, OP_POTENTIAL, base + 1)
                slots["epot"] = base + 1
        if "ekin" in self.outputs:
            g.fourier(REP_P)
            g.average_log(REP_P, OP_KINETIC, base + 2)
            slots["ekin"] = base + 2
            g.fourier(REP_X)
        self.rows.append(row)
        self._slots.append(slots)

    def _finish_rows(self) -> None:
        if not any(self._slots):
            return
        vals = self.mg.main.read_log(1 + max(k for sl in self._slots for k in sl.values()))
        for row, slots in zip(self.rows, self._slots):
            for o, k in slots.items():
                row[o] = float(vals[k])

    def run(self) -> List[dict]:
        """The time loop of SplitPropagator::run (propagator.h:442-453)."""
        self._compute_each()
        while self.step <= self.max_steps:
            self._make_step()
            self._compute_each()
            self.mg.post_compute()
        self._make_step()
        self._compute_each()
        self.mg.post_compute()
        self.mg.synchronize()
        self._finish_rows()
        return self.rows
