"""CPU oracle for QSF's split-operator step -- TEST INFRASTRUCTURE ONLY.

Only tests/, the smoke check in __graft_entry__.py and the cpu_baseline / reference
legs of bench.py import this module; the product package never does.

It wraps the C restatement in qsf_oracle.c (built into oracle/liboracle.so) and adds
the propagator loop of the reference in Python:

* ``Propagator.run``       -- SplitPropagator::run            propagator.h:420-462
* ``Propagator.make_step`` -- makeStep / chainEvolve (Strang) propagator.h:311-346,
                              Split3Base mults {0.5, 1, 0.5}  splitting.h:18-27
* ``Propagator.compute_each`` -- computeEach                   propagator.h:275-300
* ``Coupling``             -- CouplingBase / DipoleCoupling    coupling.h:43-78, 101-118
                              with PromoteFieldToA             field.h:114-123
"""
from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

MODE_IM, MODE_RE = 1, 2
REP_X, REP_P = 1, 2
OP_IDENTITY, OP_POTENTIAL, OP_KINETIC = 0, 1, 2
POT_EBERLY, POT_ECKHARDT_SACHA, POT_COULOMB, POT_NONE = 0, 1, 2, 3
ABS_CAP, ABS_COS8 = 0, 1
GAUGE_VELOCITY, GAUGE_LENGTH = 0, 1
PULSE_SIN, PULSE_SIN2_SIN, PULSE_CONST, PULSE_CHEMPHYS = 0, 1, 2, 3

BORDERS = {
    "BOX": 0, "S2CAP": 1, "D2CAP": 2, "N2S": 3, "N2D": 4, "N2D_SYM": 5, "N2D_ASYM": 6,
    "S2D": 7, "S2D_SYM": 8, "S2D_ASYM": 9, "N2T": 10, "S2T": 11, "D2T": 12, "T2CAP": 13,
}
# computations.h:68-70
ZOA_FLUX_3D = ["N2S", "N2D", "N2T", "S2D", "S2T", "S2CAP", "D2CAP", "T2CAP"]
ZOA_FLUX_2D = ["N2S", "N2D_SYM", "N2D_ASYM", "S2D_SYM", "S2D_ASYM", "S2CAP", "D2CAP"]


def build(force: bool = False) -> str:
    """Compile qsf_oracle.c into oracle/liboracle.so (gcc, no FMA contraction)."""
    so = os.path.join(_HERE, "liboracle.so")
    src = os.path.join(_HERE, "qsf_oracle.c")
    if force or not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        cmd = (f"gcc -std=c11 -O2 -ffp-contract=off -fPIC -shared -o {so}.tmp {src} -lm && "
               f"mv {so}.tmp {so}")
        rc = os.system(cmd)
        if rc != 0:
            raise RuntimeError("building the oracle failed: " + cmd)
    return so


def lib():
    global _LIB
    if _LIB is None:
        _LIB = ctypes.CDLL(build())
        L = _LIB
        dp = ctypes.POINTER(ctypes.c_double)
        lp = ctypes.POINTER(ctypes.c_long)
        ip = ctypes.POINTER(ctypes.c_int)
        L.orc_sizeof_grid.restype = ctypes.c_int
        L.orc_grid_init.argtypes = [ctypes.c_void_p, ctypes.c_int, lp, dp, ctypes.c_long, ctypes.c_int,
                                    ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_int, ctypes.c_int]
        L.orc_fft_nd.argtypes = [dp, ctypes.c_int, lp, ctypes.c_int]
        L.orc_evolve.argtypes = [ctypes.c_void_p, dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, dp]
        L.orc_fourier.argtypes = [ctypes.c_void_p, dp, ctypes.c_int]
        L.orc_average.argtypes = [ctypes.c_void_p, dp, ctypes.c_int, ctypes.c_int]
        L.orc_average.restype = ctypes.c_double
        L.orc_average_der.argtypes = [ctypes.c_void_p, dp, ctypes.c_int]
        L.orc_average_der.restype = ctypes.c_double
        L.orc_antisymmetrize.argtypes = [ctypes.c_void_p, dp, ctypes.c_int]
        L.orc_antisymmetrize.restype = None
        L.orc_normalize.argtypes = [ctypes.c_void_p, dp]
        L.orc_normalize.restype = ctypes.c_double
        L.orc_current_map.argtypes = [ctypes.c_void_p, dp, dp, dp]
        L.orc_flux.argtypes = [ctypes.c_void_p, dp, ctypes.c_int, ctypes.c_long]
        L.orc_flux.restype = ctypes.c_double
        L.orc_border.argtypes = [ctypes.c_int, ctypes.c_long, ctypes.c_int, lp, dp]
        L.orc_set_border_nodes.argtypes = [ctypes.c_long] * 4
        L.orc_mask_region.argtypes = [ctypes.c_void_p, dp, ip]
        L.orc_add_gaussian.argtypes = [ctypes.c_void_p, dp, ctypes.c_double, ctypes.c_double]
        L.orc_field_eval.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double]
        L.orc_field_eval.restype = ctypes.c_double
        L.orc_field_max_duration.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_field_max_duration.restype = ctypes.c_double
        L.orc_grid_set_region.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.orc_grid_set_absorber.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double]
        L.orc_mg_transfer.argtypes = [ctypes.c_void_p, dp, dp, ctypes.c_int, ctypes.c_int]
    return _LIB


def _dp(a: np.ndarray):
    assert a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def fft_nd(psi: np.ndarray, sign: int) -> np.ndarray:
    """Unnormalised in-place N-D DFT (sign -1 forward, +1 backward) of a complex128 array."""
    a = np.ascontiguousarray(psi, dtype=np.complex128).copy()
    n = (ctypes.c_long * a.ndim)(*a.shape)
    lib().orc_fft_nd(_dp(a.view(np.float64)), a.ndim, n, sign)
    return a


class _Pulse(ctypes.Structure):
    _fields_ = [("shape", ctypes.c_int), ("field", ctypes.c_double), ("omega", ctypes.c_double),
                ("ncycles", ctypes.c_double), ("FWHM_percent", ctypes.c_double),
                ("phase_in_pi_units", ctypes.c_double), ("delay_in_cycles", ctypes.c_double)]


@dataclass
class Pulse:
    """_FieldConfig + pulse shape (field_p.h:6-12, 30-33)."""
    field: float
    omega: float
    ncycles: float
    phase_in_pi_units: float = 0.0
    delay_in_cycles: float = 0.0
    FWHM_percent: float = 0.0
    shape: int = PULSE_SIN2_SIN


@dataclass
class Field:
    """Field<AXIS, Pulses...> (field.h:9-53); axis is a bit mask (1=X, 2=Y, 4=Z)."""
    axis: int
    pulses: List[Pulse]

    def _arr(self):
        arr = (_Pulse * len(self.pulses))()
        for i, p in enumerate(self.pulses):
            arr[i] = _Pulse(p.shape, p.field, p.omega, p.ncycles, p.FWHM_percent,
                            p.phase_in_pi_units, p.delay_in_cycles)
        return arr

    def value(self, t: float) -> float:
        a = self._arr()
        return lib().orc_field_eval(ctypes.cast(a, ctypes.c_void_p), len(self.pulses), t)

    def max_duration(self) -> float:
        a = self._arr()
        return lib().orc_field_max_duration(ctypes.cast(a, ctypes.c_void_p), len(self.pulses))


class Coupling:
    """DipoleCoupling<Gauge, Fields...>.  Velocity gauge promotes each field to A(t) by
    the rectangle rule of PromoteFieldToA (field.h:114-123); the length gauge keeps E(t)."""

    def __init__(self, gauge: int, fields: Sequence[Field] = ()):
        self.gauge = gauge
        self.fields = list(fields)
        self.last = [0.0] * len(self.fields)
        self.prev_time = [0.0] * len(self.fields)
        self.couples_in = REP_P if gauge == GAUGE_VELOCITY else REP_X

    @property
    def size(self) -> int:
        return len(self.fields)

    def max_pulse_duration(self) -> float:
        # CouplingBase::maxPulseDuration = Max(0.0, fields...)  coupling.h:53
        m = 0.0
        for f in self.fields:
            m = max(m, f.max_duration())
        return m

    def precalc(self, time: float) -> None:
        for i, f in enumerate(self.fields):
            F = f.value(time)
            if self.gauge == GAUGE_VELOCITY:
                prev = self.last[i]
                self.last[i] = prev + (self.prev_time[i] - time) * F
                self.prev_time[i] = time
            else:
                self.last[i] = F

    def vector(self, dim: int) -> List[float]:
        """operator[](Axis<d>) for d < dim  (coupling.h:63-67)."""
        out = []
        for d in range(3):
            s = 0.0
            first = True
            for f, v in zip(self.fields, self.last):
                term = v if (f.axis >> d) & 1 else 0.0
                s = term if first else s + term
                first = False
            out.append(s)
        return out


class Grid:
    """LocalGrid over CAP<CartesianGrid<dim>> with a Spin0 Hamiltonian."""

    def __init__(self, dim: int, n, dx, nCAP: int = 0, pot: int = POT_EBERLY, Ncharge: float = 1.0,
                 Echarge: float = -1.0, Nsoft: float = 1.0, Esoft: float = 1.0,
                 coupling: Optional[Coupling] = None):
        self.dim = dim
        n = [int(n)] * dim if np.isscalar(n) else [int(v) for v in n]
        dx = [float(dx)] * dim if np.isscalar(dx) else [float(v) for v in dx]
        self.n, self.dx = n, dx
        self.coupling = coupling if coupling is not None else Coupling(GAUGE_VELOCITY)
        self._buf = ctypes.create_string_buffer(lib().orc_sizeof_grid())
        nn = (ctypes.c_long * 3)(*(n + [1] * (3 - dim)))
        dd = (ctypes.c_double * 3)(*(dx + [1.0] * (3 - dim)))
        lib().orc_grid_init(self._buf, dim, nn, dd, nCAP, pot, Ncharge, Echarge, Nsoft, Esoft,
                            self.coupling.gauge, self.coupling.size)
        self.psi = np.zeros(tuple(n), dtype=np.complex128)
        self.m = int(np.prod(n))

    @property
    def shape(self):
        return tuple(self.n)

    def _p(self):
        return _dp(self.psi.view(np.float64))

    def add_gaussian(self, at: float = 0.0, delta: float = 1.0):
        lib().orc_add_gaussian(self._buf, self._p(), at, delta)

    def evolve(self, mode: int, rep: int, delta: float, cv=None):
        arr = (ctypes.c_double * 3)(*(cv if cv is not None else [0.0, 0.0, 0.0]))
        lib().orc_evolve(self._buf, self._p(), mode, rep, delta, arr)

    def fourier(self, to_rep: int):
        lib().orc_fourier(self._buf, self._p(), to_rep)

    def average(self, rep: int, op: int) -> float:
        return lib().orc_average(self._buf, self._p(), rep, op)

    def normalize(self) -> float:
        return lib().orc_normalize(self._buf, self._p())

    def current_map(self, A_vg=None) -> np.ndarray:
        curr = np.zeros(self.m * self.dim, dtype=np.float64)
        arr = None
        if A_vg is not None:
            arr = (ctypes.c_double * 3)(*A_vg)
        lib().orc_current_map(self._buf, self._p(), arr, _dp(curr))
        return curr

    def flux(self, curr: np.ndarray, border: str, box_size: int = 0) -> float:
        return lib().orc_flux(self._buf, _dp(curr), BORDERS[border], box_size)

    def mask_region(self, bounded):
        b = (ctypes.c_int * 3)(*(list(bounded) + [1] * (3 - len(bounded))))
        lib().orc_mask_region(self._buf, self._p(), b)

    def set_absorber(self, kind: int, mask_dt: float = 0.0):
        """Absorber kind: ABS_CAP (absorbers.h, the default) or ABS_COS8, the cos^(1/8)
        mask over the same nCAP-node margins applied once per mask_dt of propagation
        (orc_grid_set_absorber)."""
        lib().orc_grid_set_absorber(self._buf, int(kind), float(mask_dt))

    def set_region(self, free_mask: int, multi: bool = True):
        """Make this grid region `free_mask` (bit d: axis d kept in P space) of a
        multi-region grid (multigrid.h, mpi_logic.h:104-150): partial potentials, no
        absorber in evolve, fourier along the bounded axes only, untransposed P layout
        unless it is the main region."""
        self.free_mask = int(free_mask)
        lib().orc_grid_set_region(self._buf, int(free_mask), 1 if multi else 0)

    def mg_transfer_from(self, src: "Grid", fc: int, group: int):
        """psi += FFT_fc(margins of src.psi along axis fc, masked) (multigrid.h:454-615)."""
        lib().orc_mg_transfer(self._buf, self._p(), src._p(), int(fc), int(group))

    def average_der(self, direction: int) -> float:
        """average_der<X, direction, PotentialEnergy> (grid.h:443-465)."""
        return lib().orc_average_der(self._buf, self._p(), int(direction))

    def antisymmetrize(self, particles: int):
        """operation<M, R, AntiSymmetrize<particles>> (grid.h:611-723)."""
        lib().orc_antisymmetrize(self._buf, self._p(), int(particles))


def border_vector(border: str, dim: int, ci, box_size: int = 0) -> List[float]:
    out = (ctypes.c_double * 3)()
    c = (ctypes.c_long * 3)(*(list(ci) + [0] * (3 - len(ci))))
    lib().orc_border(BORDERS[border], box_size, dim, c, out)
    return list(out)[:dim]


def set_border_nodes(p_NS=25, p_SD=14, p_DT=10, p_CAP=40):
    """Reference globals p_NS/p_SD/p_DT/p_CAP (borders.h:30-36)."""
    lib().orc_set_border_nodes(p_NS, p_SD, p_DT, p_CAP)


# ------------------------------------------------------------------ outputs
# An output list mirrors BufferedOutputs<..., Ts...>: entries are
#   "norm"   AVG<Identity>            (rep X)
#   "epot"   AVG<PotentialEnergy>     (rep X)
#   "ekin"   AVG<KineticEnergy>       (rep P)
#   "normalize" OPERATION<Normalize>  (rep NONE, first pass)
#   ("flux", [borders...], box_size)  FLUX<B...> (rep X)
#   "etot"   ENERGY_TOTAL  = SUM<AVG<Pot>, AVG<Kin>>        (late)
#   "ediff"  ENERGY_DIFFERENCE = CHANGE<ENERGY_TOTAL>        (late)
#   "time", "step"  VALUE<Time>, VALUE<Step>                 (rep NONE)


def _rep_of(o):
    if isinstance(o, tuple):
        return REP_X
    return {"norm": REP_X, "epot": REP_X, "ekin": REP_P, "normalize": 0, "time": 0, "step": 0,
            "etot": -1, "ediff": -1}[o]


@dataclass
class Propagator:
    """SplitPropagator<M, Split3Base<X,P,X>, Spin0<...>> (propagator.h:51-494)."""
    mode: int
    dt: float
    max_steps: int
    grid: Grid
    outputs: list
    state_accuracy: float = 0.0
    step: int = 0
    timer: float = 0.0
    rows: list = field(default_factory=list)
    _last_change: float = 0.0
    dif_energy: float = float("inf")
    tot_energy: float = 0.0

    def __post_init__(self):
        if self.mode == MODE_RE:
            # propagator.h:118-127  max_steps = maxPulseDuration / dt + 1 (truncated to ind)
            self.max_steps = int(self.grid.coupling.max_pulse_duration() / self.dt + 1)
            self.state_accuracy = 0.0

    # propagator.h:304-309
    def should_continue(self) -> bool:
        if self.mode == MODE_RE:
            return self.step <= self.max_steps
        return abs(self.dif_energy) > self.state_accuracy and self.step != self.max_steps

    order: int = 1  # MultiProductSplit<Split3Base<X,P,X>, order>

    @staticmethod
    def chain_mults(chain: int) -> List[float]:
        """_SplitChain::pack for Split3Base with `chain` coefficients 1/chain, joined X
        sub-steps (splitting.h:43-58): X, then (P, X) `chain` times."""
        c = 1.0 / chain
        arr = [0.0] * (2 * chain + 1)
        for j in range(chain):
            for k, mult in enumerate((0.5, 1.0, 0.5)):
                arr[2 * j + k] += mult * c
        return arr

    @staticmethod
    def chain_value(chain: int, order: int) -> float:
        """MultiProductSplit::Chain::value (splitting.h:82-85)."""
        v = 1.0
        for j in range(1, order + 1):
            v *= (float(chain * chain) / (float(chain * chain) - float(j * j))) if j != chain else 1.0
        return v

    # propagator.h:311-328 chainEvolve
    def _chain_evolve(self, chain: int):
        g = self.grid
        c = g.coupling
        mults = self.chain_mults(chain)
        for si, mult in enumerate(mults):
            rep = REP_X if si % 2 == 0 else REP_P
            if si > 0:
                g.fourier(rep)
            if rep == c.couples_in:
                c.precalc(self.timer)
            cv = c.vector(g.dim) if (rep == c.couples_in and c.size) else None
            g.evolve(self.mode, rep, self.dt * mult, cv)
            if rep == c.couples_in:
                self.timer += self.dt * (mult * 1.0)

    # propagator.h:331-343 makeStep with chainBackup / chainRestore / chainComplete
    # (propagator.h:369-413) for order > 1, restated as written: the last chain is
    # completed at `chain == ChainCount - 1`, so for order >= 2 the result of the step
    # is the last chain's wavefunction alone.
    def make_step(self):
        g = self.grid
        K = self.order
        if K > 1:
            psi_copy = g.psi.copy()
            psi_acc = np.zeros_like(g.psi)
            timer_copy = self.timer
        for chain in range(1, K + 1):
            if K > 1 and chain > 1:
                self.timer = timer_copy
                g.psi[...] = psi_copy
            self._chain_evolve(chain)
            if K > 1:
                v = self.chain_value(chain, K)
                if chain == K - 1:
                    g.psi[...] = v * g.psi + psi_acc
                else:
                    psi_acc += v * g.psi
        self.step += 1

    # propagator.h:275-300 (+ 259-265 flux, 249-257 velocity-gauge correction)
    def compute_each(self):
        g = self.grid
        row = {}
        for o in self.outputs:
            r = _rep_of(o)
            if r in (0, REP_X):
                self._compute(o, row)
        if any(_rep_of(o) == REP_P for o in self.outputs):
            g.fourier(REP_P)
            for o in self.outputs:
                if _rep_of(o) == REP_P:
                    row["ekin"] = g.average(REP_P, OP_KINETIC)
            g.fourier(REP_X)
        for o in self.outputs:
            if _rep_of(o) == -1:
                self._compute(o, row)
        self.rows.append(row)

    def _compute(self, o, row):
        g = self.grid
        if isinstance(o, tuple):
            _, borders, box = o
            A = None
            if g.coupling.couples_in == REP_P:
                A = g.coupling.vector(g.dim)
            curr = g.current_map(A)
            row["flux"] = [g.flux(curr, b, box) for b in borders]
        elif o == "norm":
            row["norm"] = g.average(REP_X, OP_IDENTITY)
        elif o == "epot":
            row["epot"] = g.average(REP_X, OP_POTENTIAL)
        elif o == "normalize":
            g.normalize()
        elif o == "time":
            row["time"] = self.timer
        elif o == "step":
            row["step"] = float(self.step)
        elif o == "etot":
            row["etot"] = row["epot"] + row["ekin"]
            self.tot_energy = row["etot"]
        elif o == "ediff":
            curr = row["epot"] + row["ekin"]
            row["ediff"] = curr - self._last_change
            self.dif_energy = curr - self._last_change
            self._last_change = curr

    # propagator.h:420-462
    def run(self):
        self.compute_each()
        while self.should_continue():
            self.make_step()
            self.compute_each()
        self.make_step()
        self.compute_each()
        return self.rows


def region_axes(dim: int) -> List[int]:
    """Free-axis masks of the regions of MultiRegionsReduced<dim> in region order
    (mpi_logic.h:262-278): NO, X, (Y, XY) / NO, X, Y, Z, XY, XZ, YZ, XYZ."""
    return {1: [0, 1], 2: [0, 1, 2, 3], 3: [0, 1, 2, 4, 3, 5, 6, 7]}[dim]


def region_sources(dim: int) -> List[List[tuple]]:
    """Per region, its sources (region index, transferred axis) in the order of
    LocalGrid::init (multigrid.h:127-146): the regions with one free axis fewer whose
    free set differs by exactly one axis."""
    regs = region_axes(dim)
    out = []
    for fr in regs:
        src = []
        for i, fi in enumerate(regs):
            if bin(fr).count("1") - bin(fi).count("1") == 1:
                diff = fr ^ fi
                if diff in (1, 2, 4):
                    src.append((i, diff.bit_length() - 1))
        out.append(src)
    return out


class MultiRegionPropagator:
    """SplitPropagator over a multi-region grid (CAP<MultiCartesianGrid<dim>>), as the
    reference runs it with one process per region: every region makes the same Strang
    step on its own wavefunction (its own coupling state, partial potentials, fourier
    along its bounded axes); the main region alone computes the outputs
    (calcsEnabled, mpi_logic.h:247); then postCompute (multigrid.h:617-625): the
    transfer from group to group (multigrid.h:627-657) and the region masks of every
    group but the last (grid.h:582-597)."""

    def __init__(self, dt: float, grids: List[Grid], couplings: List[Coupling], outputs: list):
        self.dim = grids[0].dim
        self.regions = region_axes(self.dim)
        assert len(grids) == len(self.regions) == len(couplings)
        self.groups = [bin(f).count("1") for f in self.regions]
        self.sources = region_sources(self.dim)
        self.props = []
        for r, (g, c) in enumerate(zip(grids, couplings)):
            g.coupling = c
            g.set_region(self.regions[r], True)
            self.props.append(Propagator(MODE_RE, dt, 0, g, outputs if r == 0 else []))
        self.rows = self.props[0].rows

    def post_compute(self):
        G = max(self.groups) + 1
        grids = [p.grid for p in self.props]
        for gi in range(1, G):
            for si in range(gi):
                for r, fr in enumerate(self.regions):
                    if self.groups[r] == gi:
                        src, fc = self.sources[r][si]
                        grids[r].mg_transfer_from(grids[src], fc, gi)
        for r, fr in enumerate(self.regions):
            if self.groups[r] != G - 1:
                grids[r].mask_region([0 if (fr >> d) & 1 else 1 for d in range(self.dim)])

    def _step_all(self):
        for p in self.props:
            p.make_step()

    def run(self):
        main = self.props[0]
        main.compute_each()
        while main.should_continue():
            self._step_all()
            main.compute_each()
            self.post_compute()
        self._step_all()
        main.compute_each()
        self.post_compute()
        return self.rows
