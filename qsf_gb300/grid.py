"""Python mirror of the reference's grid / wavefunction members over the C ABI.

``Grid`` stands for LocalGrid<Spin0<CAP<CartesianGrid<dim>>, V, C>, ...>
(include/wf/grid.h:63-1301): the wavefunction lives on the GPU and every member
runs CUDA kernels of libqsfgpu.so.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np

from ._lib import DumpFormat, GridDesc, KERNEL_KINDS, StepDesc, MAX_BORDERS, check, lib

MODE_IM, MODE_RE = 1, 2
REP_X, REP_P = 1, 2
OP_IDENTITY, OP_POTENTIAL, OP_KINETIC = 0, 1, 2
POT_EBERLY, POT_ECKHARDT_SACHA, POT_COULOMB, POT_NONE = 0, 1, 2, 3
ABS_CAP, ABS_COS8 = 0, 1  # QSF_ABS_*: the reference's quartic CAP, the cos^(1/8) mask
OBS_NORM, OBS_EPOT, OBS_EKIN, OBS_FLUX = 1, 2, 4, 8
PSI_EXT = ".psi"  # io.h:25

BORDERS = {
    "BOX": 0, "S2CAP": 1, "D2CAP": 2, "N2S": 3, "N2D": 4, "N2D_SYM": 5, "N2D_ASYM": 6,
    "S2D": 7, "S2D_SYM": 8, "S2D_ASYM": 9, "N2T": 10, "S2T": 11, "D2T": 12, "T2CAP": 13,
}
# computations.h:68-70
ZOA_FLUX_3D = ["N2S", "N2D", "N2T", "S2D", "S2T", "S2CAP", "D2CAP", "T2CAP"]
ZOA_FLUX_2D_SIMPLE = ["N2S", "N2D", "S2D", "S2CAP", "D2CAP"]
ZOA_FLUX_2D = ["N2S", "N2D_SYM", "N2D_ASYM", "S2D_SYM", "S2D_ASYM", "S2CAP", "D2CAP"]


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Grid:
    """One wavefunction on the GPU (qsf_grid_create).  Axis lengths: any n >= 2 up to
    16384 on a 1D line and 4096 per axis in 2D / 3D; lengths of the built kernel list
    (2^a, 3*2^a and 5*2^a from 8 to 16384) take the fused step kernels, the others (up to
    16384 in 1D, 2048 per axis in 2D / 3D)
    Bluestein transforms and graph-replayed member-operation step programs."""

    def __init__(self, dim: int, n, dx, nCAP: int = 0, potential: int = POT_EBERLY, Ncharge: float = 1.0,
                 Echarge: float = -1.0, Nsoft: float = 1.0, Esoft: float = 1.0, gauge: int = 0,
                 n_fields: int = 0, p_axis_swap: Optional[bool] = None, border_nodes=(25, 14, 10, 40),
                 stream: Optional[int] = None, free_axes: int = 0, multi_region: bool = False,
                 absorber: int = ABS_CAP, mask_dt: float = 0.0):
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
        if p_axis_swap is None:  # the transposed P layout: main (or single) region only
            p_axis_swap = dim >= 2 and free_axes == 0
        d.p_axis_swap = int(p_axis_swap)
        d.free_axes = int(free_axes)
        d.multi_region = int(bool(multi_region))
        d.absorber = int(absorber)
        d.mask_dt = float(mask_dt)
        self.free_axes = int(free_axes)
        for k in range(4):
            d.border_nodes[k] = int(border_nodes[k])
        self.desc = d
        self.dim, self.n, self.dx = dim, n, dx
        self.shape = tuple(n)
        self.m = int(np.prod(n))
        self.gauge = gauge
        h = ctypes.c_void_p()
        check(lib().qsf_grid_create(ctypes.byref(d), ctypes.c_void_p(stream or 0), ctypes.byref(h)),
              "qsf_grid_create")
        self._h = h

    # ------------------------------------------------------------ lifetime
    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().qsf_grid_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def device_ptr(self) -> int:
        p = ctypes.c_void_p()
        check(lib().qsf_psi_device_ptr(self._h, ctypes.byref(p)), "qsf_psi_device_ptr")
        return int(p.value)

    # ------------------------------------------------------------ data
    def upload(self, psi: np.ndarray) -> None:
        a = np.ascontiguousarray(psi, dtype=np.complex128).reshape(-1)
        assert a.size == self.m
        check(lib().qsf_upload(self._h, _dp(a.view(np.float64)), self.m), "qsf_upload")

    def download(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        """psi as complex128 of the grid's shape; into `out` (C-contiguous complex128 of
        m elements, e.g. a pinned buffer) when given."""
        if out is None:
            out = np.empty(self.m, dtype=np.complex128)
        assert out.dtype == np.complex128 and out.size == self.m and out.flags.c_contiguous
        check(lib().qsf_download(self._h, _dp(out.reshape(-1).view(np.float64)), self.m), "qsf_download")
        return out.reshape(self.shape)

    def synchronize(self) -> None:
        check(lib().qsf_synchronize(self._h), "qsf_synchronize")

    # ------------------------------------------------------------ members
    def fourier(self, to_rep: int) -> None:
        check(lib().qsf_fourier(self._h, to_rep), "qsf_fourier")

    def evolve(self, mode: int, rep: int, delta: float, coupling: Optional[Sequence[float]] = None) -> None:
        c = (ctypes.c_double * 3)(*(list(coupling) + [0.0] * (3 - len(coupling)))) if coupling is not None else None
        check(lib().qsf_evolve(self._h, mode, rep, delta, c), "qsf_evolve")

    def average(self, rep: int, op: int) -> float:
        out = ctypes.c_double()
        check(lib().qsf_average(self._h, rep, op, ctypes.byref(out)), "qsf_average")
        return out.value

    def average_log(self, rep: int, op: int, slot: int) -> None:
        """average<R, Op>() into slot `slot` of the device observables log (no wait)."""
        check(lib().qsf_average_log(self._h, rep, op, int(slot)), "qsf_average_log")

    def read_log(self, n: int) -> np.ndarray:
        out = np.empty(max(int(n), 0), dtype=np.float64)
        check(lib().qsf_read_log(self._h, _dp(out), int(n)), "qsf_read_log")
        return out

    def normalize(self) -> float:
        out = ctypes.c_double()
        check(lib().qsf_normalize(self._h, ctypes.byref(out)), "qsf_normalize")
        return out.value

    def flux(self, borders: Sequence[str], box_size: int = 0, A: Optional[Sequence[float]] = None):
        nb = len(borders)
        types = (ctypes.c_int * max(nb, 1))(*[BORDERS[b] for b in borders])
        out = (ctypes.c_double * max(nb, 1))()
        a = (ctypes.c_double * 3)(*(list(A) + [0.0] * (3 - len(A)))) if A is not None else None
        check(lib().qsf_flux(self._h, a, nb, types, int(box_size), out), "qsf_flux")
        return list(out)[:nb]

    def mask_region(self, bounded: Sequence[int]) -> None:
        b = (ctypes.c_int * 3)(*(list(bounded) + [1] * (3 - len(bounded))))
        check(lib().qsf_mask_region(self._h, b), "qsf_mask_region")

    def region_transfer(self, src: "Grid", axis: int, group: int) -> None:
        """psi += DFT_axis(masked margins of src along axis) (multigrid.h:454-657)."""
        check(lib().qsf_region_transfer(self._h, src._h, int(axis), int(group)), "qsf_region_transfer")

    def add_gaussian(self, at: float = 0.0, delta: float = 1.0) -> None:
        check(lib().qsf_add_gaussian(self._h, at, delta), "qsf_add_gaussian")

    def average_der(self, direction: int) -> float:
        """average_der<X, direction, PotentialEnergy> (grid.h:443-465)."""
        out = ctypes.c_double(0.0)
        check(lib().qsf_average_der(self._h, int(direction), ctypes.byref(out)), "qsf_average_der")
        return float(out.value)

    def antisymmetrize(self, particles: int) -> None:
        """operation<M, R, AntiSymmetrize<particles>> (grid.h:611-723)."""
        check(lib().qsf_antisymmetrize(self._h, int(particles)), "qsf_antisymmetrize")

    # ------------------------------------------------------------ .psi files
    # Paths are relative to the working directory, as in the reference.
    _snapshot_counts = {}

    def save(self, path: str = "", rep: int = REP_X, complex: bool = True, downscale: int = 1,
             evo_backup: bool = False, ext: str = PSI_EXT) -> str:
        """save / _save_centered / _save (grid.h:1087-1114, 994-1071); returns the path written."""
        df = DumpFormat(rep, 1 if complex else 0, int(downscale), 1 if evo_backup else 0)
        buf = ctypes.create_string_buffer(4096)
        check(lib().qsf_save(self._h, path.encode(), ctypes.byref(df), ext.encode(), buf, 4096), "qsf_save")
        return buf.value.decode()

    def load(self, path: str, ext: str = PSI_EXT) -> float:
        """load / _load (grid.h:789-859); returns the norm after loading.  self.load_warnings
        holds the reader's warning bits (1: n differs, 2: dx differs, 4: |psi|^2 file,
        8: file shorter than the grid)."""
        w = ctypes.c_int(0)
        nrm = ctypes.c_double(0.0)
        check(lib().qsf_load(self._h, path.encode(), ext.encode(), ctypes.byref(w), ctypes.byref(nrm)), "qsf_load")
        self.load_warnings = int(w.value)
        return float(nrm.value)

    def orthogonalize_with(self, path: str, ext: str = PSI_EXT):
        """orthogonalizeWith (grid.h:909-946); returns (<psi_file|psi> dV, norm after)."""
        ov = (ctypes.c_double * 2)()
        nrm = ctypes.c_double(0.0)
        check(lib().qsf_orthogonalize_with(self._h, path.encode(), ext.encode(), ov, ctypes.byref(nrm)),
              "qsf_orthogonalize_with")
        return complex(ov[0], ov[1]), float(nrm.value)

    def backup(self, step: int, ext: str = PSI_EXT) -> None:
        """_backup (grid.h:1116-1127): backup.info and backup<ext>."""
        check(lib().qsf_backup(self._h, int(step), ext.encode()), "qsf_backup")

    def restore(self, ext: str = PSI_EXT) -> int:
        """restore (grid.h:949-953); returns the step stored in backup.info."""
        st = ctypes.c_int64(0)
        check(lib().qsf_restore(self._h, ext.encode(), ctypes.byref(st)), "qsf_restore")
        return int(st.value)

    @staticmethod
    def remove_backups(ext: str = PSI_EXT) -> None:
        check(lib().qsf_remove_backups(ext.encode()), "qsf_remove_backups")

    def snapshot(self, extra_info: str = "", rep: int = REP_X, complex: bool = True, downscale: int = 1) -> str:
        """snapshot (grid.h:1133-1152): snapshot_<count><extra_info>_rep{X,P}.psi0, one
        counter per (dimension, representation) like the reference's function statics."""
        key = (self.dim, rep)
        cnt = Grid._snapshot_counts.get(key, 0)
        Grid._snapshot_counts[key] = cnt + 1
        return self.save("snapshot_" + str(cnt) + extra_info, rep=rep, complex=complex, downscale=downscale,
                         ext=PSI_EXT + "0")

    # ------------------------------------------------------------ fused steps
    def step_desc(self, mode: int, dt: float, nsteps: int, coupling: Optional[np.ndarray] = None,
                  obs: int = OBS_NORM, normalize: bool = False, borders: Sequence[str] = (), box_size: int = 0,
                  state_accuracy: float = 0.0, last_energy: float = 0.0, energy_after_normalize: int = 0,
                  ekin_interval: int = 1):
        """A qsf_step_desc (and the coupling array it points to, which must stay alive)."""
        d = StepDesc()
        d.mode = mode
        d.dt = dt
        d.nsteps = int(nsteps)
        cp = None
        if coupling is not None:
            cp = np.ascontiguousarray(coupling, dtype=np.float64)
            d.coupling = _dp(cp)
        d.obs = obs | (OBS_FLUX if borders else 0)
        d.normalize = int(bool(normalize))
        d.nborders = len(borders)
        assert len(borders) <= MAX_BORDERS
        for i, b in enumerate(borders):
            d.border_types[i] = BORDERS[b]
        d.box_size = int(box_size)
        d.state_accuracy = state_accuracy
        d.last_energy = last_energy
        d.energy_after_normalize = int(energy_after_normalize)
        d.ekin_interval = int(ekin_interval)
        return d, cp

    def step(self, mode: int, dt: float, nsteps: int, coupling: Optional[np.ndarray] = None, obs: int = OBS_NORM,
             normalize: bool = False, borders: Sequence[str] = (), box_size: int = 0,
             state_accuracy: float = 0.0, last_energy: float = 0.0, energy_after_normalize: int = 0,
             profile: Optional[dict] = None, substeps: int = 1, ekin_interval: int = 1):
        """Run nsteps fused Strang steps; returns (rows [nsteps, 3 + nb], steps_done).

        substeps = K > 1 runs each step as MultiProductSplit<Split3Base, K> does (K
        sub-steps of dt / K; coupling then has nsteps * K rows, one per sub-step).
        With `profile` (a dict), every launch is timed with CUDA events on the grid's
        stream; per kernel kind the summed ms and launch counts are added to it.
        ekin_interval = k > 1 computes E_kin (OBS_EKIN) on every k-th step and the last
        one only (0 in the other rows); the steps between stay fused."""
        d = StepDesc()
        d.mode = mode
        d.dt = dt
        d.nsteps = int(nsteps)
        d.substeps = int(substeps)
        d.ekin_interval = int(ekin_interval)
        cp = None
        if coupling is not None:
            cp = np.ascontiguousarray(coupling, dtype=np.float64)
            d.coupling = _dp(cp)
        d.obs = obs | (OBS_FLUX if borders else 0)
        d.normalize = int(bool(normalize))
        d.nborders = len(borders)
        assert len(borders) <= MAX_BORDERS
        for i, b in enumerate(borders):
            d.border_types[i] = BORDERS[b]
        d.box_size = int(box_size)
        d.state_accuracy = state_accuracy
        d.last_energy = last_energy
        d.energy_after_normalize = int(energy_after_normalize)
        rows = np.zeros((max(int(nsteps), 1), 3 + len(borders)), dtype=np.float64)
        done = ctypes.c_int64()
        kms = kcnt = None
        if profile is not None:
            kms = (ctypes.c_float * len(KERNEL_KINDS))()
            kcnt = (ctypes.c_int64 * len(KERNEL_KINDS))()
            d.kernel_ms = kms
            d.kernel_launches = kcnt
        check(lib().qsf_step(self._h, ctypes.byref(d), _dp(rows), ctypes.byref(done)), "qsf_step")
        if profile is not None:
            for i, k in enumerate(KERNEL_KINDS):
                ms, cnt = profile.get(k, (0.0, 0))
                profile[k] = (ms + float(kms[i]), cnt + int(kcnt[i]))
        del cp
        return rows[: int(nsteps)], int(done.value)


def fft_radices(n: int):
    r = (ctypes.c_int * 32)()
    c = ctypes.c_int()
    check(lib().qsf_fft_plan_radices(int(n), r, ctypes.byref(c)), "qsf_fft_plan_radices")
    return list(r)[: c.value]


class Batch:
    """qsf_batch: many independent grids advanced together, one launch per split stage
    per (dim, line length) group, steps replayed from a captured CUDA graph."""

    def __init__(self, stream: Optional[int] = None):
        h = ctypes.c_void_p()
        check(lib().qsf_batch_create(ctypes.c_void_p(stream or 0), ctypes.byref(h)), "qsf_batch_create")
        self._h = h
        self._keep = {}

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().qsf_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, grid: "Grid", mode: int, dt: float, nsteps: int, coupling: Optional[np.ndarray] = None,
            **kw) -> int:
        d, cp = grid.step_desc(mode, dt, nsteps, coupling, **kw)
        slot = ctypes.c_int64()
        check(lib().qsf_batch_add(self._h, grid.handle, ctypes.byref(d), ctypes.byref(slot)), "qsf_batch_add")
        self._keep[slot.value] = (grid, int(nsteps), 3 + d.nborders)
        return slot.value

    def remove(self, slot: int) -> None:
        check(lib().qsf_batch_remove(self._h, int(slot)), "qsf_batch_remove")
        self._keep.pop(slot, None)

    def run(self, steps: int) -> int:
        active = ctypes.c_int64()
        check(lib().qsf_batch_run(self._h, int(steps), ctypes.byref(active)), "qsf_batch_run")
        return int(active.value)

    def result(self, slot: int):
        grid, nsteps, ncol = self._keep[slot]
        rows = np.zeros((nsteps, ncol), dtype=np.float64)
        done = ctypes.c_int64()
        check(lib().qsf_batch_result(self._h, int(slot), _dp(rows), ctypes.byref(done)), "qsf_batch_result")
        return rows, int(done.value)
