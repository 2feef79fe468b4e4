"""Size-independent checks of the fused step at the full 2D and 3D sizes and run
lengths, where the oracle cannot follow (a 2048^2 run of 6620 steps is hours of CPU).

Without an absorber the Strang step S(dt) = X(dt/2) P(dt) X(dt/2) is unitary, and the
same step with -dt and the coupling of the step (in the length gauge its two X halves'
fields swapped) is its exact inverse.  So a full run forward followed by the reversed
schedule backward must return psi_0 up to the transform's rounding, and the norm must
stay 1 throughout.  2D: 2048^2, two electrons, velocity gauge, the 3-cycle 800 nm
5e14 W/cm^2 pulse (6620 steps each way).  3D: 256^3, three electrons, length gauge, the
2-cycle 800 nm 1e15 W/cm^2 pulse (4413 steps each way).  Bar: relative L2 1e-10 (the
parity bar for psi), norm within 1e-12 at every step."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OMEGA = 45.563352529 / 800.0  # constants.h:47-51


def _field(I):
    return math.sqrt(I / 3.50944e16)  # constants.h:35


def _start(dim, n, dx, seed):
    """Seeded complex noise under a Gaussian envelope, normalised."""
    rng = np.random.default_rng(seed)
    x = (np.arange(n) - (n - 1) / 2.0) * dx
    env1 = np.exp(-x * x / (2 * (0.15 * n * dx) ** 2))
    env = env1
    for _ in range(dim - 1):
        env = np.multiply.outer(env, env1)
    shape = (n,) * dim
    psi = env * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    psi /= math.sqrt(float(np.sum(np.abs(psi) ** 2)) * dx ** dim)
    return psi


def _round_trip(Q, dim, n, dx, charge, gauge, intensity, ncycles, seed):
    from qsf_gb300.propagator import coupling_schedule
    dt = 0.05
    axis = {2: 3, 3: 7}[dim]
    g = Q.Grid(dim, n, dx, nCAP=0, potential=Q.POT_EBERLY, Ncharge=charge, gauge=gauge, n_fields=1)
    psi0 = _start(dim, n, dx, seed)
    g.upload(psi0)
    c = Q.Coupling(gauge, [Q.Field(axis, [Q.Pulse(field=_field(intensity), omega=OMEGA, ncycles=ncycles)])])
    nsteps = int(c.max_pulse_duration() / dt + 1)
    rows, _ = coupling_schedule(c, dt, nsteps)
    assert np.max(np.abs(rows)) > 0.01
    fwd, done = g.step(Q.MODE_RE, dt, nsteps, rows, obs=Q.OBS_NORM)
    assert done == nsteps
    back_rows = rows[::-1].copy()
    if rows.shape[1] == 6:  # length gauge: the reversed step's X halves swap their fields
        back_rows = np.concatenate([back_rows[:, 3:6], back_rows[:, 0:3]], axis=1)
    bwd, done = g.step(Q.MODE_RE, -dt, nsteps, back_rows, obs=Q.OBS_NORM)
    assert done == nsteps
    norms = np.concatenate([fwd[:, 0], bwd[:, 0]])
    psi = g.download()
    g.close()
    err = float(np.linalg.norm(psi - psi0) / np.linalg.norm(psi0))
    print(f"{dim}D {n}: {nsteps} steps each way, round-trip relative L2 {err:.3e}, "
          f"max |norm - 1| {float(np.max(np.abs(norms - 1.0))):.3e}")
    return nsteps, norms, err, psi0, psi


def test_2d_2048_full_run_and_back():
    import qsf_gb300 as Q
    nsteps, norms, err, psi0, psi = _round_trip(Q, 2, 2048, 0.3, 2.0, Q.GAUGE_VELOCITY, 5e14, 3, 7)
    assert nsteps == 6620  # max_steps of the run loop (propagator.h:118-127)
    assert np.max(np.abs(norms - 1.0)) < 1e-12
    assert err < 1e-10, err


def test_3d_256_full_run_and_back():
    import qsf_gb300 as Q
    nsteps, norms, err, psi0, psi = _round_trip(Q, 3, 256, 0.4, 3.0, Q.GAUGE_LENGTH, 1e15, 2, 8)
    assert nsteps == 4413  # max_steps of the run loop (propagator.h:118-127)
    assert np.max(np.abs(norms - 1.0)) < 1e-12
    assert err < 1e-10, err
