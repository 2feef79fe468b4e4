"""Physics known answers for the GPU step (closed forms and convergence rates, not the
reference's outputs): free-packet spreading, norm conservation without an absorber,
the Volkov phase of a plane wave in the velocity gauge, second-order convergence of
the Strang step, the soft-core hydrogen ground-state energy, and the transform round
trip."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def Q():
    import qsf_gb300
    return qsf_gb300


def _x(n, dx):
    return (np.arange(n) - (n - 1) / 2.0) * dx


def test_free_gaussian_spreads_as_closed_form(Q):
    """V = 0, no field, no absorber: the step is the exact free propagator, so psi(t)
    is the analytic spreading Gaussian (to the transform's rounding)."""
    n, dx, dt, steps, s = 4096, 0.2, 0.05, 200, 1.0
    x = _x(n, dx)
    psi0 = (1.0 / (math.pi * s * s)) ** 0.25 * np.exp(-x * x / (2 * s * s))
    g = Q.Grid(1, n, dx, nCAP=0, potential=Q.POT_NONE)
    g.upload(psi0.astype(np.complex128))
    g.step(Q.MODE_RE, dt, steps)
    t = dt * steps
    a = 1.0 + 1j * t / (s * s)
    exact = (1.0 / (math.pi * s * s)) ** 0.25 / np.sqrt(a) * np.exp(-x * x / (2 * s * s * a))
    assert np.linalg.norm(g.download() - exact) / np.linalg.norm(exact) < 1e-9


def test_norm_is_conserved_without_absorber(Q):
    n, dx, dt, steps = 256, 0.3, 0.05, 200
    g = Q.Grid(2, n, dx, nCAP=0, potential=Q.POT_EBERLY, Ncharge=2.0, gauge=Q.GAUGE_VELOCITY, n_fields=1)
    x = _x(n, dx)
    psi0 = np.exp(-0.5 * (x[:, None] ** 2 + (x[None, :] - 1.0) ** 2)).astype(np.complex128)
    psi0 /= math.sqrt(np.sum(np.abs(psi0) ** 2) * dx * dx)
    g.upload(psi0)
    c = Q.Coupling(Q.GAUGE_VELOCITY, [Q.Field(3, [Q.Pulse(field=0.1, omega=0.5, ncycles=2)])])
    from qsf_gb300.propagator import coupling_schedule
    rows, _ = coupling_schedule(c, dt, steps)
    out, done = g.step(Q.MODE_RE, dt, steps, rows)
    assert done == steps
    assert np.max(np.abs(out[:, 0] - 1.0)) < 1e-13 * steps


def test_volkov_phase_of_a_plane_wave(Q):
    """A grid momentum k0 in a velocity-gauge field with V = 0: each step multiplies by
    exp(-i dt (k0^2/2 + A k0)) exactly (the X halves are 1), A from the step's schedule."""
    n, dx, dt, steps = 1024, 0.2, 0.05, 300
    dp = 2 * math.pi / n / dx
    k0 = 37 * dp
    x = _x(n, dx)
    psi0 = np.exp(1j * k0 * x)
    g = Q.Grid(1, n, dx, nCAP=0, potential=Q.POT_NONE, gauge=Q.GAUGE_VELOCITY, n_fields=1)
    g.upload(psi0)
    c = Q.Coupling(Q.GAUGE_VELOCITY, [Q.Field(1, [Q.Pulse(field=0.08, omega=0.3, ncycles=2)])])
    from qsf_gb300.propagator import coupling_schedule
    rows, _ = coupling_schedule(c, dt, steps)
    g.step(Q.MODE_RE, dt, steps, rows)
    phase = np.sum(dt * (0.5 * k0 * k0 + rows[:, 0] * k0))
    assert np.max(np.abs(rows[:, 0])) > 0.05  # the field does act
    exact = psi0 * np.exp(-1j * phase)
    assert np.linalg.norm(g.download() - exact) / np.linalg.norm(exact) < 1e-10


def test_strang_step_is_second_order(Q):
    n, dx, T = 512, 0.2, 2.0
    x = _x(n, dx)
    psi0 = np.exp(-0.5 * (x - 2.0) ** 2 + 0.5j * x).astype(np.complex128)

    def run(dt):
        g = Q.Grid(1, n, dx, nCAP=0, potential=Q.POT_EBERLY, Ncharge=1.0)
        g.upload(psi0)
        g.step(Q.MODE_RE, dt, int(round(T / dt)))
        return g.download()

    ref = run(T / 640)
    err = [np.linalg.norm(run(dt) - ref) for dt in (0.1, 0.05, 0.025)]
    r1, r2 = err[0] / err[1], err[1] / err[2]
    assert 3.5 < r1 < 4.5 and 3.5 < r2 < 4.5, (err, r1, r2)


def test_soft_core_hydrogen_ground_state(Q):
    """1D soft-core hydrogen (Z = 1, a = 1): imaginary time reaches E0 = -0.66977."""
    n, dx, dt = 1024, 0.2, 0.01
    g = Q.Grid(1, n, dx, nCAP=0, potential=Q.POT_EBERLY, Ncharge=1.0, Nsoft=1.0)
    g.add_gaussian(0.0, 1.0)
    prop = Q.SplitPropagator(Q.MODE_IM, dt, 3000, g, Q.Coupling(Q.GAUGE_VELOCITY),
                             ["normalize", "norm", "epot", "ekin", "etot", "ediff"], state_accuracy=1e-12)
    rows = prop.run()
    assert abs(rows[-1]["etot"] - (-0.66977)) < 2e-4
    assert abs(rows[-1]["norm"] - 1.0) < 1e-12


def test_transform_round_trip_is_identity(Q):
    n = 512
    rng = np.random.default_rng(4)
    psi = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    g = Q.Grid(2, n, 0.3)
    g.upload(psi)
    g.fourier(Q.REP_P)
    g.fourier(Q.REP_X)
    assert np.linalg.norm(g.download() - psi) / np.linalg.norm(psi) < 1e-15
