"""Axis lengths with a prime factor above 5 (Bluestein transforms, member-operation steps).

The reference transforms any n through FFTW (wf/grid.h:251-274); the fused kernels of
this library are built for 2^a, 3*2^a and 5*2^a (8 ... 16384).  Other lengths take one chirp-z convolution per
axis through the built M-point transforms (M >= 2n - 1) and qsf_step runs the reference's
own member sequence evolve<X>(dt/2), fourier<P>, evolve<P>(dt), fourier<X>,
evolve<X>(dt/2) (propagator.h:311-346).  Checked here: transforms against numpy's FFT
(and the inverse round trip), real-time runs with a field, absorber, fluxes and
imaginary-time runs against the oracle (which transforms prime lengths by direct DFT),
and the rejection of such grids by batches."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import cases as C

pytestmark = pytest.mark.gpu

TOL_FFT = 4e-14
FLUX_RES = {1: 1e-19, 2: 1e-18, 3: 1e-18}


@pytest.mark.parametrize("n", [2, 3, 4, 5, 6, 7, 11, 97, 100, 127, 1021, 1031, 3001, 4099, 8191, 8209, 9973, 12289,
                               16383])
def test_bluestein_1d_matches_numpy(n):
    """Up to 8191 points one M-point transform (M <= 16384); above, M = M1 * M2 as a
    four-step transform."""
    import qsf_gb300 as Q
    rng = np.random.default_rng(n)
    psi = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    g = Q.Grid(1, n, 0.1)
    g.upload(psi)
    g.fourier(Q.REP_P)
    assert C.rel_l2(g.download(), np.fft.fft(psi)) < TOL_FFT
    g.fourier(Q.REP_X)
    assert C.rel_l2(g.download(), psi) < TOL_FFT
    g.close()


@pytest.mark.parametrize("dim,n", [(2, 2), (2, 5), (2, 7), (2, 63), (2, 127), (2, 1021), (3, 3), (3, 14), (3, 35),
                                   (3, 97)])
def test_bluestein_nd_matches_numpy(dim, n):
    import qsf_gb300 as Q
    rng = np.random.default_rng(11 * n + dim)
    shape = (n,) * dim
    psi = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    g = Q.Grid(dim, n, 0.1)
    g.upload(psi)
    g.fourier(Q.REP_P)
    assert C.rel_l2(g.download(), np.fft.fftn(psi)) < TOL_FFT
    g.fourier(Q.REP_X)
    assert C.rel_l2(g.download(), psi) < TOL_FFT
    g.close()


def _params(n, dx, lg):
    # flux border nodes in the proportions of the golden 2D / 3D cases (48: 6, 4, 3, 15)
    return dict(n=n, dx=dx, nCAP=max(2, n // 10), Ncharge=1.0, Echarge=-1.0, Nsoft=1.0, Esoft=1.0, F0=0.08,
                omega=1.5, ncycles=1.0, phase=0.0, re_dt=0.05, box=n // 3, lg=lg, im_dt=0.05, im_steps=40,
                p_NS=max(3, n // 8), p_SD=max(2, n // 12), p_DT=max(2, n // 16), p_CAP=max(6, (5 * n) // 16))


@pytest.mark.parametrize("dim,n,lg", [(1, 1021, 0), (1, 509, 1), (1, 9009, 1), (2, 77, 0), (2, 63, 1), (3, 21, 0)])
def test_bluestein_real_time_run_matches_oracle(dim, n, lg):
    """A full pulse (sin^2 envelope) with absorber and fluxes: rows and final psi."""
    dx = {1: 0.1, 2: 0.3, 3: 0.4}[dim]
    p = _params(n, dx, lg)
    C.set_borders(p)
    x = (np.arange(n) - (n - 1) / 2.0) * dx
    r2 = sum(np.meshgrid(*([x * x] * dim), indexing="ij"))
    psi0 = np.exp(-0.5 * r2).astype(np.complex128) * (1.0 + 0.3j * np.tanh(sum(np.meshgrid(*([x] * dim),
                                                                                        indexing="ij"))))
    psi0 /= np.sqrt(np.sum(np.abs(psi0) ** 2) * dx ** dim)
    og, orows = C.oracle_re(p, dim, psi0)
    g, rows = C.gpu_re(p, dim, psi0)
    nb = len(C.re_borders(dim))
    got = np.array([C.re_dat_row(r, nb) for r in rows])
    ref = np.array([C.re_dat_row(r, nb) for r in orows])
    assert got.shape == ref.shape and len(got) > 10
    np.testing.assert_allclose(got[:, :2], ref[:, :2], rtol=1e-14, atol=0)
    np.testing.assert_allclose(got[:, 2:5], ref[:, 2:5], rtol=1e-10, atol=0)
    # fluxes to 1e-9 relative above a fixed resolution (values far below it are floating-
    # point noise of psi's tails in both the oracle and the GPU transforms)
    np.testing.assert_allclose(got[:, 5:], ref[:, 5:], rtol=1e-9, atol=FLUX_RES[dim])
    assert C.rel_l2(g.download(), og.psi) < 1e-11
    g.close()


@pytest.mark.parametrize("dim,n", [(1, 719), (2, 91)])
def test_bluestein_imaginary_time_matches_oracle(dim, n):
    """Ground state search with Normalize and the energy convergence rule."""
    p = _params(n, 0.3 if dim == 2 else 0.1, 0)
    og, orows = C.oracle_im(p, dim)
    g, rows = C.gpu_im(p, dim)
    got = np.array([C.im_dat_row(r) for r in rows])
    ref = np.array([C.im_dat_row(r) for r in orows])
    assert got.shape == ref.shape
    np.testing.assert_allclose(got[:, 0], ref[:, 0], rtol=0, atol=0)
    np.testing.assert_allclose(got[:, 2:], ref[:, 2:], rtol=1e-10, atol=1e-13)
    np.testing.assert_allclose(got[1:, 1], ref[1:, 1], rtol=0, atol=1e-11)  # E_n - E_(n-1)
    assert C.rel_l2(g.download(), og.psi) < 1e-11
    g.close()


def test_bluestein_step_with_ekin_interval_and_substeps():
    """qsf_step's descriptor on a member-operation grid: E_kin every 4th step, and the
    multi-product chain (substeps) against the same sub-steps taken one by one."""
    import qsf_gb300 as Q
    n, steps = 77, 12
    g = Q.Grid(2, n, 0.3, nCAP=7, Ncharge=2.0, gauge=Q.GAUGE_VELOCITY, n_fields=0)
    rng = np.random.default_rng(5)
    psi0 = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    outs = {}
    for k in (1, 4):
        g.upload(psi0)
        rows, done = g.step(Q.MODE_IM, 0.05, steps, None, obs=Q.OBS_NORM | Q.OBS_EPOT | Q.OBS_EKIN,
                            normalize=True, ekin_interval=k)
        assert done == steps
        outs[k] = (rows.copy(), g.download())
    (r1, p1), (r4, p4) = outs[1], outs[4]
    # E_kin takes psi through an extra transform pair (propagator.h:284-291), so the
    # runs agree to rounding, not bit for bit
    np.testing.assert_allclose(r4[:, :2], r1[:, :2], rtol=1e-12, atol=0)
    assert C.rel_l2(p4, p1) < 1e-13
    have = np.array([(s + 1) % 4 == 0 or s == steps - 1 for s in range(steps)])
    np.testing.assert_allclose(r4[have, 2], r1[have, 2], rtol=1e-12, atol=0)
    assert np.all(r4[~have, 2] == 0.0) and np.all(r1[:, 2] > 0.0)
    # K = 3 sub-steps of dt / 3 equal three plain steps of dt / 3 observed at the end
    g.upload(psi0)
    rk, _ = g.step(Q.MODE_IM, 0.06, 2, None, obs=Q.OBS_NORM | Q.OBS_EPOT, substeps=3)
    g2 = Q.Grid(2, n, 0.3, nCAP=7, Ncharge=2.0, gauge=Q.GAUGE_VELOCITY, n_fields=0)
    g2.upload(psi0)
    rp, _ = g2.step(Q.MODE_IM, 0.02, 6, None, obs=Q.OBS_NORM | Q.OBS_EPOT)
    np.testing.assert_allclose(rk[:, :2], rp[[2, 5], :2], rtol=1e-12)
    assert C.rel_l2(g.download(), g2.download()) < 1e-12
    g.close()
    g2.close()


def test_bluestein_grids_stay_out_of_batches():
    import qsf_gb300 as Q
    g = Q.Grid(2, 63, 0.3, nCAP=6)
    g.add_gaussian(0.0, 1.0)
    b = Q.Batch()
    with pytest.raises(Q.QsfError) as e:
        b.add(g, Q.MODE_IM, 0.05, 4, None, obs=Q.OBS_NORM)
    assert e.value.code == 1
    b.close()
    g.close()


def test_server_serves_bluestein_lengths_beside_the_batch():
    """Solves of lengths without fused kernels run in the server beside the batch (their
    own streams, member operations): each result equals the same solve run alone through
    qsf_step, bit for bit, in a mix with fused-length solves."""
    import qsf_gb300 as Q
    from qsf_gb300 import serve as S
    from qsf_gb300.propagator import coupling_schedule
    nsteps, dt = 40, 0.05
    cases = [(1, 1021, 0.2, ["BOX"], 400), (2, 63, 0.3, Q.ZOA_FLUX_2D, 0), (2, 64, 0.3, Q.ZOA_FLUX_2D, 0),
             (1, 9009, 0.2, ["BOX"], 3000)]
    reqs, alone = [], []
    for dim, n, dx, borders, box in cases:
        c = Q.Coupling(Q.GAUGE_VELOCITY, [Q.Field({1: 1, 2: 3}[dim], [Q.Pulse(field=0.1, omega=1.0, ncycles=1.0)])])
        sched = coupling_schedule(c, dt, nsteps)[0]
        x = (np.arange(n) - (n - 1) / 2.0) * dx
        psi0 = np.exp(-0.5 * sum(np.meshgrid(*([x * x] * dim), indexing="ij"))).astype(np.complex128)
        psi0 /= np.sqrt(np.sum(np.abs(psi0) ** 2) * dx ** dim)
        g = Q.Grid(dim, n, dx, nCAP=n // 10, Ncharge=float(dim), gauge=Q.GAUGE_VELOCITY, n_fields=1)
        g.upload(psi0)
        rows, done = g.step(Q.MODE_RE, dt, nsteps, sched, obs=Q.OBS_NORM | Q.OBS_EPOT, borders=borders,
                            box_size=box)
        assert done == nsteps
        alone.append(rows.copy())
        g.close()
        reqs.append(dict(gdesc=S.grid_desc(dim, n, dx, nCAP=n // 10, Ncharge=float(dim), gauge=Q.GAUGE_VELOCITY,
                                           n_fields=1),
                         mode=Q.MODE_RE, dt=dt, nsteps=nsteps, coupling=sched, psi0=psi0,
                         obs=Q.OBS_NORM | Q.OBS_EPOT, borders=borders, box_size=box))
    srv = S.Server(max_slots=8, steps_per_round=16)
    try:
        tickets = [srv.submit(**r) for r in reqs]
        for t, rows, (dim, n, _, borders, _) in zip(tickets, alone, cases):
            r = srv.wait(t, 300)
            assert r["status"] == 0 and r["steps"] == nsteps, (dim, n)
            assert r["final_norm"] == rows[-1, 0] and r["final_epot"] == rows[-1, 1], (dim, n)
            for b in range(len(borders)):
                assert r["flux_integral"][b] == pytest.approx(np.sum(rows[:, 3 + b]) * dt, rel=1e-13, abs=0)
    finally:
        srv.stop()


def test_bluestein_multi_region_grid_matches_oracle():
    """A 2D multi-region grid of a length outside the built list (66 = 2 * 3 * 11):
    partial transforms and region transfers through the Bluestein transforms."""
    from qsf_gb300.multigrid import MultiGrid, MultiRegionPropagator
    import qsf_gb300 as Q
    n = 66
    p = dict(n=n, dx=0.4, nCAP=7, Ncharge=2.0, Echarge=-1.0, Nsoft=1.0, Esoft=1.0, F0=0.2, omega=1.2,
             ncycles=1, re_dt=0.05)
    rng = np.random.default_rng(17)
    x = (np.arange(n) - (n - 1) / 2.0) * p["dx"]
    env = np.exp(-(x[:, None] ** 2 + x[None, :] ** 2) / 60.0)
    psi0 = env * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    gs, orows = C.oracle_mg(p, 2, psi0)
    mg = MultiGrid(2, n, p["dx"], p["nCAP"], potential=Q.POT_EBERLY, Ncharge=p["Ncharge"], Echarge=p["Echarge"],
                   Nsoft=p["Nsoft"], Esoft=p["Esoft"], gauge=Q.GAUGE_VELOCITY, n_fields=1)
    mg.main.upload(psi0)
    pulse = Q.Pulse(field=p["F0"], omega=p["omega"], ncycles=p["ncycles"])
    prop = MultiRegionPropagator(p["re_dt"], mg, Q.Coupling(Q.GAUGE_VELOCITY, [Q.Field(3, [pulse])]), C.MG_OUTPUTS)
    rows = prop.run()
    psis = [g.download() for g in mg.regions]
    mg.close()
    np.testing.assert_allclose(np.array([C.mg_dat_row(r) for r in rows]),
                               np.array([C.mg_dat_row(r) for r in orows]), rtol=1e-9, atol=1e-12)
    for r in range(4):
        assert np.linalg.norm(gs[r].psi) > 0, r
        assert C.rel_l2(psis[r], gs[r].psi) < 1e-10, r


@pytest.mark.parametrize("dim,n", [(1, 2), (1, 5), (2, 3), (3, 4)])
def test_tiny_grids_step_like_the_oracle(dim, n):
    """The smallest grids (no fused kernels: lengths below 8 run as Bluestein lengths)
    step through the member-operation program like the oracle: norm and E_pot rows and
    the final psi."""
    import qsf_gb300 as Q
    from oracle import oracle as O
    from qsf_gb300.propagator import coupling_schedule
    dx, dt, steps = 0.7, 0.05, 12
    rng = np.random.default_rng(n + 10 * dim)
    psi0 = rng.standard_normal((n,) * dim) + 1j * rng.standard_normal((n,) * dim)
    pulse = dict(field=0.1, omega=1.0, ncycles=1.0)
    axis = {1: 1, 2: 3, 3: 7}[dim]
    oc = O.Coupling(O.GAUGE_VELOCITY, [O.Field(axis, [O.Pulse(**pulse)])])
    og = O.Grid(dim, n, dx, nCAP=0, Ncharge=float(dim), coupling=oc)
    og.psi[...] = psi0
    prop = O.Propagator(O.MODE_RE, dt, 0, og, ["norm", "epot"])
    orows = []
    for _ in range(steps):
        prop.make_step()
        prop.compute_each()
        orows.append([prop.rows[-1]["norm"], prop.rows[-1]["epot"]])
    g = Q.Grid(dim, n, dx, nCAP=0, Ncharge=float(dim), gauge=Q.GAUGE_VELOCITY, n_fields=1)
    g.upload(psi0)
    c = Q.Coupling(Q.GAUGE_VELOCITY, [Q.Field(axis, [Q.Pulse(**pulse)])])
    rows, done = g.step(Q.MODE_RE, dt, steps, coupling_schedule(c, dt, steps)[0], obs=Q.OBS_NORM | Q.OBS_EPOT)
    assert done == steps
    np.testing.assert_allclose(rows[:, :2], np.array(orows), rtol=1e-11, atol=1e-14)
    assert C.rel_l2(g.download(), og.psi) < 1e-12
    g.close()


@pytest.mark.parametrize("K,lg", [(2, 0), (3, 1)])
def test_bluestein_multiproduct_matches_oracle(K, lg):
    """MultiProductSplit<Split3Base, K> on a Bluestein length (1D, 733 points) against the
    oracle's literal chains (propagator.h:331-413): the step program's sub-steps."""
    import qsf_gb300 as Q
    n, dx = 733, 0.2
    p = _params(n, dx, lg)
    p["F0"], p["omega"], p["ncycles"] = 0.06, 1.0, 1.0
    x = (np.arange(n) - (n - 1) / 2.0) * dx
    psi0 = (np.exp(-0.5 * x * x) * (1 + 0.2j * x)).astype(np.complex128)
    psi0 /= np.sqrt(np.sum(np.abs(psi0) ** 2) * dx)
    outs = ["step", "time", "norm", "epot"]
    oc = O.Coupling(O.GAUGE_LENGTH if lg else O.GAUGE_VELOCITY, [O.Field(1, [C.pulse(p)])])
    og = C.oracle_grid(p, 1, oc)
    og.psi[...] = psi0
    orows = O.Propagator(O.MODE_RE, p["re_dt"], 0, og, outs, order=K).run()
    gauge = Q.GAUGE_LENGTH if lg else Q.GAUGE_VELOCITY
    g = C.gpu_grid(p, 1, gauge, 1)
    g.upload(psi0)
    rows = Q.SplitPropagator(Q.MODE_RE, p["re_dt"], 0, g, Q.Coupling(gauge, [Q.Field(1, [C.gpu_pulse(p)])]), outs,
                             order=K).run()
    got = np.array([[r[k] for k in outs] for r in rows])
    ref = np.array([[r[k] for k in outs] for r in orows])
    assert got.shape == ref.shape
    np.testing.assert_allclose(got[:, :2], ref[:, :2], rtol=1e-15, atol=0)
    np.testing.assert_allclose(got[:, 2:], ref[:, 2:], rtol=1e-10, atol=0)
    assert C.rel_l2(g.download(), og.psi) < 1e-11
    g.close()
