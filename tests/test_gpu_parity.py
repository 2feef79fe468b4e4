"""GPU path (libqsfgpu.so through the C ABI) against the reference's own outputs.

Golden fixtures come from the reference's header-only implementation itself
(tests/golden/make_golden.py); the CPU oracle is pinned to the same fixtures in
test_oracle_golden.py.  Tolerances: 1e-12 relative for single primitives, and the
spec bar for full runs -- relative L2 of psi <= 1e-10 after the run, norm /
energies / border fluxes within 1e-9.
"""
import numpy as np
import pytest

from tests import cases as C

pytestmark = pytest.mark.gpu

PRIM_TOL = 1e-12
PSI_TOL = 1e-10
OBS_TOL = 1e-9


@pytest.fixture(scope="module")
def Q():
    import qsf_gb300
    return qsf_gb300


# *_bs: 22^2 and 14^3, lengths with a prime factor above 5 (Bluestein transforms)
@pytest.mark.parametrize("name", ["prim2d", "prim3d", "prim2d_bs", "prim3d_bs"])
def test_primitives(Q, name):
    z = C.load(name)
    p, dim = z["params"], int(z["dim"])
    s = z["scalars"]
    lg = C.gpu_grid(p, dim, Q.GAUGE_LENGTH, 1)
    vg = C.gpu_grid(p, dim, Q.GAUGE_VELOCITY, 1)
    lg.upload(z["psi_in"])
    vg.upload(z["psi_in"])
    assert lg.average(Q.REP_X, Q.OP_IDENTITY) == pytest.approx(s[0], rel=PRIM_TOL)
    assert lg.average(Q.REP_X, Q.OP_POTENTIAL) == pytest.approx(s[1], rel=PRIM_TOL)
    names = ["S2CAP", "D2CAP", "N2S", "N2D", "S2D"]
    names += ["N2D_SYM", "N2D_ASYM", "S2D_SYM", "S2D_ASYM"] if dim == 2 else ["N2T", "S2T", "D2T", "T2CAP"]
    fl = lg.flux(["BOX"], 3) + lg.flux(names)
    np.testing.assert_allclose(fl, s[2:2 + len(fl)], rtol=PRIM_TOL, atol=1e-14)
    E = [p["F0"]] * 3
    lg.evolve(Q.MODE_RE, Q.REP_X, p["delta"], E)
    assert C.rel_l2(lg.download(), z["psi_xre"]) < PRIM_TOL
    lg.evolve(Q.MODE_IM, Q.REP_X, p["delta"], E)
    assert C.rel_l2(lg.download(), z["psi_xim"]) < PRIM_TOL
    lg.fourier(Q.REP_P)
    assert C.rel_l2(np.swapaxes(lg.download(), 0, 1), z["psi_p"]) < PRIM_TOL
    assert lg.average(Q.REP_P, Q.OP_KINETIC) == pytest.approx(s[-1], rel=PRIM_TOL)
    lg.fourier(Q.REP_X)
    assert C.rel_l2(lg.download(), z["psi_back"]) < PRIM_TOL
    vg.fourier(Q.REP_P)
    A = [-p["F0"]] * 3
    vg.evolve(Q.MODE_RE, Q.REP_P, p["delta"], A)
    vg.evolve(Q.MODE_IM, Q.REP_P, p["delta"] * 0.25, A)
    vg.fourier(Q.REP_X)
    assert C.rel_l2(vg.download(), z["psi_pvg"]) < PRIM_TOL
    vg.normalize()
    assert C.rel_l2(vg.download(), z["psi_norm"]) < PRIM_TOL


def _assert_columns(got, ref):
    """Every column at rtol OBS_TOL; the absolute floor is 1e-12 of that column's own
    largest value (border fluxes span many decades between columns)."""
    for c in range(ref.shape[1]):
        scale = float(np.max(np.abs(ref[:, c])))
        np.testing.assert_allclose(got[:, c], ref[:, c], rtol=OBS_TOL, atol=1e-12 * scale, err_msg=f"column {c}")


# *_bs: axis lengths with a prime factor above 5 (514, 46, 14), whose transforms run
# as Bluestein convolutions and whose steps run as member-operation programs
@pytest.mark.parametrize("name", ["c1_vg", "c1_lg", "c2_vg", "c3_lg", "c1_bs", "c2_bs", "c3_bs"])
def test_full_runs(Q, name):
    z = C.load(name)
    p, dim = z["params"], int(z["dim"])
    g, rows = C.gpu_im(p, dim)
    got = np.array([C.im_dat_row(r) for r in rows])
    ref = z["im_rows"]
    assert got.shape == ref.shape
    _assert_columns(got, ref)
    assert C.rel_l2(g.download(), z["im_psi"]) < PSI_TOL
    g2, rows2 = C.gpu_re(p, dim, z["re_psi0"])
    nb = len(C.re_borders(dim))
    got = np.array([C.re_dat_row(r, nb) for r in rows2])
    ref = z["re_rows"]
    assert got.shape == ref.shape
    np.testing.assert_allclose(got[:, :2], ref[:, :2], rtol=1e-14, atol=0)  # step and time are exact
    _assert_columns(got[:, 2:], ref[:, 2:])
    assert C.rel_l2(g2.download(), z["re_psi"]) < PSI_TOL


@pytest.mark.parametrize("n", [8, 12, 16, 20, 48, 64, 96, 160, 256, 384, 512, 640, 768, 1024, 2048, 4096, 8192])
def test_fft_1d_matches_numpy(Q, n):
    rng = np.random.default_rng(n)
    psi = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    g = Q.Grid(1, n, 0.1)
    g.upload(psi)
    g.fourier(Q.REP_P)
    ref = np.fft.fft(psi)
    assert C.rel_l2(g.download(), ref) < 1e-14 * max(1.0, np.log2(n))
    g.fourier(Q.REP_X)
    assert C.rel_l2(g.download(), psi) < 1e-14 * max(1.0, np.log2(n))


def _exact_dft(x):
    """DFT in extended precision: angles reduced exactly (k j mod n), long-double
    cos / sin and sums (numpy longdouble)."""
    n = len(x)
    k = np.arange(n)
    pi = np.longdouble("3.141592653589793238462643383279502884")
    ang = -2 * pi * k.astype(np.longdouble) / n
    tw = np.cos(ang) + 1j * np.sin(ang)  # the n distinct twiddles
    return tw[np.outer(k, k) % n] @ x.astype(np.clongdouble)


@pytest.mark.parametrize("n", [48, 256, 1024, 2048])
def test_fixed_point_fft_beats_fp64(Q, n):
    """The block fixed-point transform is more accurate than an FP64 FFT: normwise error
    against an extended-precision DFT, next to numpy's FP64 FFT on the same inputs."""
    if np.finfo(np.longdouble).eps >= np.finfo(np.float64).eps:
        pytest.skip("long double is not wider than double on this host")
    rng = np.random.default_rng(n + 1)
    worst_gpu = worst_fp64 = 0.0
    for _ in range(2):
        x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * np.exp(-0.5 * ((np.arange(n) - n / 2) / (n / 8)) ** 2)
        ex = _exact_dft(x)
        nrm = float(np.sqrt(np.sum(np.abs(ex) ** 2)))
        g = Q.Grid(1, n, 0.1)
        g.upload(x)
        g.fourier(Q.REP_P)
        y = g.download()
        g.close()
        worst_gpu = max(worst_gpu, float(np.sqrt(np.sum(np.abs(y.astype(np.clongdouble) - ex) ** 2))) / nrm)
        worst_fp64 = max(worst_fp64, float(np.sqrt(np.sum(np.abs(np.fft.fft(x).astype(np.clongdouble) - ex) ** 2))) / nrm)
    assert worst_gpu < 1.5e-16
    assert worst_gpu < 0.7 * worst_fp64


@pytest.mark.parametrize("dim,n", [(2, 64), (2, 384), (2, 2048), (3, 16), (3, 48), (3, 256)])
def test_fft_nd_matches_numpy(Q, dim, n):
    rng = np.random.default_rng(7 * n + dim)
    shape = (n,) * dim
    psi = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    g = Q.Grid(dim, n, 0.1)
    g.upload(psi)
    g.fourier(Q.REP_P)
    assert C.rel_l2(g.download(), np.fft.fftn(psi)) < 2e-14 * np.log2(n ** dim)
    g.fourier(Q.REP_X)
    assert C.rel_l2(g.download(), psi) < 2e-14 * np.log2(n ** dim)


def test_fused_step_is_deterministic(Q):
    z = C.load("c2_vg")
    p = z["params"]
    out = []
    for _ in range(2):
        g, rows = C.gpu_re(p, 2, z["re_psi0"])
        out.append((g.download(), np.array([C.re_dat_row(r, 7) for r in rows])))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


def test_bad_sizes_are_rejected(Q):
    # lengths without fused kernels run through Bluestein transforms of a length
    # M >= 2n - 1: any 1D line up to 16384 points, up to 2048 on the axes of a 2D/3D grid
    for dim, n in ((1, 16385), (2, 2051), (3, 2051)):
        with pytest.raises(Q.QsfError) as e:
            Q.Grid(dim, n, 0.1)
        assert e.value.code == 1
    with pytest.raises(Q.QsfError):
        Q.Grid(2, [64, 32], 0.1)
    with pytest.raises(Q.QsfError):
        Q.Grid(1, 16384 * 2, 0.1)


@pytest.mark.parametrize("n", [384, 512, 1024, 2048])
def test_fused_2d_steps_match_oracle(Q, n):
    """Fused multi-step calls at the large 2D edges (384, 512 and 2048 take the
    512-thread radix-8 row / axis kernels, 1024 the 256-thread radix-16 ones) against the oracle:
    velocity-gauge field, absorber, norm, E_pot and the ZOA_FLUX_2D fluxes every step."""
    from oracle import oracle as O
    from qsf_gb300.propagator import coupling_schedule
    steps, dx, dt, ncap = 3, 0.3, 0.05, n // 10
    rng = np.random.default_rng(n)
    x = (np.arange(n) - (n - 1) / 2.0) * dx
    env = np.exp(-(x[:, None] ** 2 + x[None, :] ** 2) / (2 * (0.35 * n * dx) ** 2))
    psi0 = env * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    pulse = dict(field=0.12, omega=0.3, ncycles=2)
    O.set_border_nodes(25, 14, 10, 40)
    oc = O.Coupling(O.GAUGE_VELOCITY, [O.Field(3, [O.Pulse(**pulse)])])
    og = O.Grid(2, n, dx, nCAP=ncap, pot=O.POT_EBERLY, Ncharge=2.0, coupling=oc)
    og.psi[...] = psi0
    prop = O.Propagator(O.MODE_RE, dt, 0, og, ["norm", "epot", ("flux", O.ZOA_FLUX_2D, 0)])
    orows = []
    for _ in range(steps):
        prop.make_step()
        prop.compute_each()
        r = prop.rows[-1]
        orows.append([r["norm"], r["epot"]] + list(r["flux"]))
    g = Q.Grid(2, n, dx, nCAP=ncap, potential=Q.POT_EBERLY, Ncharge=2.0, gauge=Q.GAUGE_VELOCITY, n_fields=1)
    g.upload(psi0)
    c = Q.Coupling(Q.GAUGE_VELOCITY, [Q.Field(3, [Q.Pulse(**pulse)])])
    rows, _ = coupling_schedule(c, dt, steps)
    out, done = g.step(Q.MODE_RE, dt, steps, rows, obs=Q.OBS_NORM | Q.OBS_EPOT, borders=Q.ZOA_FLUX_2D)
    assert done == steps
    got = np.concatenate([out[:, :2], out[:, 3:]], axis=1)
    np.testing.assert_allclose(got, np.array(orows), rtol=OBS_TOL, atol=1e-12 * float(np.max(np.abs(orows))))
    assert C.rel_l2(g.download(), og.psi) < PSI_TOL
