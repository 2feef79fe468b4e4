"""The GPU library's .psi files (qsf_save / qsf_load / qsf_backup / qsf_restore /
qsf_orthogonalize_with) against files the reference's LocalGrid wrote
(tests/golden/io{1,2,3}.npz) and against the CPU restatement (oracle/psi_io.py)."""
import json
import os

import numpy as np
import pytest

from oracle import psi_io as IO

HERE = os.path.dirname(os.path.abspath(__file__))

pytestmark = pytest.mark.gpu


# (fixture, dim): io1..3 at 16, 8^2, 8^3 points; *_bs at 22, 14^2, 14^3 (lengths outside
# the built list: Bluestein transforms in the P-representation saves)
IO_CASES = [("io1", 1), ("io2", 2), ("io3", 3), ("io1_bs", 1), ("io2_bs", 2), ("io3_bs", 3)]


def _golden(dim, name=None):
    z = np.load(os.path.join(HERE, "golden", f"{name or 'io%d' % dim}.npz"))
    p = json.loads(str(z["params"]))
    return z, p


def _grid(dim, p, psi):
    import qsf_gb300 as Q
    g = Q.Grid(dim, int(p["n"]), float(p["dx"]), nCAP=int(p["nCAP"]))
    g.upload(psi)
    return g


def _payload(raw: bytes, dim: int):
    h = IO.parse_header(raw)
    dt = np.complex128 if h["complex"] else np.float64
    return raw[:h["offset"]], np.frombuffer(raw[h["offset"]:], dtype=dt)


@pytest.mark.parametrize("name,dim", IO_CASES)
def test_save_matches_reference_files(name, dim, tmp_path, monkeypatch):
    import qsf_gb300 as Q
    monkeypatch.chdir(tmp_path)
    z, p = _golden(dim, name)
    g = _grid(dim, p, z["psi_in"])
    # X representation: the same bytes as the reference
    for kw, fname in ((dict(), "sx_repX.psi"), (dict(downscale=2), "sd_scale2_repX.psi"),
                      (dict(complex=False), "sn_repX.psi")):
        base = fname.split("_")[0]
        path = g.save(base, **kw)
        assert path == fname
        assert open(path, "rb").read() == z["file:" + fname].tobytes(), fname
    # P representation: same header, payload within the transform's rounding
    for kw, fname in ((dict(rep=Q.REP_P), "sp_repP.psi"), (dict(rep=Q.REP_P, downscale=2), "sdp_scale2_repP.psi")):
        base = fname.split("_")[0]
        path = g.save(base, **kw)
        assert path == fname
        h_gpu, d_gpu = _payload(open(path, "rb").read(), dim)
        h_ref, d_ref = _payload(z["file:" + fname].tobytes(), dim)
        assert h_gpu == h_ref
        assert np.max(np.abs(d_gpu - d_ref)) <= 1e-13 * np.max(np.abs(d_ref)), fname
    # the P saves transformed psi and back
    psi = g.download()
    assert np.linalg.norm(psi - z["psi_in"]) <= 1e-14 * np.linalg.norm(z["psi_in"])
    g.close()


@pytest.mark.parametrize("name,dim", IO_CASES)
def test_load_backup_restore(name, dim, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    z, p = _golden(dim, name)
    for fname in ("sx_repX.psi", "sn_repX.psi"):
        (tmp_path / fname).write_bytes(z["file:" + fname].tobytes())
    g = _grid(dim, p, z["psi_b"])
    nrm = g.load("sx_repX")
    assert np.array_equal(g.download(), z["psi_load_sx"])
    assert g.load_warnings == 0
    dV = float(p["dx"]) ** dim
    assert nrm == pytest.approx(float(np.sum(np.abs(z["psi_load_sx"]) ** 2)) * dV, rel=1e-13)
    g.upload(z["psi_b"])
    g.load("sn_repX")
    assert g.load_warnings == 4
    # each element becomes its modulus through the host libm's hypot (as std::abs does
    # in the reference); libm builds may differ in the last bit
    np.testing.assert_allclose(g.download(), z["psi_load_sn"], rtol=2.3e-16, atol=0)
    # backup / restore
    g.upload(z["psi_in"])
    g.backup(7)
    assert open("backup.psi", "rb").read() == z["file:backup.psi"].tobytes()
    assert open("backup.info", "rb").read() == z["file:backup.info"].tobytes()
    g.upload(z["psi_b"])
    assert g.restore() == 7
    assert np.array_equal(g.download(), z["psi_in"])
    g.remove_backups()
    assert not os.path.exists("backup.psi")
    g.close()


@pytest.mark.parametrize("name,dim", IO_CASES)
def test_orthogonalize_matches_oracle(name, dim, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    z, p = _golden(dim, name)
    dx = [float(p["dx"])] * dim
    dV = float(np.prod(dx))
    f = z["psi_in"] / np.sqrt(np.sum(np.abs(z["psi_in"]) ** 2) * dV)
    path = IO.save(f, dx, "f")
    ref, sp_ref, nrm_ref = IO.orthogonalize_with(path, z["psi_b"], dx, offset=IO.header_size(dim))
    g = _grid(dim, p, z["psi_b"])
    sp, nrm = g.orthogonalize_with("f_repX")
    assert sp == pytest.approx(sp_ref, rel=1e-13)
    assert nrm == pytest.approx(nrm_ref, rel=1e-12)
    out = g.download()
    assert np.linalg.norm(out - ref) <= 1e-13 * np.linalg.norm(ref)
    g.close()


def test_snapshot_names(tmp_path, monkeypatch):
    import qsf_gb300 as Q
    monkeypatch.chdir(tmp_path)
    z, p = _golden(2)
    g = _grid(2, p, z["psi_in"])
    Q.Grid._snapshot_counts.clear()
    a = g.snapshot("_a")
    b = g.snapshot("_b")
    assert (a, b) == ("snapshot_0_a_repX.psi0", "snapshot_1_b_repX.psi0")
    assert open(a, "rb").read() == z["file:snapshot_0_a_repX.psi0"].tobytes()
    g.close()


def test_bad_files_are_errors(tmp_path, monkeypatch):
    import qsf_gb300 as Q
    monkeypatch.chdir(tmp_path)
    z, p = _golden(2)
    (tmp_path / "one_d.psi").write_bytes(_golden(1)[0]["file:sx_repX.psi"].tobytes())
    g = _grid(2, p, z["psi_in"])
    with pytest.raises(Q.QsfError):
        g.load("one_d")
    with pytest.raises(Q.QsfError):
        g.load("missing")
    with pytest.raises(Q.QsfError):
        g.save("x", downscale=3)
    g.close()


def _re_prop():
    import qsf_gb300 as Q
    n, dx = 256, 0.2
    g = Q.Grid(1, n, dx, nCAP=25, n_fields=1)
    x = (np.arange(n) - (n - 1) / 2.0) * dx
    psi = np.exp(-0.5 * x * x).astype(np.complex128)
    psi /= np.sqrt(np.sum(np.abs(psi) ** 2) * dx)
    g.upload(psi)
    c = Q.Coupling(Q.GAUGE_VELOCITY, [Q.Field(1, [Q.Pulse(field=0.05, omega=0.5, ncycles=1.0)])])
    return g, Q.SplitPropagator(Q.MODE_RE, 0.05, 0, g, c, ["norm", "epot"])


def test_run_restore_continues_the_same_run(tmp_path, monkeypatch):
    """run(restore=True) after a backup at step k ends in the same state, bit for bit,
    as the uninterrupted run (propagator.h:420-462)."""
    monkeypatch.chdir(tmp_path)
    ga, pa = _re_prop()
    rows_a = pa.run()
    psi_a = ga.download()
    gb, pb = _re_prop()
    pb.rows.append(pb.compute_at_start())
    pb.run_steps(40)
    gb.backup(pb.step)
    gc, pc = _re_prop()
    rows_c = pc.run(restore=True)
    assert pc.step == pa.step
    assert np.array_equal(gc.download(), psi_a)
    assert [r["norm"] for r in rows_c] == [r["norm"] for r in rows_a[41:]]
    assert not os.path.exists("backup.info") and not os.path.exists("backup.psi")
    for g in (ga, gb, gc):
        g.close()
