"""The CPU restatement of the .psi files (oracle/psi_io.py) against files the
reference's own LocalGrid wrote (tests/golden/io{1,2,3}.npz, made by
tests/golden/make_golden.py from grid.h:789-1153 compiled unmodified)."""
import json
import os
import warnings

import numpy as np
import pytest

from oracle import psi_io as IO

HERE = os.path.dirname(os.path.abspath(__file__))


# (fixture, dim): io1..3 at 16, 8^2, 8^3 points; *_bs at 22, 14^2, 14^3 (lengths outside
# the GPU library's built list)
IO_CASES = [("io1", 1), ("io2", 2), ("io3", 3), ("io1_bs", 1), ("io2_bs", 2), ("io3_bs", 3)]


def _golden(dim, name=None):
    z = np.load(os.path.join(HERE, "golden", f"{name or 'io%d' % dim}.npz"))
    p = json.loads(str(z["params"]))
    return z, [float(p["dx"])] * dim


def _ref_file(z, name):
    return z["file:" + name].tobytes()


SAVES = [  # (base, kwargs, file the reference wrote)
    ("sx", dict(), "sx_repX.psi"),
    ("sp", dict(rep=IO.REP_P), "sp_repP.psi"),
    ("sd", dict(downscale=2), "sd_scale2_repX.psi"),
    ("sdp", dict(rep=IO.REP_P, downscale=2), "sdp_scale2_repP.psi"),
    ("sn", dict(complex_=False), "sn_repX.psi"),
]


@pytest.mark.parametrize("name,dim", IO_CASES)
@pytest.mark.parametrize("base,kw,fname", SAVES)
def test_save_bytes_equal_reference(name, dim, base, kw, fname, tmp_path):
    z, dx = _golden(dim, name)
    path = IO.save(z["psi_in"], dx, base, directory=str(tmp_path), **kw)
    assert os.path.basename(path) == fname
    assert open(path, "rb").read() == _ref_file(z, fname)


@pytest.mark.parametrize("name,dim", IO_CASES)
def test_backup_and_snapshot_bytes(name, dim, tmp_path):
    z, dx = _golden(dim, name)
    IO.backup(z["psi_in"], dx, 7, directory=str(tmp_path))
    assert open(tmp_path / "backup.psi", "rb").read() == _ref_file(z, "backup.psi")
    assert open(tmp_path / "backup.info", "rb").read() == _ref_file(z, "backup.info")
    # a snapshot is the X-representation save under its own name and extension
    assert _ref_file(z, "snapshot_0_a_repX.psi0") == _ref_file(z, "sx_repX.psi")
    psi, step = IO.restore(z["psi_b"], directory=str(tmp_path))
    assert step == 7 and np.array_equal(psi, z["psi_in"])


@pytest.mark.parametrize("name,dim", IO_CASES)
def test_load_equals_reference(name, dim, tmp_path):
    z, dx = _golden(dim, name)
    for fname, key in (("sx_repX.psi", "psi_load_sx"), ("sn_repX.psi", "psi_load_sn")):
        (tmp_path / fname).write_bytes(_ref_file(z, fname))
        psi, h = IO.load(str(tmp_path / fname), z["psi_b"])
        assert h["dim"] == dim and h["downscale"] == 1
        assert np.array_equal(psi, z[key]), fname


@pytest.mark.parametrize("name,dim", [c for c in IO_CASES if c[1] < 3])
def test_orthogonalize_reproduces_reference_offset(name, dim, tmp_path):
    """The reference reads the payload 3 bytes early; where its result is finite the
    restatement with the same offset gives the same values."""
    z, dx = _golden(dim, name)
    (tmp_path / "sx_repX.psi").write_bytes(_ref_file(z, "sx_repX.psi"))
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        out, _, _ = IO.orthogonalize_with(str(tmp_path / "sx_repX.psi"), z["psi_b"], dx)
    ref = z["psi_orth"]
    fin = np.isfinite(ref)
    assert fin.any() and np.array_equal(out[fin], ref[fin])


@pytest.mark.parametrize("name,dim", IO_CASES)
def test_orthogonalize_at_payload_projects_out(name, dim, tmp_path):
    """psi -= <f|psi> dV f removes f from psi when f is normalised (<f|f> dV = 1)."""
    z, dx = _golden(dim, name)
    dV = float(np.prod(dx))
    f = z["psi_in"] / np.sqrt(np.sum(np.abs(z["psi_in"]) ** 2) * dV)
    path = IO.save(f, dx, "s", directory=str(tmp_path))
    out, sp, nrm = IO.orthogonalize_with(path, z["psi_b"], dx, offset=IO.header_size(dim))
    assert sp == pytest.approx(np.vdot(f, z["psi_b"]) * dV, rel=1e-13)
    assert abs(np.vdot(f, out) * dV) < 1e-12 * abs(sp)
    assert nrm == pytest.approx(float(np.sum(np.abs(out) ** 2)) * dV, rel=1e-13)


def test_downscale_must_divide(tmp_path):
    z, dx = _golden(2)
    with pytest.raises(ValueError):
        IO.save(z["psi_in"], dx, "x", downscale=3, directory=str(tmp_path))
