"""The .dat observable files (BufferedOutputs, buffer.h:89-91, 296-338).

The golden fixtures hold the binary .dat rows the reference's own BufferedOutputs
wrote for the harness runs, so the column order of `dat_columns` and the bytes of
`write_dat` are pinned against them through the oracle's rows.
"""
import os

import numpy as np
import pytest

from qsf_gb300 import propagator as P
from tests import cases as C


def test_im_columns_follow_buffer_classes():
    cols = [name for name, _ in P.dat_columns(C.IM_OUTPUTS)]
    assert cols == C.IM_DAT


def test_re_columns_with_flux():
    cols = P.dat_columns(C.re_outputs(2, 0))
    assert cols[:5] == [("step", None), ("time", None), ("norm", None), ("epot", None), ("ekin", None)]
    assert cols[5:] == [("flux", i) for i in range(7)]


def test_operation_and_change_placement():
    outs = ["norm", "normalize", ("flux", ["BOX"], 10), "ediff", "time", "etot"]
    assert P.dat_columns(outs) == [("ediff", None), ("time", None), ("norm", None), ("flux", 0), ("etot", None)]


@pytest.mark.parametrize("name", ["c1_vg", "c2_vg"])
def test_binary_dat_matches_reference_rows(tmp_path, name):
    z = C.load(name)
    p, dim = z["params"], int(z["dim"])
    C.set_borders(p)
    g, rows = C.oracle_im(p, dim)
    path = os.path.join(tmp_path, "im.dat")
    P.write_dat(path, rows, C.IM_OUTPUTS, binary=True)
    got = P.read_dat(path, C.IM_OUTPUTS, binary=True)
    assert os.path.getsize(path) == z["im_rows"].size * 8
    np.testing.assert_allclose(got, z["im_rows"], rtol=1e-11, atol=1e-13)
    _, rows2 = C.oracle_re(p, dim, z["re_psi0"])
    outs = C.re_outputs(dim, int(p.get("box", 0)))
    P.write_dat(path, rows2, outs, binary=True)
    got = P.read_dat(path, outs, binary=True)
    np.testing.assert_allclose(got, z["re_rows"], rtol=1e-10, atol=1e-13)


def test_text_rows_use_fmt_double(tmp_path):
    rows = [{"step": 0.0, "time": 0.0, "norm": 1.0, "flux": [1.234567e-9, -2.0]},
            {"step": 1.0, "time": 0.05, "norm": 0.999999871, "flux": [3.0e-3, 12345678.0]}]
    outs = ["step", "time", "norm", ("flux", ["A", "B"], 0)]
    path = os.path.join(tmp_path, "x.dat")
    P.write_dat(path, rows, outs)
    with open(path) as f:
        text = f.read()
    assert text.splitlines()[0] == "|            0 |            0 |            1 |   1.2346e-09 |           -2 "
    assert text.splitlines()[1] == "|            1 |         0.05 |            1 |        0.003 |   1.2346e+07 "
    back = P.read_dat(path, outs)
    np.testing.assert_allclose(back, P.dat_values(rows, outs), rtol=1e-4)
