"""The C ABI library: it loads without a GPU and exports every declared symbol.

No compute call is made here (no GPU in this container); host-only helpers of the
ABI (FFT planning) are exercised.
"""
import ctypes
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "qsf_gpu.h")


@pytest.fixture(scope="module")
def lib():
    from qsf_gb300 import build as B
    B.build()
    from qsf_gb300 import _lib
    return _lib.lib()


def test_header_declares_entry_points():
    from qsf_gb300 import _lib
    names = _lib.exported_symbols(HEADER)
    for must in ("qsf_grid_create", "qsf_step", "qsf_fourier", "qsf_evolve", "qsf_average", "qsf_flux",
                 "qsf_normalize", "qsf_mask_region"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    from qsf_gb300 import _lib
    missing = [n for n in _lib.exported_symbols(HEADER) if not hasattr(lib, n)]
    assert not missing, missing


def test_fft_plans(lib):
    import qsf_gb300 as Q
    assert Q.fft_radices(2048) == [16, 16, 8]
    assert Q.fft_radices(4096) == [16, 16, 16]
    assert Q.fft_radices(384) == [16, 8, 3]
    assert Q.fft_radices(640) == [16, 8, 5]
    with pytest.raises(Q.QsfError):
        Q.fft_radices(7 * 64)


def test_status_names_match_the_header():
    """The binding's names of the QSF_E* status codes are the header's."""
    import re
    from qsf_gb300 import _lib
    codes = {int(v): k for k, v in re.findall(r"#define QSF_(E[A-Z]+)\s+(\d+)", open(HEADER).read())}
    assert codes and codes == _lib.ERRORS
    assert re.search(r"#define QSF_OK 0\b", open(HEADER).read()) and _lib.QSF_OK == 0


def test_struct_layouts_match_the_header(tmp_path):
    """Every ctypes mirror of a header struct has the C compiler's size and field
    offsets (a probe program compiled against include/qsf_gpu.h prints them)."""
    import shutil
    import subprocess
    from qsf_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    pairs = {"qsf_grid_desc": _lib.GridDesc, "qsf_step_desc": _lib.StepDesc, "qsf_request": _lib.Request,
             "qsf_result": _lib.Result, "qsf_server_config": _lib.ServerConfig,
             "qsf_server_stats": _lib.ServerStats, "qsf_dump_format": _lib.DumpFormat}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "qsf_gpu.h"', "int main(void) {"]
    for cname, py in pairs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            # a trailing underscore in Python stands for a C name that is a Python keyword
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname.rstrip("_")}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(ln.split()[:2]): int(ln.split()[2]) for ln in out if ln.strip()}
    for cname, py in pairs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


def test_kernel_kinds_match_the_header():
    """qsf_step's per-kernel timing slots (QSF_K_*) in the binding's order."""
    import re
    from qsf_gb300 import _lib
    kinds = dict(re.findall(r"#define QSF_K_([A-Z_]+)\s+(\d+)", open(HEADER).read()))
    count = int(kinds.pop("COUNT"))
    order = [k.lower() for k, _ in sorted(kinds.items(), key=lambda kv: int(kv[1]))]
    assert order == _lib.KERNEL_KINDS and count == len(order)


def test_python_constants_match_the_header():
    """Every QSF_<NAME> integer the package also exports as <NAME> (modes,
    representations, potentials, gauges, observables, operators, absorbers) and every
    border type QSF_B_<NAME> (BORDERS) has the header's value."""
    import re
    import qsf_gb300 as Q
    from qsf_gb300 import _lib
    defs = {k: int(v) for k, v in re.findall(r"#define QSF_([A-Z0-9_]+)\s+(\d+)u?\b", open(HEADER).read())}
    shared = [k for k in defs if hasattr(Q, k)]
    assert len(shared) >= 15, shared
    for k in shared:
        assert getattr(Q, k) == defs[k], k
    borders = {k[2:]: v for k, v in defs.items() if k.startswith("B_")}
    assert borders == Q.BORDERS
    assert defs["MAX_BORDERS"] == _lib.MAX_BORDERS
