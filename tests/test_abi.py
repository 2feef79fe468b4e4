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
