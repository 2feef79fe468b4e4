"""Yields from the observables rows (qsf_gb300/yields.py, flx.wl:97-104 restated)."""
import numpy as np
import pytest

from tests import cases as C


def test_derived_rates_and_integrals_from_reference_rows():
    from qsf_gb300 import yields as Y
    from qsf_gb300.grid import ZOA_FLUX_2D
    z = C.load("c2_vg")
    ref = z["re_rows"]  # step, time, norm, epot, ekin, 7 ZOA_FLUX_2D fluxes
    rows = [{"flux": list(r[5:12]), "norm": r[2]} for r in ref]
    f = Y.flux_table(rows, ZOA_FLUX_2D)
    d = Y.derived_rates(f)
    np.testing.assert_allclose(d["N2*"], ref[:, 5] + ref[:, 6] + ref[:, 7])
    np.testing.assert_allclose(d["*2D"], ref[:, 6] + ref[:, 7] + ref[:, 8] + ref[:, 9])
    np.testing.assert_allclose(d["*2S"], ref[:, 5] - ref[:, 8] - ref[:, 9])
    y = Y.flux_yields(rows, ZOA_FLUX_2D, dt=0.05)
    assert y["*2CAP"] == pytest.approx(float(np.sum(ref[:, 10] + ref[:, 11]) * 0.05))
    assert Y.ionization_from_rows(rows) == pytest.approx(1.0 - ref[-1, 2])


def test_one_electron_yields():
    from qsf_gb300 import yields as Y
    y = Y.one_electron_yields(0.9, 0.8 + 0.3j)
    assert y["1-norm"] == pytest.approx(0.1)
    assert y["1-|<psi0|psi>|^2"] == pytest.approx(1 - 0.73)
