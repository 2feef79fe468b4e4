"""Ionization yields from the step observables.

The reference computes border fluxes but no yields; its Mathematica post-processing
combines the ZOA_FLUX_2D fluxes into derived rates (flx.wl:97-104) and integrates them
over time.  These helpers do the same on the rows `SplitPropagator.run` returns
(dicts with a "flux" list in the order of the flux output's borders):

* derived rates: N2* = N2S + N2D_SYM + N2D_ASYM (out of the neutral region),
  *2S = N2S - S2D_SYM - S2D_ASYM (net single ionization), *2D = N2D_SYM + N2D_ASYM +
  S2D_SYM + S2D_ASYM (double ionization), *2D_SYM, *2D_ASYM, *2CAP = S2CAP + D2CAP;
* yields: the time integrals of the rates (rectangle rule, the same sum the serving loop
  reports as flux integrals), and for one electron 1 - norm(T) and
  1 - |<psi_0|psi(T)>|^2 (the projection orthogonalizeWith removes, grid.h:909-946).
"""
from __future__ import annotations

from typing import Dict, List, Sequence

import numpy as np

DERIVED = {
    "N2*": (("N2S", 1), ("N2D_SYM", 1), ("N2D_ASYM", 1)),
    "*2S": (("N2S", 1), ("S2D_SYM", -1), ("S2D_ASYM", -1)),
    "*2D": (("N2D_SYM", 1), ("N2D_ASYM", 1), ("S2D_SYM", 1), ("S2D_ASYM", 1)),
    "*2D_SYM": (("N2D_SYM", 1), ("S2D_SYM", 1)),
    "*2D_ASYM": (("N2D_ASYM", 1), ("S2D_ASYM", 1)),
    "*2CAP": (("S2CAP", 1), ("D2CAP", 1)),
}


def flux_table(rows: Sequence[dict], borders: Sequence[str]) -> Dict[str, np.ndarray]:
    """Per-border flux time series from propagator rows (rows without fluxes are skipped)."""
    data = [r["flux"] for r in rows if r.get("flux")]
    arr = np.array(data, dtype=np.float64).reshape(len(data), len(borders))
    return {b: arr[:, i] for i, b in enumerate(borders)}


def derived_rates(fluxes: Dict[str, np.ndarray]) -> Dict[str, np.ndarray]:
    """FLXDerivedData (flx.wl:97-104) for the borders present."""
    out = {}
    for name, terms in DERIVED.items():
        if all(b in fluxes for b, _ in terms):
            out[name] = sum(s * fluxes[b] for b, s in terms)
    return out


def flux_yields(rows: Sequence[dict], borders: Sequence[str], dt: float) -> Dict[str, float]:
    """Time integrals (sum of rate * dt over the steps) of every border flux and derived rate."""
    f = flux_table(rows, borders)
    rates = dict(f)
    rates.update(derived_rates(f))
    return {k: float(np.sum(v) * dt) for k, v in rates.items()}


def one_electron_yields(norm_T: float, overlap_with_initial: complex) -> Dict[str, float]:
    """1 - norm(T) and 1 - |<psi_0|psi(T)>|^2 (psi_0 normalised)."""
    return {"1-norm": 1.0 - float(norm_T), "1-|<psi0|psi>|^2": 1.0 - abs(complex(overlap_with_initial)) ** 2}


def ionization_from_rows(rows: List[dict]) -> float:
    """1 - norm at the last row (absorbed probability)."""
    return 1.0 - float(rows[-1]["norm"])
