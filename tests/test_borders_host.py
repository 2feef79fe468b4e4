"""The library's host-side border vectors (qsf_gb300/csrc/qsf_borders.h, which build the
sparse flux point lists) against the oracle's restatement of fluxes/borders*.h, point
by point on the CPU: every border type of 1D / 2D / 3D grids, over every centred index
within the borders' reach, with the reference's default node positions and with small
ones.  Bit-exact: both evaluate the same integer region tests and one normalisation."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "qsf_gb300", "csrc")
INCLUDE = os.path.join(ROOT, "include")

DRIVER = r"""
#include <cstdio>
#include <cstdlib>
#include "qsf_borders.h"
// argv: dim type box NS SD DT CAP reach -> one line per centred index: ok w0 w1 w2
int main(int argc, char** argv) {
  const int dim = atoi(argv[1]), type = atoi(argv[2]);
  const long long box = atoll(argv[3]);
  qsf::BorderNodes B;
  B.NS = atoll(argv[4]); B.SD = atoll(argv[5]); B.DT = atoll(argv[6]); B.CAP = atoll(argv[7]);
  const long long R = atoll(argv[8]);
  const long long lo1 = dim > 1 ? -R : 0, hi1 = dim > 1 ? R : 0, lo2 = dim > 2 ? -R : 0, hi2 = dim > 2 ? R : 0;
  for (long long i = -R; i <= R; ++i)
    for (long long j = lo1; j <= hi1; ++j)
      for (long long k = lo2; k <= hi2; ++k) {
        const int64_t ci[3] = {i, j, k};
        double w[3];
        const bool ok = qsf::border_vector(type, box, dim, ci, B, w);
        printf("%d %.17g %.17g %.17g\n", ok ? 1 : 0, w[0], w[1], w[2]);
      }
  return 0;
}
"""

TYPES = {1: ["BOX"], 2: ["BOX", "S2CAP", "D2CAP", "N2S", "N2D", "N2D_SYM", "N2D_ASYM", "S2D", "S2D_SYM", "S2D_ASYM"],
         3: ["BOX", "S2CAP", "D2CAP", "N2S", "N2D", "S2D", "N2T", "S2T", "D2T", "T2CAP"]}
NODES = [(25, 14, 10, 40), (6, 4, 3, 12)]


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("borders")
    src = d / "borders.cpp"
    src.write_text(DRIVER)
    exe = d / "borders"
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", CSRC, "-I", INCLUDE, str(src), "-o", str(exe)], check=True)
    return str(exe)


def _host(driver, dim, btype, box, nodes, reach):
    out = subprocess.run([driver, str(dim), str(O.BORDERS[btype]), str(box)] + [str(v) for v in nodes] + [str(reach)],
                         check=True, capture_output=True, text=True).stdout
    a = np.array([[float(x) for x in ln.split()] for ln in out.splitlines()])
    return a[:, 0], a[:, 1:1 + dim]


@pytest.mark.parametrize("nodes", NODES)
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_border_vectors_match_oracle(driver, dim, nodes):
    O.set_border_nodes(*nodes)
    try:
        # every centred index within the set's reach; 3D with the default nodes on a
        # band of it (the whole cube would be 91^3 oracle calls per type)
        band = dim == 3 and nodes == NODES[0]
        for btype in TYPES[dim]:
            for box in ((0, 7, 20) if btype == "BOX" else (0,)):
                reach = 14 if band else max(max(nodes), box) + 2
                ok, got = _host(driver, dim, btype, box, nodes, reach)
                assert ok.all(), (dim, btype)
                rng = range(-reach, reach + 1)
                if dim == 1:
                    pts = [(i,) for i in rng]
                elif dim == 2:
                    pts = [(i, j) for i in rng for j in rng]
                else:
                    pts = [(i, j, k) for i in rng for j in rng for k in rng]
                ref = np.array([O.border_vector(btype, dim, p, box) for p in pts])
                assert np.array_equal(got, ref), (dim, btype, box, int(np.sum(np.any(got != ref, axis=1))))
                if not band and (btype != "BOX" or box):
                    assert np.any(ref != 0.0), (dim, btype, box)  # the region lies within the reach
    finally:
        O.set_border_nodes()
