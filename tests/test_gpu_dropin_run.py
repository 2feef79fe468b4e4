"""The reference's own SplitPropagator::run (propagator.h:420-462), unmodified, driving
the GPU grid through the LocalGrid drop-in (include/qsf_gpu_localgrid.hpp): the user
program tests/cpp/dropin_main.cpp is compiled against the reference headers and run,
and the .dat rows its BufferedOutputs write are compared with the oracle's run of the
same system.  Imaginary time (50 steps, Normalize, E_kin, E_tot) on 64^2, then the
velocity-gauge sin^2 pulse with ZOA_FLUX_2D.

Needs the reference headers at build time ($QSF_REF_INCLUDE, or the oracle recipe's
default location) and a GPU; skipped where either is missing.
"""
import os
import re
import subprocess

import numpy as np
import pytest

import oracle
from tests import cases as C

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = oracle.ref_include()


@pytest.mark.skipif(not REF or not os.path.isdir(REF), reason="reference headers not present")
def test_reference_propagator_runs_on_the_gpu_grid(tmp_path):
    from qsf_gb300 import build as B
    from qsf_gb300 import propagator as P
    from oracle import oracle as O
    lib = B.build()
    O.build()
    exe = tmp_path / "dropin"
    cmd = ["g++", "-std=c++20", "-O1", "-w", "-DDEBUG=0", "-D_NSL", "-D_NFL", "-DPROJNAME=dropin",
           "-I", os.path.join(ROOT, "oracle", "ref", "shim"), "-I", REF, "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "dropin_main.cpp"), os.path.join(ROOT, "oracle", "liboracle.so"),
           "-L", os.path.dirname(lib), "-lqsfgpu", "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    run = subprocess.run([str(exe), "64"], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert run.returncode == 0, (run.stdout[-2000:], run.stderr[-2000:])
    # the oracle on the same system
    n, dx = 64, 0.3
    O.set_border_nodes(25, 14, 10, 40)
    gi = O.Grid(2, n, dx, nCAP=n // 10, pot=O.POT_EBERLY, Ncharge=2.0, Echarge=-1.0, Nsoft=1.0, Esoft=1.0,
                coupling=O.Coupling(O.GAUGE_VELOCITY))
    gi.add_gaussian(0.0, 1.0)
    im_rows = O.Propagator(O.MODE_IM, 0.01, 50, gi, C.IM_OUTPUTS).run()
    pulse = O.Pulse(field=0.1, omega=1.0, ncycles=1.0, shape=O.PULSE_SIN2_SIN)
    gr = O.Grid(2, n, dx, nCAP=n // 10, pot=O.POT_EBERLY, Ncharge=2.0, Echarge=-1.0, Nsoft=1.0, Esoft=1.0,
                coupling=O.Coupling(O.GAUGE_VELOCITY, [O.Field(3, [pulse])]))
    gr.psi[...] = gi.psi
    re_out = ["step", "time", "norm", "epot", ("flux", O.ZOA_FLUX_2D, 0)]
    re_rows = O.Propagator(O.MODE_RE, 0.05, 0, gr, re_out).run()
    got_im = P.read_dat(str(tmp_path / "IM.dat"), C.IM_OUTPUTS, binary=True)
    want_im = P.dat_values(im_rows, C.IM_OUTPUTS)
    assert got_im.shape == want_im.shape
    for c in range(want_im.shape[1]):
        scale = float(np.max(np.abs(want_im[:, c])))
        np.testing.assert_allclose(got_im[:, c], want_im[:, c], rtol=1e-9, atol=1e-12 * scale)
    got_re = P.read_dat(str(tmp_path / "RE.dat"), re_out, binary=True)
    want_re = P.dat_values(re_rows, re_out)
    assert got_re.shape == want_re.shape
    np.testing.assert_allclose(got_re[:, :2], want_re[:, :2], rtol=1e-14, atol=0)
    for c in range(2, want_re.shape[1]):
        scale = float(np.max(np.abs(want_re[:, c])))
        np.testing.assert_allclose(got_re[:, c], want_re[:, c], rtol=1e-9, atol=1e-12 * scale)
    m = re.search(r"norm after the pulse: (\S+)", run.stdout)
    assert m, run.stdout[-1000:]
    gr_norm = float(np.sum(np.abs(gr.psi) ** 2) * dx * dx)
    # orthogonalizeWith("ground_repX") removed the ground-state part before this norm
    assert 0.0 < float(m.group(1)) < gr_norm
