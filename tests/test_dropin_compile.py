"""The LocalGrid drop-in (include/qsf_gpu_localgrid.hpp) compiles and links against the
reference's own unmodified headers and libqsfgpu.so.

Needs the reference checkout (development container only); running the binary needs a
GPU and the reference headers at build time together, which no single machine here
has, so this test stops at the link.  The single-rank MPI / FFTW stand-ins of the
oracle harness satisfy the reference's includes of mpi.h and fftw3.h.
"""
import os
import subprocess

import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = oracle.ref_include()  # $QSF_REF_INCLUDE or the oracle recipe's default


@pytest.mark.skipif(not REF or not os.path.isdir(REF), reason="reference checkout not present")
def test_reference_propagator_with_gpu_grid_compiles_and_links(tmp_path):
    from qsf_gb300 import build as B
    lib = B.build()
    from oracle import oracle as O
    O.build()
    exe = tmp_path / "dropin"
    cmd = ["g++", "-std=c++20", "-O1", "-w", "-DDEBUG=0", "-D_NSL", "-D_NFL", "-DPROJNAME=dropin",
           "-I", os.path.join(ROOT, "oracle", "ref", "shim"), "-I", REF, "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "dropin_main.cpp"), os.path.join(ROOT, "oracle", "liboracle.so"),
           "-L", os.path.dirname(lib), "-lqsfgpu", "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    assert exe.exists()
