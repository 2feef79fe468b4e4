"""The autotuner's choice logic (qsf_gb300/autotune.py) on fixed timings, and the
committed tuning table it generated: per edge the thread count with the least summed
step time over that edge's workloads (2D grid and 3D cube share kernels)."""
import os
import re

from qsf_gb300 import autotune as A

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_choice_sums_over_the_workloads_of_an_edge():
    times = {("2d256", 256): 0.089, ("2d256", 512): 0.079, ("3d256", 256): 2.13, ("3d256", 512): 2.21,
             ("2d2048", 256): 0.60, ("2d2048", 512): 0.51}
    ch = A.choose(times)
    assert ch == {256: 256, 2048: 512}   # the cube outweighs the grid at 256


def test_header_encodes_the_choice():
    times = {(w, t): 1.0 for w, _ in A.TUNE_WORKLOADS for t in A.CANDIDATES}
    txt = A.header_text({384: 512, 512: 512, 2048: 512, 256: 256}, times)
    assert "return (n == 384 || n == 512 || n == 2048) ? 512 : 256;" in txt
    assert "return (false) ? 512 : 256;" in A.header_text({256: 256}, times)


def test_committed_table_is_the_autotuner_output():
    txt = open(os.path.join(ROOT, "qsf_gb300", "csrc", "qsf_tuning.h")).read()
    assert "python -m qsf_gb300.autotune --write" in txt
    rows = dict(re.findall(r"//\s+(\S+)\s+ms/step\s+256: ([0-9.]+)\s+512: [0-9.]+", txt))
    assert set(rows) == {w for w, _ in A.TUNE_WORKLOADS}
    times = {}
    for line in re.findall(r"//\s+(\S+)\s+ms/step\s+256: ([0-9.]+)\s+512: ([0-9.]+)", txt):
        w, a, b = line
        times[(w, 256)] = float(a)
        times[(w, 512)] = float(b)
    cond = re.search(r"return \((.*)\) \? 512 : 256;", txt).group(1)
    big = {int(v) for v in re.findall(r"n == (\d+)", cond)}
    assert big == {n for n, t in A.choose(times).items() if t == 512}
