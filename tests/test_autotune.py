"""The autotuner's choice logic (qsf_gb300/autotune.py) on fixed timings, and the
committed tuning table it generated: per edge the thread count with the least summed
step time over that edge's workloads (2D grid and 3D cube share kernels)."""
import os
import re

from qsf_gb300 import autotune as A

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_choice_sums_over_the_workloads_of_an_edge():
    A4, A5, B2 = (4096, 256), (4096, 512), (2048, 256)
    times = {("2d256", A4): 0.089, ("2d256", A5): 0.079, ("2d256", B2): 0.083,
             ("3d256", A4): 2.13, ("3d256", A5): 2.21, ("3d256", B2): 2.40,
             ("2d2048", A4): 0.60, ("2d2048", A5): 0.51, ("2d2048", B2): 0.70}
    ch = A.choose(times)
    assert ch == {256: A4, 2048: A5}   # the cube outweighs the grid at 256


def test_header_encodes_the_choice():
    times = {(w, c): 1.0 for w, _ in A.TUNE_WORKLOADS for c in A.ALL_CANDIDATES}
    txt = A.header_text({384: (4096, 512), 512: (2048, 256), 2048: (4096, 512), 256: (2048, 128),
                         1024: (4096, 256)}, times)
    assert "return n == 384 ? 512 : n == 2048 ? 512 : n == 256 ? 128 : 256;" not in txt  # ordered by n
    assert "return n == 256 ? 128 : n == 384 ? 512 : n == 2048 ? 512 : 256;" in txt
    assert "return n == 256 ? 2048 : n == 512 ? 2048 : 4096;" in txt
    plain = A.header_text({256: A.DEFAULT_SHAPE}, times)
    assert "tuned_row_threads(int n) {\n  return 256;" in plain and "tuned_tile(int n) {\n  return 4096;" in plain


def test_committed_table_is_the_autotuner_output():
    txt = open(os.path.join(ROOT, "qsf_gb300", "csrc", "qsf_tuning.h")).read()
    assert "python -m qsf_gb300.autotune --write" in txt
    times = A.committed_row_times()
    assert times and {w for w, _ in times} <= {w for w, _ in A.TUNE_WORKLOADS}
    ch = A.choose({k: v for k, v in times.items() if k[1] in A.CANDIDATES})
    threads = re.search(r"tuned_row_threads\(int n\) \{\s*return (.*);", txt).group(1)
    tile = re.search(r"tuned_tile\(int n\) \{\s*return (.*);", txt).group(1)
    assert threads == A.shape_function(ch, 1, A.DEFAULT_SHAPE[1])
    assert tile == A.shape_function(ch, 0, A.DEFAULT_SHAPE[0])


def test_line_plans_choose_the_fastest_valid_plan_per_length():
    lt = {("1d1024", 4): 0.030, ("1d1024", 8): 0.031, ("1d1024", 16): 0.039,
          ("1d2048", 4): 0.055, ("1d2048", 8): 0.051, ("1d2048", 16): 0.053,
          ("1d4096", 4): 0.010,  # a plan that does not fit (4 points x 512 threads < 4096): ignored
          ("1d4096", 8): 0.073, ("1d4096", 16): 0.069}
    ch = A.choose_lines(lt)
    assert ch == {1024: 4, 2048: 8, 4096: 16}
    assert not A.line_valid(4096, 4) and A.line_valid(4096, 8)
    assert A.line_function({1024: 4, 2048: 8, 4096: 16}) == "n <= 1024 ? 4 : n <= 2048 ? 8 : 16"
    assert A.line_function({1024: 16, 4096: 16}) == "16"


def test_committed_line_plans_match_their_timings():
    txt = open(os.path.join(ROOT, "qsf_gb300", "csrc", "qsf_tuning.h")).read()
    lt = {}
    for w, cells in re.findall(r"//\s+(1d\d+)\s+ms/step\s+(.*)", txt):
        for p, ms in re.findall(r"(\d+): ([0-9.]+)", cells):
            lt[(w, int(p))] = float(ms)
    assert lt, "no line plan timings in the table"
    expr = re.search(r"tuned_line_ppt\(int n\) \{\s*return (.*);", txt).group(1)
    assert expr == A.line_function(A.choose_lines(lt))
