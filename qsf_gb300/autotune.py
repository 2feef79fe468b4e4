"""Autotuner of the row / axis pass kernels: threads per block per line length.

The count sets the radix plan with it: 256 threads carry 16 points of a 4096-point tile
each (radix-16 passes, 128 registers), 512 threads 8 points (radix-8 passes, 64
registers, twice the resident warps).  For each candidate count the library is built
with every line length forced to it (`QSF_ROW_THREADS`, in qsf_gb300/_build/tune_<T>/);
each tuning workload's fused step is timed as a user runs it (`profile_step --timed`:
one call of K graph-replayed steps after a warm-up call) in a subprocess that loads that
build; per line length the count with the least summed step time over the workloads of
that edge wins (the 2D grid and the 3D cube of one edge share their kernels).  With
--write the choice goes to qsf_gb300/csrc/qsf_tuning.h, which the default build
compiles in.  Needs a GPU.

    python -m qsf_gb300.autotune [--repeat 2] [--write]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys

from . import build as B
from .profile_step import WORKLOADS

CANDIDATES = (256, 512)
# (workload of profile_step, steps per timed call)
TUNE_WORKLOADS = [("2d256", 400), ("2d384", 400), ("2d512", 400), ("2d768", 300), ("2d1024", 300),
                  ("2d2048", 100), ("2d4096", 30), ("3d128", 100), ("3d256", 30)]
HEADER = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc", "qsf_tuning.h")


def time_workload(lib_path: str, workload: str, steps: int, repeat: int) -> float:
    """Least ms per step over `repeat` timed calls in a process that loads `lib_path`."""
    env = dict(os.environ, QSF_LIB=lib_path)
    best = float("inf")
    for _ in range(repeat):
        r = subprocess.run([sys.executable, "-m", "qsf_gb300.profile_step", "--workload", workload, "--steps",
                            str(steps), "--timed"], capture_output=True, text=True, env=env)
        if r.returncode != 0:
            raise RuntimeError(f"{workload} with {lib_path} failed:\n{r.stderr[-2000:]}")
        best = min(best, json.loads(r.stdout.strip().splitlines()[-1])["timed_ms_per_step"])
    return best


def choose(times: dict) -> dict:
    """times[(workload, T)] -> ms per step; returns edge -> chosen T (summed over the
    workloads of each edge)."""
    edges = {}
    for (w, t), ms in times.items():
        edges.setdefault(WORKLOADS[w][1], {}).setdefault(t, 0.0)
        edges[WORKLOADS[w][1]][t] += ms
    return {n: min(per, key=lambda t: per[t]) for n, per in edges.items()}


def header_text(choice: dict, times: dict) -> str:
    rows = []
    for w, _ in TUNE_WORKLOADS:
        cells = "  ".join(f"{t}: {times[(w, t)]:.4f}" for t in CANDIDATES if (w, t) in times)
        rows.append(f"//   {w:7s} ms/step  {cells}")
    big = sorted(n for n, t in choice.items() if t != 256)
    cond = " || ".join(f"n == {n}" for n in big) or "false"
    return f"""// qsf_tuning.h -- threads per block of the row / axis pass kernels per line length.
//
// Written by the autotuner (qsf_gb300/autotune.py) from step times measured on a GB300:
//   python -m qsf_gb300.autotune --write
// 256 threads carry 16 points of a 4096-point tile each (radix-16 plans, 128 registers),
// 512 threads 8 points (radix-8 plans, 64 registers, twice the resident warps).  Line
// lengths not listed take 256.  Measured (one call of graph-replayed steps per
// workload, threads per block: ms per step):
{chr(10).join(rows)}
#pragma once

namespace qsf {{

__host__ __device__ constexpr int tuned_row_threads(int n) {{
  return ({cond}) ? 512 : 256;
}}

}}  // namespace qsf
"""


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--repeat", type=int, default=2)
    ap.add_argument("--write", action="store_true", help="rewrite qsf_gb300/csrc/qsf_tuning.h")
    args = ap.parse_args()
    times = {}
    for t in CANDIDATES:
        lib_path = B.build(defines=[f"QSF_ROW_THREADS={t}"], tag=f"tune_{t}")
        for w, steps in TUNE_WORKLOADS:
            times[(w, t)] = time_workload(lib_path, w, steps, args.repeat)
            print(json.dumps({"workload": w, "threads": t, "ms_per_step": times[(w, t)]}), flush=True)
    choice = choose(times)
    print(json.dumps({"choice": {str(n): t for n, t in sorted(choice.items())}}), flush=True)
    if args.write:
        with open(HEADER, "w") as f:
            f.write(header_text(choice, times))


if __name__ == "__main__":
    main()
