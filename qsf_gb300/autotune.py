"""Autotuner of the pass kernels: the shape of the row / axis passes per line length
(points per block and threads per block), and the radix plan (points per thread) of the
one-CTA 1D line kernel per length.

A row / axis shape is a tile of whole lines (1024, 2048 or 4096 points per block, or
one line when lines are longer) and a thread count; their ratio, the points each thread
carries per pass, sets the radix plan (16: radix 16, 128 registers; 8: radix 8).
Smaller tiles give small grids more blocks (a 256^2 grid is 16 blocks of 4096 points
on 152 SMs).  For each candidate shape the library is built with every line length
forced to it (`QSF_TILE`, `QSF_ROW_THREADS`, in qsf_gb300/_build/tune_<tile>_<threads>/);
each tuning workload's fused step is timed as a user runs it (`profile_step --timed`:
one call of K graph-replayed steps after a warm-up call) in a subprocess that loads that
build; per line length the shape with the least summed step time over the workloads of
that edge wins (the 2D grid and the 3D cube of one edge share their kernels).  With
--write the choice goes to qsf_gb300/csrc/qsf_tuning.h, which the default build
compiles in.  The 1D line kernel's plan is tuned the same way: candidate builds force 4,
8 or 16 points per thread (`QSF_LINE_PPT`, at least n / 512), the 1D workloads are
timed, and each measured length keeps its fastest plan; a length between measured ones
takes the plan of the next longer measured length.  Needs a GPU.

    python -m qsf_gb300.autotune [--repeat 2] [--write] [--only rows|lines]
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys

from . import build as B
from .profile_step import WORKLOADS

# (points per block, threads per block) of the row / axis passes.  The committed table
# comes from the 4096-point tiles: smaller tiles (--shapes all) make small grids faster
# alone (2D 512^2 0.0725 -> 0.0499 ms per step with 1024 x 128) but the 256-solve batch
# slower (1.25e10 -> 1.19e10 grid-pt-steps/s), where the solves already fill the GPU.
CANDIDATES = ((4096, 256), (4096, 512))
ALL_CANDIDATES = ((4096, 256), (4096, 512), (2048, 128), (2048, 256), (1024, 128))
DEFAULT_SHAPE = (4096, 256)
LINE_CANDIDATES = (4, 8, 16)
LINE_WORKLOADS = [("1d1024", 400), ("1d1536", 400), ("1d2048", 400), ("1d3072", 400), ("1d4096", 400)]
# (workload of profile_step, steps per timed call)
TUNE_WORKLOADS = [("2d256", 400), ("2d320", 400), ("2d384", 400), ("2d512", 400), ("2d640", 300), ("2d768", 300),
                  ("2d1024", 300), ("2d2048", 100), ("2d4096", 30), ("3d128", 100), ("3d256", 30)]
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
    """times[(workload, shape)] -> ms per step; returns edge -> chosen shape (summed over
    the workloads of each edge)."""
    edges = {}
    for (w, t), ms in times.items():
        edges.setdefault(WORKLOADS[w][1], {}).setdefault(t, 0.0)
        edges[WORKLOADS[w][1]][t] += ms
    return {n: min(per, key=lambda t: per[t]) for n, per in edges.items()}


def line_valid(n: int, p: int) -> bool:
    """A plan of p points per thread fits a line of n points on the kernel's 512 threads."""
    return p * 512 >= n


def choose_lines(ltimes: dict) -> dict:
    """ltimes[(workload, p)] -> ms per step; returns line length -> fastest valid p."""
    per = {}
    for (w, p), ms in ltimes.items():
        n = WORKLOADS[w][1]
        if line_valid(n, p):
            per.setdefault(n, {})[p] = ms
    return {n: min(c, key=lambda p: c[p]) for n, c in per.items()}


def line_function(lchoice: dict) -> str:
    """tuned_line_ppt(n): the plan of the smallest measured length >= n (16 above them);
    a threshold whose plan equals the next longer one's is left out."""
    expr, nxt = "16", 16
    for n in sorted(lchoice, reverse=True):
        if lchoice[n] != nxt:
            expr, nxt = f"n <= {n} ? {lchoice[n]} : {expr}", lchoice[n]
    return expr


def shape_function(choice: dict, k: int, default: int) -> str:
    """An expression of n giving component k of the chosen shape (default elsewhere)."""
    expr = str(default)
    for n in sorted(choice, reverse=True):
        v = choice[n][k]
        if v != default:
            expr = f"n == {n} ? {v} : {expr}"
    return expr


def header_text(choice: dict, times: dict, lchoice: dict = None, ltimes: dict = None) -> str:
    lchoice = lchoice if lchoice is not None else {1024: 4, 2048: 8, 4096: 16}
    rows = []
    for w, _ in TUNE_WORKLOADS:
        cells = "  ".join(f"{c[0]}x{c[1]}: {times[(w, c)]:.4f}" for c in ALL_CANDIDATES if (w, c) in times)
        if cells:
            rows.append(f"//   {w:7s} ms/step  {cells}")
    lrows = []
    for w, _ in LINE_WORKLOADS:
        cells = "  ".join(f"{p}: {ltimes[(w, p)]:.4f}" for p in LINE_CANDIDATES if ltimes and (w, p) in ltimes)
        if cells:
            lrows.append(f"//   {w:7s} ms/step  {cells}")
    return f"""// qsf_tuning.h -- pass kernel shapes per line length: points and threads per block of
// the row / axis passes, and the radix plan of the one-CTA 1D line kernel.
//
// Written by the autotuner (qsf_gb300/autotune.py) from step times measured on a GB300:
//   python -m qsf_gb300.autotune --write
// Row / axis shapes: points per block x threads per block (16 points per thread:
// radix-16 plans, 128 registers; 8: radix-8 plans); lengths not listed take
// {DEFAULT_SHAPE[0]}x{DEFAULT_SHAPE[1]}.  Chosen among {", ".join(f"{c[0]}x{c[1]}" for c in CANDIDATES)}; smaller tiles, timed
// beside them, speed up small grids run alone but slow the batched form down.
// Measured (one call of graph-replayed steps per workload, ms per step):
{chr(10).join(rows)}
#pragma once

namespace qsf {{

__host__ __device__ constexpr int tuned_row_threads(int n) {{
  return {shape_function(choice, 1, DEFAULT_SHAPE[1])};
}}

__host__ __device__ constexpr int tuned_tile(int n) {{
  return {shape_function(choice, 0, DEFAULT_SHAPE[0])};
}}

// Points per thread of the one-CTA 1D line kernel per line length (4: radix-4 plans,
// 8: radix 8, 16: radix 16); a length between measured ones takes the plan of the next
// longer measured length.  Measured (one call of graph-replayed steps, points per
// thread: ms per step):
{chr(10).join(lrows)}
__host__ __device__ constexpr int tuned_line_ppt(int n) {{
  return {line_function(lchoice)};
}}

}}  // namespace qsf
"""


def committed_row_times() -> dict:
    """The row / axis timings of the committed table (kept when only the lines are tuned)."""
    if not os.path.exists(HEADER):
        return {}
    txt = open(HEADER).read()
    times = {}
    for w, cells in re.findall(r"//\s+([23]d\d+)\s+ms/step\s+(.*)", txt):
        for tile, thr, ms in re.findall(r"(\d+)x(\d+): ([0-9.]+)", cells):
            times[(w, (int(tile), int(thr)))] = float(ms)
    return times


def committed_line_times() -> dict:
    """The 1D line-plan timings of the committed table (kept when only the rows are tuned)."""
    if not os.path.exists(HEADER):
        return {}
    lt = {}
    for w, cells in re.findall(r"//\s+(1d\d+)\s+ms/step\s+(.*)", open(HEADER).read()):
        for p, ms in re.findall(r"(\d+): ([0-9.]+)", cells):
            lt[(w, int(p))] = float(ms)
    return lt


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--repeat", type=int, default=2)
    ap.add_argument("--write", action="store_true", help="rewrite qsf_gb300/csrc/qsf_tuning.h")
    ap.add_argument("--only", choices=["rows", "lines"], default=None)
    ap.add_argument("--shapes", choices=["tiles4096", "all"], default="tiles4096",
                    help="row / axis candidates: 4096-point tiles (the committed table) or all shapes")
    args = ap.parse_args()
    cands = CANDIDATES if args.shapes == "tiles4096" else ALL_CANDIDATES
    times, ltimes = {}, {}
    if args.only != "lines":
        for c in cands:
            lib_path = B.build(defines=[f"QSF_TILE={c[0]}", f"QSF_ROW_THREADS={c[1]}"], tag=f"tune_{c[0]}_{c[1]}")
            for w, steps in TUNE_WORKLOADS:
                times[(w, c)] = time_workload(lib_path, w, steps, args.repeat)
                print(json.dumps({"workload": w, "tile": c[0], "threads": c[1], "ms_per_step": times[(w, c)]}),
                      flush=True)
    if args.only != "rows":
        for p in LINE_CANDIDATES:
            lib_path = B.build(defines=[f"QSF_LINE_PPT={p}"], tag=f"tune_line{p}")
            for w, steps in LINE_WORKLOADS:
                if not line_valid(WORKLOADS[w][1], p):
                    continue
                ltimes[(w, p)] = time_workload(lib_path, w, steps, args.repeat)
                print(json.dumps({"workload": w, "points_per_thread": p, "ms_per_step": ltimes[(w, p)]}), flush=True)
    if not times:
        times = committed_row_times()
    choice = choose({k: v for k, v in times.items() if k[1] in cands})
    if not ltimes:
        ltimes = committed_line_times()
    lchoice = choose_lines(ltimes) if ltimes else None
    print(json.dumps({"choice": {str(n): list(t) for n, t in sorted(choice.items())},
                      "line_choice": {str(n): p for n, p in sorted((lchoice or {}).items())}}), flush=True)
    if args.write:
        with open(HEADER, "w") as f:
            f.write(header_text(choice, times, lchoice, ltimes))


if __name__ == "__main__":
    main()
