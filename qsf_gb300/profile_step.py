"""Run a few fused steps of one workload, for profilers (ncu) and quick timing.

    python -m qsf_gb300.profile_step --workload 2d2048 --steps 3

Workloads: 1d4096 (1 electron, length gauge, BOX flux), 2d2048 (2 electrons,
velocity gauge, ZOA_FLUX_2D), 3d256 (3 electrons, length gauge, ZOA_FLUX_3D),
2d1024.  Each starts from a normalised Gaussian and runs `steps` Strang steps with
norm, E_pot and the workload's fluxes every step; prints the event-timed ms per step
and the per-kernel split.
"""
from __future__ import annotations

import argparse
import json
import math

import numpy as np

WORKLOADS = {
    # dim, n, dx, nCAP, Ncharge, gauge, intensity W/cm^2, wavelength nm, cycles, borders, box
    "1d4096": (1, 4096, 0.2, 410, 1.0, 1, 1e14, 800.0, 2.0, ["BOX"], 1638),
    "2d1024": (2, 1024, 0.3, 102, 2.0, 0, 5e14, 800.0, 3.0, "ZOA_FLUX_2D", 0),
    "2d2048": (2, 2048, 0.3, 205, 2.0, 0, 5e14, 800.0, 3.0, "ZOA_FLUX_2D", 0),
    "3d256": (3, 256, 0.4, 26, 3.0, 1, 1e15, 800.0, 2.0, "ZOA_FLUX_3D", 0),
    # further edges of the batched / served 2D mix and a smaller 3D cube
    "2d256": (2, 256, 0.3, 26, 2.0, 0, 5e14, 800.0, 3.0, "ZOA_FLUX_2D", 0),
    "2d320": (2, 320, 0.3, 32, 2.0, 0, 5e14, 800.0, 3.0, "ZOA_FLUX_2D", 0),
    "2d384": (2, 384, 0.3, 38, 2.0, 0, 5e14, 800.0, 3.0, "ZOA_FLUX_2D", 0),
    "2d640": (2, 640, 0.3, 64, 2.0, 0, 5e14, 800.0, 3.0, "ZOA_FLUX_2D", 0),
    "2d512": (2, 512, 0.3, 51, 2.0, 0, 5e14, 800.0, 3.0, "ZOA_FLUX_2D", 0),
    "2d768": (2, 768, 0.3, 77, 2.0, 0, 5e14, 800.0, 3.0, "ZOA_FLUX_2D", 0),
    "2d4096": (2, 4096, 0.3, 410, 2.0, 0, 5e14, 800.0, 3.0, "ZOA_FLUX_2D", 0),
    "3d128": (3, 128, 0.4, 13, 3.0, 1, 1e15, 800.0, 2.0, "ZOA_FLUX_3D", 0),
    "1d1024": (1, 1024, 0.2, 102, 1.0, 1, 1e14, 800.0, 2.0, ["BOX"], 400),
    "1d2048": (1, 2048, 0.2, 205, 1.0, 1, 1e14, 800.0, 2.0, ["BOX"], 800),
    "1d8192": (1, 8192, 0.2, 819, 1.0, 1, 1e14, 800.0, 2.0, ["BOX"], 1638),
    "1d1536": (1, 1536, 0.2, 153, 1.0, 1, 1e14, 800.0, 2.0, ["BOX"], 600),
    # lengths outside the built list: Bluestein transforms, member-operation programs
    "1d4099": (1, 4099, 0.2, 410, 1.0, 1, 1e14, 800.0, 2.0, ["BOX"], 1638),
    "2d1000": (2, 1000, 0.3, 100, 2.0, 0, 5e14, 800.0, 3.0, "ZOA_FLUX_2D", 0),
    "1d3072": (1, 3072, 0.2, 307, 1.0, 1, 1e14, 800.0, 2.0, ["BOX"], 1200),
}


def make(workload: str):
    import qsf_gb300 as Q
    dim, n, dx, ncap, charge, gauge, inten, lam, cyc, borders, box = WORKLOADS[workload]
    if isinstance(borders, str):
        borders = getattr(Q, borders)
    g = Q.Grid(dim, n, dx, nCAP=ncap, potential=Q.POT_EBERLY, Ncharge=charge, gauge=gauge, n_fields=1)
    x = (np.arange(n) - (n - 1) / 2.0) * dx
    line = np.exp(-0.5 * x * x)
    psi = line
    for _ in range(dim - 1):
        psi = np.multiply.outer(psi, line)
    psi = psi.astype(np.complex128)
    psi /= math.sqrt(float(np.sum(np.abs(psi) ** 2)) * dx ** dim)
    g.upload(psi)
    axis = {1: 1, 2: 3, 3: 7}[dim]
    c = Q.Coupling(gauge, [Q.Field(axis, [Q.Pulse(field=Q.field_from_intensity(inten),
                                                  omega=Q.omega_from_wavelength(lam), ncycles=cyc)])])
    prop = Q.SplitPropagator(Q.MODE_RE, 0.05, 0, g, c, ["norm", "epot", ("flux", borders, box)])
    return g, prop, borders, box


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="2d2048", choices=sorted(WORKLOADS))
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--ekin", action="store_true", help="also compute the kinetic energy every step")
    ap.add_argument("--fourier", type=int, default=0, help="instead time this many forward+backward transforms")
    ap.add_argument("--timed", action="store_true",
                    help="instead time one call of --steps steps as a user runs it (graph-replayed, wall clock "
                         "around the call after a warm-up call)")
    args = ap.parse_args()
    import time
    import qsf_gb300 as Q
    g, prop, borders, box = make(args.workload)
    if args.fourier:
        g.fourier(Q.REP_P)
        g.fourier(Q.REP_X)
        g.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.fourier):
            g.fourier(Q.REP_P)
            g.fourier(Q.REP_X)
        g.synchronize()
        ms = (time.perf_counter() - t0) * 1e3 / args.fourier
        print(json.dumps({"workload": args.workload, "fourier_pairs": args.fourier, "ms_per_pair": ms}))
        return
    obs = Q.OBS_NORM | Q.OBS_EPOT | (Q.OBS_EKIN if args.ekin else 0)
    prof = {}
    sched = prop._schedule(args.steps)
    if args.timed:
        g.step(Q.MODE_RE, 0.05, args.steps, sched, obs=obs, borders=borders, box_size=box)
        g.synchronize()
        t0 = time.perf_counter()
        g.step(Q.MODE_RE, 0.05, args.steps, sched, obs=obs, borders=borders, box_size=box)
        g.synchronize()
        ms = (time.perf_counter() - t0) * 1e3 / args.steps
        print(json.dumps({"workload": args.workload, "steps": args.steps, "timed_ms_per_step": ms}))
        return
    g.step(Q.MODE_RE, 0.05, args.steps, sched, obs=obs, borders=borders, box_size=box, profile=prof)
    tot = sum(v[0] for v in prof.values())
    print(json.dumps({"workload": args.workload, "steps": args.steps, "ms_per_step": tot / args.steps,
                      "kernels_ms_per_step": {k: v[0] / args.steps for k, v in prof.items() if v[1]}}))


if __name__ == "__main__":
    main()
