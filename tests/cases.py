"""Shared case builders: turn a golden fixture's parameters into oracle runs.

The golden fixtures (tests/golden/*.npz) hold the reference's own outputs for small
seeded cases.  These helpers rebuild the same cases on the CPU oracle so that tests
can pin the oracle to the reference, and the GPU tests can pin the GPU path to both.
"""
import json
import os

import numpy as np

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# BufferedOutputs used by the harness (oracle/ref/ref_driver.cpp)
IM_OUTPUTS = ["step", "norm", "normalize", "epot", "ekin", "etot", "ediff"]
# .dat row = non-reduced columns first (VALUE, CHANGE), then reduced ones (AVG, SUM, FLUX)
IM_DAT = ["step", "ediff", "norm", "epot", "ekin", "etot"]


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    out = {k: z[k] for k in z.files}
    out["params"] = json.loads(str(out["params"]))
    return out


def set_borders(p):
    O.set_border_nodes(int(p.get("p_NS", 25)), int(p.get("p_SD", 14)), int(p.get("p_DT", 10)),
                       int(p.get("p_CAP", 40)))


def pulse(p):
    return O.Pulse(field=p["F0"], omega=p["omega"], ncycles=p["ncycles"],
                   phase_in_pi_units=p.get("phase", 0.0), delay_in_cycles=p.get("delay", 0.0),
                   shape=O.PULSE_SIN2_SIN)


def field_axis(dim):
    return {1: 1, 2: 3, 3: 7}[dim]


def re_borders(dim):
    if dim == 1:
        return ["BOX"]
    return O.ZOA_FLUX_2D if dim == 2 else O.ZOA_FLUX_3D


def re_outputs(dim, box):
    return ["step", "time", "norm", "epot", "ekin", ("flux", re_borders(dim), box)]


def re_dat_row(row, nb):
    return [row["step"], row["time"], row["norm"], row["epot"], row["ekin"]] + list(row["flux"][:nb])


def im_dat_row(row):
    return [row[k] for k in IM_DAT]


def oracle_grid(p, dim, coupling):
    return O.Grid(dim, int(p["n"]), p["dx"], nCAP=int(p["nCAP"]), pot=O.POT_EBERLY, Ncharge=p["Ncharge"],
                  Echarge=p["Echarge"], Nsoft=p["Nsoft"], Esoft=p["Esoft"], coupling=coupling)


def oracle_im(p, dim, psi0=None):
    g = oracle_grid(p, dim, O.Coupling(O.GAUGE_VELOCITY))
    if psi0 is None:
        g.add_gaussian(0.0, 1.0)
    else:
        g.psi[...] = psi0
    prop = O.Propagator(O.MODE_IM, p["im_dt"], int(p["im_steps"]), g, IM_OUTPUTS)
    rows = prop.run()
    return g, rows


def oracle_re(p, dim, psi0):
    gauge = O.GAUGE_LENGTH if p.get("lg", 0) else O.GAUGE_VELOCITY
    c = O.Coupling(gauge, [O.Field(field_axis(dim), [pulse(p)])])
    g = oracle_grid(p, dim, c)
    g.psi[...] = psi0
    prop = O.Propagator(O.MODE_RE, p["re_dt"], 0, g, re_outputs(dim, int(p.get("box", 0))))
    rows = prop.run()
    return g, rows


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


# ---------------------------------------------------------------- GPU side
def gpu_grid(p, dim, gauge, n_fields):
    import qsf_gb300 as Q
    nodes = (int(p.get("p_NS", 25)), int(p.get("p_SD", 14)), int(p.get("p_DT", 10)), int(p.get("p_CAP", 40)))
    return Q.Grid(dim, int(p["n"]), p["dx"], nCAP=int(p["nCAP"]), potential=Q.POT_EBERLY, Ncharge=p["Ncharge"],
                  Echarge=p["Echarge"], Nsoft=p["Nsoft"], Esoft=p["Esoft"], gauge=gauge, n_fields=n_fields,
                  border_nodes=nodes)


def gpu_pulse(p):
    import qsf_gb300 as Q
    return Q.Pulse(field=p["F0"], omega=p["omega"], ncycles=p["ncycles"], phase_in_pi_units=p.get("phase", 0.0),
                   delay_in_cycles=p.get("delay", 0.0), shape=Q.PULSE_SIN2_SIN)


def gpu_im(p, dim, psi0=None):
    import qsf_gb300 as Q
    g = gpu_grid(p, dim, Q.GAUGE_VELOCITY, 0)
    if psi0 is None:
        g.add_gaussian(0.0, 1.0)
    else:
        g.upload(psi0)
    prop = Q.SplitPropagator(Q.MODE_IM, p["im_dt"], int(p["im_steps"]), g, Q.Coupling(Q.GAUGE_VELOCITY),
                             IM_OUTPUTS)
    rows = prop.run()
    return g, rows


def gpu_re(p, dim, psi0):
    import qsf_gb300 as Q
    gauge = Q.GAUGE_LENGTH if p.get("lg", 0) else Q.GAUGE_VELOCITY
    c = Q.Coupling(gauge, [Q.Field(field_axis(dim), [gpu_pulse(p)])])
    g = gpu_grid(p, dim, gauge, 1)
    g.upload(psi0)
    prop = Q.SplitPropagator(Q.MODE_RE, p["re_dt"], 0, g, c, re_outputs(dim, int(p.get("box", 0))))
    rows = prop.run()
    return g, rows


MG_OUTPUTS = ["step", "time", "norm", "epot", "ekin"]


def mg_dat_row(row):
    return [row[k] for k in MG_OUTPUTS]


def oracle_mg(p, dim, psi0):
    """The fixture's multi-region run on the oracle: one grid and one coupling per
    region (each region's process keeps its own coupling state in the reference)."""
    regs = O.region_axes(dim)
    cs = [O.Coupling(O.GAUGE_VELOCITY, [O.Field(field_axis(dim), [pulse(p)])]) for _ in regs]
    gs = [oracle_grid(p, dim, c) for c in cs]
    gs[0].psi[...] = psi0
    mp = O.MultiRegionPropagator(p["re_dt"], gs, cs, MG_OUTPUTS)
    rows = mp.run()
    return gs, rows
