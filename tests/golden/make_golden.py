"""Generate the golden fixtures in tests/golden/ from the reference's own code.

Runs oracle/_ref/qsf_ref (the reference's unmodified header-only implementation,
compiled by `make -C oracle ref` against the single-rank MPI / FFTW stand-ins) on small
seeded cases and stores its outputs -- the binary .dat rows written by the reference's
BufferedOutputs and the raw complex128 wavefunctions -- as compressed .npz files.

Needs the reference checkout (so it runs in the development container only); the
fixtures it writes are committed and are all the tests need elsewhere.

    python tests/golden/make_golden.py
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, "oracle", "_ref", "qsf_ref")

# name -> (harness case, params, IM dat columns, RE dat columns, grid dims)
CASES = {
    "prim2d": ("prim2d", dict(n=16, dx=0.4, nCAP=3, Ncharge=2, Echarge=-1, Nsoft=1, Esoft=1, p_NS=4, p_SD=3,
                              p_DT=2, p_CAP=6, seed=7, delta=0.37, F0=0.11), 0, 0, 2),
    "prim3d": ("prim3d", dict(n=12, dx=0.5, nCAP=2, Ncharge=3, Echarge=-1, Nsoft=1, Esoft=1, p_NS=4, p_SD=3,
                              p_DT=2, p_CAP=5, seed=11, delta=0.29, F0=0.07), 0, 0, 3),
    "c1_vg": ("c1", dict(n=512, dx=0.2, nCAP=51, Ncharge=1, Echarge=-1, Nsoft=1, Esoft=1, im_dt=0.01, im_steps=100,
                         re_dt=0.05, F0=0.05338, omega=0.5, ncycles=2, phase=0.0, box=100, lg=0), 6, 6, 1),
    "c1_lg": ("c1", dict(n=512, dx=0.2, nCAP=51, Ncharge=1, Echarge=-1, Nsoft=1, Esoft=1, im_dt=0.01, im_steps=100,
                         re_dt=0.05, F0=0.05338, omega=0.5, ncycles=2, phase=0.25, box=100, lg=1), 6, 6, 1),
    "c2_vg": ("c2", dict(n=48, dx=0.3, nCAP=5, Ncharge=2, Echarge=-1, Nsoft=1, Esoft=1, im_dt=0.01, im_steps=40,
                         re_dt=0.05, F0=0.11936, omega=1.0, ncycles=2, phase=0.0, p_NS=6, p_SD=4, p_DT=3, p_CAP=15,
                         lg=0), 6, 12, 2),
    "c3_lg": ("c3", dict(n=16, dx=0.4, nCAP=2, Ncharge=3, Echarge=-1, Nsoft=1, Esoft=1, im_dt=0.01, im_steps=20,
                         re_dt=0.05, F0=0.1688, omega=1.5, ncycles=1, phase=0.0, p_NS=4, p_SD=3, p_DT=2, p_CAP=6,
                         lg=1), 6, 13, 3),
    # the same runs at axis lengths with a prime factor above 5 (514 = 2 * 257,
    # 46 = 2 * 23, 14 = 2 * 7): the reference's FFTW plans take any n, the GPU path
    # transforms them by Bluestein's convolution
    "c1_bs": ("c1", dict(n=514, dx=0.2, nCAP=51, Ncharge=1, Echarge=-1, Nsoft=1, Esoft=1, im_dt=0.01, im_steps=100,
                         re_dt=0.05, F0=0.05338, omega=0.5, ncycles=2, phase=0.25, box=100, lg=1), 6, 6, 1),
    "c2_bs": ("c2", dict(n=46, dx=0.3, nCAP=5, Ncharge=2, Echarge=-1, Nsoft=1, Esoft=1, im_dt=0.01, im_steps=40,
                         re_dt=0.05, F0=0.11936, omega=1.0, ncycles=2, phase=0.0, p_NS=6, p_SD=4, p_DT=3, p_CAP=15,
                         lg=0), 6, 12, 2),
    "c3_bs": ("c3", dict(n=14, dx=0.4, nCAP=2, Ncharge=3, Echarge=-1, Nsoft=1, Esoft=1, im_dt=0.01, im_steps=20,
                         re_dt=0.05, F0=0.1688, omega=1.5, ncycles=1, phase=0.0, p_NS=4, p_SD=3, p_DT=2, p_CAP=6,
                         lg=1), 6, 13, 3),
    # .psi files written by the reference's own save / backup / snapshot, and the
    # wavefunctions its load / orthogonalizeWith produce (grid.h:789-1153)
    # MultiProductSplit<Split3Base, K> real-time runs, K = 2, 3, both gauges
    "mp": ("mp", dict(n=256, dx=0.2, nCAP=25, Ncharge=1, Echarge=-1, Nsoft=1, Esoft=1, re_dt=0.05, F0=0.05,
                      omega=0.5, ncycles=1, phase=0.0), 0, 4, 1),
    # average_der of the potential, AntiSymmetrize<2> (2D, 3D) and <3> (3D)
    "as2": ("as2", dict(n=12, dx=0.5, nCAP=1, Ncharge=2, Echarge=-1, Nsoft=1, Esoft=1, seed=5), 0, 0, 2),
    "as3": ("as3", dict(n=8, dx=0.5, nCAP=1, Ncharge=3, Echarge=-1, Nsoft=1, Esoft=1, seed=6), 0, 0, 3),
    # multi-region grids (multigrid.h), one process per region: the main region's .dat
    # rows and every region's final wavefunction
    "mg1": ("mg1", dict(n=128, dx=0.3, nCAP=16, Ncharge=1, Echarge=-1, Nsoft=1, Esoft=1, seed=3, F0=0.1, omega=1.0,
                        ncycles=1, re_dt=0.05), 0, 5, 1),
    "mg2": ("mg2", dict(n=32, dx=0.4, nCAP=4, Ncharge=2, Echarge=-1, Nsoft=1, Esoft=1, seed=5, F0=0.1, omega=1.0,
                        ncycles=1, re_dt=0.05), 0, 5, 2),
    "mg3": ("mg3", dict(n=8, dx=0.5, nCAP=3, Ncharge=3, Echarge=-1, Nsoft=1, Esoft=1, seed=9, F0=0.12, omega=1.5,
                        ncycles=1, re_dt=0.05), 0, 5, 3),
    # multi-region grids and multi-product chains at lengths with a prime factor above 5
    # (130 = 2 * 5 * 13, 34 = 2 * 17, 14 = 2 * 7, 258 = 2 * 3 * 43)
    "mg1_bs": ("mg1", dict(n=130, dx=0.3, nCAP=16, Ncharge=1, Echarge=-1, Nsoft=1, Esoft=1, seed=3, F0=0.1,
                           omega=1.0, ncycles=1, re_dt=0.05), 0, 5, 1),
    "mg2_bs": ("mg2", dict(n=34, dx=0.4, nCAP=4, Ncharge=2, Echarge=-1, Nsoft=1, Esoft=1, seed=5, F0=0.1,
                           omega=1.0, ncycles=1, re_dt=0.05), 0, 5, 2),
    "mg3_bs": ("mg3", dict(n=14, dx=0.5, nCAP=3, Ncharge=3, Echarge=-1, Nsoft=1, Esoft=1, seed=9, F0=0.12,
                           omega=1.5, ncycles=1, re_dt=0.05), 0, 5, 3),
    "mp_bs": ("mp", dict(n=258, dx=0.2, nCAP=25, Ncharge=1, Echarge=-1, Nsoft=1, Esoft=1, re_dt=0.05, F0=0.05,
                         omega=0.5, ncycles=1, phase=0.0), 0, 4, 1),
    # primitives and .psi files at lengths with a prime factor above 5 (22 = 2 * 11, 14)
    "prim2d_bs": ("prim2d", dict(n=22, dx=0.4, nCAP=3, Ncharge=2, Echarge=-1, Nsoft=1, Esoft=1, p_NS=4, p_SD=3,
                                 p_DT=2, p_CAP=6, seed=7, delta=0.37, F0=0.11), 0, 0, 2),
    "prim3d_bs": ("prim3d", dict(n=14, dx=0.5, nCAP=2, Ncharge=3, Echarge=-1, Nsoft=1, Esoft=1, p_NS=4, p_SD=3,
                                 p_DT=2, p_CAP=5, seed=11, delta=0.29, F0=0.07), 0, 0, 3),
    "io1_bs": ("io1", dict(n=22, dx=0.3, nCAP=2, seed=3), 0, 0, 1),
    "io2_bs": ("io2", dict(n=14, dx=0.5, nCAP=1, seed=5), 0, 0, 2),
    "io3_bs": ("io3", dict(n=14, dx=0.4, nCAP=1, seed=9), 0, 0, 3),
    "io1": ("io1", dict(n=16, dx=0.3, nCAP=2, seed=3), 0, 0, 1),
    "io2": ("io2", dict(n=8, dx=0.5, nCAP=1, seed=5), 0, 0, 2),
    "io3": ("io3", dict(n=8, dx=0.4, nCAP=1, seed=9), 0, 0, 3),
}

IO_FILES = ("sx_repX.psi", "sp_repP.psi", "sd_scale2_repX.psi", "sdp_scale2_repP.psi", "sn_repX.psi",
            "backup.psi", "backup.info", "snapshot_0_a_repX.psi0")


def _read_psi(path, shape):
    return np.fromfile(path, dtype=np.complex128).reshape(shape)


def make(name):
    case, params, im_cols, re_cols, dim = CASES[name]
    shape = (int(params["n"]),) * dim
    with tempfile.TemporaryDirectory() as tmp:
        args = [REF, case, tmp] + [f"{k}={v}" for k, v in params.items()]
        env = dict(os.environ)
        if case.startswith("mg"):  # one rank per region of MultiRegionsReduced<dim>
            env["QSF_SHIM_NP"] = str(2 ** dim)
        subprocess.run(args, check=True, stdout=subprocess.DEVNULL, env=env)
        out = {"params": json.dumps(params), "case": case, "dim": dim}
        if case in ("as2", "as3"):
            out["psi_in"] = _read_psi(os.path.join(tmp, "psi_in.bin"), shape)
            out["psi_as2"] = _read_psi(os.path.join(tmp, "psi_as2.bin"), shape)
            if case == "as3":
                out["psi_as3"] = _read_psi(os.path.join(tmp, "psi_as3.bin"), shape)
            out["der"] = np.fromfile(os.path.join(tmp, "der.bin"), dtype=np.float64)
        elif case == "mp":
            for tag in ("MP2VG", "MP3VG", "MP2LG", "MP3LG"):
                out[tag + "_psi0"] = _read_psi(os.path.join(tmp, tag + "_psi0.bin"), shape)
                out[tag + "_psi"] = _read_psi(os.path.join(tmp, tag + "_psi.bin"), shape)
                out[tag + "_rows"] = np.fromfile(os.path.join(tmp, tag + ".dat"), dtype=np.float64).reshape(-1, re_cols)
        elif case.startswith("mg"):
            out["psi_in"] = _read_psi(os.path.join(tmp, "psi_in.bin"), shape)
            for r in range(2 ** dim):
                sub = "" if r == 0 else "rank%d" % r
                out["psi_r%d" % r] = _read_psi(os.path.join(tmp, sub, "psi_r%d.bin" % r), shape)
            out["re_rows"] = np.fromfile(os.path.join(tmp, "RE.dat"), dtype=np.float64).reshape(-1, re_cols)
        elif case.startswith("io"):
            for f in ("psi_in", "psi_b", "psi_after_sp", "psi_load_sx", "psi_load_sn", "psi_orth"):
                out[f] = _read_psi(os.path.join(tmp, f + ".bin"), shape)
            for f in IO_FILES:
                out["file:" + f] = np.fromfile(os.path.join(tmp, f), dtype=np.uint8)
        elif case.startswith("prim"):
            for f in ("psi_in", "psi_xre", "psi_xim", "psi_p", "psi_back", "psi_pvg", "psi_norm"):
                out[f] = _read_psi(os.path.join(tmp, f + ".bin"), shape)
            out["scalars"] = np.fromfile(os.path.join(tmp, "prim.bin"), dtype=np.float64)
        else:
            for f in ("im_psi0", "im_psi", "re_psi0", "re_psi"):
                out[f] = _read_psi(os.path.join(tmp, f + ".bin"), shape)
            out["im_rows"] = np.fromfile(os.path.join(tmp, "IM.dat"), dtype=np.float64).reshape(-1, im_cols)
            out["re_rows"] = np.fromfile(os.path.join(tmp, "RE.dat"), dtype=np.float64).reshape(-1, re_cols)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return out


if __name__ == "__main__":
    if not os.path.exists(REF):
        sys.exit("build the harness first: make -C oracle ref")
    for name in (sys.argv[1:] or CASES):
        o = make(name)
        print(name, {k: getattr(v, "shape", v) for k, v in o.items() if k != "params"})
