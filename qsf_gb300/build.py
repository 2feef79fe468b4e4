"""Build libqsfgpu.so (the sm_103a kernels + C ABI) in-tree with nvcc.

Each translation unit under qsf_gb300/csrc/ is compiled in parallel with
`-gencode arch=compute_103a,code=sm_103a`, then linked into qsf_gb300/libqsfgpu.so.
Objects go to qsf_gb300/_build/ and are rebuilt only when a source or header changed.

    python -m qsf_gb300.build          # or qsf_gb300.build.build()
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libqsfgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include")]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _newest(paths) -> float:
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def build(verbose: bool = False, force: bool = False, defines=(), tag: str = "") -> str:
    """Compile and link; returns the library path.  `defines` (NAME=VALUE strings) and a
    `tag` give a variant build in qsf_gb300/_build/<tag>/ (the autotuner's candidates);
    the default build is qsf_gb300/libqsfgpu.so."""
    out = os.path.join(OUT, tag) if tag else OUT
    lib_path = os.path.join(out, "libqsfgpu.so") if tag else LIB
    os.makedirs(out, exist_ok=True)
    extra = ["-D" + d for d in defines]
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))
    hdr_time = _newest(headers)
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(out, os.path.basename(src)[:-3] + ".o")
        if not force and os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_time):
            return obj
        cmd = [nvcc] + ARCH + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, sources))
    if force or not os.path.exists(lib_path) or os.path.getmtime(lib_path) < _newest(objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", lib_path + ".tmp"] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr)
        os.replace(lib_path + ".tmp", lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
