"""CPU restatement of the reference's .psi wavefunction files -- TEST INFRASTRUCTURE ONLY.

Only tests/ import this module.  It restates, in numpy, what LocalGrid does with .psi
files (include/wf/grid.h), so the GPU library's files can be compared with it and it
can be compared with files the reference itself wrote:

* ``save``        -- _save_centered / _save / coarse            grid.h:955-1114
* ``load``        -- _load                                       grid.h:789-859
* ``orthogonalize_with`` -- orthogonalizeWith                    grid.h:909-946
* ``backup`` / ``restore`` -- _backup / restore                  grid.h:949-953, 1116-1131

File layout (grid.h:1025-1035): dim u8 | rep u8 | complex u8 | downscale i64 |
n[dim] i64 | dx[dim] f64 | bounded[dim] u8 | payload (native little-endian).  The
payload is the wavefunction in memory order (complex128) or, when downscaled or saved
without phase, block sums of |psi|^2 (float64) in C order over the coarse grid.
"""
from __future__ import annotations

import math
import os
import struct
from typing import Tuple

import numpy as np

from . import oracle as O

REP_X, REP_P = 1, 2
PSI_EXT = ".psi"


def header(dim: int, rep: int, complex_: bool, downscale: int, n, dx, bounded=None) -> bytes:
    """grid.h:1025-1035 (bounded[] is all true for a single-region grid, mpi_logic.h:149-150)."""
    if bounded is None:
        bounded = [True] * dim
    h = struct.pack("<BBBq", dim, rep, 1 if complex_ else 0, int(downscale))
    h += struct.pack("<%dq" % dim, *[int(v) for v in n])
    h += struct.pack("<%dd" % dim, *[float(v) for v in dx])
    h += bytes(1 if b else 0 for b in bounded)
    return h


def header_size(dim: int) -> int:
    return 11 + 17 * dim


def parse_header(raw: bytes):
    dim, rep, cplx, ds = struct.unpack_from("<BBBq", raw, 0)
    off = 11
    n = list(struct.unpack_from("<%dq" % dim, raw, off))
    off += 8 * dim
    dx = list(struct.unpack_from("<%dd" % dim, raw, off))
    off += 8 * dim
    bounded = [bool(b) for b in raw[off:off + dim]]
    off += dim
    return dict(dim=dim, rep=rep, complex=bool(cplx), downscale=ds, n=n, dx=dx, bounded=bounded, offset=off)


def phase_shift_trick(psi: np.ndarray) -> np.ndarray:
    """psi * (-1)^(i0 + i1 + ...)  (grid.h:1074-1085)."""
    sign = np.ones(psi.shape)
    for d, nd in enumerate(psi.shape):
        shp = [1] * psi.ndim
        shp[d] = nd
        sign = sign * np.where(np.arange(nd) % 2 == 1, -1.0, 1.0).reshape(shp)
    return psi * sign


def p_memory(psi: np.ndarray) -> np.ndarray:
    """The reference's P-representation array in memory after fourier<P>: the forward
    transform of the phase-shifted psi, axes 0 and 1 transposed for D > 1
    (FFTW_MPI_TRANSPOSED_OUT, grid.h:251-274)."""
    p = O.fft_nd(phase_shift_trick(psi), -1)
    if psi.ndim > 1:
        p = np.swapaxes(p, 0, 1)
    return np.ascontiguousarray(p)


def file_name(base: str, rep: int, complex_: bool, downscale: int, evo_backup: bool = False,
              ext: str = PSI_EXT) -> str:
    """Name rules of _save (grid.h:996-1005)."""
    if not evo_backup:
        if downscale > 1:
            base += "_scale" + str(downscale)
        base += "_repX" if rep == REP_X else "_repP"
    return base + ext


def payload(psi: np.ndarray, dx, rep: int = REP_X, complex_: bool = True, downscale: int = 1,
            evo_backup: bool = False) -> Tuple[bytes, bool]:
    """Data written by _save / coarse (grid.h:955-992, 1063-1066); returns (bytes, complex flag)."""
    if not evo_backup and downscale > 1:
        complex_ = False
    src = psi if (evo_backup or rep == REP_X) else p_memory(psi)
    if evo_backup or (downscale == 1 and complex_ and rep == REP_X):
        return np.ascontiguousarray(psi, dtype=np.complex128).tobytes(), complex_
    dim = psi.ndim
    dV = 1.0
    for v in dx:
        dV *= v
    p_scale = dV / math.pow(math.sqrt(2 * math.pi), dim)
    ds = int(downscale)
    n = psi.shape
    if any(nd % ds for nd in n):
        raise ValueError("downscale must divide every axis length")
    if complex_:
        sub = np.array(src[tuple(slice(0, nd, ds) for nd in n)], dtype=np.complex128)
        if rep == REP_P:
            sub.real = sub.real * p_scale
            sub.imag = sub.imag * p_scale
        return np.ascontiguousarray(sub, dtype=np.complex128).tobytes(), True
    # block sums of |psi|^2, offsets with the last axis fastest, accumulated in that order
    coarse_shape = tuple(nd // ds for nd in n)
    acc = np.zeros(coarse_shape)
    for ofs in np.ndindex(*([ds] * dim)):
        blk = src[tuple(slice(o, nd, ds) for o, nd in zip(ofs, n))]
        acc = acc + (blk.real * blk.real + blk.imag * blk.imag)
    if rep == REP_P:
        acc = acc * (p_scale * p_scale)
    return acc.tobytes(), False


def save(psi: np.ndarray, dx, base: str, rep: int = REP_X, complex_: bool = True, downscale: int = 1,
         evo_backup: bool = False, ext: str = PSI_EXT, directory: str = ".") -> str:
    """_save_centered + _save: writes the file and returns its path."""
    data, cplx = payload(psi, dx, rep, complex_, downscale, evo_backup)
    ds = int(downscale)
    if not evo_backup and ds > 1:
        cplx = False
    path = os.path.join(directory, file_name(base, rep, cplx, ds, evo_backup, ext))
    with open(path, "wb") as f:
        f.write(header(psi.ndim, REP_X if evo_backup else rep, cplx, ds, psi.shape, dx))
        f.write(data)
    return path


def load(path: str, psi: np.ndarray) -> Tuple[np.ndarray, dict]:
    """_load (grid.h:789-859) into a grid currently holding psi; returns (new psi, header).

    A file of doubles is read the way the reference reads it: m doubles land in the
    first 8 m bytes of psi's buffer, then every element is replaced by its modulus."""
    raw = open(path, "rb").read()
    h = parse_header(raw)
    if h["dim"] != psi.ndim:
        raise ValueError("dimensionality of the file differs from the grid's")
    m = psi.size
    buf = np.ascontiguousarray(psi, dtype=np.complex128).copy().reshape(-1)
    data = raw[h["offset"]:]
    if h["complex"]:
        vals = np.frombuffer(data[:16 * m], dtype=np.complex128)
        buf[:vals.size] = vals
    else:
        vals = np.frombuffer(data[:8 * m], dtype=np.float64)
        fl = buf.view(np.float64)
        fl[:vals.size] = vals
        buf = np.hypot(buf.real, buf.imag).astype(np.complex128)  # std::abs -> cabs -> libm hypot
    return buf.reshape(psi.shape), h


def orthogonalize_with(path: str, psi: np.ndarray, dx, offset=None) -> Tuple[np.ndarray, complex, float]:
    """orthogonalizeWith (grid.h:909-946): reads m complex values, projects them out and
    returns (psi, <psi_file|psi> dV, norm after).  The reference reads them at the byte
    offset it computes (8 + 17 dim, grid.h:917-918), 3 bytes before the payload of the
    files it writes (11 + 17 dim), so on its own files it projects out misaligned
    bytes; offset=None reproduces that, offset=header_size(dim) reads the payload."""
    dim = psi.ndim
    off = (1 + 1 + 1 + 1 + 4 + dim * (8 + 8 + 1)) if offset is None else int(offset)
    raw = open(path, "rb").read()
    m = psi.size
    tmp = np.frombuffer(raw[off:off + 16 * m], dtype=np.complex128).reshape(psi.shape)
    dV = 1.0
    for v in dx:
        dV *= v
    sp = complex(0.0)
    for a, b in zip(tmp.reshape(-1), psi.reshape(-1)):
        sp += a.conjugate() * b
    sp *= dV
    # psi[i] -= sp * tmp[i] (grid.h:939), the complex product as separate real
    # multiplies and adds: numpy's vector loops for complex products may fuse them into
    # multiply-adds, which the reference's compiled code does not (-ffp-contract=off)
    prod = np.empty_like(tmp)
    prod.real = sp.real * tmp.real - sp.imag * tmp.imag
    prod.imag = sp.real * tmp.imag + sp.imag * tmp.real
    out = psi - prod
    nrm = float(np.sum(out.real * out.real + out.imag * out.imag)) * dV
    return out, sp, nrm


def backup(psi: np.ndarray, dx, step: int, ext: str = PSI_EXT, directory: str = ".") -> str:
    """_backup (grid.h:1116-1126): backup.info holds the step (int64), backup<ext> the
    raw wavefunction with an X / complex / downscale-1 header."""
    with open(os.path.join(directory, "backup.info"), "wb") as f:
        f.write(struct.pack("<q", int(step)))
    return save(psi, dx, "backup", evo_backup=True, ext=ext, directory=directory)


def restore(psi: np.ndarray, ext: str = PSI_EXT, directory: str = ".") -> Tuple[np.ndarray, int]:
    with open(os.path.join(directory, "backup.info"), "rb") as f:
        step = struct.unpack("<q", f.read(8))[0]
    out, _ = load(os.path.join(directory, "backup" + ext), psi)
    return out, step
