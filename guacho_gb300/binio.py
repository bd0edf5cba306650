"""Guacho's BIN output format: the on-disk form of the state on both sides of
the timestep path (output, checkpoint and warm start).

  write_bin   src/Out_BIN_Module.f90:40-166 (write_header + write_BIN): an
              ASCII header closed by achar(255), a binary header, then the
              whole u(neq, nxmin:nxmax, nymin:nymax, nzmin:nzmax) with
              ghost cells in Fortran order
  write_divb  src/Out_BIN_Module.f90:208-246: the centred div B of the
              interior, with a header of neq=1 and nghost=0
  read_bin    the warm-start reader of src/init.f90:437-467 (skip to
              achar(255), read the binary header, then u)
  bin_path    the file naming of src/Out_BIN_Module.f90:129-130

Files are written as the reference's DOUBLEP=Y build writes them: 'd' kind,
4-byte integers, 8-byte reals, native (little-endian) byte order.
"""
from __future__ import annotations

import os
import struct
from pathlib import Path

import numpy as np

from .params import NGHOST, Params

LF = b"\n"


def _es(x: float) -> str:
    """Fortran es10.3."""
    return f"{x:10.3E}"


def _header(p: Params, neq_out: int, nghost_out: int, scal=(1.0, 1.0, 1.0)) -> bytes:
    rsc, vsc, rhosc = scal
    neqdyn = 8 if p.bfield else 5
    lines = [
        "**************** Output for Guacho v1.3****************",
        f"Dimensions    : {p.nx} {p.ny} {p.nz}",
        f"Spacings      : {_es(p.dx)}{_es(p.dy)}{_es(p.dz)}",
        "Block Origin, cells    : 0 0 0",
        "MPI blocks (X, Y, Z)   : 1 1 1",
        f"Number of Equations/dynamical ones  {neq_out}/{neqdyn}",
        f"Number of Ghost Cells  {nghost_out}",
        "Scalings",
        f"r_sc: {_es(rsc)} v_sc: {_es(vsc)} rho_sc: {_es(rhosc)}",
        f"Specfic heat at constant volume Cv: {p.cv:7.2f}",
        "Double precision 8 byte floats",
        "*******************************************************",
    ]
    out = b"".join(line.rstrip().encode() + LF for line in lines)
    out += bytes([255]) + LF + b"d"
    out += struct.pack("<3i", p.nx, p.ny, p.nz)
    out += struct.pack("<3d", p.dx, p.dy, p.dz)
    out += struct.pack("<3i", 0, 0, 0)          # block origin (one domain)
    out += struct.pack("<3i", 1, 1, 1)          # MPI blocks
    out += struct.pack("<2i", neq_out, neqdyn)
    out += struct.pack("<i", nghost_out)
    out += struct.pack("<3d", rsc, vsc, rhosc)
    out += struct.pack("<d", p.cv)
    return out


def bin_path(outputpath: str | os.PathLike, itprint: int, rank: int = 0,
             base: str = "points") -> Path:
    """outputpath/BIN/points<rank>.<itprint>.bin (MPI naming, rank 0)."""
    return Path(outputpath) / "BIN" / f"{base}{rank:03d}.{itprint:03d}.bin"


def write_bin(path, u: np.ndarray, p: Params, scal=(1.0, 1.0, 1.0),
              prim0: np.ndarray | None = None) -> None:
    """u in the host layout (nz+4, ny+4, nx+4, neq) float64: its bytes are
    the Fortran u(neq, nxmin:nxmax, ...) in column-major order.  With the
    split solver's background prim0 the file holds the total state, as
    src/Out_BIN_Module.f90:144-158 writes it: rho + rho0, the momenta,
    E + cv p0 + B0^2/2 and B + B0."""
    u = np.ascontiguousarray(u, dtype="<f8")
    assert u.shape == p.shape
    if prim0 is not None:
        q = np.asarray(prim0, dtype=np.float64)
        assert q.shape == p.shape
        u = u.copy()
        u[..., 0] = u[..., 0] + q[..., 0]
        u[..., 4] = (u[..., 4] + p.cv * q[..., 4]
                     + 0.5 * (q[..., 5] * q[..., 5] + q[..., 6] * q[..., 6] + q[..., 7] * q[..., 7]))
        for c in (5, 6, 7):
            u[..., c] = u[..., c] + q[..., c]
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    with open(path, "wb") as f:
        f.write(_header(p, p.neq, NGHOST, scal))
        f.write(u.tobytes())


def divb(u: np.ndarray, p: Params) -> np.ndarray:
    """Centred div B of the interior, src/Out_BIN_Module.f90:214-222,
    as (nz, ny, nx)."""
    bx, by, bz = u[..., 5], u[..., 6], u[..., 7]
    return ((bx[2:-2, 2:-2, 3:-1] - bx[2:-2, 2:-2, 1:-3]) / (2.0 * p.dx)
            + (by[2:-2, 3:-1, 2:-2] - by[2:-2, 1:-3, 2:-2]) / (2.0 * p.dy)
            + (bz[3:-1, 2:-2, 2:-2] - bz[1:-3, 2:-2, 2:-2]) / (2.0 * p.dz))


def write_divb(path, u: np.ndarray, p: Params, scal=(1.0, 1.0, 1.0)) -> None:
    d = np.ascontiguousarray(divb(u, p), dtype="<f8")
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    with open(path, "wb") as f:
        f.write(_header(p, 1, 0, scal))
        f.write(d.tobytes())


def read_bin(path) -> tuple[dict, np.ndarray]:
    """Warm-start read (src/init.f90:455-467): returns the binary header
    fields and the array as (nz+2g, ny+2g, nx+2g, neq) float64."""
    data = Path(path).read_bytes()
    i = data.index(bytes([255]))
    off = i + 2  # achar(255) and its line feed
    kind = data[off:off + 1]
    off += 1
    if kind != b"d":
        raise ValueError(f"{path}: only 8-byte ('d') files are supported, found {kind!r}")

    def take(fmt):
        nonlocal off
        vals = struct.unpack_from(fmt, data, off)
        off += struct.calcsize(fmt)
        return vals

    nx, ny, nz = take("<3i")
    dx, dy, dz = take("<3d")
    x0, y0, z0 = take("<3i")
    mx, my, mz = take("<3i")
    neq, neqdyn = take("<2i")
    (ng,) = take("<i")
    scal = take("<3d")
    (cv,) = take("<d")
    shape = (nz + 2 * ng, ny + 2 * ng, nx + 2 * ng, neq)
    count = int(np.prod(shape))
    arr = np.frombuffer(data, dtype="<f8", count=count, offset=off).reshape(shape)
    hdr = dict(nx=nx, ny=ny, nz=nz, dx=dx, dy=dy, dz=dz, origin=(x0, y0, z0),
               mpi=(mx, my, mz), neq=neq, neqdyn=neqdyn, nghost=ng, scal=scal, cv=cv)
    return hdr, arr.copy()
