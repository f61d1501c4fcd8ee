"""Fortran unformatted sequential records, the on-disk format of every .dat
file the SeidarT driver writes and the backend writes back.

One record = int32 byte count, payload, int32 byte count (the gfortran
default and what ``scipy.io.FortranFile`` writes; used by ``tensor2dat``,
``atten2dat``, ``writesrc`` and the initial conditions in
``src/seidart/routines/classes.py:608-750, 882-898`` and read by
``read_dat`` in ``src/seidart/routines/definitions.py:77-136``).  Arrays are
stored x fastest (the driver writes ``arr.T`` of an (nx, nz) array).
"""
from __future__ import annotations

import os
import struct

import numpy as np


def read_record(path, dtype=np.float64) -> np.ndarray:
    """The first record of ``path`` as a flat array of ``dtype``."""
    with open(path, "rb") as f:
        head = f.read(4)
        if len(head) != 4:
            raise ValueError(f"{path}: empty or truncated record")
        (n,) = struct.unpack("<i", head)
        payload = f.read(n)
        tail = f.read(4)
    if len(payload) != n or len(tail) != 4 or struct.unpack("<i", tail)[0] != n:
        raise ValueError(f"{path}: record marker mismatch (truncated or not a Fortran sequential file)")
    itemsize = np.dtype(dtype).itemsize
    if n % itemsize:
        raise ValueError(f"{path}: record of {n} bytes is not a whole number of {np.dtype(dtype).name}")
    return np.frombuffer(payload, dtype=dtype).copy()


def write_record(path, array, dtype=np.float32) -> None:
    """Write ``array`` (flattened in C order) as one record of ``dtype``."""
    data = np.ascontiguousarray(array, dtype=dtype)
    n = struct.pack("<i", data.nbytes)
    tmp = f"{path}.tmp"
    with open(tmp, "wb") as f:
        f.write(n)
        f.write(memoryview(data.reshape(-1)).cast("B"))
        f.write(n)
    os.replace(tmp, path)


def read_plane(path, shape) -> np.ndarray:
    """A (NZ, NX) or (NZ, NY, NX) FP64 model array written x fastest."""
    a = read_record(path, np.float64)
    if a.size != int(np.prod(shape)):
        raise ValueError(f"{path}: {a.size} values, expected {int(np.prod(shape))} for shape {shape}")
    return a.reshape(shape)
