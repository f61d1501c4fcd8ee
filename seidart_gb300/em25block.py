"""SEIDART_EM25B1 block files: 2.5-D electromagnetic snapshots as
block-floating int16.

The reference reads 2.5-D EM snapshots from these files
(``src/seidart/routines/definitions.py:140-212``, ``read_block``; its
viewer globs ``EM25.*.blk*``, ``src/seidart/visualization/imgen.py:63-70``).
A file holds consecutive steps of every channel, all little-endian:

====================  ================================================
16 bytes              ASCII magic ``SEIDART_EM25B1``, space padded
int32                 version, 1
3 x int32             nx, ny, nz (full grid)
3 x int32             first_step, step_count, component_count
per step, per channel int32 step; 2 ASCII bytes channel ("Ex", "Ey",
                      "Ez"); 2 x float32 min, max; nx*ny*nz int16
                      codes, x fastest, then y, then z
====================  ================================================

A code c stands for (c + 32767) / 65534 * (max - min) + min; a record whose
max equals its min holds min everywhere.  The codes are produced on the GPU
(``sfd_encode_field_i16``); this module writes and reads the files.
"""
from __future__ import annotations

import gzip
import struct
from pathlib import Path
from typing import Dict, Iterable, Optional

import numpy as np

MAGIC = b"SEIDART_EM25B1  "
VERSION = 1
_HEAD = struct.Struct("<16si3i3i")
_REC = struct.Struct("<i2s2f")
_COUNTS_OFFSET = 16 + 4 + 12 + 4  # step_count, component_count


def block_name(xind: int, yind: int, zind: int, first_step: int) -> str:
    """File name of the block that starts at ``first_step`` for the source
    at cell (xind, yind, zind): ``EM25.{xind}.{yind}.{zind}.{first:06d}.blk``."""
    return f"EM25.{xind}.{yind}.{zind}.{first_step:06d}.blk"


class BlockWriter:
    """Appends the records of consecutive steps to one block file.  The step
    count in the header is filled in by ``close``."""

    def __init__(self, path, nx: int, ny: int, nz: int, first_step: int, channels: Iterable[str]):
        self.path = Path(path)
        self.shape = (int(nx), int(ny), int(nz))
        self.first = int(first_step)
        self.channels = tuple(channels)
        self.records = 0
        self.f = open(self.path, "wb")
        self.f.write(_HEAD.pack(MAGIC, VERSION, *self.shape, self.first, 0, len(self.channels)))

    @property
    def steps(self) -> int:
        return self.records // len(self.channels)

    def add(self, step: int, channel: str, vmin: float, vmax: float, codes) -> None:
        """One record; records come step by step, in ``channels`` order."""
        want_step = self.first + self.steps
        want_ch = self.channels[self.records % len(self.channels)]
        if step != want_step or channel != want_ch:
            raise ValueError(f"record ({step}, {channel}) out of order: expected ({want_step}, {want_ch})")
        codes = np.ascontiguousarray(codes, dtype="<i2").reshape(-1)
        if codes.size != self.shape[0] * self.shape[1] * self.shape[2]:
            raise ValueError("a record holds nx*ny*nz codes")
        self.f.write(_REC.pack(int(step), channel.encode("ascii"), float(vmin), float(vmax)))
        self.f.write(memoryview(codes).cast("B"))
        self.records += 1

    def close(self) -> None:
        if self.f is None:
            return
        if self.records % len(self.channels):
            raise ValueError("a block ends in the middle of a step")
        self.f.seek(_COUNTS_OFFSET)
        self.f.write(struct.pack("<2i", self.steps, len(self.channels)))
        self.f.close()
        self.f = None


def read(path, channels: Optional[Iterable[str]] = None, dtype=np.float32) -> Dict:
    """Decode a block file (gzip-compressed too).  Returns ``metadata`` and
    ``fields``: {channel: array (step_count, nz, ny, nx)}, the memory order
    of the solver's fields, and ``scales``: {channel: [(step, min, max)]}."""
    want = None if channels is None else set(channels)
    opener = gzip.open if str(path).endswith(".gz") else open
    with opener(path, "rb") as f:
        magic, version, nx, ny, nz, first, nsteps, ncomp = _HEAD.unpack(f.read(_HEAD.size))
        if magic.decode("ascii").strip() != "SEIDART_EM25B1":
            raise ValueError(f"{path} is not an EM25 block file")
        if version != VERSION:
            raise ValueError(f"unsupported EM25 block version {version}")
        n = nx * ny * nz
        fields: Dict[str, np.ndarray] = {}
        scales: Dict[str, list] = {}
        for _ in range(nsteps * ncomp):
            step, ch, vmin, vmax = _REC.unpack(f.read(_REC.size))
            ch = ch.decode("ascii")
            codes = np.frombuffer(f.read(2 * n), dtype="<i2")
            if want is not None and ch not in want:
                continue
            out = fields.setdefault(ch, np.empty((nsteps, nz, ny, nx), dtype=dtype))
            t = step - first
            if vmax == vmin:
                out[t] = vmin
            else:
                u = (codes.astype(dtype) + dtype(32767.0)) / dtype(65534.0)
                out[t] = (u * (dtype(vmax) - dtype(vmin)) + dtype(vmin)).reshape(nz, ny, nx)
            scales.setdefault(ch, []).append((step, float(vmin), float(vmax)))
    meta = dict(version=version, nx=nx, ny=ny, nz=nz, first_step=first, step_count=nsteps, component_count=ncomp)
    return {"metadata": meta, "fields": fields, "scales": scales}
