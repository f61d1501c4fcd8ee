"""SEIDART_EM25B1 block files (2.5-D EM snapshots as block-floating int16).

CPU: the byte layout of the header and records the reference's reader
expects (src/seidart/routines/definitions.py:140-212), the round trip through
the writer and the reader, gzip input and the ordering checks.  GPU: the
device encoding of real fields and the seidartfdtd ``--em25-blocks`` output
against the FP32 snapshots of the same run, within 0.51 of a code step.
"""
import gzip
import shutil
import struct

import numpy as np
import pytest

from seidart_gb300 import ELECTROMAG25, em25block
from seidart_gb300 import synthetic as sy


def _codes(rng, n):
    return rng.integers(-32767, 32768, n).astype(np.int16)


def test_header_and_record_layout(tmp_path):
    rng = np.random.default_rng(0)
    nx, ny, nz = 5, 3, 4
    n = nx * ny * nz
    path = tmp_path / "b.blk"
    w = em25block.BlockWriter(path, nx, ny, nz, 7, ("Ex", "Ey", "Ez"))
    recs = []
    for step in (7, 8):
        for ch in ("Ex", "Ey", "Ez"):
            c = _codes(rng, n)
            w.add(step, ch, -1.5, 2.5, c)
            recs.append((step, ch, c))
    w.close()
    raw = path.read_bytes()
    assert raw[:16].decode("ascii").strip() == "SEIDART_EM25B1"
    assert struct.unpack("<i", raw[16:20]) == (1,)
    assert struct.unpack("<3i", raw[20:32]) == (nx, ny, nz)
    assert struct.unpack("<3i", raw[32:44]) == (7, 2, 3)
    off = 44
    for step, ch, c in recs:
        assert struct.unpack("<i", raw[off:off + 4]) == (step,)
        assert raw[off + 4:off + 6] == ch.encode()
        assert struct.unpack("<2f", raw[off + 6:off + 14]) == (-1.5, 2.5)
        assert np.array_equal(np.frombuffer(raw[off + 14:off + 14 + 2 * n], dtype="<i2"), c)
        off += 14 + 2 * n
    assert off == len(raw)


def test_round_trip_and_gzip(tmp_path):
    rng = np.random.default_rng(1)
    nx, ny, nz = 6, 2, 5
    path = tmp_path / "r.blk"
    w = em25block.BlockWriter(path, nx, ny, nz, 1, ("Ex", "Ez"))
    codes = {}
    for step in (1, 2, 3):
        for ch, (lo, hi) in (("Ex", (-2.0, 3.0)), ("Ez", (0.5, 0.5))):
            c = _codes(rng, nx * ny * nz)
            codes[step, ch] = (c, lo, hi)
            w.add(step, ch, lo, hi, c)
    w.close()
    with open(path, "rb") as src, gzip.open(str(path) + ".gz", "wb") as dst:
        shutil.copyfileobj(src, dst)
    for p in (path, str(path) + ".gz"):
        out = em25block.read(p)
        assert out["metadata"] == dict(version=1, nx=nx, ny=ny, nz=nz, first_step=1, step_count=3, component_count=2)
        for (step, ch), (c, lo, hi) in codes.items():
            got = out["fields"][ch][step - 1]
            assert got.shape == (nz, ny, nx)
            want = np.full(c.shape, lo, np.float32) if hi == lo else \
                (c.astype(np.float32) + 32767) / 65534 * np.float32(hi - lo) + np.float32(lo)
            assert np.array_equal(got.reshape(-1), want)
        assert [s[0] for s in out["scales"]["Ex"]] == [1, 2, 3]
    only = em25block.read(path, channels=["Ez"])
    assert list(only["fields"]) == ["Ez"]


def test_records_must_come_in_order(tmp_path):
    w = em25block.BlockWriter(tmp_path / "o.blk", 2, 1, 2, 3, ("Ex", "Ey", "Ez"))
    c = np.zeros(4, np.int16)
    with pytest.raises(ValueError):
        w.add(3, "Ey", 0, 1, c)
    w.add(3, "Ex", 0, 1, c)
    with pytest.raises(ValueError):
        w.add(4, "Ex", 0, 1, c)
    with pytest.raises(ValueError):
        w.add(3, "Ey", 0, 1, np.zeros(5, np.int16))
    with pytest.raises(ValueError):
        w.close()  # the block ends in the middle of step 3
    assert em25block.block_name(10, 2, 7, 41) == "EM25.10.2.7.000041.blk"


def _quantum(field):
    """One code step.  Encoding and decoding in FP32 each add up to about
    65534 x 2^-24 = 0.004 of a step to the half step of rounding to a code,
    hence the 0.51-step bounds below."""
    return float(field.max() - field.min()) / 65534.0


@pytest.mark.gpu
def test_device_encoding_of_fields(gpu):
    import torch
    from helpers import make_solver
    from seidart_gb300.solver import FIELDS
    case = sy.small_case(ELECTROMAG25, seed=4, nx=30, nz=26, ny=14, npml=4, nstep=40)
    n = case.grid.nx * case.grid.ny * case.grid.nz
    codes = torch.empty(n, dtype=torch.int16, device=gpu)
    mm = torch.empty(2, dtype=torch.float32, device=gpu)
    with make_solver(case) as s:
        s.run(40)
        for name in FIELDS[ELECTROMAG25][:3]:
            f = s.field(name)
            s.encode_i16(name, codes, mm)
            lo, hi = (float(v) for v in mm.cpu())
            assert lo == float(f.min()) and hi == float(f.max())
            c = codes.cpu().numpy()
            dec = (c.astype(np.float64) + 32767) / 65534 * (hi - lo) + lo
            err = np.abs(dec - f.reshape(-1).astype(np.float64)).max()
            assert err <= 0.51 * _quantum(f) + 1e-30, (name, err, _quantum(f))


@pytest.mark.gpu
def test_cli_em25_blocks_match_fp32_snapshots(gpu, tmp_path):
    import glob
    from project_helpers import write_project
    from seidart_gb300 import cli, fortran_io as fio
    case = sy.small_case(ELECTROMAG25, seed=6, nx=28, nz=24, ny=12, npml=4, nstep=10)
    g = case.grid
    a, b = tmp_path / "blocks", tmp_path / "dat"
    a.mkdir()
    b.mkdir()
    path_a, (xi, yi, zi) = write_project(case, a)
    path_b, _ = write_project(case, b)
    assert cli.run([path_a, "seismic=false", "--workdir", str(a), "--em25-blocks", "4"]) == 0
    assert cli.run([path_b, "seismic=false", "--workdir", str(b)]) == 0
    files = sorted(glob.glob(str(a / "EM25.*.blk")))
    assert [f.split(".")[-2] for f in files] == ["000001", "000005", "000009"]
    for f in files:
        blk = em25block.read(f)
        m = blk["metadata"]
        for ch, arr in blk["fields"].items():
            for t in range(m["step_count"]):
                step = m["first_step"] + t
                ref = fio.read_record(b / f"{ch}.{step:06d}.{xi}.{yi}.{zi}.dat", np.float32).reshape(g.nz, g.ny, g.nx)
                err = np.abs(arr[t] - ref).max()
                assert err <= 0.51 * _quantum(ref) + 1e-30, (f, ch, step, err)
