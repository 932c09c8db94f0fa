"""Host-side I/O next to the path: MRC stacks (MRC_Reader / MRC_Writer) and alignment
files (AffineAlignment.loadFromFile / saveToFile)."""
from __future__ import annotations

import math
import struct

import numpy as np
import pytest

from tomoj_gb300 import mrc
from tomoj_gb300.tiltseries import IDENTITY, TiltSeries, concatenate, inverse, rotation


def test_mrc_roundtrip_and_header_fields(tmp_path):
    rng = np.random.default_rng(1)
    stack = rng.normal(0, 1, (3, 5, 7)).astype(np.float32)
    p = str(tmp_path / "a.mrc")
    mrc.write(p, stack)
    raw = open(p, "rb").read()
    assert len(raw) == 1024 + stack.nbytes
    nx, ny, nz, mode = struct.unpack_from("<4i", raw, 0)
    assert (nx, ny, nz, mode) == (7, 5, 3, 2)
    assert struct.unpack_from("<3i", raw, 64) == (1, 2, 3)
    mn, mx, mean = struct.unpack_from("<3f", raw, 76)
    ref = mrc._stats(stack)
    assert (mn, mx) == (np.float32(ref[0]), np.float32(ref[1])) and mean == np.float32(ref[2])
    got, info = mrc.read(p)
    assert info["little_endian"] and info["mode"] == 2 and not info["fei"]
    assert np.array_equal(got, stack)


def test_mrc_writer_min_max_follow_the_reference_else_if():
    # the first value 5 is the running max; 9 is a new max and is never tested as a
    # minimum; 1 is then the minimum.  A descending start keeps the first value as max.
    for vals in ([5, 9, 1, 7], [3, 2, 8, 1, 9], [4, 4, 4], [9, 1, 10, 0.5]):
        a = np.array(vals, np.float32).reshape(1, 1, -1)
        assert mrc._stats(a) == mrc._stats_fast(a)
    rng = np.random.default_rng(2)
    a = rng.normal(0, 1, (2, 30, 40)).astype(np.float32)
    assert mrc._stats(a) == mrc._stats_fast(a)


@pytest.mark.parametrize("mode,dtype", [(0, np.uint8), (1, np.int16), (6, np.uint16), (2, np.float32)])
def test_mrc_reads_big_and_little_endian_modes(tmp_path, mode, dtype):
    rng = np.random.default_rng(3)
    stack = (rng.uniform(0, 200, (2, 4, 6))).astype(dtype)
    for little in (True, False):
        e = "<" if little else ">"
        h = bytearray(1024)
        struct.pack_into(e + "4i", h, 0, 6, 4, 2, mode)
        p = str(tmp_path / f"m{mode}{int(little)}.mrc")
        with open(p, "wb") as f:
            f.write(h)
            f.write(stack.astype(np.dtype(dtype).newbyteorder(e)).tobytes())
        got, info = mrc.read(p, as_float32=False)
        assert info["little_endian"] == little
        assert np.array_equal(got, stack)


def test_mrc_fei_extended_header_tilt_angles(tmp_path):
    nz = 3
    h = bytearray(1024)
    struct.pack_into("<4i", h, 0, 4, 2, nz, 2)
    struct.pack_into("<i", h, 92, mrc.FEI_EXTENDED_BYTES)
    ext = bytearray(mrc.FEI_EXTENDED_BYTES)
    for i, a in enumerate((-60.0, 0.5, 60.0)):
        struct.pack_into("<f", ext, 128 * i, a)
    data = np.arange(4 * 2 * nz, dtype=np.float32)
    p = str(tmp_path / "fei.mrc")
    with open(p, "wb") as f:
        f.write(h + ext + data.tobytes())
    got, info = mrc.read(p)
    assert info["fei"] and info["offset"] == 1024 + mrc.FEI_EXTENDED_BYTES
    assert np.allclose(info["tilt_angles"], (-60.0, 0.5, 60.0))
    assert np.array_equal(got.ravel(), data)


def _ts(n=5):
    return TiltSeries(np.zeros((n, 8, 8), np.float32), np.linspace(-40, 40, n))


def test_imod_xf_final_transforms_become_consecutive(tmp_path):
    ts = _ts()
    al = ts.getAlignment()
    rng = np.random.default_rng(4)
    finals = []
    lines = []
    for i in range(5):
        a = math.radians(rng.uniform(-3, 3))
        T = (math.cos(a), math.sin(a), -math.sin(a), math.cos(a), rng.uniform(-4, 4), rng.uniform(-4, 4))
        finals.append(T)
        lines.append(" ".join(f"{v:.7f}" for v in T))
    p = str(tmp_path / "s.xf")
    open(p, "w").write("\n".join(lines) + "\n")
    al.loadFromFile(p, binning=1.0)
    assert al.combine
    # the combined transform of every image equals its final transform (tilt axis 0)
    for i in range(5):
        got = al.getTransform(i)
        exp = tuple(float(f"{v:.7f}") for v in finals[i])
        assert np.allclose(got, exp, atol=1e-9), i


def test_imod_xf_binning_and_tiff2mrc(tmp_path):
    ts = _ts(3)
    al = ts.getAlignment()
    p = str(tmp_path / "b.xf")
    open(p, "w").write("1 0 0 1 2 3\n1 0 0 1 -1 4\n1 0 0 1 0.5 0.5\n")
    al.loadFromFile(p, binning=2.0)
    assert np.allclose(al.getTransform(0), (1, 0, 0, 1, 4, 6))
    assert np.allclose(al.getTransform(2), (1, 0, 0, 1, 1, 1))
    al2 = _ts(3).getAlignment()
    al2.loadFromFile(p, binning=1.0, tiff2mrc=True)
    assert np.allclose(al2.getTransform(1), (-1, 0, 0, -1, 1, -4))


def test_tomoj_csv_roundtrip(tmp_path):
    ts = _ts(4)
    al = ts.getAlignment()
    ts.setTiltAxis(0.0)
    for i in range(4):
        al.setTransform(i, concatenate(rotation(math.radians(0.3 * i)), (1, 0, 0, 1, i, -i)))
    al.setZeroTransform((1, 0, 0, 1, 0.25, -0.5))
    p = str(tmp_path / "t.csv")
    al.saveToFile(p)
    ts2 = _ts(4)
    al2 = ts2.getAlignment()
    al2.loadFromFile(p)
    assert np.allclose(ts2.tiltAngles, ts.tiltAngles)
    for i in range(4):
        assert np.allclose(al2.transforms[i], al.transforms[i], atol=1e-15)
    assert np.allclose(al2.zeroT, al.zeroT)
    text = open(p).read().splitlines()
    assert text[0].startswith("-40.0;0.0;") and text[0].endswith(";")
