"""MRC stacks in and out (tilt-series in, tomograms out).

Mirrors the reference's InputOutput plug-ins:
  * MRC_Reader (InputOutput/src/main/java/fr/curie/InputOutput/MRC_Reader.java):
    1024-byte header; modes 0 (8-bit), 1 (signed 16-bit), 2 (float32) and 6
    (unsigned 16-bit); the byte order is found by reading the mode big-endian
    first (for mode 0, dimensions outside [0, 65536) mean little-endian; any other
    mode than 1, 2, 6 means little-endian) (:160-207); data starts at
    1024 + the extended-header size in word 23 (:208-212); an extended header of
    131072 bytes marks an FEI file whose per-image tilt angle is the first float
    of each 128-byte record (:214-220, :222-245).
  * MRC_Writer (InputOutput/src/main/java/fr/curie/InputOutput/MRC_Writer.java):
    little-endian header with nx, ny, nz, mode (0 for 8-bit, 1 or 6 for 16-bit
    by the sign of the minimum, 2 for float), axis order 1, 2, 3 in words 16-18,
    and min, max, mean as float bits in words 19-21, computed as the reference
    does (an `else if` that never tests a new maximum as a minimum; the mean is
    (float)(double sum / count)) (:86-160); then the raw little-endian data.
Stacks are numpy arrays (nz, ny, nx), x fastest: the [N][h][w] tilt-series and
[D][H][W] volume layouts of the engine.
"""
from __future__ import annotations

import struct

import numpy as np

HEADER_BYTES = 1024
FEI_EXTENDED_BYTES = 131072
_MODES = {0: np.uint8, 1: np.int16, 2: np.float32, 6: np.uint16}


def _word(header: bytes, index: int, little: bool) -> int:
    return struct.unpack_from("<i" if little else ">i", header, index)[0]


def read_header(path: str) -> dict:
    """Parsed header fields {nx, ny, nz, mode, little_endian, offset, extended, fei}."""
    with open(path, "rb") as f:
        header = f.read(HEADER_BYTES)
    if len(header) < HEADER_BYTES:
        raise IOError(f"{path}: shorter than an MRC header")
    little = False
    mode = _word(header, 12, little)
    if mode == 0:
        nx, ny, nz = (_word(header, 4 * k, little) for k in range(3))
        if not all(0 <= v < 65536 for v in (nx, ny, nz)):
            little = True
    elif mode not in (1, 2, 6):
        little = True
        mode = _word(header, 12, little)
        if mode not in (1, 2, 6):
            raise IOError(f"Unimplemented ImageData mode={mode} in MRC file.")
    nx, ny, nz = (_word(header, 4 * k, little) for k in range(3))
    extended = _word(header, 23 * 4, little)
    return dict(nx=nx, ny=ny, nz=nz, mode=mode, little_endian=little, offset=HEADER_BYTES + extended,
                extended=extended, fei=extended == FEI_EXTENDED_BYTES)


def read(path: str, as_float32: bool = True):
    """Returns (stack (nz, ny, nx), info).  info["tilt_angles"] holds the FEI
    per-image tilt angles when the file carries them (else None)."""
    info = read_header(path)
    dt = np.dtype(_MODES[info["mode"]]).newbyteorder("<" if info["little_endian"] else ">")
    n = info["nx"] * info["ny"] * info["nz"]
    with open(path, "rb") as f:
        f.seek(info["offset"])
        data = np.fromfile(f, dtype=dt, count=n)
        if data.size != n:
            raise IOError(f"{path}: truncated data ({data.size} of {n} values)")
        tilts = None
        if info["fei"]:
            f.seek(HEADER_BYTES)
            ext = f.read(FEI_EXTENDED_BYTES)
            fmt = "<f" if info["little_endian"] else ">f"
            tilts = np.array([struct.unpack_from(fmt, ext, 128 * i)[0] for i in range(info["nz"])], np.float64)
    stack = data.reshape(info["nz"], info["ny"], info["nx"])
    stack = stack.astype(np.float32) if as_float32 else stack.astype(dt.newbyteorder("="))
    info["tilt_angles"] = tilts
    return stack, info


def _stats(stack: np.ndarray):
    # MRC_Writer.createHeader: min/max with the reference's `else if`, mean from a double sum
    flat = stack.reshape(-1).astype(np.float32)
    if flat.size == 0:
        return float("nan"), float("nan"), float("nan")
    mn = mx = float(flat[0])
    for v in flat[1:]:
        v = float(v)
        if mx < v:
            mx = v
        elif mn > v:
            mn = v
    mean = float(np.float32(np.sum(flat, dtype=np.float64) / flat.size))
    return mn, mx, mean


def _stats_fast(stack: np.ndarray):
    """The same figures without a Python loop: a new maximum is never tested as a
    minimum, so the minimum is taken over the values that were not a running maximum
    when they arrived (the first value counts as both)."""
    flat = np.ascontiguousarray(stack.reshape(-1), np.float32).astype(np.float64)
    if flat.size == 0:
        return float("nan"), float("nan"), float("nan")
    run_max = np.maximum.accumulate(flat)
    new_max = np.empty(flat.size, bool)
    new_max[0] = False
    new_max[1:] = flat[1:] > run_max[:-1]
    cand = flat[~new_max]
    mn = float(np.min(cand)) if cand.size else float(flat[0])
    mx = float(run_max[-1])
    mean = float(np.float32(np.sum(flat) / flat.size))
    return mn, mx, mean


def header_bytes(stack: np.ndarray) -> bytes:
    """The 1024-byte header MRC_Writer writes for `stack` (nz, ny, nx)."""
    nz, ny, nx = stack.shape
    if stack.dtype == np.uint8:
        mode = 0
    elif stack.dtype in (np.int16, np.uint16):
        mode = 1 if (stack.size and int(stack.min()) < 0) else 6
    else:
        mode = 2
    mn, mx, mean = _stats_fast(stack)
    h = bytearray(HEADER_BYTES)
    for k, v in enumerate((nx, ny, nz, mode)):
        struct.pack_into("<i", h, 4 * k, v)
    for k, v in ((16, 1), (17, 2), (18, 3)):
        struct.pack_into("<i", h, 4 * k, v)
    for k, v in ((19, mn), (20, mx), (21, mean)):
        struct.pack_into("<f", h, 4 * k, v)
    return bytes(h)


def write(path: str, stack: np.ndarray) -> None:
    """MRC_Writer: little-endian header and data; float stacks are written as mode 2."""
    stack = np.asarray(stack)
    if stack.ndim == 2:
        stack = stack[None]
    if stack.dtype not in (np.uint8, np.int16, np.uint16):
        stack = stack.astype(np.float32)
    dt = stack.dtype.newbyteorder("<")
    with open(path, "wb") as f:
        f.write(header_bytes(stack))
        f.write(np.ascontiguousarray(stack, dtype=dt).tobytes())
