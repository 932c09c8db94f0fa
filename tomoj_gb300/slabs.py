"""Y-slab partitioning of one reconstruction across ranks.

With the tilt axis vertical (AffineAlignment.java:18, 389-395) projection row j
only sees volume row j - (pc1 - vc1), so contiguous row slabs are independent:
each rank reconstructs rows [y0, y1) of the volume from the matching rows of
every aligned projection, with the full volume's centres expressed in slab
coordinates.  The reference partitions the same way across OpenCL devices
(ReconstructionThreadManagerGPU.doGPURec, ReconstructionThreadManagerGPU.java:172-308).
The only exchange is the per-projection FP64 residual of every update (summed
across ranks before osartIteration's error summary) and the final gather.

Every slab but the last carries one extra volume row (a halo whose values are
never used): the reference's sampler returns the raw floor voxel on the
volume's last row (TomoReconstruction2.java:163-164), and without the halo a
slab's last row would be treated as the volume's last row.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Slab:
    y0: int           # first volume row owned by the rank
    y1: int           # one past the last owned volume row
    halo: int         # 1 if the sub-volume carries row y1 as a halo
    j0: int           # first projection row of the sub-series
    j1: int           # one past its last projection row
    vol_center: tuple  # (cx, cy, cz) in slab coordinates
    proj_center: tuple  # (centerX, centerY, projectionCenterX, projectionCenterY) in slab coordinates

    @property
    def rows(self) -> int:
        """Rows of the sub-volume, halo included."""
        return self.y1 - self.y0 + self.halo

    @property
    def proj_rows(self) -> int:
        return self.j1 - self.j0


def _centres(W, H, D, w, h, vol_center, proj_center):
    vc = tuple(vol_center) if vol_center is not None else ((W - 1) / 2.0, (H - 1) / 2.0, (D - 1) / 2.0)
    pc = tuple(proj_center) if proj_center is not None else ((w - 1.0) / 2, (h - 1.0) / 2, (w - 1) / 2.0,
                                                             (h - 1) / 2.0)
    off_fp = pc[1] - vc[1]
    off_bp = pc[3] - vc[1]
    if off_fp != off_bp or off_fp != int(off_fp):
        raise ValueError("slabs need equal, integral row offsets for projection and backprojection")
    return vc, pc, int(off_fp)


def slab(W: int, H: int, D: int, w: int, h: int, y0: int, y1: int, vol_center=None, proj_center=None) -> Slab:
    """The slab of volume rows [y0, y1) (0 <= y0 <= y1 <= H): its halo, projection rows
    and centres in slab coordinates."""
    if not 0 <= y0 <= y1 <= H:
        raise ValueError("slab rows out of range")
    vc, pc, off = _centres(W, H, D, w, h, vol_center, proj_center)
    halo = 1 if y1 < H else 0
    j0 = min(max(y0 + off, 0), h)
    j1 = min(max(y1 + halo + off, 0), h)
    return Slab(y0, y1, halo, j0, j1, (vc[0], vc[1] - y0, vc[2]), (pc[0], pc[1] - j0, pc[2], pc[3] - j0))


def plan(W: int, H: int, D: int, w: int, h: int, world: int, vol_center=None, proj_center=None) -> list[Slab]:
    """Contiguous, balanced row slabs for `world` ranks (rank r gets slabs[r]).
    Centres default to TomoJ's ((n - 1) / 2) convention."""
    _centres(W, H, D, w, h, vol_center, proj_center)
    out = []
    base, extra = divmod(H, world)
    y = 0
    for r in range(world):
        n = base + (1 if r < extra else 0)
        out.append(slab(W, H, D, w, h, y, y + n, vol_center, proj_center))
        y += n
    return out


def crop_series(series: np.ndarray, slab: Slab, halo_nan: bool = True) -> np.ndarray:
    """Rows [j0, j1) of every aligned projection (N, h, w) -> (N, j1 - j0, w).  For the
    iterative methods the halo row's measurements are NaN, so its pixels add nothing to
    the difference images or to the residual (VoxelProjector3D.difference skips NaN
    measurements).  For WBP, which backprojects the measurements themselves, pass
    halo_nan=False: the backprojection's bilinear read of the slab's last row blends in
    the halo row with weight 0 (ImageJ getInterpolatedValue), and a NaN there would
    void the sample."""
    out = np.array(series[:, slab.j0:slab.j1, :], np.float32, copy=True, order="C")
    if halo_nan and slab.halo and slab.j1 > slab.j0:
        out[:, -1, :] = np.nan
    return out


def error_summary(per_proj: np.ndarray, order, W: int, H: int) -> np.ndarray:
    """osartIteration's summary (TomoReconstruction2.java:692-730) from the per-projection
    sums of squared differences in update order, including its else-if."""
    som, errmin, errmax, imin, imax = 0.0, float(np.finfo(np.float32).max), 0.0, 0, 0
    for t, e in enumerate(per_proj):
        som += e
        if e > errmax:
            errmax, imax = e, int(order[t])
        elif e < errmin:
            errmin, imin = e, int(order[t])
    n = len(per_proj)
    return np.array([np.sqrt(som / (n * W * H)), np.sqrt(errmin / (W * H)), imin, np.sqrt(errmax / (W * H)), imax])
