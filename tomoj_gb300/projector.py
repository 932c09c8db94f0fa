"""GB300 drop-in for TomoJ's Projector plug-in surface.

Mirrors Projector (TomoJ_Base/.../projectors/Projector.java:14-159) and the
VoxelProjector3D setters (VoxelProjector3D.java:69-104) with the same method
names and argument meanings; every call goes through the C ABI of
libtomoj_gb300.so (include/tomoj_gb300.h).  The volume and the tilt-series stay
resident in HBM; `rec` is updated in place on the device and read back with
TomoReconstruction2.getVolume().
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import check


class Projector:
    """Abstract projector surface (Projector.java:130-156)."""

    def addProjection(self, index: int) -> None:
        raise NotImplementedError

    def clearAllProjections(self) -> None:
        raise NotImplementedError

    def project(self, startY: int = 0, endY: int | None = None) -> None:
        raise NotImplementedError

    def projectAndDifference(self, factor: float, startY: int = 0, endY: int | None = None) -> np.ndarray:
        raise NotImplementedError

    def backproject(self, startY: int = 0, endY: int | None = None) -> None:
        raise NotImplementedError

    def startOfIteration(self) -> None:
        raise NotImplementedError

    def endOfIteration(self) -> None:
        raise NotImplementedError

    def getProjection(self, index: int) -> np.ndarray:
        raise NotImplementedError


class VoxelProjector3D(Projector):
    """Ray-driven forward projector / voxel-driven backprojector on the GPU.

    Construction captures dimensions and centres from the tilt-series and the
    reconstruction (Projector.java:30-40); the tilt-series (aligned by the
    series' AffineAlignment, TiltSeries.getPixels) is uploaded once.
    `weighting` is None or a (kind, radius) pair (WBP filter).  `precision` selects the
    volume storage ("fp32", "bf16" or "fp16"; 16-bit forms keep per-row slab scales)."""

    def __init__(self, ts, rec, weighting=None, positivity=False, long_object=False, scale=None, precision="fp32"):
        self.ts = ts
        self.rec = rec
        lib = _abi.load()
        W, H, D = rec.getWidth(), rec.getHeight(), rec.getSizez()
        w, h, n = ts.getWidth(), ts.getHeight(), ts.getImageStackSize()
        if scale is None:
            scale = w / float(W)  # ReconstructionParameters.rescaleData (ReconstructionParameters.java:328)
        self._geom = _abi.make_geom(W, H, D, w, h, n, vol_center=rec.centers(),
                                    proj_center=(ts.getCenterX(), ts.getCenterY(), ts.getProjectionCenterX(),
                                                 ts.getProjectionCenterY()), scale=scale)
        self._params = _abi.make_params(positivity=positivity, long_object=long_object, fill=ts.getFillType(),
                                        normalize=ts.isNormalized(), precision=_abi.precision_code(precision))
        h_ = C.c_void_p()
        check(lib.tomo_create(C.byref(self._geom), C.byref(self._params), C.byref(h_)))
        self._h = h_
        self._lib = lib
        self._n_added = 0
        self.weighting = None
        self._upload_series()
        rec._attach(self)
        if weighting is not None:
            self.setWeighting(*weighting)

    # --- lifetime --------------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self.rec._detach(self)
            self._lib.tomo_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def _upload_series(self):
        ts = self.ts
        eul = np.ascontiguousarray(ts.eulers(), np.float64)
        T = np.ascontiguousarray(ts.transforms(), np.float64)
        need_stats = ts.isNormalized() or ts.getFillType() == _abi.FILL_AVG
        stats = np.ascontiguousarray(ts.statistics(), np.float64) if need_stats else None
        pix = np.ascontiguousarray(ts.pixels, np.float32)
        check(self._lib.tomo_load_series(self._h, pix.ctypes.data, 0, _abi.ptr(eul, C.c_double),
                                         _abi.ptr(T, C.c_double),
                                         None if stats is None else _abi.ptr(stats, C.c_double)))

    # --- setters (VoxelProjector3D.java:78-104) ----------------------------------------
    def setPositivityConstraint(self, enabled: bool):
        check(self._lib.tomo_set_positivity(self._h, int(bool(enabled))))

    def setLongObjectCompensation(self, enabled: bool):
        check(self._lib.tomo_set_long_object(self._h, int(bool(enabled))))

    def setScale(self, value: float):
        """Projection width / reconstruction width (VoxelProjector3D.setScale)."""
        check(self._lib.tomo_set_scale(self._h, float(value)))

    def setVolumeCenters(self, cx, cy=None, cz=None):
        """Projector.setVolumeCenters(rec) or (cx, cy, cz) (Projector.java:60-65, 104-108)."""
        if cy is None:
            cx, cy, cz = cx.centers()
        vc = np.ascontiguousarray([cx, cy, cz], np.float64)
        check(self._lib.tomo_set_centers(self._h, _abi.ptr(vc, C.c_double), None))

    def setProjectionCenter(self, pcx, pcy=None):
        """Projector.setProjectionCenter(ts) (all four centres) or (pcx, pcy) (the tilt-axis
        position on the projections only) (Projector.java:52-58, 99-102)."""
        if pcy is None:
            ts = pcx
            pc = [ts.getCenterX(), ts.getCenterY(), ts.getProjectionCenterX(), ts.getProjectionCenterY()]
        else:
            pc = [np.nan, np.nan, pcx, pcy]
        pc = np.ascontiguousarray(pc, np.float64)
        check(self._lib.tomo_set_centers(self._h, None, _abi.ptr(pc, C.c_double)))

    def getTiltSeries(self):
        return self.ts

    def getReconstruction(self):
        return self.rec

    def getWeightingFilter(self):
        return self.weighting

    def setWeightingFilter(self, weighting):
        """None or a (kind, radius) pair (Projector.setWeightingFilter)."""
        if weighting is None:
            check(self._lib.tomo_set_weighting(self._h, _abi.WEIGHT_NONE, 0.0, None, None))
            self.weighting = None
        else:
            self.setWeighting(*weighting)

    def getCompletion(self) -> float:
        return float(getattr(self.rec, "completion", 0.0))

    def setNbRaysPerPixels(self, n: float):
        """Kept for the reference's interface: its Joseph projector reads one ray per
        pixel whatever this value (VoxelProjector3D.java:471, 671-821)."""
        self.nbRaysPerPixels = float(n)

    def setWeighting(self, kind: int, radius: float = 0.0):
        """new FFTWeighting(ts, radius * w) (ReconstructionParameters.java:320): the mask
        reads every tilt angle and the tilt axis (FFTWeighting.java:67-81)."""
        ts = self.ts
        n = ts.getImageStackSize()
        tilts = np.ascontiguousarray([ts.getTiltAngle(i) for i in range(n)], np.float64)
        axes = np.full(n, float(ts.getTiltAxis()), np.float64)
        check(self._lib.tomo_set_weighting(self._h, int(kind), float(radius), _abi.ptr(tilts, C.c_double),
                                           _abi.ptr(axes, C.c_double)))
        self.weighting = (kind, radius)

    def isWeighting(self) -> bool:
        return self.weighting is not None and self.weighting[0] != _abi.WEIGHT_NONE

    def setTVM(self, theta=25.0, g=1.0, dt=0.1, iterations=5):
        check(self._lib.tomo_set_tvm(self._h, theta, g, dt, int(iterations)))

    def setFista(self, enabled: bool):
        check(self._lib.tomo_set_fista(self._h, int(bool(enabled))))

    # --- Projector surface --------------------------------------------------------------
    def _rows(self, startY, endY):
        return int(startY), int(self.rec.getHeight() if endY is None else endY)

    def addProjection(self, index: int) -> None:
        check(self._lib.tomo_add_projection(self._h, int(index)))
        self._n_added += 1

    def clearAllProjections(self) -> None:
        check(self._lib.tomo_clear_projections(self._h))
        self._n_added = 0

    def project(self, startY: int = 0, endY: int | None = None) -> None:
        y0, y1 = self._rows(startY, endY)
        check(self._lib.tomo_project(self._h, y0, y1))

    def projectAndDifference(self, factor: float, startY: int = 0, endY: int | None = None) -> np.ndarray:
        y0, y1 = self._rows(startY, endY)
        n = self._lib.tomo_projection_count(self._h)
        err = np.zeros(max(n, 1), np.float64)
        check(self._lib.tomo_project_and_difference(self._h, float(factor), y0, y1, _abi.ptr(err, C.c_double)))
        return err[:n]

    def backproject(self, startY: int = 0, endY: int | None = None) -> None:
        y0, y1 = self._rows(startY, endY)
        check(self._lib.tomo_backproject(self._h, y0, y1))

    def startOfIteration(self) -> None:
        check(self._lib.tomo_start_iteration(self._h))

    def endOfIteration(self) -> None:
        check(self._lib.tomo_end_iteration(self._h))

    def _slot(self, fn, index):
        out = np.empty((self.ts.getHeight(), self.ts.getWidth()), np.float32)
        check(fn(self._h, int(index), _abi.ptr(out)))
        return out

    def getProjection(self, index: int) -> np.ndarray:
        return self._slot(self._lib.tomo_get_projection, index)

    def getNormImage(self, index: int) -> np.ndarray:
        return self._slot(self._lib.tomo_get_norm, index)

    def getDifferenceImage(self, index: int) -> np.ndarray:
        return self._slot(self._lib.tomo_get_difference, index)

    def getAlignedProjection(self, index: int) -> np.ndarray:
        """TiltSeries.getPixels(index) as resident on the device."""
        return self._slot(self._lib.tomo_get_aligned, index)

    # --- device drivers ---------------------------------------------------------------------
    def run_wbp(self, startY=0, endY=None):
        y0, y1 = self._rows(startY, endY)
        check(self._lib.tomo_run_wbp(self._h, y0, y1))

    def run_ossart(self, n_iter, relax, update, seed=0, startY=0, endY=None, use_graph=True):
        y0, y1 = self._rows(startY, endY)
        err = np.zeros((max(n_iter, 1), 5), np.float64)
        check(self._lib.tomo_run_ossart(self._h, int(n_iter), float(relax), int(update), int(seed), y0, y1,
                                        int(bool(use_graph)), _abi.ptr(err, C.c_double)))
        return err[:n_iter]

    def order(self, first: int) -> np.ndarray:
        out = np.zeros(self.ts.getImageStackSize(), np.int32)
        check(self._lib.tomo_order(self._h, int(first), _abi.ptr(out, C.c_int32)))
        return out

    def cancel(self):
        check(self._lib.tomo_cancel(self._h))

    # volume plumbing used by TomoReconstruction2
    def _share_volume(self, owner):
        """Work on `owner`'s device volume (two projectors on one TomoReconstruction2);
        None takes a private copy."""
        check(self._lib.tomo_share_volume(self._h, None if owner is None else owner._h))

    def _shares_with(self, other) -> bool:
        """Whether this projector can work on `other`'s device volume."""
        return (isinstance(other, VoxelProjector3D) and getattr(other, "_h", None) is not None
                and self._params.precision == _abi.PREC_FP32 and other._params.precision == _abi.PREC_FP32)

    def _set_volume(self, vol: np.ndarray):
        vol = np.ascontiguousarray(vol, np.float32)
        check(self._lib.tomo_set_volume(self._h, vol.ctypes.data, 0, 0, vol.shape[1]))

    def _get_volume(self) -> np.ndarray:
        D, H, W = self.rec.getSizez(), self.rec.getHeight(), self.rec.getWidth()
        out = np.empty((D, H, W), np.float32)
        check(self._lib.tomo_get_volume(self._h, out.ctypes.data, 0, 0, H))
        return out


class BayesianVoxelProjector3D(VoxelProjector3D):
    """BayesianVoxelProjector3D (TomoJ_AdvancedReconstruction/.../projectors/
    BayesianVoxelProjector3D.java): the differences of an iteration accumulate in a
    distance volume seeded with -lambda times the 27-point [1,-2,1]^3 stencil of the
    volume, and alpha times it is added to the volume at the end of the iteration."""

    def __init__(self, ts, rec, weighting=None, **kw):
        super().__init__(ts, rec, weighting, **kw)
        self.regularizationLambda = 0.1
        self.regularizationAlpha = 0.1
        self._apply()

    def _apply(self):
        check(self._lib.tomo_set_bayesian(self._h, float(self.regularizationLambda),
                                          float(self.regularizationAlpha), 1))

    def setRegularizationLambda(self, v: float):
        self.regularizationLambda = float(v)
        self._apply()

    def setRegularizationAlpha(self, v: float):
        self.regularizationAlpha = float(v)
        self._apply()


class BgARTVoxelProjector3D(VoxelProjector3D):
    """BgARTVoxelProjector3D (TomoJ_AdvancedReconstruction/.../projectors/
    BgARTVoxelProjector3D.java): cross median before and histogram collapse filter
    after every iteration; the constructor collapses the starting volume once."""

    def __init__(self, ts, rec, weighting, k, darkBG=True, doMedian=True, **kw):
        super().__init__(ts, rec, weighting, **kw)
        self.k, self.darkBG, self.doMedian = float(k), bool(darkBG), bool(doMedian)
        self.bgValue = float("nan")
        check(self._lib.tomo_set_bgart(self._h, self.k, int(self.darkBG), int(self.doMedian), self.bgValue, 1))


class CompressedSensingProjector(VoxelProjector3D):
    """CompressedSensingProjector (TomoJ_AdvancedReconstruction/.../projectors/
    CompressedSensingProjector.java:16-201): after every iteration the volume goes through
    the separable 3-D fractional spline wavelet transform, is soft-thresholded at the level
    that zeroes softThresholdingPercentageOfZeros of the coefficients and is transformed
    back.  The wavelet filters are restated from the published fractional spline wavelets
    (the reference calls a third-party library for them)."""

    WAVELET_ORTHONORMAL, WAVELET_BSPLINE, WAVELET_DUAL = 0, 3, 6

    def __init__(self, ts, rec, weighting=None, waveletType=3, waveletDegree=3.0, waveletShift=0.0,
                 softThresholdingPercentageOfZeros=0.95, **kw):
        super().__init__(ts, rec, weighting, **kw)
        self.waveletDegree = float(waveletDegree)
        self.waveletShift = float(waveletShift)
        self.waveletType = int(waveletType)
        self.softThresholdingPercentageOfZeros = float(softThresholdingPercentageOfZeros)
        self.iters = self.findBestWaveletsIteration(rec)
        self._apply()

    @staticmethod
    def findBestWaveletsIteration(rec):
        """CompressedSensingProjector.java:127-151: levels from 64 doubling up to the width,
        the same count on all three axes (the reference sizes every axis from the width)."""
        n, s = 1, 64
        while s < rec.getWidth():
            s *= 2
            n += 1
        return [n, n, n]

    def _apply(self):
        lv = (C.c_int32 * 3)(*[int(v) for v in self.iters])
        check(self._lib.tomo_set_compressed_sensing(self._h, int(self.waveletType), float(self.waveletDegree),
                                                    float(self.waveletShift),
                                                    float(self.softThresholdingPercentageOfZeros), lv, 1))

    def getLastThreshold(self) -> float:
        """The soft threshold of the last end-of-iteration filter."""
        out = C.c_double()
        check(self._lib.tomo_compressed_sensing_threshold(self._h, C.byref(out)))
        return out.value

    def getWaveletDegree(self):
        return self.waveletDegree

    def setWaveletDegree(self, v):
        self.waveletDegree = float(v)
        self._apply()

    def getWaveletShift(self):
        return self.waveletShift

    def setWaveletShift(self, v):
        self.waveletShift = float(v)
        self._apply()

    def getWaveletType(self):
        return self.waveletType

    def setWaveletType(self, v):
        self.waveletType = int(v)
        self._apply()

    def getSoftThresholdingPercentageOfZeros(self):
        return self.softThresholdingPercentageOfZeros

    def setSoftThresholdingPercentageOfZeros(self, v):
        self.softThresholdingPercentageOfZeros = float(v)
        self._apply()

    def getWaveletsIterations(self):
        return list(self.iters)

    def setWaveletsIterations(self, x, y=None, z=None):
        self.iters = list(x) if y is None else [int(x), int(y), int(z)]
        self._apply()


class VoxelProjector3DGPU(VoxelProjector3D):
    """VoxelProjector3DGPU / ProjectorGPU (TomoJ_GPU/.../projectors/ProjectorGPU.java:70-403):
    the reference's OpenCL projector surface over the same engine handle.  The engine keeps
    the whole volume on the device, so the slab calls act on rows of it:

    * initForBP(startY, endY, updateNb) zeroes rows [startY, endY): the reference
      backprojects into a new zero buffer (:175-193);
    * initForIterative(startY, endY, update, kernelType, errorVolume[, other]) uploads those
      rows from the reconstruction's host copy (:211-216), or, with `other`, works on
      other's device volume (:217-235);
    * copyInGPUBuffer uploads rows, updateFromGPU(startY, endY[, usableStartY, usableEndY])
      downloads the usable rows into the reconstruction's host copy (:297-330);
    * releaseCL_Memory frees the device memory and leaves the host copy as the last
      updateFromGPU left it (:376-403);
    * computeMaximumSizeForVolume is 40 % of the device memory (:162-166).

    Kernel choices (setKernelToUse, setUseImage3D, kernelType) pick among OpenCL kernels of
    one computation and are recorded only.  The debugging error volume (errorVolume =
    True) is not provided."""

    SEPARATE_PROJ_DIFF, ONE_KERNEL_PROJ_DIFF, ONE_KERNEL_PROJ_DIFF_WITH_ALIGNMENT = 0, 1, 2

    def __init__(self, ts, rec, device=None, weightingFilter=None, **kw):
        super().__init__(ts, rec, weightingFilter, **kw)
        self.device = device
        self.kernelusage = self.SEPARATE_PROJ_DIFF
        self.useImage3D = False
        self.currentStartY, self.currentEndY = 0, rec.getHeight()

    def setKernelToUse(self, kernelusage: int):
        self.kernelusage = int(kernelusage)

    def setUseImage3D(self, useImage3D: bool):
        self.useImage3D = bool(useImage3D)

    def computeMaximumSizeForVolume(self) -> int:
        free, total = C.c_uint64(), C.c_uint64()
        check(self._lib.tomo_device_memory(C.byref(free), C.byref(total)))
        return int(0.4 * total.value)

    def _slab(self, startY, endY):
        if not 0 <= startY <= endY <= self.rec.getHeight():
            raise ValueError(f"rows [{startY}, {endY}) outside the volume")
        self.currentStartY, self.currentEndY = int(startY), int(endY)

    def initForBP(self, startY: int, endY: int, updateNb: int):
        self._slab(startY, endY)
        zeros = np.zeros((self.rec.getSizez(), endY - startY, self.rec.getWidth()), np.float32)
        check(self._lib.tomo_set_volume(self._h, zeros.ctypes.data, 0, startY, endY))
        self.kernelusage = self.SEPARATE_PROJ_DIFF

    def initForIterative(self, startY: int, endY: int, update: int, kernelType: int, errorVolume: bool = False,
                         other=None):
        if errorVolume:
            raise NotImplementedError("the debugging error volume of the OpenCL projector is not provided")
        self._slab(startY, endY)
        self.kernelusage = int(kernelType)
        if other is not None:
            self._share_volume(other)
            return
        self.copyInGPUBuffer(startY, endY)

    def copyInGPUBuffer(self, startY: int, endY: int):
        rows = np.ascontiguousarray(self.rec._host[:, startY:endY, :])
        check(self._lib.tomo_set_volume(self._h, rows.ctypes.data, 0, startY, endY))

    def updateFromGPU(self, startY: int, endY: int, usableStartY=None, usableEndY=None):
        a = startY if usableStartY is None else int(usableStartY)
        b = endY if usableEndY is None else int(usableEndY)
        out = np.empty((self.rec.getSizez(), b - a, self.rec.getWidth()), np.float32)
        check(self._lib.tomo_get_volume(self._h, out.ctypes.data, 0, a, b))
        self.rec._host[:, a:b, :] = out

    def releaseCL_Memory(self):
        host = self.rec._host
        self.close()
        self.rec._host = host


def first_index(seed: int, iteration: int, nproj: int) -> int:
    """Deterministic replacement of orderShuffleART's Math.random() first index."""
    return int(_abi.load().tomo_first_index(int(seed), int(iteration), int(nproj)))
