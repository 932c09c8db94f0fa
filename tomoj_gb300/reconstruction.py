"""Host-side mirror of TomoReconstruction2's drivers and the parameter factories.

TomoReconstruction2 (TomoJ_Base/.../tomography/TomoReconstruction2.java) is the
volume container plus the WBP / OSSART / regularization iteration drivers;
ReconstructionParameters (ReconstructionParameters.java:279-333) and
AdvancedReconstructionParameters (AdvancedReconstructionParameters.java:112-221)
build the projector for a method.  Same names and argument meanings; the
drivers run device-resident through the C ABI (one graph-captured launch
sequence per iteration) when the projector is the GB300 VoxelProjector3D, and
through the plain Projector surface otherwise.
"""
from __future__ import annotations

import numpy as np

from . import _abi
from .projector import Projector, VoxelProjector3D, first_index

# ReconstructionParameters (:13-15) and AdvancedReconstructionParameters (:10-13) types
BP, WBP, OSSART = 0, 1, 2
TVM, BAYESIAN, COMPRESSED_SENSING, BGART = 3, 4, 5, 6


class TomoReconstruction2:
    """Reconstruction volume float32 (D, H, W) with TomoJ's centre convention."""

    def __init__(self, width: int, height: int, depth: int, data: np.ndarray | None = None):
        self.W, self.H, self.D = int(width), int(height), int(depth)
        self._host = np.zeros((self.D, self.H, self.W), np.float32) if data is None else \
            np.ascontiguousarray(data, np.float32).reshape(self.D, self.H, self.W).copy()
        self.centerx = (self.W - 1) / 2.0
        self.centery = (self.H - 1) / 2.0
        self.centerz = (self.D - 1) / 2.0
        self._proj = None      # the projector holding the volume on the device
        self._sharers = []     # projectors working on the same device volume
        self.completion = 0.0

    # --- container ------------------------------------------------------------------
    def getWidth(self):
        return self.W

    def getHeight(self):
        return self.H

    def getSizez(self):
        return self.D

    def centers(self):
        return (self.centerx, self.centery, self.centerz)

    def setCenter(self, cx, cy, cz):
        self.centerx, self.centery, self.centerz = float(cx), float(cy), float(cz)

    def _attach(self, projector):
        # projectors built on the same reconstruction work on one volume (the dual-axis
        # drivers construct two), as the reference's projectors share `rec`
        owner = self._proj
        if owner is not None and owner is not projector and projector._shares_with(owner):
            projector._share_volume(owner)
            self._sharers.append(projector)
            return
        self._proj = projector
        self._sharers = []
        projector._set_volume(self._host)

    def _detach(self, projector):
        if self._proj is projector:
            self._host = projector._get_volume()
            # the engine hands the device volume to the first sharer
            self._proj = self._sharers.pop(0) if self._sharers else None
        elif projector in self._sharers:
            self._sharers.remove(projector)

    def getVolume(self) -> np.ndarray:
        if self._proj is not None:
            self._host = self._proj._get_volume()
        return self._host

    def setVolume(self, data: np.ndarray):
        self._host = np.ascontiguousarray(data, np.float32).reshape(self.D, self.H, self.W).copy()
        if self._proj is not None:
            self._proj._set_volume(self._host)

    def interrupt(self):
        self.completion = -1000
        for p in ([self._proj] if self._proj is not None else []) + self._sharers:
            p.cancel()

    # --- drivers ----------------------------------------------------------------------
    def WBP(self, ts, projector: Projector, params=None, startY=0, endY=None):
        """WBP with update 0 (TomoReconstruction2.java:499-538)."""
        endY = self.H if endY is None else endY
        if isinstance(projector, VoxelProjector3D):
            projector.run_wbp(startY, endY)
            return
        for i in range(ts.getImageStackSize()):
            projector.addProjection(i)
            projector.backproject(startY, endY)
            projector.clearAllProjections()

    def OSSART(self, ts, projector: Projector, params, startY=0, endY=None, seed=0, use_graph=True):
        """OS-SART / SIRT / ART (TomoReconstruction2.java:548-634).  Returns the per-iteration
        error rows [average, min, argmin, max, argmax]."""
        endY = self.H if endY is None else endY
        if isinstance(projector, VoxelProjector3D):
            return projector.run_ossart(params.getNbIterations(), params.getRelaxationCoefficient(),
                                        params.getUpdateNb(), seed, startY, endY, use_graph)
        return self._ossart_surface(ts, projector, params, startY, endY, seed)

    def regularization(self, ts, projector: Projector, params, startY=0, endY=None, seed=0, use_graph=True):
        """TomoReconstruction2.regularization (TomoReconstruction2.java:783-878): the same
        iteration with the projector's endOfIteration regularisation (TVM)."""
        return self.OSSART(ts, projector, params, startY, endY, seed, use_graph)

    def _ossart_surface(self, ts, projector, params, startY, endY, seed):
        n = ts.getImageStackSize()
        out = []
        for it in range(params.getNbIterations()):
            projector.startOfIteration()
            out.append(self.osartIteration(projector, ts, params, startY, endY, first_index(seed, it, n)))
            projector.endOfIteration()
        return np.array(out)

    def osartIteration(self, projector, ts, params, startY, endY, first):
        """One iteration through the Projector surface (TomoReconstruction2.osartIteration,
        :640-733); `first` is orderShuffleART's first index.  Returns [average, min, argmin,
        max, argmax]."""
        n = ts.getImageStackSize()
        order = order_shuffle(ts.eulers(), first)
        upd = n if params.getUpdateNb() == 0 else params.getUpdateNb()
        factor = float(np.float32(params.getRelaxationCoefficient() / upd))
        som, errmin, errmax, imin, imax = 0.0, float(np.finfo(np.float32).max), 0.0, 0, 0
        pending = 0
        projector.clearAllProjections()
        for t in range(n):
            projector.addProjection(int(order[t]))
            pending += 1
            if pending == upd or t == n - 1:
                err = projector.projectAndDifference(factor, startY, endY)
                for e, v in enumerate(err):
                    som += v
                    if v > errmax:
                        errmax, imax = v, order[t - len(err) + e + 1]
                    elif v < errmin:
                        errmin, imin = v, order[t - len(err) + e + 1]
                projector.backproject(startY, endY)
                projector.clearAllProjections()
                pending = 0
        wh = self.W * self.H
        return [np.sqrt(som / (n * wh)), np.sqrt(errmin / wh), imin, np.sqrt(errmax / wh), imax]

    def osartIterationDual(self, projector1, ts1, projector2, ts2, params, startY, endY, first1, first2):
        """TomoReconstruction2.osartIterationDual (:1282-1428): the two series alternate two
        projections at a time with one update counter shared by both projectors; the loop
        runs t < n1 - 1 (the last projection of an odd-length first series is not used) and
        a projector's pending projections are flushed when the shared counter reaches
        `update` or at its series' last index."""
        n1, n2 = ts1.getImageStackSize(), ts2.getImageStackSize()
        upd = params.getUpdateNb()  # used as given: 0 is not replaced by the series length here
        factor = float(np.float32(params.getRelaxationCoefficient() / upd)) if upd else float(np.float32(np.inf))
        projector1.clearAllProjections()
        projector2.clearAllProjections()
        idx = (order_shuffle(ts1.eulers(), first1), order_shuffle(ts2.eulers(), first2))
        state = {"diff": 0, "som": 0.0, "min": float(np.finfo(np.float32).max), "max": 0.0, "imin": 0, "imax": 0}

        def step(proj, ts, order, t, i):
            proj.addProjection(int(order[t + i]))
            state["diff"] += 1
            if state["diff"] == upd or t + i == ts.getImageStackSize() - 1:
                err = proj.projectAndDifference(factor, startY, endY)
                for e, v in enumerate(err):
                    state["som"] += v
                    if v > state["max"]:
                        state["max"], state["imax"] = v, int(order[t + i - len(err) + e + 1])
                    elif v < state["min"]:
                        state["min"], state["imin"] = v, int(order[t + i - len(err) + e + 1])
                proj.backproject(startY, endY)
                proj.clearAllProjections()
                state["diff"] = 0

        for t in range(0, n1 - 1, 2):
            for i in range(2):
                if t + 1 >= n1 or self.completion < 0:
                    break
                step(projector1, ts1, idx[0], t, i)
            for i in range(2):
                if t + 1 >= n2 or self.completion < 0:
                    break
                step(projector2, ts2, idx[1], t, i)
        wh = self.W * self.H
        return [np.sqrt(state["som"] / ((n1 + n2) * wh)), np.sqrt(state["min"] / wh), state["imin"],
                np.sqrt(state["max"] / wh), state["imax"]]

    def _until_diverging(self, iteration, n_iter):
        """The dual-axis drivers' loop: stop once the average residual grows by more than
        10 % over the previous iteration's.  Returns the average of every iteration run."""
        out, err0 = [], float("inf")
        for i in range(n_iter):
            if self.completion < 0:
                break
            err = iteration(i)
            out.append(err[0])
            if err[0] > err0 * 1.1:
                self.completion = -1000
            else:
                err0 = err[0]
        return out

    def ADASIRT(self, ts1, projector1, ts2, projector2, params, startY=0, endY=None, seed=0):
        """TomoReconstruction2.ADASIRT (:880-999): alternate whole iterations of the two
        series on one volume.  As the reference, projector1.endOfIteration() runs after
        both halves (projector2's never does).  Iteration i orders series 1 and 2 with
        first indexes first_index(seed, 2i, n1) and first_index(seed, 2i + 1, n2)."""
        endY = self.H if endY is None else endY
        self.completion = 0.0
        n1, n2 = ts1.getImageStackSize(), ts2.getImageStackSize()

        def iteration(i):
            projector1.startOfIteration()
            self.osartIteration(projector1, ts1, params, startY, endY, first_index(seed, 2 * i, n1))
            projector1.endOfIteration()
            projector2.startOfIteration()
            err = self.osartIteration(projector2, ts2, params, startY, endY, first_index(seed, 2 * i + 1, n2))
            projector1.endOfIteration()
            return err

        return self._until_diverging(iteration, params.getNbIterations())

    def ADOSSART(self, ts1, projector1, ts2, projector2, params, startY=0, endY=None, seed=0):
        """TomoReconstruction2.ADOSSART (:1001-1100): iterations of osartIterationDual, then
        both projectors' endOfIteration."""
        endY = self.H if endY is None else endY
        self.completion = 0.0
        n1, n2 = ts1.getImageStackSize(), ts2.getImageStackSize()

        def iteration(i):
            err = self.osartIterationDual(projector1, ts1, projector2, ts2, params, startY, endY,
                                          first_index(seed, 2 * i, n1), first_index(seed, 2 * i + 1, n2))
            projector1.endOfIteration()
            projector2.endOfIteration()
            return err

        return self._until_diverging(iteration, params.getNbIterations())

    def ADASIRT2Single(self, ts, projector, params, startY=0, endY=None, seed=0):
        """TomoReconstruction2.ADASIRT2Single (:1102-1181): osartIteration + endOfIteration
        with the dual drivers' stop rule."""
        endY = self.H if endY is None else endY
        self.completion = 0.0
        n = ts.getImageStackSize()

        def iteration(i):
            err = self.osartIteration(projector, ts, params, startY, endY, first_index(seed, i, n))
            projector.endOfIteration()
            return err

        return self._until_diverging(iteration, params.getNbIterations())


def order_shuffle(eulers, first: int) -> np.ndarray:
    """orderShuffleART with a given first index, through the engine's host code."""
    import ctypes as C
    e = np.ascontiguousarray(eulers, np.float64)
    out = np.zeros(e.shape[0], np.int32)
    _abi.check(_abi.load().tomo_order_shuffle(e.shape[0], _abi.ptr(e, C.c_double), int(first),
                                              _abi.ptr(out, C.c_int32)))
    return out


class ReconstructionParameters:
    """ReconstructionParameters (ReconstructionParameters.java:12-333)."""

    def __init__(self, width, height, depth):
        self.width, self.height, self.depth = width, height, depth
        self.reconstructionType = OSSART
        self.nbIterations = 0
        self.relaxationCoefficient = 1.0
        self.updateNb = 0
        self.positivityConstraint = False
        self.fista = False
        self.weightingRadius = float("nan")
        self.weightingType = _abi.WEIGHT_RADERMACHER
        self.rescaleData = True
        self.longObjectCompensation = False
        # TVM (AdvancedReconstructionParameters)
        self.tvmTheta, self.tvmG, self.tvmDt, self.tvmIterations = 25.0, 1.0, 0.1, 5
        self.regularizationWeight = 0.1
        # BgART and compressed sensing (AdvancedReconstructionParameters)
        self.bgartK, self.bgartMedian, self.bgartDarkBG = 0.0, True, True
        self.waveletPercentageOfZeros, self.waveletType, self.waveletDegree, self.waveletShift = 0.95, 3, 3.0, 0.0
        # volume storage precision (engine option; the reference stores float32)
        self.precision = _abi.PREC_FP32
        # shifts of the volume centre (ReconstructionParameters.getReconstructionCenterModifiers)
        self.reconstructionCenterModifiers = None

    @staticmethod
    def createOSSARTParameters(width, height, depth, nbIterations, relaxationCoefficient, updateNb):
        p = ReconstructionParameters(width, height, depth)
        p.reconstructionType = OSSART
        p.nbIterations = nbIterations
        p.relaxationCoefficient = relaxationCoefficient
        p.updateNb = updateNb
        return p

    @staticmethod
    def createWBPParameters(width, height, depth, weightingRadius, weightingType=_abi.WEIGHT_RADERMACHER):
        p = ReconstructionParameters(width, height, depth)
        radial = weightingType == _abi.WEIGHT_RADERMACHER
        p.reconstructionType = BP if (radial and (np.isnan(weightingRadius) or weightingRadius <= 0)) else WBP
        p.weightingRadius = weightingRadius
        p.weightingType = weightingType
        p.updateNb = 0
        p.nbIterations = 0
        p.relaxationCoefficient = float("nan")
        return p

    @staticmethod
    def createTVMParameters(width, height, depth, nbIterations, relaxationCoefficient, tvmTheta, tvmG, tvmDt,
                            tvmIterations):
        """AdvancedReconstructionParameters.createTVMParameters (AdvancedReconstructionParameters.java:122-134).
        TVMProjector3D.endOfIteration uses the regularisation weight (lambda) as dt
        (TVMProjector3D.java:152); pass lambda as tvmDt."""
        p = ReconstructionParameters(width, height, depth)
        p.reconstructionType = TVM
        p.nbIterations = nbIterations
        p.relaxationCoefficient = relaxationCoefficient
        p.tvmTheta, p.tvmG, p.tvmDt, p.tvmIterations = tvmTheta, tvmG, tvmDt, tvmIterations
        p.updateNb = 0
        return p

    @staticmethod
    def createBayesianParameters(width, height, depth, nbIterations, regularizationAlpha, regularizationWeight):
        """AdvancedReconstructionParameters.createBayesianParameters (:135-144): the
        relaxation coefficient carries alpha."""
        p = ReconstructionParameters(width, height, depth)
        p.reconstructionType = BAYESIAN
        p.nbIterations = nbIterations
        p.relaxationCoefficient = regularizationAlpha
        p.regularizationWeight = regularizationWeight
        p.updateNb = 0
        return p

    @staticmethod
    def createBgARTParameters(width, height, depth, nbIterations, relaxationCoefficient, updateNb, bgartK,
                              bgartMedian, bgartDarkBG):
        """AdvancedReconstructionParameters.createBgARTParameters (:145-156)."""
        p = ReconstructionParameters(width, height, depth)
        p.reconstructionType = BGART
        p.nbIterations = nbIterations
        p.relaxationCoefficient = relaxationCoefficient
        p.updateNb = updateNb
        p.bgartK, p.bgartMedian, p.bgartDarkBG = float(bgartK), bool(bgartMedian), bool(bgartDarkBG)
        return p

    @staticmethod
    def createCompressedSensingParameters(width, height, depth, nbIterations, relaxationCoefficient,
                                          waveletPercentageOfZeros, waveletType, waveletDegree, waveletShift):
        """AdvancedReconstructionParameters.createCompressedSensingParameters (:157-168)."""
        p = ReconstructionParameters(width, height, depth)
        p.reconstructionType = COMPRESSED_SENSING
        p.nbIterations = nbIterations
        p.relaxationCoefficient = relaxationCoefficient
        p.waveletPercentageOfZeros, p.waveletType = waveletPercentageOfZeros, waveletType
        p.waveletDegree, p.waveletShift = waveletDegree, waveletShift
        p.updateNb = 0
        return p

    def getRegularizationWeight(self):
        return self.regularizationWeight

    def getWidth(self):
        return self.width

    def getHeight(self):
        return self.height

    def getDepth(self):
        return self.depth

    def getReconstructionType(self):
        return self.reconstructionType

    def getReconstructionCenterModifiers(self):
        return self.reconstructionCenterModifiers

    def setReconstructionCenterModifiers(self, dx, dy, dz):
        self.reconstructionCenterModifiers = (float(dx), float(dy), float(dz))

    def getNbIterations(self):
        return self.nbIterations

    def getRelaxationCoefficient(self):
        return self.relaxationCoefficient

    def getUpdateNb(self):
        return self.updateNb

    def setPositivityConstraint(self, v):
        self.positivityConstraint = bool(v)

    def setFista(self, v):
        self.fista = bool(v)

    def setLongObjectCompensation(self, v):
        self.longObjectCompensation = bool(v)

    def setPrecision(self, v):
        """Volume storage: "fp32" (default), "bf16" or "fp16" (or a PREC_* value)."""
        self.precision = _abi.precision_code(v)

    def getProjector(self, ts, rec) -> VoxelProjector3D:
        """ReconstructionParameters.getProjector (ReconstructionParameters.java:313-333) and
        AdvancedReconstructionParameters.getProjector (AdvancedReconstructionParameters.java:171-221)."""
        from .projector import BayesianVoxelProjector3D, BgARTVoxelProjector3D, CompressedSensingProjector
        scale = ts.getWidth() / float(rec.getWidth()) if self.rescaleData else 1.0
        kind = self.reconstructionType
        if kind == COMPRESSED_SENSING:
            # CompressedSensingProjector keeps the projector defaults (no positivity / long object)
            proj = CompressedSensingProjector(ts, rec, None, self.waveletType, self.waveletDegree, self.waveletShift,
                                              self.waveletPercentageOfZeros, scale=scale, precision=self.precision)
            if self.fista:
                proj.setFista(True)
            return proj
        if kind == BAYESIAN:
            proj = BayesianVoxelProjector3D(ts, rec, None, positivity=self.positivityConstraint,
                                            long_object=self.longObjectCompensation, scale=scale,
                                            precision=self.precision)
            proj.setRegularizationAlpha(self.relaxationCoefficient)
            proj.setRegularizationLambda(self.regularizationWeight)
            return proj
        if kind == BGART:
            # BgARTVoxelProjector3D keeps the projector defaults (no positivity / long object)
            proj = BgARTVoxelProjector3D(ts, rec, None, self.bgartK, self.bgartDarkBG, self.bgartMedian, scale=scale,
                                         precision=self.precision)
            if self.fista:
                proj.setFista(True)
            return proj
        pos = self.positivityConstraint if kind in (OSSART, TVM) else False
        proj = VoxelProjector3D(ts, rec, None, positivity=pos, long_object=self.longObjectCompensation, scale=scale,
                                precision=self.precision)
        if self.reconstructionType == WBP:
            proj.setWeighting(self.weightingType, self.weightingRadius if self.weightingRadius == self.weightingRadius
                              else 0.0)
        if self.reconstructionType == TVM:
            proj.setTVM(self.tvmTheta, self.tvmG, self.tvmDt, self.tvmIterations)
        if self.fista:
            proj.setFista(True)
        return proj


def project_volume(volume: np.ndarray, tilt_angle_start=-60.0, tilt_angle_end=60.0, tilt_angle_increment=2.0,
                   center=None) -> tuple[np.ndarray, np.ndarray]:
    """Project_Volume (TomoJ_Base/.../plugins/Project_Volume.java:41-70): a tilt-series of
    the volume [D][H][W] at angles start, start + increment, ... <= end about the vertical
    axis, projections W x H, through VoxelProjector3D.  center = (cx, cy, cz) of the tilt
    axis in the volume (default (n - 1) / 2).  The reference sizes its angle array as
    (int)((end - start + 1) / increment), one short when the increment does not divide
    end - start + 1; every angle of the loop is kept here.  Returns (projections, angles)."""
    from .tiltseries import TiltSeries
    vol = np.ascontiguousarray(volume, np.float32)
    D, H, W = vol.shape
    angles = []
    a = float(tilt_angle_start)
    while a <= tilt_angle_end:
        angles.append(a)
        a += tilt_angle_increment
    angles = np.array(angles)
    ts = TiltSeries(np.zeros((angles.size, H, W), np.float32), angles)
    ts.setNormalize(False)  # the blank series is never compared with the projections
    rec = TomoReconstruction2(W, H, D, vol)
    if center is not None:
        rec.setCenter(*center)
    proj = VoxelProjector3D(ts, rec)
    try:
        for i in range(angles.size):
            proj.addProjection(i)
        proj.project(0, H)
        return np.array([proj.getProjection(i) for i in range(angles.size)], np.float32), angles
    finally:
        proj.close()


class ReconstructionThreadManager:
    """ReconstructionThreadManager (TomoJ_Base/.../tomography/ReconstructionThreadManager.java):
    the reference's driver from a ReconstructionParameters to a reconstruction.
    reconstruct() makes or reuses the volume (createRec2, :169-196: reused when the sizes
    match, so further calls add iterations) and runs doCPUrec (:218-255): the parameters'
    projector, then WBP for BP / WBP, OSSART for OSSART, regularization for the other
    types.  The run is synchronous (the reference runs it on a worker thread behind a
    progress window).  The debugging error volumes (saveErrorVolume) are not provided.
    The projector stays open for getProjection until the next reconstruction or close()."""

    def __init__(self, parentWindow=None, ts=None, other=None):
        self.parentWindow = parentWindow if other is None else other.parentWindow
        self.ts = ts
        self.rec2 = None
        self.projector = None
        self.errors = None
        self.numberofsteps = 0.0
        self._thprojs = None
        self.seed = 0  # orderShuffleART's first-index seed

    def reconstruct(self, parameters, showProgressWindow=False):
        self.createRec2(parameters)
        self.performReconstruction(parameters, showProgressWindow)
        return self.rec2

    def createRec2(self, parameters):
        self._thprojs = None
        w, h, d = parameters.getWidth(), parameters.getHeight(), parameters.getDepth()
        r = self.rec2
        if r is None or (r.getWidth(), r.getHeight(), r.getSizez()) != (w, h, d):
            self.close()
            self.rec2 = TomoReconstruction2(w, h, d)
            mod = parameters.getReconstructionCenterModifiers()
            if mod is not None:
                c = self.rec2.centers()
                self.rec2.setCenter(c[0] + mod[0], c[1] + mod[1], c[2] + mod[2])

    def performReconstruction(self, parameters, showProgressWindow=False):
        self._thprojs = None
        self.rec2.completion = 0.0
        n = self.ts.getImageStackSize()
        self.numberofsteps = n * parameters.getNbIterations() * 2 if parameters.getReconstructionType() > WBP else n
        self.errors = self.doCPUrec(parameters, False, False)

    def doRec(self, parameters, saveErrorVol=False, saveForAll=False, time=None):
        return self.doCPUrec(parameters, saveErrorVol, saveForAll)

    def doCPUrec(self, params, saveError=False, saveForAll=False):
        if saveError or saveForAll:
            raise NotImplementedError("the debugging error volume is not provided")
        self.close()
        self.projector = params.getProjector(self.ts, self.rec2)
        kind = params.getReconstructionType()
        if kind in (BP, WBP):
            self.rec2.WBP(self.ts, self.projector, params, 0, self.rec2.getHeight())
            return None
        if kind == OSSART:
            return self.rec2.OSSART(self.ts, self.projector, params, 0, self.rec2.getHeight(), seed=self.seed)
        return self.rec2.regularization(self.ts, self.projector, params, 0, self.rec2.getHeight(), seed=self.seed)

    def getProjection(self, index: int) -> np.ndarray:
        """The projection of the reconstruction at tilt `index` (cached, :257-270)."""
        if self._thprojs is None:
            self._thprojs = {}
        if index not in self._thprojs:
            p = self.projector
            p.addProjection(index)
            p.project(0, self.rec2.getHeight())
            self._thprojs[index] = p.getProjection(0).copy()
            p.clearAllProjections()
        return self._thprojs[index]

    def close(self):
        if self.projector is not None:
            self.projector.close()
            self.projector = None

    def setRec2(self, rec2):
        self._thprojs = None
        self.close()
        self.rec2 = rec2

    def resetRec2(self):
        self.setRec2(None)

    def getRec2(self):
        return self.rec2

    def setTiltSeries(self, ts):
        self.ts = ts

    def getNumberofsteps(self):
        return self.numberofsteps

    def getReconstructionDissimilarities(self):
        return self.errors

    def getCompletion(self):
        if self.rec2 is not None and self.numberofsteps:
            return self.rec2.completion / self.numberofsteps * 100
        return -123456789
