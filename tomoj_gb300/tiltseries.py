"""Host-side mirror of TomoJ's TiltSeries and AffineAlignment for the fields
the projection path reads (TomoJ_Base/.../tomography/TiltSeries.java,
TomoJ_Base/.../align/AffineAlignment.java).

Transforms are java.awt.geom.AffineTransform flat matrices
{m00, m10, m01, m11, m02, m12}; composition follows AffineTransform.concatenate
(T <- T * other).  Euler matrices follow MatrixUtils.eulerAngles2Matrix with
the tilt axis made vertical (AffineAlignment.getEulerMatrix, AffineAlignment.java:382-395).
"""
from __future__ import annotations

import math

import numpy as np

FILL_NONE, FILL_AVG, FILL_NAN = 0, 1, 2
IDENTITY = (1.0, 0.0, 0.0, 1.0, 0.0, 0.0)


def _mat(T):
    m00, m10, m01, m11, m02, m12 = T
    return np.array([[m00, m01, m02], [m10, m11, m12], [0.0, 0.0, 1.0]])


def _flat(M):
    return (M[0, 0], M[1, 0], M[0, 1], M[1, 1], M[0, 2], M[1, 2])


def concatenate(T, other):
    """AffineTransform.concatenate: returns T * other."""
    return _flat(_mat(T) @ _mat(other))


def rotation(theta_rad):
    c, s = math.cos(theta_rad), math.sin(theta_rad)
    if s == 0.0 and c == 1.0:
        return IDENTITY
    return (c, s, -s, c, 0.0, 0.0)


def inverse(T):
    """AffineTransform.createInverse (general case)."""
    m00, m10, m01, m11, m02, m12 = T
    det = m00 * m11 - m01 * m10
    if abs(det) <= 5e-324:
        raise ValueError("transform is not invertible")
    return (m11 / det, -m10 / det, -m01 / det, m00 / det, (m01 * m12 - m11 * m02) / det,
            (m10 * m02 - m00 * m12) / det)


def euler_angles_to_matrix(phi, theta, psi):
    """MatrixUtils.eulerAngles2Matrix (Utility/.../MatrixUtils.java:226-251), degrees."""
    phi, theta, psi = math.radians(phi), math.radians(theta), math.radians(psi)
    cphi, sphi, ct, st = math.cos(phi), math.sin(phi), math.cos(theta), math.sin(theta)
    cpsi, spsi = math.cos(psi), math.sin(psi)
    return np.array([[cpsi * ct * cphi - spsi * sphi, cpsi * ct * sphi + spsi * cphi, -cpsi * st],
                     [-spsi * ct * cphi - cpsi * sphi, -spsi * ct * sphi + cpsi * cphi, spsi * st],
                     [st * cphi, st * sphi, ct]])


class AffineAlignment:
    """Per-tilt 2-D transforms (AffineAlignment.java:13-303)."""

    def __init__(self, ts: "TiltSeries", combine: bool = True):
        self.ts = ts
        n = ts.getImageStackSize()
        self.transforms = [IDENTITY] * n
        self.zeroT = IDENTITY
        self.combine = combine
        self.tiltaxis = 0.0
        self.tiltAxisVertical = True
        self.expand = False

    def setTransform(self, index, T):
        self.transforms[index] = tuple(float(v) for v in T)

    def setCombineTransforms(self, value: bool):
        self.combine = bool(value)

    def setZeroTransform(self, T):
        self.zeroT = tuple(float(v) for v in T)

    def setTiltAxis(self, tiltaxis: float):
        self.tiltaxis = float(tiltaxis)

    def getInverseTransform(self, index):
        return inverse(self.transforms[index])

    def getTransform(self, index, combine=None):
        """AffineAlignment.getTransform(index, combineTransforms) (AffineAlignment.java:269-303)."""
        combine = self.combine if combine is None else combine
        T = IDENTITY
        if self.tiltAxisVertical:
            T = concatenate(T, rotation(math.radians(-self.tiltaxis)))
        if combine:
            z = self.ts.zeroindex
            T = concatenate(T, self.zeroT)
            if index < z:
                for i in range(z - 1, index - 1, -1):
                    T = concatenate(T, self.transforms[i])
            elif index > z:
                for i in range(z, index):
                    T = concatenate(T, self.getInverseTransform(i))
        else:
            T = concatenate(T, self.transforms[index])
        if self.expand:
            f = 1.0 / math.cos(math.radians(self.ts.getTiltAngle(index)))
            E = concatenate(concatenate(rotation(math.radians(self.tiltaxis)), (f, 0.0, 0.0, 1.0, 0.0, 0.0)),
                            rotation(-math.radians(self.tiltaxis)))
            T = _flat(_mat(E) @ _mat(T))
        return T

    def addTransform(self, index, T):
        """AffineAlignment.addTransform (AffineAlignment.java:97-102): transforms[i] <- transforms[i] * T."""
        self.transforms[index] = concatenate(self.transforms[index], tuple(float(v) for v in T))

    def addToZeroTransform(self, T):
        """AffineAlignment.addToZeroTransform (:118-124)."""
        self.zeroT = concatenate(self.zeroT, tuple(float(v) for v in T))

    def getZeroTransform(self):
        return self.zeroT

    def setTiltAxisVertical(self, value: bool):
        self.tiltAxisVertical = bool(value)

    def convertTolocalTransform(self):
        """AffineAlignment.convertTolocalTransform (:337-380): final (per-image) transforms
        become the zero-tilt transform plus transforms between consecutive images, going
        forward from the zero tilt with getTransform(i - 1) of the state built so far, and
        backward with the inverse of getTransform(i + 1)."""
        self.combine = True
        old = list(self.transforms)
        self.transforms = [IDENTITY] * len(old)
        z = self.ts.zeroindex
        self.setZeroTransform(old[z])
        for i in range(z + 1, len(old)):
            T = concatenate(inverse(old[i]), self.getTransform(i - 1))
            self.transforms[i - 1] = T
        for i in range(z - 1, -1, -1):
            T0 = inverse(self.getTransform(i + 1))
            self.transforms[i] = concatenate(T0, old[i])  # T.preConcatenate(T0) = T0 * T

    def loadFromFile(self, path: str, binning: float = 1.0, finalTransforms: bool = False,
                     combineWithExisting: bool = False, tiff2mrc: bool = False):
        """AffineAlignment.loadFromFile (:420-507): IMOD .xf / .prexg (final transforms
        a11 a12 a21 a22 dx dy per line, read as AffineTransform's flat matrix, shifts
        times binning, all negated for tiff2mrc stacks, then converted to local
        transforms), IMOD .prexf (consecutive transforms, shifts negated, the first
        line belongs to the last image), or a TomoJ csv / txt file (angle, tilt axis and
        six matrix values per image; the zero-tilt transform on the last line unless
        the transforms are final)."""
        n = self.ts.getImageStackSize()

        def lines():
            with open(path) as f:
                for raw in f:
                    yield raw

        it = lines()

        def next_data(strip=True):
            line = next(it)
            line = line.strip() if strip else line.rstrip("\n")
            while line.startswith(";") or line.startswith("#"):
                line = next(it)
                line = line.strip() if strip else line.rstrip("\n")
            return line

        if path.endswith(".xf") or path.endswith(".prexg"):
            for i in range(n):
                words = next_data().split()
                tmp = []
                for j in range(6):
                    v = float(words[j])
                    if j > 3:
                        v *= binning
                    if tiff2mrc:
                        v = -v
                    tmp.append(v)
                if combineWithExisting:
                    self.addTransform(i, tmp)
                else:
                    self.setTransform(i, tmp)
            self.convertTolocalTransform()
        elif path.endswith(".prexf"):
            for i in range(n):
                words = next_data().split()
                tmp = [float(words[0]), float(words[1]), float(words[2]), float(words[3]),
                       -float(words[4]) * binning,
                       float(words[5]) * binning if finalTransforms else -float(words[5]) * binning]
                self.setTransform(n - 1 if i == 0 else i - 1, tmp)
        else:
            import re
            sep = ";" if path.lower().endswith("csv") else None
            split = (lambda ln: ln.split(";")) if sep else (lambda ln: re.split(r"\s+", ln))
            for i in range(n):
                words = split(next_data(strip=False))
                self.ts.setTiltAngle(i, float(words[0]))
                self.ts.setTiltAxis(float(words[1]))
                tmp = [float(words[j + 2]) * (binning if j > 3 else 1.0) for j in range(6)]
                if combineWithExisting:
                    self.addTransform(i, tmp)
                else:
                    self.setTransform(i, tmp)
            if finalTransforms:
                self.convertTolocalTransform()
            else:
                words = split(next(it).rstrip("\n"))
                tmp = [float(words[j]) * (binning if j > 3 else 1.0) for j in range(6)]
                if combineWithExisting:
                    self.addToZeroTransform(tmp)
                else:
                    self.setZeroTransform(tmp)

    def saveToFile(self, path: str, finalTransforms: bool = False):
        """AffineAlignment.saveToFile (:509-539): angle, tilt axis and the six matrix
        values per image (';' for .csv, tab otherwise, each value followed by the
        separator), written with the tilt axis not put vertical; then the zero-tilt
        transform unless the transforms are final."""
        sep = ";" if path.lower().endswith("csv") else "\t"
        vertical = self.tiltAxisVertical
        self.tiltAxisVertical = False
        try:
            with open(path, "w") as f:
                for i in range(self.ts.getImageStackSize()):
                    f.write(f"{_jd(self.ts.getTiltAngle(i))}{sep}{_jd(self.tiltaxis)}{sep}")
                    t = self.getTransform(i, True) if finalTransforms else self.getTransform(i, False)
                    for v in t:
                        f.write(f"{_jd(v)}{sep}")
                    f.write("\n")
                if not finalTransforms:
                    for v in self.zeroT:
                        f.write(f"{_jd(v)}{sep}")
                f.write("\n")
        finally:
            self.tiltAxisVertical = vertical

    def getEulerMatrix(self, index):
        ta = 0.0 if self.tiltAxisVertical else self.tiltaxis
        return euler_angles_to_matrix(ta, self.ts.getTiltAngle(index), -ta)


def _jd(v: float) -> str:
    """Java's Double.toString for the values an alignment file holds (repr, with
    Java's forms of integral values and of exponents)."""
    v = float(v)
    if v != v:
        return "NaN"
    if v in (float("inf"), float("-inf")):
        return "Infinity" if v > 0 else "-Infinity"
    a = abs(v)
    if a == 0 or 1e-3 <= a < 1e7:
        r = repr(v)
        if "e" in r or "E" in r:  # repr switches to exponents earlier than Java
            r = f"{v:.17f}".rstrip("0")
            if r.endswith("."):
                r += "0"
        return r if "." in r else r + ".0"
    # shortest round-trip mantissa
    m, e = f"{v:.16e}".split("e")
    for digits in range(1, 17):
        cand = f"{v:.{digits}e}"
        if float(cand) == v:
            m, e = cand.split("e")
            break
    if "." not in m:
        m += ".0"
    return f"{m}E{int(e)}"


class TiltSeries:
    """Tilt-series container: unaligned projections float32 (N, h, w) and angles in degrees."""

    def __init__(self, pixels: np.ndarray, tilt_angles):
        pixels = np.ascontiguousarray(pixels, np.float32)
        if pixels.ndim != 3:
            raise ValueError("pixels must be (N, h, w)")
        self.pixels = pixels
        self.tiltAngles = np.asarray(tilt_angles, np.float64).copy()
        if self.tiltAngles.size != pixels.shape[0]:
            raise ValueError("one tilt angle per projection is required")
        # TiltSeries.firstInit (TiltSeries.java:123-159)
        self.normalize = True
        self.fill = FILL_AVG
        self.zeroindex = int(np.argmin(np.abs(self.tiltAngles))) if self.tiltAngles.size else 0
        # zeroindex keeps the first minimum of |angle|, as the reference's strict '<' scan does
        self.alignment = AffineAlignment(self, True)
        self.stats = None

    def setTiltAngle(self, index: int, angleDeg: float):
        """TiltSeries.setTiltAngle / updateZeroIndex (TiltSeries.java:366-392): the zero
        index moves only to a strictly smaller |angle| than |angle[0]|."""
        self.tiltAngles[index] = float(angleDeg)
        tmp = abs(self.tiltAngles[0])
        for i in range(self.tiltAngles.size):
            if abs(self.tiltAngles[i]) < tmp:
                tmp = abs(self.tiltAngles[i])
                self.zeroindex = i

    def setTiltAxis(self, angleDeg: float):
        """TiltSeries.setTiltAxis (:1440-1447): also puts the tilt axis vertical."""
        self.alignment.setTiltAxis(angleDeg)
        self.alignment.setTiltAxisVertical(True)

    def getTiltAxis(self) -> float:
        return self.alignment.tiltaxis

    # --- TiltSeries accessors used by the projectors ---------------------------------
    def getWidth(self) -> int:
        return int(self.pixels.shape[2])

    def getHeight(self) -> int:
        return int(self.pixels.shape[1])

    def getImageStackSize(self) -> int:
        return int(self.pixels.shape[0])

    def getTiltAngle(self, i) -> float:
        return float(self.tiltAngles[i])

    def getTiltAngles(self):
        return self.tiltAngles

    def getCenterX(self):
        return (self.getWidth() - 1.0) / 2

    def getCenterY(self):
        return (self.getHeight() - 1.0) / 2

    def getProjectionCenterX(self):
        return (self.getWidth() - 1) / 2.0

    def getProjectionCenterY(self):
        return (self.getHeight() - 1) / 2.0

    def setNormalize(self, value: bool):
        self.normalize = bool(value)

    def isNormalized(self) -> bool:
        return self.normalize

    def setFillType(self, fill: int):
        self.fill = int(fill)

    def getFillType(self) -> int:
        return self.fill

    def getAlignment(self) -> AffineAlignment:
        return self.alignment

    def getOriginalPixels(self, i):
        return self.pixels[i]

    def transforms(self) -> np.ndarray:
        return np.array([self.alignment.getTransform(i) for i in range(self.getImageStackSize())], np.float64)

    def eulers(self) -> np.ndarray:
        return np.array([self.alignment.getEulerMatrix(i) for i in range(self.getImageStackSize())], np.float64)

    def setStatistics(self, stats):
        """Per-tilt {mean, stdDev} used by normalisation and FILL_AVG."""
        self.stats = np.asarray(stats, np.float64).reshape(-1, 2)

    def getImageStatistics(self, i):
        """Mean / stdDev over the tilt-dependent central region (TiltSeries.java:809-835).

        The reference measures ImageJ statistics inside a PolygonRoi; the polygon is
        rasterised here with an even-odd pixel-centre test (ImageJ's own rasteriser
        is not available, so this is unpinned)."""
        if self.stats is not None:
            return tuple(self.stats[i])
        w, h = self.getWidth(), self.getHeight()
        cx, cy = self.getCenterX(), self.getCenterY()
        roisx = int(max(round(w * math.cos(math.radians(self.getTiltAngle(i)))), 10))
        x0 = (w - roisx) // 2 - cx
        pts = np.array([[x0, -cy], [x0 + roisx, -cy], [x0 + roisx, h - cy], [x0, h - cy]])
        m00, m10, m01, m11, m02, m12 = self.alignment.getTransform(i)
        xs = [int(m00 * x + m01 * y + m02 + cx) for x, y in pts]
        ys = [int(m10 * x + m11 * y + m12 + cy) for x, y in pts]
        yy, xx = np.mgrid[0:h, 0:w] + 0.5
        inside = np.zeros((h, w), bool)
        n = len(xs)
        for k in range(n):
            xa, ya, xb, yb = xs[k], ys[k], xs[(k + 1) % n], ys[(k + 1) % n]
            cond = (ya > yy) != (yb > yy)
            with np.errstate(divide="ignore", invalid="ignore"):
                xint = xa + (yy - ya) * (xb - xa) / np.where(yb == ya, 1, yb - ya)
            inside ^= cond & (xx < xint)
        vals = self.pixels[i][inside].astype(np.float64)
        if vals.size == 0:
            vals = self.pixels[i].astype(np.float64).ravel()
        return float(vals.mean()), float(vals.std(ddof=1) if vals.size > 1 else 0.0)

    def statistics(self) -> np.ndarray:
        return np.array([self.getImageStatistics(i) for i in range(self.getImageStackSize())], np.float64)
