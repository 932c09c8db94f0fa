"""Host-side logic of the engine without a GPU: the C-ABI library loads and exports
every symbol include/tomoj_gb300.h declares, the ctypes binding covers them, the
host code (ordering, seeded first index, tables' helpers) agrees with the oracle,
and the reference-interface mirror (TiltSeries / AffineAlignment / parameters)
behaves like the reference."""
from __future__ import annotations

import ctypes as C
import math
import os
import re

import numpy as np
import pytest

from oracle import oracle as O
from tomoj_gb300 import _abi, phantom as P
from tomoj_gb300.tiltseries import (IDENTITY, AffineAlignment, TiltSeries, concatenate, euler_angles_to_matrix,
                                    inverse)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "tomoj_gb300.h")


def header_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(tomo_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(engine):
    syms = header_symbols()
    assert len(syms) > 30
    for name in syms:
        assert hasattr(engine, name), name


def test_binding_covers_the_header(engine):
    assert sorted(_abi.SIGNATURES) == header_symbols()
    assert engine.tomo_abi_version() == 1


def test_no_device_fails_loudly_without_fallback(engine):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    g = _abi.make_geom(8, 2, 8, 8, 2, 3)
    p = _abi.make_params()
    h = C.c_void_p()
    rc = engine.tomo_create(C.byref(g), C.byref(p), C.byref(h))
    assert rc == -2 and not h.value  # TOMO_ERR_CUDA: no device, nothing created


def test_invalid_arguments_are_rejected(engine):
    g = _abi.make_geom(0, 2, 8, 8, 2, 3)
    h = C.c_void_p()
    assert engine.tomo_create(C.byref(g), None, C.byref(h)) == -1
    e = np.zeros((3, 9))
    out = np.zeros(3, np.int32)
    assert engine.tomo_order_shuffle(3, _abi.ptr(e, C.c_double), 5, _abi.ptr(out, C.c_int32)) == -1
    assert b"first index" in engine.tomo_last_error()
    # a thread's 16 voxels are addressed with 32-bit offsets: 16 * W * H must stay below 2^32
    g = _abi.make_geom(65535, 4097, 8, 64, 8, 3)
    assert engine.tomo_create(C.byref(g), None, C.byref(h)) == _abi.ERR_UNSUPPORTED
    assert b"2^28" in engine.tomo_last_error()


@pytest.mark.parametrize("first", [0, 7, 30, 60])
def test_engine_ordering_matches_oracle(engine, oracle_lib, first):
    from tomoj_gb300.reconstruction import order_shuffle
    eul = np.array([O.euler_tilt_y(a) for a in np.arange(-60, 61, 2.0)])
    assert np.array_equal(order_shuffle(eul, first), O.order_shuffle(eul, first))


def test_first_index_is_seeded_and_in_range(engine):
    a = [engine.tomo_first_index(1234, it, 61) for it in range(50)]
    b = [engine.tomo_first_index(1234, it, 61) for it in range(50)]
    c = [engine.tomo_first_index(1235, it, 61) for it in range(50)]
    assert a == b and a != c and all(0 <= v < 61 for v in a)
    assert len(set(a)) > 10


def test_euler_matrix_matches_oracle(oracle_lib):
    for th in (-70.0, -1.0, 0.0, 33.3, 60.0):
        assert np.allclose(euler_angles_to_matrix(0.0, th, -0.0), O.euler_tilt_y(th), atol=1e-15)
    assert np.allclose(euler_angles_to_matrix(12.0, 40.0, -7.0), O.euler(12.0, 40.0, -7.0), atol=1e-15)


def test_affine_transform_composition_and_inverse():
    T = (math.cos(0.3), math.sin(0.3), -math.sin(0.3), math.cos(0.3), 4.0, -1.5)
    I = concatenate(T, inverse(T))
    assert np.allclose(I, IDENTITY, atol=1e-12)
    S = (2.0, 0.0, 0.0, 1.0, 0.0, 0.0)
    TS = concatenate(T, S)  # AffineTransform.concatenate: apply S first
    x, y = 1.0, 2.0
    sx, sy = 2.0 * x, y
    m00, m10, m01, m11, m02, m12 = TS
    tx = T[0] * sx + T[2] * sy + T[4]
    assert math.isclose(m00 * x + m01 * y + m02, tx, rel_tol=1e-12)


def test_combined_transforms_chain_from_zero_tilt():
    """AffineAlignment.getTransform with combineTransforms (AffineAlignment.java:275-288):
    images before the zero tilt concatenate the forward transforms, after it the inverses."""
    px = np.zeros((5, 4, 4), np.float32)
    ts = TiltSeries(px, [-20, -10, 0, 10, 20])
    al = ts.getAlignment()
    shifts = [(1.0, 0.0), (2.0, 0.0), (0.0, 0.0), (0.0, 3.0), (0.0, 4.0)]
    for i, (sx, sy) in enumerate(shifts):
        al.setTransform(i, (1.0, 0.0, 0.0, 1.0, sx, sy))
    assert ts.zeroindex == 2
    assert np.allclose(al.getTransform(0)[4:], [3.0, 0.0])      # T1 * T0
    assert np.allclose(al.getTransform(3)[4:], [0.0, 0.0])      # inv(T2)
    assert np.allclose(al.getTransform(4)[4:], [0.0, -3.0])     # inv(T2) * inv(T3)
    al.setCombineTransforms(False)
    assert np.allclose(al.getTransform(4)[4:], [0.0, 4.0])


def test_tiltseries_defaults_follow_reference():
    ts = TiltSeries(np.zeros((3, 4, 6), np.float32), [-5.0, 0.0, 5.0])
    assert ts.isNormalized() and ts.getFillType() == 1  # TiltSeries.firstInit: normalize, FILL_AVG
    assert ts.getCenterX() == 2.5 and ts.getProjectionCenterY() == 1.5
    assert isinstance(ts.getAlignment(), AffineAlignment)


def test_phantom_and_schemes_are_seeded():
    a = P.ellipsoid_phantom(16, 4, 12, 5, 7)
    b = P.ellipsoid_phantom(16, 4, 12, 5, 7)
    assert np.array_equal(a, b) and a.max() > 0 and a.min() == 0
    s = P.saxton_tilts(60.0, 61)
    assert len(s) == 61 and np.allclose(s, -s[::-1]) and abs(s[-1] - 60.0) < 2.0
    d = P.dose_symmetric_tilts(60.0, 61)
    assert d[0] == 0 and sorted(np.round(d, 6)) == sorted(np.round(np.linspace(-60, 60, 61), 6))
    u = P.uniform_tilts(-60, 60, 2)
    assert len(u) == 61


def test_unalign_is_inverse_of_oracle_alignment(oracle_lib):
    img = P.ellipsoid_phantom(64, 48, 1, 6, 3)[0] + np.float32(0.5)
    T = P.misalignment(1, 5, 3.0, 1.0)[0]
    back = O.align(P.unalign(img, T), T, fill=O.FILL_NAN)
    inner = (slice(8, -8), slice(8, -8))
    # two bilinear resamples of a piecewise-constant image: small mean error
    assert np.nanmean(np.abs(back[inner] - img[inner])) < 0.02
    shift = np.array([1.0, 0.0, 0.0, 1.0, 2.0, 1.0])  # integer shifts round-trip exactly
    back = O.align(P.unalign(img, shift), shift, fill=O.FILL_NAN)
    assert np.array_equal(back[inner], img[inner])


def test_reconstruction_type_codes_follow_the_reference():
    # ReconstructionParameters.java:13-15, AdvancedReconstructionParameters.java:10-13
    from tomoj_gb300 import reconstruction as R
    assert (R.BP, R.WBP, R.OSSART, R.TVM, R.BAYESIAN, R.COMPRESSED_SENSING, R.BGART) == (0, 1, 2, 3, 4, 5, 6)


def test_advanced_parameter_factories_fill_their_fields():
    from tomoj_gb300 import reconstruction as R
    params = R.ReconstructionParameters.createCompressedSensingParameters(8, 2, 8, 2, 1.0, 0.9, 0, 2.0, 0.25)
    assert params.reconstructionType == R.COMPRESSED_SENSING and params.updateNb == 0
    assert (params.waveletPercentageOfZeros, params.waveletType, params.waveletDegree, params.waveletShift) == \
        (0.9, 0, 2.0, 0.25)
    p = R.ReconstructionParameters.createBgARTParameters(8, 2, 8, 3, 0.5, 2, 1.5, False, True)
    assert (p.reconstructionType, p.bgartK, p.bgartMedian, p.bgartDarkBG, p.updateNb) == (R.BGART, 1.5, False, True, 2)
    b = R.ReconstructionParameters.createBayesianParameters(8, 2, 8, 4, 0.3, 0.02)
    assert (b.reconstructionType, b.relaxationCoefficient, b.getRegularizationWeight()) == (R.BAYESIAN, 0.3, 0.02)
