"""Parity of the CUDA type-1 NUFFT (plan API and FINUFFT-compatible drop-ins) with the FP64
direct-sum oracle.  Tolerances: the requested eps for FP64 (bound 5*eps on the relative l2
error) and for FP32 1e-4, 2e-5 and 3e-6 at eps 1e-5, 1e-6 and 1e-7 (kernel widths 6, 7, 8)."""
import ctypes as C

import numpy as np
import pytest

import oracle
from helpers import plan_type1, rel_l2
from mp_tools_gb300 import _lib

pytestmark = pytest.mark.gpu


def _pts(rng, n, dim, span=np.pi):
    xs = [rng.uniform(-span, span, n) for _ in range(dim)]
    c = rng.normal(size=n) + 1j * rng.normal(size=n)
    return xs, c


CASES = [(_lib.FP64, 1e-9, 5e-9), (_lib.FP64, 1e-12, 5e-12), (_lib.FP32, 1e-5, 1e-4),
         (_lib.FP32, 1e-6, 2e-5), (_lib.FP32, 1e-7, 3e-6)]


@pytest.mark.parametrize("prec,eps,tol", CASES)
@pytest.mark.parametrize("iflag", [-1, 1])
def test_plan_2d_vs_direct(cuda, prec, eps, tol, iflag):
    rng = np.random.default_rng(10 + iflag)
    (x, y), c = _pts(rng, 4000, 2, span=3 * np.pi)
    ms, mt = 50, 37
    got = plan_type1(cuda, 2, (ms, mt), x, y, None, c, iflag, eps, prec)[0]
    ref = oracle.dirft2d1(x, y, c, iflag, ms, mt)
    assert rel_l2(got, ref) < tol


@pytest.mark.parametrize("prec,eps,tol", CASES)
@pytest.mark.parametrize("iflag", [-1, 1])
def test_plan_3d_vs_direct(cuda, prec, eps, tol, iflag):
    rng = np.random.default_rng(20 + iflag)
    (x, y, z), c = _pts(rng, 3000, 3)
    modes = (20, 17, 12)
    got = plan_type1(cuda, 3, modes, x, y, z, c, iflag, eps, prec)[0]
    ref = oracle.dirft3d1(x, y, z, c, iflag, *modes)
    assert rel_l2(got, ref) < tol


def test_plan_many_transforms_share_points(cuda):
    rng = np.random.default_rng(30)
    (x, y, z), _ = _pts(rng, 1500, 3)
    c = rng.normal(size=(3, 1500)) + 1j * rng.normal(size=(3, 1500))
    got = plan_type1(cuda, 3, (16, 16, 16), x, y, z, c.ravel(), -1, 1e-9, _lib.FP64, ntrans=3)
    for t in range(3):
        ref = oracle.dirft3d1(x, y, z, c[t], -1, 16, 16, 16)
        assert rel_l2(got[t], ref) < 5e-9


def test_plan_clustered_points_and_tile_edges(cuda):
    # many points in one tile, points on tile boundaries and at the periodic seam
    rng = np.random.default_rng(31)
    n = 5000
    x = np.concatenate([rng.normal(0.0, 1e-3, n // 2), np.full(n // 4, -np.pi), np.full(n - n // 2 - n // 4, np.pi * (1 - 1e-12))])
    y = np.concatenate([rng.normal(0.0, 1e-3, n // 2), rng.uniform(-np.pi, np.pi, n - n // 2)])
    z = rng.uniform(-np.pi, np.pi, n)
    c = rng.normal(size=n) + 1j * rng.normal(size=n)
    got = plan_type1(cuda, 3, (24, 24, 24), x, y, z, c, -1, 1e-9, _lib.FP64)[0]
    ref = oracle.dirft3d1(x, y, z, c, -1, 24, 24, 24)
    assert rel_l2(got, ref) < 5e-9


@pytest.mark.parametrize("modes", [(1, 1), (2, 1), (1, 7), (3, 5)])
def test_plan_tiny_mode_grids(cuda, modes):
    rng = np.random.default_rng(32)
    (x, y), c = _pts(rng, 200, 2)
    got = plan_type1(cuda, 2, modes, x, y, None, c, -1, 1e-10, _lib.FP64)[0]
    ref = oracle.dirft2d1(x, y, c, -1, *modes)
    assert rel_l2(got, ref) < 1e-9


def test_plan_no_points_gives_zeros(cuda):
    got = plan_type1(cuda, 2, (8, 6), np.zeros(0), np.zeros(0), None, np.zeros(0, complex), -1, 1e-6,
                     _lib.FP64)
    assert np.all(got == 0)


# ------------------------------------------------------------------ FINUFFT-compatible ABI
def _dp(a):
    return a.ctypes.data_as(C.c_void_p)


def test_fortran_finufft2d1_matches_oracle(lib):
    """The call mp_sqom makes (mp_sqom56.f90:1148): everything by reference, NULL opts,
    complex(8) arrays, fk(n_qx, n_qy) column-major, ier out."""
    rng = np.random.default_rng(40)
    n = 20000
    x, y = rng.uniform(-np.pi, np.pi, (2, n))
    c = np.exp(-1j * rng.uniform(0, 2 * np.pi, n))
    ms, mt = 160, 160
    fk = np.zeros(ms * mt, np.complex128)
    nj = C.c_int64(n)
    iflag = C.c_int(-1)
    eps = C.c_double(1e-6)
    m1, m2 = C.c_int64(ms), C.c_int64(mt)
    ier = C.c_int(-99)
    lib.finufft2d1_(C.byref(nj), _dp(x), _dp(y), _dp(c), C.byref(iflag), C.byref(eps), C.byref(m1),
                    C.byref(m2), _dp(fk), None, C.byref(ier))
    assert ier.value == 0
    ref = oracle.dirft2d1(x, y, c, -1, ms, mt)
    assert rel_l2(fk.reshape(mt, ms), ref) < 5e-6


def test_c_finufft3d1_and_float_variants(lib):
    rng = np.random.default_rng(41)
    n = 3000
    x, y, z = rng.uniform(-np.pi, np.pi, (3, n))
    c = rng.normal(size=n) + 1j * rng.normal(size=n)
    m = (18, 14, 10)
    ref = oracle.dirft3d1(x, y, z, c, 1, *m)
    fk = np.zeros(np.prod(m), np.complex128)
    rc = lib.finufft3d1(n, _dp(x), _dp(y), _dp(z), _dp(c), 1, 1e-10, *m, _dp(fk), None)
    assert rc == 0 and rel_l2(fk.reshape(m[::-1]), ref) < 5e-10
    xf, yf, zf = (a.astype(np.float32) for a in (x, y, z))
    cf = c.astype(np.complex64)
    fkf = np.zeros(np.prod(m), np.complex64)
    rc = lib.finufftf3d1(n, _dp(xf), _dp(yf), _dp(zf), _dp(cf), 1, C.c_float(1e-6), *m, _dp(fkf), None)
    ref32 = oracle.dirft3d1(xf, yf, zf, cf, 1, *m)
    assert rc == 0 and rel_l2(fkf.reshape(m[::-1]), ref32) < 2e-5
    fk2 = np.zeros(m[0] * m[1], np.complex64)
    rc = lib.finufftf2d1(n, _dp(xf), _dp(yf), _dp(cf), -1, C.c_float(1e-6), m[0], m[1], _dp(fk2), None)
    ref2 = oracle.dirft2d1(xf, yf, cf, -1, m[0], m[1])
    assert rc == 0 and rel_l2(fk2.reshape(m[1], m[0]), ref2) < 2e-5


def test_3d_equals_stack_of_z_phased_2d_calls(lib):
    """mp_sql's construction (mp_sql56.f90:1106-1131): slice kz of the 3D transform equals a
    finufft2d1 call with strengths exp(-i kz z)."""
    rng = np.random.default_rng(42)
    n = 2000
    x, y, z = rng.uniform(-np.pi, np.pi, (3, n))
    m = (16, 12, 9)
    f3 = np.zeros(np.prod(m), np.complex128)
    assert lib.finufft3d1(n, _dp(x), _dp(y), _dp(z), _dp(np.ones(n, complex)), -1, 1e-11, *m, _dp(f3), None) == 0
    f3 = f3.reshape(m[::-1])
    for l in range(m[2]):
        kz = l - m[2] // 2
        cf = np.exp(-1j * kz * z)
        f2 = np.zeros(m[0] * m[1], np.complex128)
        assert lib.finufft2d1(n, _dp(x), _dp(y), _dp(cf), -1, 1e-11, m[0], m[1], _dp(f2), None) == 0
        assert rel_l2(f2.reshape(m[1], m[0]), f3[l]) < 1e-9


def test_dropin_error_reporting(lib):
    fk = np.zeros(4, np.complex128)
    ier = C.c_int(0)
    nj = C.c_int64(-5)
    iflag, eps = C.c_int(-1), C.c_double(1e-6)
    m = C.c_int64(2)
    x = np.zeros(1)
    lib.finufft2d1_(C.byref(nj), _dp(x), _dp(x), _dp(x), C.byref(iflag), C.byref(eps), C.byref(m),
                    C.byref(m), _dp(fk), None, C.byref(ier))
    assert ier.value == 1  # MPSQ_ERR_ARG
    assert b"nj" in lib.mpsq_last_error()
    # zero modes: nothing to do, success
    assert lib.finufft2d1(0, None, None, None, -1, 1e-6, 0, 5, _dp(fk), None) == 0
    # zero points: zero output
    fk[:] = 7
    assert lib.finufft2d1(0, None, None, None, -1, 1e-6, 2, 2, _dp(fk), None) == 0
    assert np.all(fk == 0)
