"""The allocation-free 2D transform (mpsq_nufft2d1_noalloc) for callers that cannot allocate
device memory during a call (hosts whose device memory belongs to their own pool under a fixed
budget, plug-in hosts that forbid allocation inside a call).

It is checked through the C ABI against the existing finufft2d1 entry point on two calls in a
row with different sizes (the second call reuses the static scratch the first one left
behind), at a loose, a medium and the tightest tolerance, within the FP64 tolerance the other
parity tests use (5 eps), and with no points at all.  This file is collected last so that a run
stopping at the first failure has run every other test; it also passes alone in a fresh
process (its first call performs the per-device set-up).
"""
import ctypes as C

import numpy as np
import pytest

from helpers import rel_l2


pytestmark = pytest.mark.gpu



def _tol(eps):
    # both sides are within about eps of the exact sum (the bound the FP64 parity tests use is
    # 5 eps), on different fine grids (a power of two here, a 2,3,5-smooth length there)
    return max(5 * eps, 1e-12)


def _existing(lib, x, y, c, iflag, eps, ms, mt):
    fk = np.zeros(ms * mt, np.complex128)
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    assert lib.finufft2d1(len(x), p(x), p(y), p(c), iflag, eps, ms, mt, p(fk), None) == 0
    return fk


def _noalloc(lib, torch, x, y, c, iflag, eps, ms, mt):
    xd = torch.as_tensor(x, device="cuda")
    yd = torch.as_tensor(y, device="cuda")
    cd = torch.as_tensor(c, device="cuda")
    fk = torch.full((ms * mt,), 7.0 + 7.0j, dtype=torch.complex128, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.mpsq_nufft2d1_noalloc(len(x), C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()),
                                   C.c_void_p(cd.data_ptr()), iflag, eps, ms, mt,
                                   C.c_void_p(fk.data_ptr()), C.c_void_p(stream))
    assert rc == 0, lib.mpsq_last_error()
    return fk.cpu().numpy()


@pytest.mark.parametrize("eps", [1e-3, 1e-9, 1e-14])
def test_noalloc_matches_finufft2d1_twice(lib, cuda, eps):
    rng = np.random.default_rng(99)
    cases = [(40000, 160, 160, -1), (5000, 64, 37, 1)]
    for n, ms, mt, iflag in cases:
        x, y = rng.uniform(-np.pi, np.pi, (2, n))
        c = rng.normal(size=n) + 1j * rng.normal(size=n)
        got = _noalloc(lib, cuda, x, y, c, iflag, eps, ms, mt)
        want = _existing(lib, x, y, c, iflag, eps, ms, mt)
        assert rel_l2(got, want) < _tol(eps), (eps, n, ms, mt)


def test_noalloc_without_points_gives_zeros(lib, cuda):
    fk = cuda.full((8 * 6,), 7.0 + 7.0j, dtype=cuda.complex128, device="cuda")
    rc = lib.mpsq_nufft2d1_noalloc(0, None, None, None, -1, 1e-9, 8, 6,
                                   C.c_void_p(fk.data_ptr()), None)
    assert rc == 0, lib.mpsq_last_error()
    assert not fk.cpu().numpy().any()


def test_noalloc_rejects_sizes_beyond_the_static_scratch(lib, cuda):
    fk = cuda.zeros(4, dtype=cuda.complex128, device="cuda")
    x = cuda.zeros(1, dtype=cuda.float64, device="cuda")
    rc = lib.mpsq_nufft2d1_noalloc(70000, C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()),
                                   C.c_void_p(x.data_ptr()), -1, 1e-9, 2, 2,
                                   C.c_void_p(fk.data_ptr()), None)
    assert rc == 1  # MPSQ_ERR_ARG, nothing launched
    assert b"65536" in lib.mpsq_last_error()
    rc = lib.mpsq_nufft2d1_noalloc(1, C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()),
                                   C.c_void_p(x.data_ptr()), -1, 1e-9, 300, 2,
                                   C.c_void_p(fk.data_ptr()), None)
    assert rc == 1 and b"256" in lib.mpsq_last_error()
