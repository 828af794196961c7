"""ORACLE — test infrastructure only, never the product path.

Only tests/, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` (``cpu_baseline`` and
``--impl reference``) import this package, and only as the checker or the timed CPU baseline.

Contents
  * ``dirft2d1`` / ``dirft3d1`` / ``dirft_modes`` / ``dirft_modes_tab`` — FP64 direct type-1
    sums (C, OpenMP), the
    definition the reference's own check path uses (code/src/mp_sqom56.f90:2530-2547).
  * ``es_nufft`` — a CPU port of the exponential-of-semicircle type-1 NUFFT (FP64 spreading in
    C/OpenMP with the points counting-sorted into 8^dim blocks and threads owning disjoint
    planes, scipy/pocketfft FFT, deconvolution by quadrature of the kernel transform), the
    stand-in for FINUFFT+OpenMP, which is not available on either machine; with
    ``weight_accumulate`` / ``abs2_accumulate`` (OpenMP) it is the timed CPU baseline.
  * ``sqom_ref`` — numpy restatement of the mp_sqom loops around the NUFFT call.
  * ``sql_ref`` — numpy restatement of mp_sql's spherical average (Q cube, FP32 |Q| binning,
    normalisation, smoothing, X-ray output modes).

Parity status
  * Pinned on the reference's own outputs: ``es_nufft`` + ``sql_ref`` reproduce the four mp_sql
    result tables of the reference's amorphous Al92U8 example (examples/amorphous_Al92U08,
    files _40.._43: Z(Q), I(Q), S(Q), unscaled I(Q), total and partial columns) from the
    example's own input frame, within 7e-7 of each column's maximum for Q <= 7.9 A^-1
    (tests/test_golden_alu.py).  This pins the type-1 transform itself (the same finufft2d1
    boundary mp_sqom calls), its mode order and sign, and the radial post-processing.
  * The mp_sqom-specific loops (selection, phases, species weights, time windows) have no
    runnable golden output in the reference tree (its BZO map files need frame files that
    are absent; only three map rows serve as a text-format check); they are checked against
    known-answer identities (tests/test_oracle.py) and the reference's formulas line by line.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"
SRC = [HERE / "dirft.c"]

_lib = None


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and all(s.stat().st_mtime <= LIB.stat().st_mtime for s in SRC):
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-o", str(tmp), *map(str, SRC), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def _load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        vp, i64 = C.c_void_p, C.c_int64
        lib.oracle_dirft2d1.argtypes = [i64, vp, vp, vp, C.c_int, i64, i64, vp]
        lib.oracle_dirft3d1.argtypes = [i64, vp, vp, vp, vp, C.c_int, i64, i64, i64, vp]
        lib.oracle_dirft_modes.argtypes = [C.c_int, i64, vp, vp, vp, vp, C.c_int, i64, vp, vp]
        lib.oracle_dirft_modes_tab.argtypes = [C.c_int, i64, vp, vp, vp, vp, C.c_int, i64, vp, vp,
                                               vp, vp]
        lib.oracle_es_spread.argtypes = [C.c_int, i64, vp, vp, C.c_int, C.c_double, i64, i64, i64, vp]
        lib.oracle_zero.argtypes = [vp, i64]
        lib.oracle_weight_accumulate.argtypes = [i64, vp, vp, vp, C.c_int]
        lib.oracle_abs2_accumulate.argtypes = [i64, vp, vp]
        lib.oracle_es_extract.argtypes = [C.c_int, vp, i64, i64, i64, i64, i64, i64, vp, vp, vp, vp]
        lib.oracle_num_threads.restype = C.c_int
        _lib = lib
    return _lib


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _c128(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


def dirft2d1(x, y, c, iflag, ms, mt):
    """Direct FP64 sum; returns complex128 array of shape (mt, ms) (k1 fastest)."""
    x, y, c = _f64(x), _f64(y), _c128(c)
    out = np.zeros((mt, ms), np.complex128)
    _load().oracle_dirft2d1(len(x), x.ctypes.data, y.ctypes.data, c.ctypes.data, int(iflag),
                            ms, mt, out.ctypes.data)
    return out


def dirft3d1(x, y, z, c, iflag, ms, mt, mu):
    """Direct FP64 sum; returns complex128 array of shape (mu, mt, ms)."""
    x, y, z, c = _f64(x), _f64(y), _f64(z), _c128(c)
    out = np.zeros((mu, mt, ms), np.complex128)
    _load().oracle_dirft3d1(len(x), x.ctypes.data, y.ctypes.data, z.ctypes.data, c.ctypes.data,
                            int(iflag), ms, mt, mu, out.ctypes.data)
    return out


def dirft_modes(x, y, z, c, iflag, kq):
    """Direct FP64 sum at integer modes kq (nq x 2 or nq x 3); z may be None for 2D."""
    kq = np.asarray(kq, dtype=np.int64)
    dim = kq.shape[1]
    k3 = np.zeros((kq.shape[0], 3), np.int64)
    k3[:, :dim] = kq
    x, y, c = _f64(x), _f64(y), _c128(c)
    z = _f64(z) if z is not None else np.zeros_like(x)
    out = np.zeros(kq.shape[0], np.complex128)
    _load().oracle_dirft_modes(dim, len(x), x.ctypes.data, y.ctypes.data, z.ctypes.data,
                               c.ctypes.data, int(iflag), kq.shape[0], k3.ctypes.data,
                               out.ctypes.data)
    return out


def dirft_modes_tab(x, y, z, c, iflag, kq):
    """dirft_modes for large point sets and many modes: per point, phase tables along each
    axis over the span of the selected mode indices (exact every 16 steps), then one product per
    selected mode.  Same result as dirft_modes to ~1e-13 relative."""
    kq = np.asarray(kq, dtype=np.int64)
    dim = kq.shape[1]
    k3 = np.zeros((kq.shape[0], 3), np.int64)
    k3[:, :dim] = kq
    kmin = k3.min(axis=0).astype(np.int64)
    span = (k3.max(axis=0) - kmin + 1).astype(np.int64)
    x, y, c = _f64(x), _f64(y), _c128(c)
    z = _f64(z) if z is not None else np.zeros_like(x)
    out = np.zeros(kq.shape[0], np.complex128)
    _load().oracle_dirft_modes_tab(dim, len(x), x.ctypes.data, y.ctypes.data, z.ctypes.data,
                                   c.ctypes.data, int(iflag), kq.shape[0], k3.ctypes.data,
                                   kmin.ctypes.data, span.ctypes.data, out.ctypes.data)
    return out


def num_threads() -> int:
    return int(_load().oracle_num_threads())


# ------------------------------------------------------------------------ CPU NUFFT port
def es_params(eps: float):
    """Width and shape parameter of the ES kernel for upsampling 2 (Barnett et al. 2019)."""
    eps = min(max(eps, 1e-14), 1e-1)
    w = int(np.ceil(np.log10(1.0 / eps))) + 1
    w = max(2, min(16, w))
    return w, 2.30 * w


def _smooth(n):
    for p in (2, 3, 5, 7):
        while n % p == 0:
            n //= p
    return n == 1


def fine_size(m, w):
    n = max(2 * m, 2 * w, 16)
    n += (-n) % 2
    while not _smooth(n):
        n += 2
    return n


def es_phihat(w, beta, nf, m):
    """Kernel Fourier transform at k = -m/2 .. (m-1)/2 by Gauss-Legendre quadrature."""
    xq, wq = np.polynomial.legendre.leggauss(4 * w + 40)
    u = 0.5 * w * xq
    f = 0.5 * w * wq * np.exp(beta * (np.sqrt(np.maximum(0.0, 1.0 - xq * xq)) - 1.0))
    k = np.arange(m) - m // 2
    return (f[None, :] * np.cos(2 * np.pi * k[:, None] * u[None, :] / nf)).sum(axis=1)


def weight_accumulate(cs, w, A, first):
    """cs = (0 if first else cs) + w * A over the flattened Q grid, in place (complex128 cs and
    A, float64 w; OpenMP)."""
    assert cs.dtype == np.complex128 and cs.flags.c_contiguous and cs.size == A.size == w.size
    A, w = _c128(A), _f64(w)
    _load().oracle_weight_accumulate(cs.size, w.ctypes.data, A.ctypes.data, cs.ctypes.data,
                                     int(bool(first)))


def abs2_accumulate(s, cs):
    """s += |cs|^2 in place (float64 s, complex128 cs; OpenMP)."""
    assert s.dtype == np.float64 and s.flags.c_contiguous and s.size == cs.size
    cs = _c128(cs)
    _load().oracle_abs2_accumulate(s.size, cs.ctypes.data, s.ctypes.data)


_grid_cache = None


def _fine_grid(shape):
    """A zeroed complex128 fine grid; the buffer of the previous call of the same shape is
    reused (zeroed in parallel in C), as a plan reuses its grid across repeated transforms."""
    global _grid_cache
    if _grid_cache is None or _grid_cache.shape != shape:
        _grid_cache = None
        _grid_cache = np.empty(shape, np.complex128)
    _load().oracle_zero(_grid_cache.ctypes.data, 2 * _grid_cache.size)
    return _grid_cache


def es_nufft(coords, c, iflag, eps, modes, workers=None):
    """CPU type-1 NUFFT (FP64).  coords: list of 2 or 3 coordinate arrays (radians);
    modes: (m1, m2[, m3]).  Returns complex128 of shape modes[::-1] (k1 fastest)."""
    import scipy.fft

    dim = len(modes)
    w, beta = es_params(eps)
    nf = [fine_size(m, w) for m in modes]
    nj = len(coords[0])
    g = np.zeros((nj, 3), np.float64)
    for d in range(dim):
        gd = _f64(coords[d]) * (nf[d] / (2 * np.pi))
        gd -= nf[d] * np.floor(gd / nf[d])
        gd[gd >= nf[d]] -= nf[d]
        g[:, d] = gd
    c = _c128(c)
    shape = (nf[2] if dim == 3 else 1, nf[1], nf[0])
    grid = _fine_grid(shape)
    _load().oracle_es_spread(dim, nj, g.ctypes.data, c.ctypes.data, w, beta, nf[0], nf[1],
                             nf[2] if dim == 3 else 1, grid.ctypes.data)
    axes = tuple(range(3 - dim, 3))
    workers = workers or num_threads()
    if iflag >= 0:
        G = scipy.fft.ifftn(grid, axes=axes, workers=workers, overwrite_x=True, norm="forward")
    else:
        G = scipy.fft.fftn(grid, axes=axes, workers=workers, overwrite_x=True)
    corr = [np.ascontiguousarray(1.0 / es_phihat(w, beta, n, m)) for m, n in zip(modes, nf)]
    G = np.ascontiguousarray(G, dtype=np.complex128)
    out = np.empty(tuple(modes[::-1]), np.complex128)
    m = list(modes) + [1] * (3 - dim)
    _load().oracle_es_extract(dim, G.ctypes.data, nf[0], nf[1], nf[2] if dim == 3 else 1, m[0],
                              m[1], m[2], corr[0].ctypes.data, corr[1].ctypes.data,
                              corr[2].ctypes.data if dim == 3 else None, out.ctypes.data)
    return out
