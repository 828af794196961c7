"""Oracle self-checks against known answers (CPU only)."""
import os
from pathlib import Path

import numpy as np
import pytest

import oracle
from oracle import sqom_ref


def test_single_atom_at_origin_gives_unit_amplitudes():
    f = oracle.dirft2d1([0.0], [0.0], [1.0], -1, 8, 6)
    assert np.allclose(f, 1.0)
    g = oracle.dirft3d1([0.0], [0.0], [0.0], [1.0], 1, 5, 4, 3)
    assert np.allclose(g, 1.0)


def test_mode_order_and_sign():
    x, y = 0.3, -1.1
    f = oracle.dirft2d1([x], [y], [1.0], -1, 6, 5)
    for i in range(6):
        for j in range(5):
            k1, k2 = i - 3, j - 2
            assert np.isclose(f[j, i], np.exp(-1j * (k1 * x + k2 * y)))
    g = oracle.dirft2d1([x], [y], [1.0], +1, 6, 5)
    assert np.allclose(g, np.conj(f))


def test_perfect_lattice_bragg_peaks():
    # 8x8 CELL lattice: x = 2pi*i/8 -> amplitude N at multiples of 8, 0 elsewhere
    i, j = np.meshgrid(np.arange(8), np.arange(8), indexing="ij")
    x = (2 * np.pi * i.ravel() / 8) - np.pi
    y = (2 * np.pi * j.ravel() / 8) - np.pi
    f = oracle.dirft2d1(x, y, np.ones(64), -1, 32, 32)
    k = np.arange(32) - 16
    peak = (k[:, None] % 8 == 0) & (k[None, :] % 8 == 0)
    assert np.allclose(np.abs(f[peak]), 64)
    assert np.max(np.abs(f[~peak])) < 1e-9


def test_q_center_shift_equals_strength_phase():
    rng = np.random.default_rng(3)
    x, y = rng.uniform(-np.pi, np.pi, (2, 50))
    c = np.exp(-1j * (2 * x + (-3) * y))  # shift by (2,-3) modes
    f = oracle.dirft2d1(x, y, c, -1, 16, 16)
    g = oracle.dirft2d1(x, y, np.ones(50), -1, 24, 24)
    # f(k) = g(k + (2,-3))
    assert np.allclose(f[8 - 8:16, :], g[12 - 8 - 3:12 + 8 - 3, 12 - 8 + 2:12 + 8 + 2])


def test_3d_slices_equal_z_phased_2d():
    # the mp_sql construction: slice kz of the 3D sum = 2D sum with strengths exp(-i kz z)
    rng = np.random.default_rng(4)
    x, y, z = rng.uniform(-np.pi, np.pi, (3, 40))
    f3 = oracle.dirft3d1(x, y, z, np.ones(40), -1, 10, 8, 6)
    for l in range(6):
        kz = l - 3
        f2 = oracle.dirft2d1(x, y, np.exp(-1j * kz * z), -1, 10, 8)
        assert np.allclose(f3[l], f2)


@pytest.mark.parametrize("eps", [1e-6, 1e-9, 1e-12])
def test_cpu_nufft_port_meets_tolerance_2d(eps):
    rng = np.random.default_rng(5)
    n = 3000
    x, y = rng.uniform(-3 * np.pi, 3 * np.pi, (2, n))
    c = rng.normal(size=n) + 1j * rng.normal(size=n)
    ref = oracle.dirft2d1(x, y, c, -1, 48, 30)
    got = oracle.es_nufft([x, y], c, -1, eps, (48, 30))
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 5 * eps


def test_cpu_nufft_port_3d():
    rng = np.random.default_rng(6)
    n = 2000
    x, y, z = rng.uniform(-np.pi, np.pi, (3, n))
    c = rng.normal(size=n) + 1j * rng.normal(size=n)
    ref = oracle.dirft3d1(x, y, z, c, 1, 14, 12, 9)
    got = oracle.es_nufft([x, y, z], c, 1, 1e-9, (14, 12, 9))
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-8


@pytest.mark.parametrize("modes", [(5, 3, 4), (2, 2, 2), (33, 1, 7)])
def test_cpu_nufft_port_small_grids(modes):
    """Fine grids narrower than a sorting block plus the kernel width, and points on the
    periodic edges: every block's support reaches every thread's planes."""
    rng = np.random.default_rng(8)
    n = 500
    x, y, z = rng.uniform(-np.pi, np.pi, (3, n))
    x[:4] = [-np.pi, np.pi - 1e-12, 0.0, -1e-15]
    c = rng.normal(size=n) + 1j * rng.normal(size=n)
    ref = oracle.dirft3d1(x, y, z, c, -1, *modes)
    got = oracle.es_nufft([x, y, z], c, -1, 1e-9, modes)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-8


def test_cpu_nufft_port_independent_of_thread_count():
    """Each cell is summed in the sorted point order by the one thread owning its plane, so
    the port gives the same bits with 1 thread and with several."""
    import subprocess
    import sys
    code = (
        "import numpy as np, oracle\n"
        "rng = np.random.default_rng(10)\n"
        "x, y, z = rng.uniform(-np.pi, np.pi, (3, 4000))\n"
        "c = rng.normal(size=4000) + 1j * rng.normal(size=4000)\n"
        "f = oracle.es_nufft([x, y, z], c, -1, 1e-6, (12, 10, 8))\n"
        "g = oracle.es_nufft([x, y], c, 1, 1e-6, (20, 14))\n"
        "import sys; sys.stdout.write(np.concatenate([f.ravel(), g.ravel()]).tobytes().hex())\n")
    root = str(Path(__file__).resolve().parents[1])
    outs = []
    for n in ("1", "3"):
        env = dict(os.environ, OMP_NUM_THREADS=n, PYTHONPATH=root)
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env,
                           cwd=root, timeout=120)
        assert r.returncode == 0, r.stderr
        outs.append(r.stdout)
    assert outs[0] == outs[1]


def test_weighting_helpers_match_numpy():
    """The CPU baseline's species weighting and |F|^2 accumulation (OpenMP loops)."""
    rng = np.random.default_rng(9)
    n = 1001
    a, b = rng.normal(size=(2, n)) + 1j * rng.normal(size=(2, n))
    w1, w2 = rng.normal(size=(2, n))
    cs = np.empty(n, np.complex128)
    oracle.weight_accumulate(cs, w1, a, first=True)
    oracle.weight_accumulate(cs, w2, b, first=False)
    assert np.array_equal(cs, w1 * a + w2 * b)
    s = np.ones(n)
    oracle.abs2_accumulate(s, cs)
    assert np.allclose(s, 1.0 + np.abs(cs) ** 2, rtol=1e-15, atol=0)


def test_dirft_modes_matches_full_sum():
    rng = np.random.default_rng(7)
    x, y, z = rng.uniform(-np.pi, np.pi, (3, 300))
    c = rng.normal(size=300) + 0j
    full = oracle.dirft3d1(x, y, z, c, -1, 8, 6, 4)
    kq = np.array([[-4, -3, -2], [3, 2, 1], [0, 0, 0], [1, -1, 0]])
    got = oracle.dirft_modes(x, y, z, c, -1, kq)
    for q, (a, b, cc) in enumerate(kq):
        assert np.isclose(got[q], full[cc + 2, b + 3, a + 4])


def test_time_transforms_identities():
    rng = np.random.default_rng(8)
    F, nq = 40, 7
    cs = rng.normal(size=(F, nq)) + 1j * rng.normal(size=(F, nq))
    n_int = 21
    w = sqom_ref.hann_window(n_int)
    assert w[0] == 0 and np.isclose(w[n_int // 2], 1.0)
    # E=const and dispersion give the same |X|^2 (the centring phase drops out)
    for jf in (1, 4, 9):
        e = sqom_ref.econst(cs, n_int, w, jf)
        d = sqom_ref.dispersion(cs, n_int, w, np.arange(nq), 11)[:, jf - 1]
        assert np.allclose(e, d)
    # Parseval for a flat window over the full run
    X = sqom_ref.dispersion(cs, F, np.ones(F), np.arange(nq), F)
    x = sqom_ref.centered(cs)
    assert np.allclose(X.sum(axis=1), F * (np.abs(x) ** 2).sum(axis=0))


def test_single_exponential_peaks_at_its_bin():
    F = 64
    t = np.arange(F)
    cs = np.exp(-2j * np.pi * 5 * t / F)[:, None] * np.ones((1, 3))
    cs = cs + 0.0
    s = sqom_ref.gauss_spectrum(cs, F / 2, F)
    assert np.all(np.argmax(s, axis=0) == (-5) % F)
    cs2 = np.exp(+2j * np.pi * 5 * t / F)[:, None] * np.ones((1, 3))
    s2 = sqom_ref.gauss_spectrum(cs2, F / 2, F)
    assert np.all(np.argmax(s2, axis=0) == 5)


def test_iqt_identities():
    """I(Q,t) at lag 0 over the whole run is the mean-subtracted power; the path cut at lag t
    equals n_int times the map at lag t on the path's pixels; atom-pair maps of a centred
    series equal the weighted-series maps."""
    rng = np.random.default_rng(11)
    F, nq = 16, 40
    cs = rng.normal(size=(F, nq)) + 1j * rng.normal(size=(F, nq))
    x = sqom_ref.centered(cs)
    np.testing.assert_allclose(sqom_ref.iqt_map(cs, F, 0), (np.abs(x) ** 2).mean(axis=0), rtol=1e-12)
    path = np.array([3, 7, 30])
    cut = sqom_ref.iqt_dispersion(cs, 6, path)
    assert cut.shape == (3, F - 6 + 1)
    for lag in (0, 4, 10):
        np.testing.assert_allclose(cut[:, lag], 6 * sqom_ref.iqt_map(cs, 6, lag)[path], rtol=1e-12)
    w = sqom_ref.hann_window(5)
    a = sqom_ref.econst(cs, 5, w, 2)
    b = sqom_ref.econst(x, 5, w, 2, center=False)
    np.testing.assert_allclose(a, b, rtol=1e-12)


def test_hann_leakage_pattern_of_a_pure_tone():
    """E=const map of a pure tone exp(2 pi i k0 t / n_int): every start frame contributes the
    same |X|^2, so bin f holds n0 |H(f - 1 - k0)|^2 with H the DFT of the reference's Hann
    window; the main lobe sits at bin k0 + 1 and the first neighbours carry about a quarter of
    it (the symmetric window's -6 dB points), the far bins much less."""
    n_int, k0 = 65, 5
    F = 130                                   # ten whole periods: the elastic mean is zero
    t = np.arange(F)
    cs = np.exp(2j * np.pi * k0 * t / n_int)[:, None] * np.ones((1, 2))
    h = sqom_ref.hann_window(n_int)
    H = np.fft.fft(h)
    n0 = F - n_int + 1
    maps = np.array([sqom_ref.econst(cs, n_int, h, f)[0] for f in range(1, n_int // 2 + 2)])
    want = n0 * np.abs(H[(np.arange(n_int // 2 + 1) - k0) % n_int]) ** 2
    np.testing.assert_allclose(maps, want, rtol=1e-9, atol=1e-9 * maps.max())
    assert np.argmax(maps) == k0
    assert 0.23 < maps[k0 + 1] / maps[k0] < 0.27 and 0.23 < maps[k0 - 1] / maps[k0] < 0.27
    assert np.all(maps[k0 + 3:] < 1e-3 * maps[k0])


def test_plane_wave_displacement_satellites():
    """A longitudinal plane wave u(R, t) = A e cos(2 pi q.R - 2 pi nu t) on a simple cubic
    lattice: to first order in A the amplitude at G - q is -pi i (Q.e) A N exp(+2 pi i nu t) and
    at G + q the same with exp(-2 pi i nu t); elsewhere off the lattice it vanishes.  In the
    E=const map at the bin of nu (mp_sqom's phase convention) G - q carries
    n0 (sum h)^2 |pi (Q.e) A N|^2 and G + q nothing."""
    n, A = 8, 0.002
    n_int, k0 = 33, 3
    F = 66                                     # 6 periods of 11 frames
    nu = k0 / n_int
    R = np.stack(np.meshgrid(*(np.arange(n) - n // 2,) * 3, indexing="ij"), -1).reshape(-1, 3)
    N = len(R)
    q = np.array([1.0 / n, 0.0, 0.0])
    kq = np.array([[n - 1, 0, 0], [n + 1, 0, 0], [n, 0, 0], [n + 1, 1, 0]])  # G-q, G+q, G, off
    amps = np.empty((F, len(kq)), np.complex128)
    for t in range(F):
        r = R.astype(np.float64).copy()
        r[:, 0] += A * np.cos(2 * np.pi * (R @ q) - 2 * np.pi * nu * t)
        x, y, z = (2 * np.pi * r / n).T
        amps[t] = oracle.dirft_modes(x, y, z, np.ones(N), -1, kq)
    tt = np.arange(F)
    for col, sign in ((0, +1), (1, -1)):
        Qe = kq[col, 0] / n
        want = -np.pi * 1j * Qe * A * N * np.exp(sign * 2j * np.pi * nu * tt)
        assert np.abs(amps[:, col] - want).max() < 2e-3 * abs(want[0])
    assert np.abs(amps[:, 2] - N).max() < 1e-3 * N            # Bragg: constant to O(A^2)
    assert np.abs(amps[:, 3]).max() < 1e-6 * N                 # off-lattice, no satellite
    h = sqom_ref.hann_window(n_int)
    m = sqom_ref.econst(amps, n_int, h, k0 + 1)
    n0 = F - n_int + 1
    lo = n0 * h.sum() ** 2 * (np.pi * (kq[0, 0] / n) * A * N) ** 2
    assert abs(m[0] / lo - 1) < 5e-3
    assert m[1] < 1e-4 * m[0] and m[3] < 1e-9 * m[0]
