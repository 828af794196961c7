"""Seeded synthetic trajectories with the shapes, sizes and value distributions of the
benchmark workloads (the reference publishes no benchmark data set).

Coordinates follow the reference's conventions: CELL supercells in lattice units centred on
the box (at_pos = cell index - n/2 + basis + displacement, as mp_latt writes them), BULK boxes
in Angstrom centred on 0, atoms species-major, float4 records (x, y, z, charge=0).
"""
from __future__ import annotations

import numpy as np

ABO3_BASIS = np.array([[0, 0, 0], [0.5, 0.5, 0.5], [0.5, 0.5, 0.0], [0.5, 0.0, 0.5], [0.0, 0.5, 0.5]])
ABO3_B_COH_FM = [5.07, 7.16, 5.803, 5.803, 5.803]   # A, B, O, O, O (fm)
# Cromer-Mann coefficients (a1 b1 a2 b2 a3 b3 a4 b4 c), International Tables
XFF = {
    "Al": [6.4202, 3.0387, 1.9002, 0.7426, 1.5936, 31.5472, 1.9646, 85.0886, 1.1151],
    "U": [36.0228, 0.5293, 23.4128, 3.3253, 14.9491, 16.0927, 4.1880, 100.6130, 13.3966],
}


def abo3_cells(n: int):
    """Cell origins (n^3, 3) in centred lattice units and 1-based cell indices."""
    i = np.stack(np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij"), -1).reshape(-1, 3)
    return (i - n // 2).astype(np.float64), (i + 1).astype(np.int32)


def abo3_static(n: int, a: float, rng, sigma_ab=0.05, sigma_o=0.08, extra_b=None):
    """ABO3 supercell with Gaussian displacements (Angstrom -> lattice units).  Returns
    (positions (5 n^3, 4) float32, at_ind (5 n^3, 4) int32, species counts)."""
    cells, ind = abo3_cells(n)
    sig = [sigma_ab, sigma_ab, sigma_o, sigma_o, sigma_o]
    pos = np.zeros((5 * len(cells), 4), np.float32)
    at_ind = np.zeros((5 * len(cells), 4), np.int32)
    for s in range(5):
        p = cells + ABO3_BASIS[s] + rng.normal(0.0, sig[s] / a, size=cells.shape)
        if extra_b is not None and s == 1:
            p = p + extra_b
        sl = slice(s * len(cells), (s + 1) * len(cells))
        pos[sl, :3] = p
        at_ind[sl, :3] = ind
        at_ind[sl, 3] = s + 1
    return pos, at_ind, [len(cells)] * 5


def domain_wall_shift(n: int, a: float, rng, slab=17, dz=0.1):
    """B-site z shifts of +-dz (Angstrom) in alternating slabs of `slab` cells along a seeded
    axis and phase (90-degree domain-wall pattern)."""
    cells, _ = abo3_cells(n)
    axis = int(rng.integers(0, 3))
    phase = int(rng.integers(0, slab))
    sign = np.where(((cells[:, axis] + n // 2 + phase) // slab) % 2 == 0, 1.0, -1.0)
    shift = np.zeros_like(cells)
    shift[:, 2] = sign * dz / a
    return shift


def planewave_modes(n: int, rng, n_modes=48):
    """48 seeded modes: commensurate wavevector (h,k,l)/n, unit polarisation, frequency
    U(1,20) THz, amplitude U(0.01,0.03) Angstrom, phase U(0, 2pi)."""
    q = rng.integers(-n // 2, n // 2, size=(n_modes, 3)) / n
    e = rng.normal(size=(n_modes, 3))
    e /= np.linalg.norm(e, axis=1, keepdims=True)
    nu = rng.uniform(1.0, 20.0, n_modes)
    amp = rng.uniform(0.01, 0.03, n_modes)
    phi = rng.uniform(0, 2 * np.pi, n_modes)
    return q, e, nu, amp, phi


def abo3_planewave_frames(n: int, frames: int, dt_ps: float, a: float, rng, device="cpu"):
    """ABO3 n^3 ideal sites displaced by a superposition of plane-wave modes; returns a torch
    tensor (frames, 5 n^3, 4) float32 on `device` plus species counts and the modes."""
    import torch
    q, e, nu, amp, phi = planewave_modes(n, rng)
    cells, _ = abo3_cells(n)
    R = np.concatenate([cells + ABO3_BASIS[s] for s in range(5)])  # (5n^3, 3) l.u.
    Rt = torch.as_tensor(R, dtype=torch.float64, device=device)
    qt = torch.as_tensor(q, dtype=torch.float64, device=device)
    et = torch.as_tensor(e * (amp[:, None] / a), dtype=torch.float64, device=device)
    phase0 = 2 * np.pi * (Rt @ qt.T) + torch.as_tensor(phi, device=device)  # (N, M)
    out = torch.zeros((frames, len(R), 4), dtype=torch.float32, device=device)
    w = torch.as_tensor(2 * np.pi * nu, dtype=torch.float64, device=device)
    for t in range(frames):
        u = torch.cos(phase0 - w * (t * dt_ps)) @ et  # (N, 3)
        out[t, :, :3] = (Rt + u).to(torch.float32)
    return out, [n ** 3] * 5, (q, e, nu, amp, phi)


def rsa_hard_spheres(n_atoms: int, box: float, dmin: float, seed: int):
    """Uniform random sequential addition of n_atoms points in a periodic cubic box with
    minimum distance dmin (C helper, cell list).  Positions in [-box/2, box/2)."""
    import ctypes as C

    from . import build as _b
    lib = C.CDLL(str(_b.build_synth()))
    f = lib.mpsq_rsa_hard_spheres
    f.restype = C.c_int64
    f.argtypes = [C.c_int64, C.c_double, C.c_double, C.c_uint64, C.c_int64, C.c_void_p]
    pos = np.zeros((n_atoms, 3), np.float64)
    got = f(n_atoms, box, dmin, seed, 400 * n_atoms + 10_000_000, pos.ctypes.data)
    if got != n_atoms:
        raise RuntimeError(f"hard-sphere packing stalled at {got} of {n_atoms} atoms")
    return pos - box / 2


def amorphous_alloy(n_atoms=1_000_000, rho=0.06, frac_b=0.08, dmin=2.2, seed=20261205):
    """Al(1-x)U(x) amorphous box (species-major: Al then U) at number density rho (1/A^3)."""
    rng = np.random.default_rng(seed)
    box = (n_atoms / rho) ** (1.0 / 3.0)
    pos = rsa_hard_spheres(n_atoms, box, dmin, seed)
    n_b = int(round(frac_b * n_atoms))
    perm = rng.permutation(n_atoms)
    pos = pos[perm]
    out = np.zeros((n_atoms, 4), np.float32)
    out[:, :3] = pos
    return out, [n_atoms - n_b, n_b], box


def random_walk_frames(pos0, frames: int, sigma: float, box: float, seed: int, device="cuda"):
    """Frames k+1 = frame k + N(0, sigma) per axis, wrapped into the periodic box; a torch
    tensor (frames, N, 4) float32 on `device` (seeded torch generator)."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    p = torch.as_tensor(pos0[:, :3], dtype=torch.float32, device=device).clone()
    out = torch.zeros((frames, p.shape[0], 4), dtype=torch.float32, device=device)
    half = box / 2
    for t in range(frames):
        if t > 0:
            p += sigma * torch.randn(p.shape, generator=g, device=device, dtype=torch.float32)
            p = torch.remainder(p + half, box) - half
        out[t, :, :3] = p
    return out
