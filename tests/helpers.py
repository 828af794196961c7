"""Shared helpers for the parity tests: small seeded systems and C-ABI call wrappers."""
import ctypes as C

import numpy as np

from mp_tools_gb300 import _lib
from mp_tools_gb300._lib import check


def rel_l2(a, b):
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def plan_type1(torch, dim, modes, x, y, z, c, iflag, eps, precision, ntrans=1):
    """Runs the device-pointer plan API; returns fk as numpy complex (ntrans, *modes[::-1])."""
    L = _lib.load()
    rdt = torch.float64 if precision == _lib.FP64 else torch.float32
    cdt = torch.complex128 if precision == _lib.FP64 else torch.complex64
    dev = "cuda"
    xd = torch.as_tensor(np.asarray(x), dtype=rdt, device=dev).contiguous()
    yd = torch.as_tensor(np.asarray(y), dtype=rdt, device=dev).contiguous()
    zd = torch.as_tensor(np.asarray(z), dtype=rdt, device=dev).contiguous() if dim == 3 else None
    cd = torch.as_tensor(np.asarray(c), dtype=cdt, device=dev).contiguous()
    nm = int(np.prod(modes))
    fk = torch.empty(ntrans * nm, dtype=cdt, device=dev)
    m = (C.c_int64 * 3)(*(list(modes) + [1] * (3 - len(modes))))
    plan = C.c_void_p()
    stream = torch.cuda.current_stream().cuda_stream
    check(L.mpsq_nufft_makeplan(dim, m, iflag, ntrans, eps, precision, C.c_void_p(stream),
                                C.byref(plan)), "makeplan")
    try:
        check(L.mpsq_nufft_setpts(plan, len(x), C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()),
                                  C.c_void_p(zd.data_ptr() if zd is not None else 0)), "setpts")
        check(L.mpsq_nufft_execute(plan, C.c_void_p(cd.data_ptr()), C.c_void_p(fk.data_ptr())), "execute")
        check(L.mpsq_nufft_check_error(plan), "check_error")
        torch.cuda.synchronize()
        out = fk.cpu().numpy()
    finally:
        L.mpsq_nufft_destroy(plan)
    return out.reshape((ntrans,) + tuple(modes[::-1]))


def abo3_cell(n, rng, sigma=(0.05, 0.05, 0.08), a=4.19):
    """ABO3 supercell of n^3 cubic cells in centred lattice units (species-major: A, B, O1..O3),
    Gaussian displacements sigma (Angstrom) per species kind."""
    base = np.array([[0, 0, 0], [0.5, 0.5, 0.5], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    i = np.stack(np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij"), -1).reshape(-1, 3)
    cells = i - (n // 2)
    sig = [sigma[0], sigma[1], sigma[2], sigma[2], sigma[2]]
    pos, ind = [], []
    for s in range(5):
        p = cells + base[s] + rng.normal(0.0, sig[s] / a, size=cells.shape)
        pos.append(p)
        ind.append(np.concatenate([i + 1, np.full((len(i), 1), s + 1)], axis=1))
    pos = np.concatenate(pos).astype(np.float32)
    out = np.zeros((len(pos), 4), np.float32)
    out[:, :3] = pos
    return out, np.concatenate(ind).astype(np.int32), [n ** 3] * 5
