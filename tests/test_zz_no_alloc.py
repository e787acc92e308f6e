"""The allocation-free banded solve, checked against the allocating path.

mafem_band_solve_noalloc is for callers that must not call cudaMalloc (their
device memory belongs to their own allocator, e.g. a CUDA.jl memory pool, or
they cannot afford cudaMalloc's device-wide synchronisation).  It factors and
solves in a static scratch array inside the library.  Here it is called through
the C ABI with device buffers the test allocates itself (the test is not such a
caller), several times in a row on different systems, and every result must
equal the handle-based path's K \\ r (mafem_solve) within the FP64 solve
tolerance of the other parity tests.

This file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from _cases import M, params_pair, rel, state

pytestmark = pytest.mark.gpu


class _Cudart:
    def __init__(self):
        self.lib = None
        for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
            try:
                self.lib = C.CDLL(name)
                break
            except OSError:
                continue
        assert self.lib is not None, "libcudart not found"
        self.bufs = []

    def to_device(self, a: np.ndarray) -> C.c_void_p:
        a = np.ascontiguousarray(a, dtype=np.float64)
        p = C.c_void_p()
        assert self.lib.cudaMalloc(C.byref(p), C.c_size_t(max(a.nbytes, 8))) == 0
        self.bufs.append(p)
        assert self.lib.cudaMemcpy(p, a.ctypes.data_as(C.c_void_p), C.c_size_t(a.nbytes), 1) == 0  # H2D
        return p

    def from_device(self, p, n: int) -> np.ndarray:
        out = np.zeros(n)
        assert self.lib.cudaMemcpy(out.ctypes.data_as(C.c_void_p), p, C.c_size_t(out.nbytes), 2) == 0  # D2H
        return out

    def free(self):
        for p in self.bufs:
            self.lib.cudaFree(p)
        self.bufs = []


def _system(motion, n1, n2, seed):
    """K (LAPACK band, column j at row j of the array) and r of one assembly, and
    the allocating path's solution x = K \\ r = -mafem_solve(r)."""
    p, _ = params_pair(motion, M.F_PULL, n1, n2)
    mesh = M.Mesh(p)
    xms, cps = state(p, mesh, seed=seed, amp=1e-2, vel_amp=0.02)
    with M.Solver(mesh, p) as s:
        r, ab = s.calc_r_K(xms, cps, 0.01, 0.01)
        x_ref = -s.solve(r)
    return ab, r, mesh.half_bw, x_ref


def _noalloc_solve(cu, ab, r, kl):
    lib = M.lib()
    f = lib.mafem_band_solve_noalloc
    f.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    n, ldab = ab.shape
    d_band = cu.to_device(ab)        # row j of `ab` = band column j: the LAPACK layout
    d_rhs = cu.to_device(r)
    d_x = cu.to_device(np.zeros(n))
    rc = f(d_band, n, kl, kl, ldab, d_rhs, d_x, None)
    assert rc == 0, lib.mafem_last_error(None).decode()
    return cu.from_device(d_x, n)


def test_noalloc_solve_matches_allocating_solve():
    cu = _Cudart()
    try:
        systems = [_system(M.ALEVB, 7, 7, seed=1), _system(M.LAG, 8, 6, seed=2)]
        # two different systems back to back, then the first again: each call
        # must be correct whatever the previous call left in the shared scratch
        for ab, r, kl, x_ref in systems + systems[:1]:
            x = _noalloc_solve(cu, ab, r, kl)
            assert rel(x, x_ref) < 1e-10
    finally:
        cu.free()


def test_noalloc_rejects_oversize_systems():
    lib = M.lib()
    f = lib.mafem_band_solve_noalloc
    f.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    # 33262 unknowns with half bandwidth 1055 need ~1 GB of scratch: refused
    # before any device work (the pointers are never dereferenced)
    rc = f(C.c_void_p(16), 33262, 1055, 1055, 3 * 1055 + 1, C.c_void_p(16), C.c_void_p(16), None)
    assert rc == M.ERR_ARG
    assert "scratch" in lib.mafem_last_error(None).decode()
