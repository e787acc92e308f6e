"""The allocation-free banded solve, checked against the allocating path and
against a dense solve.

mafem_band_solve_noalloc is for callers that must not call cudaMalloc (their
device memory belongs to their own allocator, e.g. a CUDA.jl memory pool, or
they cannot afford cudaMalloc's device-wide synchronisation).  It factors and
solves in a static scratch array inside the library.  Here it is called through
the C ABI with device buffers the test allocates itself (the test is not such a
caller), several times in a row on different systems, and every result must
equal the handle-based path's K \\ r (mafem_solve) and numpy's dense solve of
the same matrix within the FP64 solve tolerance of the other parity tests.  The
free device memory must not change across calls once the library's kernels are
loaded, and singular or non-finite systems and bad arguments must be refused
with their status codes.

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


def _dense(ab, kl):
    n = ab.shape[0]
    A = np.zeros((n, n))
    for j in range(n):
        for i in range(max(0, j - kl), min(n, j + kl + 1)):
            A[i, j] = ab[j, 2 * kl + i - j]
    return A


def _free_bytes(cu):
    free, total = C.c_size_t(), C.c_size_t()
    assert cu.lib.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value


def test_noalloc_solve_matches_allocating_solve():
    cu = _Cudart()
    try:
        systems = [_system(M.ALEVB, 7, 7, seed=1), _system(M.LAG, 8, 6, seed=2)]
        # two different systems back to back, then the first again: each call
        # must be correct whatever the previous call left in the shared scratch
        for ab, r, kl, x_ref in systems + systems[:1]:
            x = _noalloc_solve(cu, ab, r, kl)
            assert rel(x, x_ref) < 1e-10
            assert rel(x, np.linalg.solve(_dense(ab, kl), r)) < 1e-10
    finally:
        cu.free()


def test_noalloc_allocates_no_device_memory():
    """Free device memory before and after a second pass of calls (the first pass
    loads the library's kernels and the scratch array's module, which lazy
    module loading may defer to first use) is the same to the byte."""
    cu = _Cudart()
    try:
        systems = [_system(M.ALEVB, 7, 7, seed=3), _system(M.LAG, 8, 6, seed=4)]
        staged = []
        for ab, r, kl, _ in systems:
            staged.append((cu.to_device(ab), cu.to_device(r), cu.to_device(np.zeros(ab.shape[0])), ab.shape, kl))
        f = _noalloc_fn()
        for d_band, d_rhs, d_x, (n, ldab), kl in staged:  # warm-up pass
            assert f(d_band, n, kl, kl, ldab, d_rhs, d_x, None) == 0
        assert cu.lib.cudaDeviceSynchronize() == 0
        before = _free_bytes(cu)
        for _ in range(2):
            for d_band, d_rhs, d_x, (n, ldab), kl in staged:
                assert f(d_band, n, kl, kl, ldab, d_rhs, d_x, None) == 0
        assert cu.lib.cudaDeviceSynchronize() == 0
        assert _free_bytes(cu) == before
    finally:
        cu.free()


def _noalloc_fn():
    f = M.lib().mafem_band_solve_noalloc
    f.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def _small_band(n, kl, seed):
    rng = np.random.default_rng(seed)
    A = np.zeros((n, n))
    for j in range(n):
        lo, hi = max(0, j - kl), min(n, j + kl + 1)
        A[lo:hi, j] = rng.uniform(-1, 1, hi - lo)
    A[np.arange(n), np.arange(n)] += 2.0 * kl
    ab = np.zeros((n, 3 * kl + 1))
    for j in range(n):
        for i in range(max(0, j - kl), min(n, j + kl + 1)):
            ab[j, 2 * kl + i - j] = A[i, j]
    return ab


# A NaN or infinity below the pivot of a column poisons its row, which can then
# never be a pivot: whether the factorisation ends at a zero pivot or the
# solution turns non-finite first, the call must refuse, never return
# MAFEM_OK with a non-finite x.
@pytest.mark.parametrize("case,codes,text", [("zero column", (M.ZERO_PIVOT,), "column 6"),
                                             ("inf alone in a column", (M.ZERO_PIVOT,), "column 4"),
                                             ("nan in the right-hand side", (M.NAN_DETECTED,), "NaN"),
                                             ("inf in the right-hand side", (M.NAN_DETECTED,), "NaN"),
                                             ("nan below a pivot", (M.ZERO_PIVOT, M.NAN_DETECTED), ""),
                                             ("inf below a pivot", (M.ZERO_PIVOT, M.NAN_DETECTED), "")])
def test_noalloc_reports_singular_and_non_finite_systems(case, codes, text):
    n, kl = 40, 5
    ab = _small_band(n, kl, seed=11)
    rhs = np.ones(n)
    if case == "zero column":
        ab[5, :] = 0.0  # column 5 (0-based): every entry zero
    elif case == "inf alone in a column":
        ab[3, :] = 0.0
        ab[3, 2 * kl + 1] = np.inf  # A(4, 3) = Inf, the column's only entry
    elif case == "nan in the right-hand side":
        rhs[17] = np.nan
    elif case == "inf in the right-hand side":
        rhs[3] = -np.inf
    elif case == "nan below a pivot":
        ab[10, 2 * kl + 3] = np.nan  # A(13, 10)
    else:
        ab[10, 2 * kl + 3] = np.inf
    cu = _Cudart()
    try:
        f = _noalloc_fn()
        d_band, d_rhs, d_x = cu.to_device(ab), cu.to_device(rhs), cu.to_device(np.zeros(n))
        rc = f(d_band, n, kl, kl, 3 * kl + 1, d_rhs, d_x, None)
        assert rc in codes, (case, rc)
        assert text in M.lib().mafem_last_error(None).decode()
        d_rhs = cu.to_device(np.ones(n))
        # the next call on a regular system is correct
        good = _small_band(n, kl, seed=12)
        d_band2 = cu.to_device(good)
        assert f(d_band2, n, kl, kl, 3 * kl + 1, d_rhs, d_x, None) == 0
        assert rel(cu.from_device(d_x, n), np.linalg.solve(_dense(good, kl), np.ones(n))) < 1e-12
    finally:
        cu.free()


def test_noalloc_rejects_bad_arguments():
    """Refused before any device work (the pointers are never dereferenced)."""
    f = _noalloc_fn()
    p = C.c_void_p(16)
    cases = [(p, 40, 5, 4, 16, p, p),            # kl != ku
             (p, 40, 5, 5, 15, p, p),            # ldab < 2 kl + ku + 1
             (None, 40, 5, 5, 16, p, p),         # null band
             (p, 40, 5, 5, 16, None, p),         # null rhs
             (p, 40, 5, 5, 16, p, None),         # null x
             (p, 0, 5, 5, 16, p, p),             # n < 1
             (p, 40, 1 << 33, 1 << 33, 3 << 33 | 1, p, p)]  # a bandwidth beyond int: no narrowing
    for band, n, kl, ku, ldab, rhs, x in cases:
        assert f(band, n, kl, ku, ldab, rhs, x, None) == M.ERR_ARG, (n, kl, ku, ldab)


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
