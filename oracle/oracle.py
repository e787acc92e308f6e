"""ctypes wrapper of the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module.  The product path never loads it.

The oracle is a C++ restatement of MembraneAleFem.jl; see mafem_oracle.cpp for
the reference file:line each function follows.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

# enums (src/input/Enums.jl, src/input/Dof.jl)
F_CAVI, F_COUE, F_POIS, F_PULL, F_BEND = 1, 2, 3, 4, 5
STATIC, EUL, LAG, ALEV, ALEVB = 1, 2, 3, 4, 5
BOTTOM, RIGHT, TOP, LEFT = 1, 2, 3, 4
SHEAR, STRETCH, MOMENT = 1, 2, 3
CLAMPED, CLOSED = 1, 2


class AssertionFailed(AssertionError):
    """The restated reference code hit one of the reference's @asserts."""


class _Params(C.Structure):
    _fields_ = [
        ("motion", C.c_int), ("scenario", C.c_int), ("num1el", C.c_int), ("num2el", C.c_int),
        ("length", C.c_double), ("kb", C.c_double), ("kg", C.c_double), ("zv", C.c_double),
        ("pn", C.c_double), ("poly", C.c_int), ("gp1d", C.c_int), ("nders", C.c_int),
        ("nen", C.c_int), ("adb", C.c_double), ("am", C.c_double), ("eps_k", C.c_double),
        ("eps_nr", C.c_double), ("pull_speed", C.c_double), ("bend_tm", C.c_double),
        ("bend_mf", C.c_double), ("lambda0", C.c_double), ("pull_centre", C.c_int),
    ]


@dataclass
class Params:
    """Mirror of the reference's ``Params`` (src/input/Params.jl:36-55) plus the
    keyword arguments the hot path reads (pull_speed, bend_tm, bend_mf), and two
    F_PULL extensions with no reference keyword: lambda0 (edge tension and
    initial λ; 0 = the reference's kb / 4) and pull_centre (1 = pull the centre
    element (floor(n1/2) + 1, floor(n2/2) + 1) instead of ceil(numel / 2))."""

    motion: int = ALEVB
    scenario: int = F_PULL
    num1el: int = 17
    num2el: int = 17
    length: float = 64.0
    kb: float = 1.0
    kg: float = -0.5
    zv: float = 1.0
    pn: float = 0.0
    poly: int = 2
    gp1d: int = 3
    nders: int = 2
    nen: int = 9
    adb: float | None = None  # defaults to length^2, as in the reference
    am: float = 1.0
    eps_k: float = 1e-15
    eps_nr: float = 1e-12
    pull_speed: float = 0.0
    bend_tm: float = 1.0
    bend_mf: float = 0.0
    lambda0: float = 0.0
    pull_centre: int = 0

    def to_c(self) -> _Params:
        adb = self.length ** 2 if self.adb is None else self.adb
        return _Params(self.motion, self.scenario, self.num1el, self.num2el, self.length,
                       self.kb, self.kg, self.zv, self.pn, self.poly, self.gp1d, self.nders,
                       self.nen, adb, self.am, self.eps_k, self.eps_nr, self.pull_speed,
                       self.bend_tm, self.bend_mf, self.lambda0, self.pull_centre)


def build() -> str:
    """Compile the oracle with its Makefile (g++, a few seconds)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_last_error.restype = C.c_char_p
        L.orc_mesh_destroy.argtypes = [C.c_void_p]
        for name in ("orc_mesh_sizes", "orc_mesh_dofs", "orc_mesh_IX", "orc_mesh_ID",
                     "orc_mesh_LM", "orc_mesh_ID_inv", "orc_mesh_knots", "orc_mesh_area",
                     "orc_mesh_bdry", "orc_mesh_bdry_elems", "orc_mesh_bdry_nodes",
                     "orc_mesh_neu", "orc_mesh_dir", "orc_prepare_input", "orc_gds",
                     "orc_elem_r_K", "orc_calc_r_K", "orc_update_xms", "orc_time_step", "orc_pull_force"):
            getattr(L, name).argtypes = None
        _lib = L
    return _lib


def _chk(rc: int):
    if rc == 1:
        raise AssertionFailed(lib().orc_last_error().decode())
    if rc != 0:
        raise RuntimeError(lib().orc_last_error().decode())


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


# ---- spline / Gauss / basis-level functions ---------------------------------

class KnotVector:
    """Knot list + polynomial order + curve (src/input/Spline.jl:20-61)."""

    def __init__(self, zs, poly: int, curve: int = CLAMPED):
        self.zs = _f64(zs)
        self.poly = int(poly)
        self.curve = int(curve)
        nel = C.c_int()
        _chk(lib().orc_knot_vector_check(_dp(self.zs), len(self.zs), self.poly, self.curve,
                                         C.byref(nel)))
        self.nel = nel.value

    @classmethod
    def uniform(cls, nel: int, poly: int, curve: int = CLAMPED):
        out = np.zeros(nel + 2 * poly + 1)
        _chk(lib().orc_knot_vector_uniform(nel, poly, curve, _dp(out)))
        return cls(out, poly, curve)

    def __eq__(self, o):
        return (np.array_equal(self.zs, o.zs) and self.poly == o.poly and self.curve == o.curve)

    def __hash__(self):
        return hash((self.zs.tobytes(), self.poly, self.curve))

    def _a(self):
        return (_dp(self.zs), len(self.zs), self.poly, self.curve)


def get_fine_zs(nel: int, poly: int) -> np.ndarray:
    out = np.zeros(nel + 2 * poly + 1)
    _chk(lib().orc_fine_zs(nel, poly, _dp(out)))
    return out


def get_knot_span_index(kv: KnotVector, z: float) -> int:
    out = C.c_int()
    _chk(lib().orc_knot_span(*kv._a(), C.c_double(z), C.byref(out)))
    return out.value


def get_bspline_vals(kv: KnotVector, z: float) -> np.ndarray:
    out = np.zeros(kv.poly + 1)
    _chk(lib().orc_bspline_vals(*kv._a(), C.c_double(z), _dp(out)))
    return out


def get_bspline_ders(kv: KnotVector, z: float, nders: int) -> np.ndarray:
    out = np.zeros((kv.poly + 1) * (max(nders, 0) + 1))
    _chk(lib().orc_bspline_ders(*kv._a(), C.c_double(z), int(nders), _dp(out)))
    return out.reshape((max(nders, 0) + 1, kv.poly + 1)).T


def get_bspline_indices(kv: KnotVector, z: float) -> list:
    out = np.zeros(kv.poly + 1, dtype=np.int32)
    _chk(lib().orc_bspline_indices(*kv._a(), C.c_double(z), _ip(out)))
    return [int(v) for v in out]


def collocate_z(kv: KnotVector) -> np.ndarray:
    out = np.zeros(len(kv.zs))
    n = C.c_int()
    _chk(lib().orc_collocate(*kv._a(), _dp(out), C.byref(n)))
    return out[: n.value]


_FN1 = C.CFUNCTYPE(C.c_double, C.c_double)
_FN2 = C.CFUNCTYPE(C.c_double, C.c_double, C.c_double)


def get_1d_bspline_cps(kv: KnotVector, f) -> np.ndarray:
    out = np.zeros(len(kv.zs))
    n = C.c_int()
    cb = _FN1(lambda z: float(f(z)))
    _chk(lib().orc_1d_cps(*kv._a(), cb, _dp(out), C.byref(n)))
    return out[: n.value]


def get_2d_bspline_cps(kv1: KnotVector, kv2: KnotVector, f) -> np.ndarray:
    n1 = len(kv1.zs) - kv1.poly - 1
    n2 = len(kv2.zs) - kv2.poly - 1
    out = np.zeros(n1 * n2)
    cb = _FN2(lambda a, b: float(f(a, b)))
    _chk(lib().orc_2d_cps(_dp(kv1.zs), len(kv1.zs), _dp(kv2.zs), len(kv2.zs), kv1.poly, cb,
                          _dp(out)))
    return out


def get_unique_1d_elements(kv: KnotVector):
    ne = len(kv.zs)
    un, nel = C.c_int(), C.c_int()
    ids = np.zeros(ne, dtype=np.int32)
    lst = np.zeros(2 * ne)
    _chk(lib().orc_unique_1d(*kv._a(), C.byref(un), C.byref(nel), _ip(ids), _dp(lst)))
    u = un.value
    return u, nel.value, [int(v) for v in ids[: nel.value]], [
        (float(lst[2 * q]), float(lst[2 * q + 1])) for q in range(u)]


def gauss_xi(ngp: int):
    xs, ws = np.zeros(ngp), np.zeros(ngp)
    _chk(lib().orc_gauss_xi(ngp, _dp(xs), _dp(ws)))
    return xs, ws


def gauss_zeta(ngp: int, lo: float, hi: float):
    zs, ws = np.zeros(ngp), np.zeros(ngp)
    _chk(lib().orc_gauss_zeta(ngp, C.c_double(lo), C.c_double(hi), _dp(zs), _dp(ws)))
    return zs, ws


@dataclass
class Fz:
    """GpBasisFnsζ (src/input/GpBasisFn.jl:20-55)."""
    w: float
    N: np.ndarray
    dN: np.ndarray
    ddN: np.ndarray

    @classmethod
    def unpack(cls, a):
        a = np.asarray(a)
        return cls(float(a[0]), a[1:4].copy(), a[4:7].copy(), a[7:10].copy())

    def pack(self):
        return np.concatenate([[self.w], self.N, self.dN, self.ddN])

    def __eq__(self, o):
        return np.array_equal(self.pack(), o.pack())


def gp_basis_fns_z(w: float, z: float, kv: KnotVector) -> Fz:
    out = np.zeros(10)
    _chk(lib().orc_gp_fns_z(C.c_double(w), C.c_double(z), *kv._a(), _dp(out)))
    return Fz.unpack(out)


@dataclass
class Fza:
    """GpBasisFnsζα (src/input/GpBasisFn.jl:96-112)."""
    w: float
    N: np.ndarray      # (9,)
    dN: np.ndarray     # (9, 2)
    ddN: np.ndarray    # (9, 3)

    @classmethod
    def unpack(cls, a):
        a = np.asarray(a)
        return cls(float(a[0]), a[1:10].copy(), a[10:28].reshape(2, 9).T.copy(),
                   a[28:55].reshape(3, 9).T.copy())


def gp_basis_fns_za(f1: Fz, f2: Fz) -> Fza:
    out = np.zeros(55)
    _chk(lib().orc_gp_fns_za(_dp(_f64(f1.pack())), _dp(_f64(f2.pack())), _dp(out)))
    return Fza.unpack(out)


class LineGpBasisFns:
    """src/input/GpBasisFn.jl:143-202."""

    def __init__(self, kv: KnotVector, ngp: int):
        ne = len(kv.zs)
        nel, nu = C.c_int(), C.c_int()
        ids = np.zeros(ne, dtype=np.int32)
        uf = np.zeros(ne * ngp * 10)
        zmin, zmax = np.zeros(10), np.zeros(10)
        _chk(lib().orc_line_gp_fns(*kv._a(), ngp, C.byref(nel), C.byref(nu), _ip(ids), _dp(uf),
                                   _dp(zmin), _dp(zmax)))
        self.nel = nel.value
        self.uel_ids = [int(v) for v in ids[: self.nel]]
        self.ufns = [[Fz.unpack(uf[10 * (q * ngp + g): 10 * (q * ngp + g) + 10])
                      for g in range(ngp)] for q in range(nu.value)]
        self.zmin_fns = Fz.unpack(zmin)
        self.zmax_fns = Fz.unpack(zmax)


# ---- mesh-level ------------------------------------------------------------

class Mesh:
    """The reference's ``Mesh`` (src/input/Mesh.jl:48-80), built by the oracle.

    Integer maps are returned with the reference's conventions: 1-based, column
    major, 0 = Dirichlet in ID/LM.
    """

    def __init__(self, p: Params):
        self.p = p
        self._cp = p.to_c()
        h = C.c_void_p()
        _chk(lib().orc_mesh_create(C.byref(self._cp), C.byref(h)))
        self.h = h
        s = np.zeros(12, dtype=np.int32)
        lib().orc_mesh_sizes(self.h, _ip(s))
        (self.num1el, self.num2el, self.numel, self.num1np, self.num2np, self.numnp,
         self.ndf, self.nmdf, self.n_uel, self.half_bw, self.n_neu, self.n_dir) = [int(v) for v in s]
        d = np.zeros(8, dtype=np.int32)
        lib().orc_mesh_dofs(self.h, _ip(d))
        self.dofs = [int(v) for v in d]  # dofs[u-1] for Unknown u = vx..pm

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().orc_mesh_destroy(self.h)
        except Exception:
            pass

    @property
    def IX(self):
        a = np.zeros(9 * self.numel, dtype=np.int32)
        lib().orc_mesh_IX(self.h, _ip(a))
        return a.reshape(self.numel, 9).T

    @property
    def ID(self):
        a = np.zeros(self.ndf * self.numnp, dtype=np.int32)
        lib().orc_mesh_ID(self.h, _ip(a))
        return a.reshape(self.numnp, self.ndf).T

    @property
    def LM(self):
        a = np.zeros(9 * self.ndf * self.numel, dtype=np.int32)
        lib().orc_mesh_LM(self.h, _ip(a))
        return a.reshape(self.numel, 9 * self.ndf).T

    @property
    def ID_inv(self):
        a = np.zeros(2 * self.nmdf, dtype=np.int32)
        lib().orc_mesh_ID_inv(self.h, _ip(a))
        return a.reshape(self.nmdf, 2)

    def knots(self):
        k1 = np.zeros(self.num1el + 5)
        k2 = np.zeros(self.num2el + 5)
        lib().orc_mesh_knots(self.h, _dp(k1), _dp(k2))
        return k1, k2

    def area_tables(self):
        ids = np.zeros(self.numel, dtype=np.int32)
        uf = np.zeros(self.n_uel * 9 * 55)
        lib().orc_mesh_area(self.h, _ip(ids), _dp(uf))
        return ids, uf.reshape(self.n_uel, 9, 55)

    def bdry_tables(self, b: int):
        nel, nu = C.c_int(), C.c_int()
        lib().orc_mesh_bdry(self.h, b, C.byref(nel), C.byref(nu), None, None)
        ids = np.zeros(nel.value, dtype=np.int32)
        uf = np.zeros(nu.value * 3 * 55)
        lib().orc_mesh_bdry(self.h, b, C.byref(nel), C.byref(nu), _ip(ids), _dp(uf))
        return ids, uf.reshape(nu.value, 3, 55)

    def bdry_elems(self, b: int):
        n = self.num1el if b in (BOTTOM, TOP) else self.num2el
        a = np.zeros(n, dtype=np.int32)
        lib().orc_mesh_bdry_elems(self.h, b, _ip(a))
        return a

    def bdry_nodes(self, b: int, inner: bool = False):
        n = self.num1np if b in (BOTTOM, TOP) else self.num2np
        a = np.zeros(n, dtype=np.int32)
        lib().orc_mesh_bdry_nodes(self.h, b, int(inner), _ip(a))
        return a

    def neumann(self):
        n = self.n_neu
        b, t, v = np.zeros(n, np.int32), np.zeros(n, np.int32), np.zeros(n)
        lib().orc_mesh_neu(self.h, _ip(b), _ip(t), _dp(v))
        return list(zip(b.tolist(), t.tolist(), v.tolist()))

    def dirichlet(self):
        n = self.n_dir
        u, nd, v = np.zeros(n, np.int32), np.zeros(n, np.int32), np.zeros(n)
        lib().orc_mesh_dir(self.h, _ip(u), _ip(nd), _dp(v))
        return list(zip(u.tolist(), nd.tolist(), v.tolist()))

    # -- analysis ----------------------------------------------------------
    def prepare_input(self):
        """Default initial state of src/Input.jl:22-121 (xms numnp x 3, cps numnp x ndf)."""
        xms = np.zeros((self.numnp, 3), order="F")
        cps = np.zeros((self.numnp, self.ndf), order="F")
        _chk(lib().orc_prepare_input(self.h, _dp(xms), _dp(cps)))
        return xms, cps

    def gds(self, xms, cps, el_id: int, gp_id: int, bdry: int = 0) -> dict:
        xms, cps = np.asfortranarray(xms, dtype=np.float64), np.asfortranarray(cps, dtype=np.float64)
        out = np.zeros(64)
        _chk(lib().orc_gds(self.h, _dp(xms), _dp(cps), int(el_id), int(gp_id), int(bdry), _dp(out)))
        return _unpack_gds(out)

    def elem_r_K(self, xms, cps, el_id: int, time: float, dt: float, area=True, bdry=True,
                 tangent=True):
        xms, cps = np.asfortranarray(xms, dtype=np.float64), np.asfortranarray(cps, dtype=np.float64)
        nd = 9 * self.ndf
        r = np.zeros(nd)
        K = np.zeros((nd, nd), order="F") if tangent else None
        _chk(lib().orc_elem_r_K(self.h, _dp(xms), _dp(cps), int(el_id), C.c_double(time),
                                C.c_double(dt), int(area), int(bdry), _dp(r),
                                _dp(K) if tangent else None))
        return r, K

    def calc_r_K(self, xms, cps, time: float, dt: float, nthreads: int = 0, tangent=True):
        """Residual (nmdf) and band tangent (LAPACK layout, kl = ku = half_bw,
        ldab = 3*half_bw + 1; the top kl rows are fill space)."""
        xms, cps = np.asfortranarray(xms, dtype=np.float64), np.asfortranarray(cps, dtype=np.float64)
        nthreads = nthreads or os.cpu_count() or 1
        b = self.half_bw
        ldab = 3 * b + 1
        r = np.zeros(self.nmdf)
        ab = np.zeros((self.nmdf, ldab)) if tangent else None  # row q = band column q
        _chk(lib().orc_calc_r_K(self.h, _dp(xms), _dp(cps), C.c_double(time), C.c_double(dt),
                                int(nthreads), _dp(r), _dp(ab) if tangent else None, b, b, ldab))
        return r, ab

    def update_xms(self, xms, c, dt: float):
        assert xms.flags.f_contiguous and c.flags.f_contiguous
        lib().orc_update_xms(self.h, _dp(xms), _dp(np.asfortranarray(c)), C.c_double(dt))

    def pull_force(self, xms, cps) -> np.ndarray:
        """calc_pull_force (src/analysis/PullForce.jl:61-80) at the given state: 3-vector."""
        f = np.zeros(3)
        _chk(lib().orc_pull_force(self.h, _dp(np.asfortranarray(xms)), _dp(np.asfortranarray(cps)), _dp(f)))
        return f

    def time_step(self, xms, cps, time: float, dt: float, nthreads: int = 0):
        """time_step! (src/analysis/FiniteElement.jl:11-63), band-LU solve; in place."""
        assert xms.flags.f_contiguous and cps.flags.f_contiguous
        nthreads = nthreads or os.cpu_count() or 1
        it = C.c_int()
        eps = np.zeros(14)
        _chk(lib().orc_time_step(self.h, _dp(xms), _dp(cps), C.c_double(time), C.c_double(dt),
                                 int(nthreads), C.byref(it), _dp(eps)))
        return eps[: it.value]


def bend_errors(mesh: Mesh, xms, cps) -> tuple[float, float, float]:
    """The error norms of ``analyze_output`` (src/Output.jl:129-180) for the
    bending scenario at L = kb = 1, whose state should approach the arc of
    radius 1 about (sin 1, ·, cos 1) with λ = 1/4 and H = 1/2.  Summed over the
    elements and Gauss points in the reference's order, w the parametric Gauss
    weight (get_gpw): Er = Σ w (√((x - sin 1)² + (z - cos 1)²) - 1)² (left
    without the square root, as there), Eλ = √Σ w (λ - 1/4)²,
    EH = √Σ w (H - 1/2)²."""
    import math
    ids, uf = mesh.area_tables()
    er = el = eh = 0.0
    for e2 in range(mesh.num2el):
        for e1 in range(mesh.num1el):
            e = e1 + mesh.num1el * e2
            for g2 in range(3):
                for g1 in range(3):
                    g = g1 + 3 * g2
                    w = uf[ids[e] - 1, g, 0]
                    d = mesh.gds(xms, cps, e + 1, g + 1)
                    x = d["x"]
                    er += w * (math.sqrt((x[0] - math.sin(1.0)) ** 2 + (x[2] - math.cos(1.0)) ** 2) - 1.0) ** 2
                    el += w * (d["lam"] - 0.25) ** 2
                    eh += w * (d["H"] - 0.5) ** 2
    return er, math.sqrt(el), math.sqrt(eh)


def band_to_dense(ab: np.ndarray, kl: int, ku: int, n: int) -> np.ndarray:
    """Band storage (row q = column q of the matrix, offset kl+ku+i-j) -> dense."""
    A = np.zeros((n, n))
    for j in range(n):
        for i in range(max(0, j - ku), min(n, j + kl + 1)):
            A[i, j] = ab[j, kl + ku + i - j]
    return A


def band_to_csr(ab: np.ndarray, kl: int, ku: int, n: int):
    """Band storage -> scipy CSR of the structural band (zeros dropped)."""
    import scipy.sparse as sp
    off = np.arange(-ku, kl + 1)  # i - j
    cols = np.repeat(np.arange(n), len(off))
    rows = cols + np.tile(off, n)
    vals = ab[:, kl + ku + off].reshape(-1)
    keep = (rows >= 0) & (rows < n) & (vals != 0.0)
    return sp.csr_matrix((vals[keep], (rows[keep], cols[keep])), shape=(n, n))


def band_lu(ab: np.ndarray, n: int, kl: int, ku: int):
    ldab = ab.shape[1]
    ipiv = np.zeros(n, dtype=np.int32)
    info = C.c_int()
    _chk(lib().orc_band_lu(n, kl, ku, _dp(ab), ldab, _ip(ipiv), C.byref(info)))
    return ipiv, info.value


def band_solve(ab: np.ndarray, n: int, kl: int, ku: int, ipiv, b):
    x = _f64(b).copy()
    _chk(lib().orc_band_solve(n, kl, ku, _dp(ab), ab.shape[1], _ip(ipiv), _dp(x)))
    return x


_GDS_FIELDS = [("x", (3,)), ("a", (3, 2)), ("aup", (3, 2)), ("J", ()), ("n", (3,)), ("b", (2, 2)),
               ("H", ()), ("K", ()), ("v", (3,)), ("dv", (3, 2)), ("lam", ()), ("pm", ()),
               ("vm", (3,)), ("sig", (3,)), ("sigm", (3,)), ("M", (3,)), ("Gam", (3, 2)), ("ainv", (2, 2))]


def _unpack_gds(out):
    d, o = {}, 0
    for name, shp in _GDS_FIELDS:
        sz = int(np.prod(shp)) if shp else 1
        v = out[o: o + sz]
        o += sz
        d[name] = float(v[0]) if not shp else v.reshape(shp[::-1]).T.copy()
    return d


def time_step_sparse(mesh: Mesh, xms, cps, time: float, dt: float, nthreads: int = 0,
                     max_iter: int = 14):
    """time_step! (FiniteElement.jl:11-63) with the oracle's threaded complex-step
    assembly and scipy's sparse LU (SuperLU) in place of the reference's UMFPACK
    `K \\ r`.  The CPU baseline of the benchmarks.  Updates xms/cps in place and
    returns the list of ε = ‖Δu‖/nmdf."""
    import scipy.sparse.linalg as sla
    assert xms.flags.f_contiguous and cps.flags.f_contiguous
    ID_inv = mesh.ID_inv
    nodes, dofs = ID_inv[:, 0] - 1, ID_inv[:, 1] - 1
    mmo = {LAG: [1, 2, 3], STATIC: []}.get(mesh.p.motion, [4, 5, 6])
    mmo = [mesh.dofs[d - 1] for d in mmo]
    eps = []
    for _ in range(max_iter):
        r, ab = mesh.calc_r_K(xms, cps, time, dt, nthreads=nthreads)
        K = band_to_csr(ab, mesh.half_bw, mesh.half_bw, mesh.nmdf)
        du = -sla.spsolve(K.tocsc(), r)
        dc = np.zeros_like(cps)
        dc[nodes, dofs] = du
        cps += dc
        for j, d in enumerate(mmo):
            if d:
                xms[:, j] += dt * dc[:, d - 1]
        eps.append(float(np.linalg.norm(du) / mesh.nmdf))
        if eps[-1] < mesh.p.eps_nr:
            break
    if not eps[-1] < mesh.p.eps_nr:
        raise AssertionFailed("did not reach Newton--Raphson tolerance")
    return eps


# ---- seeded initial states -------------------------------------------------------------
# The benchmarks' synthetic input: prepare_input's flat patch plus an out-of-plane
# perturbation of the interior nodes drawn from SplitMix64 (Steele, Lea and Flood,
# "Fast splittable pseudorandom number generators", OOPSLA 2014; the published
# constants).  The product's Python layer draws the same numbers; this copy lets the
# CPU baseline build its input without loading the product library.

def splitmix64(seed: int, n: int) -> np.ndarray:
    """n uniform doubles in [0, 1): the top 53 bits of successive SplitMix64 outputs."""
    mask = (1 << 64) - 1
    s = seed & mask
    out = np.empty(n, dtype=np.float64)
    for i in range(n):
        s = (s + 0x9E3779B97F4A7C15) & mask
        z = s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & mask
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & mask
        z ^= z >> 31
        out[i] = (z >> 11) * (1.0 / 9007199254740992.0)
    return out


def perturb_interior_z(mesh: Mesh, xms: np.ndarray, seed: int = 0, amp: float = 1e-4) -> np.ndarray:
    """z += amp (2u - 1), u ~ SplitMix64(seed), on the nodes off the outer boundary."""
    u = splitmix64(seed, mesh.numnp)
    s1 = np.arange(mesh.numnp) % mesh.num1np
    s2 = np.arange(mesh.numnp) // mesh.num1np
    interior = (s1 > 0) & (s1 < mesh.num1np - 1) & (s2 > 0) & (s2 < mesh.num2np - 1)
    xms[:, 2] += np.where(interior, amp * (2.0 * u - 1.0), 0.0)
    return xms


# ---- state files ---------------------------------------------------------------------
# The reference writes xms / cps with DelimitedFiles.writedlm (src/Analysis.jl:76-77,
# src/Input.jl:113-114): print(io, x) of each Float64, '\t' between the entries of a
# row, '\n' after each row.  print(::Float64) is Julia Base's Ryu shortest printer
# (base/ryu/shortest.jl, `writeshortest`; Julia 1.10, the reference's compat): the
# shortest digit string that reads back to x, closest to x, written in fixed notation
# when the decimal point position pt (x = 0.d1d2... x 10^pt) satisfies -4 < pt <= 6,
# else as d.ddd "e" exponent, with ".0" when there is a single digit.  This restatement
# takes the digits from Python's repr, which produces the same shortest-closest digits.

def julia_print_float64(x: float) -> str:
    """print(::Float64) of Julia Base (base/ryu/shortest.jl), restated."""
    import math
    x = float(x)
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "Inf" if x > 0 else "-Inf"
    if x == 0.0:
        return "-0.0" if math.copysign(1.0, x) < 0 else "0.0"
    sign = "-" if x < 0 else ""
    mant, _, ex = f"{abs(x)!r}".partition("e")  # repr: '123.45', '1e-05', '1.5e+16'
    exp10 = int(ex) if ex else 0
    ip, _, fp = mant.partition(".")
    digits = (ip + fp).lstrip("0")
    pt = len(ip.lstrip("0")) + exp10 if ip.strip("0") else exp10 - (len(fp) - len(fp.lstrip("0")))
    digits = digits.rstrip("0") or "0"
    if -4 < pt <= 6:
        if pt <= 0:
            return sign + "0." + "0" * (-pt) + digits
        if pt >= len(digits):
            return sign + digits + "0" * (pt - len(digits)) + ".0"
        return sign + digits[:pt] + "." + digits[pt:]
    return sign + digits[0] + "." + (digits[1:] or "0") + "e" + str(pt - 1)


def writedlm_text(a) -> str:
    """The text writedlm produces for a Float64 matrix (rows joined by '\\n')."""
    a = np.atleast_2d(np.asarray(a, dtype=np.float64))
    return "".join("\t".join(julia_print_float64(v) for v in row) + "\n" for row in a)
