"""numpy model of the batched FP32 factorisation and its refinement (test
infrastructure: a numerical model, never the thing measured or shipped).

It restates, in float32 numpy, the algorithm the batched FP32 form runs one
CTA per patch.  Per panel of whole node blocks (at most 32 columns):

1. Factor the w x w diagonal block with node-block pivoting.  The pivot of
   column k is the largest entry among the not-yet-eliminated rows of k's
   node block; rows below the panel never pivot.
2. Form explicit inverses Li = L11^-1, Ui = U11^-1 and Mi = Ui Li.
3. Form U12 = Li P A12 and Y = Mi P A12, and update A22 -= A21 Y with the raw
   A21 (FP32 accumulation).

The FP32 substitutions use the same stored quantities.  The refinement
repeats x += LU^-1 (b - A0 x), with the residual taken in FP64 against the
FP32 tangent A0.  It stops when the last correction is at most tol |x|.

`double_float_residual` restates how the batched refinement forms that
residual on the FP32 pipe (double-float arithmetic).

The model answers numerical questions about that scheme on the oracle's
tangents (growth, refinement contraction, sweeps per solve, residual
accuracy) without a GPU.
Dense float32 storage: meant for patches up to 32 x 32 elements.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sl


def band_matvec(ab: np.ndarray, kl: int, x: np.ndarray) -> np.ndarray:
    """A x for the oracle's band layout (row q holds column q, A[i, q] at
    ab[q, 2 kl + i - q], kl = ku), in FP64."""
    n = ab.shape[0]
    y = np.zeros(n)
    q = np.arange(n)
    for off in range(-kl, kl + 1):
        i = q + off
        ok = (i >= 0) & (i < n)
        y[i[ok]] += ab[q[ok], 2 * kl + off] * x[q[ok]]
    return y


def dense_from_band(ab: np.ndarray, kl: int, dtype=np.float32) -> np.ndarray:
    n = ab.shape[0]
    A = np.zeros((n, n), dtype=dtype)
    q = np.arange(n)
    for off in range(-kl, kl + 1):
        i = q + off
        ok = (i >= 0) & (i < n)
        A[i[ok], q[ok]] = ab[q[ok], 2 * kl + off]
    return A


def node_blocks(id_inv: np.ndarray) -> np.ndarray:
    """blk_end[k]: one past the last unknown of k's node (ID_inv rows are
    (node, dof), 1-based, node-major as src/input/Mesh.jl:291-296 builds them)."""
    node = np.asarray(id_inv)[:, 0]
    n = len(node)
    blk_end = np.zeros(n, dtype=int)
    q = 0
    while q < n:
        e = q
        while e < n and node[e] == node[q]:
            e += 1
        blk_end[q:e] = e
        q = e
    return blk_end


def panels_of(blk_end: np.ndarray, wmax: int = 32) -> tuple[list[int], int]:
    """Panel starts (runs of whole node blocks, at most wmax wide) and ndfp
    (largest block - 1: the U fill beyond ku)."""
    n = len(blk_end)
    ps, j0, ndfp = [0], 0, 0
    while j0 < n:
        j1 = j0
        while j1 < n and blk_end[j1] - j0 <= wmax:
            ndfp = max(ndfp, int(blk_end[j1]) - j1 - 1)
            j1 = int(blk_end[j1])
        if j1 == j0:
            raise ValueError("a node block wider than the panel")
        ps.append(j1)
        j0 = j1
    return ps, ndfp


class PatchLU:
    """The FP32 factors of one patch's tangent."""

    def __init__(self, ab0: np.ndarray, kl: int, blk_end: np.ndarray):
        A = dense_from_band(ab0, kl, np.float32)
        n = A.shape[0]
        ps, ndfp = panels_of(blk_end)
        kuf = kl + ndfp
        f32 = np.float32
        self.panels, self.growth = [], 0.0
        for p in range(len(ps) - 1):
            j0, j1 = ps[p], ps[p + 1]
            w = j1 - j0
            R, C = min(n - j0, w + kl), min(n, j1 + kuf) - j1
            D = A[j0:j1, j0:j1].copy()
            eliminated = np.zeros(w, bool)
            perm = np.zeros(w, int)
            bend = np.asarray(blk_end[j0:j1]) - j0
            for k in range(w):
                cand = np.nonzero(~eliminated & (np.arange(w) < bend[k]))[0]
                pr = cand[np.argmax(np.abs(D[cand, k]))]
                if D[pr, k] == 0.0 or not np.isfinite(D[pr, k]):
                    raise ZeroDivisionError(f"no usable pivot in column {j0 + k}")
                perm[k] = pr
                eliminated[pr] = True
                act = ~eliminated
                l = D[act, k] / D[pr, k]
                D[act, k + 1:] -= np.outer(l, D[pr, k + 1:]).astype(f32)
                D[act, k] = l
            PD = D[perm]
            L11 = np.tril(PD, -1) + np.eye(w, dtype=f32)
            U11 = np.triu(PD)
            eye = np.eye(w, dtype=f32)
            Li = sl.solve_triangular(L11, eye, lower=True, unit_diagonal=True).astype(f32)
            Ui = sl.solve_triangular(U11, eye, lower=False).astype(f32)
            Mi = (Ui @ Li).astype(f32)
            a = A[j0:j1, j1:j1 + C][perm]
            U12 = (Li @ a).astype(f32)
            Y = (Mi @ a).astype(f32)
            A21 = A[j1:j0 + R, j0:j1].copy()
            A[j1:j0 + R, j1:j1 + C] -= (A21 @ Y).astype(f32)
            A[j0:j1, j1:j1 + C] = U12
            self.growth = max(self.growth, float(np.abs(U11).max()), float(np.abs(U12).max()) if C else 0.0)
            self.panels.append((j0, j1, R, C, perm, Li, Ui, U12, A21))

    def solve(self, b: np.ndarray) -> np.ndarray:
        """LU^-1 b in FP32 with the stored inverses (forward, then backward)."""
        f32 = np.float32
        z = b.astype(f32)
        for (j0, j1, R, C, perm, Li, Ui, U12, A21) in self.panels:
            y = (Li @ z[j0:j1][perm]).astype(f32)
            z[j1:j0 + R] -= (A21 @ (Ui @ y).astype(f32)).astype(f32)
            z[j0:j1] = y
        for (j0, j1, R, C, perm, Li, Ui, U12, A21) in reversed(self.panels):
            z[j0:j1] = (Ui @ (z[j0:j1] - U12 @ z[j1:j1 + C]).astype(f32)).astype(f32)
        return z.astype(np.float64)


def refine(lu: PatchLU, ab0: np.ndarray, kl: int, b: np.ndarray, tol: float = 1e-4, max_sweeps: int = 30,
           predicted: bool = False):
    """x with |last correction| <= tol |x|; returns (x, corrections |d_k| / |x|).
    predicted=True: the batched kernel's rule (patch_refine_kernel) -- also stop
    once the predicted next correction rho |d_k|, rho = |d_k| / |d_k-1|, is at
    most tol |x| while the sweeps contract (rho <= 1/2)."""
    x = np.zeros(len(b))
    res = b.copy()
    hist = []
    prev = np.inf
    for k in range(max_sweeps):
        d = lu.solve(res)
        x += d
        dn, xn = float(np.linalg.norm(d)), float(np.linalg.norm(x))
        hist.append(dn / max(xn, 1e-300))
        rho = dn / prev
        if dn <= tol * xn or (predicted and k >= 1 and rho <= 0.5 and rho * dn <= tol * xn):
            break
        prev = dn
        res = b - band_matvec(ab0, kl, x)
    return x, hist


def _fma32(a, b, c):
    """fmaf(a, b, c) for float32 arrays: the product is exact in float64 and the
    sum is rounded to float32 (double rounding through float64 can differ from a
    true FMA in the last bit, far below what the model measures)."""
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(np.float32)


def double_float_residual(ab0: np.ndarray, kl: int, b: np.ndarray, x: np.ndarray) -> np.ndarray:
    """b - A0 x as the batched refinement forms it on the FP32 pipe: x split into
    two floats (xh + xl), each term a xh = p + e exactly by FMA (plus a xl), and
    the row sum kept as an unevaluated float pair (sh, sl) updated by Knuth's
    TwoSum with explicit roundings, one column at a time from the left edge of
    the band; the pair is added in FP64 at the end."""
    n = ab0.shape[0]
    f32 = np.float32
    a0 = ab0.astype(f32)
    xh = x.astype(f32)
    xl = (x - xh.astype(np.float64)).astype(f32)
    sh = np.zeros(n, f32)
    sl = np.zeros(n, f32)
    rows = np.arange(n)
    for off in range(-kl, kl + 1):  # column j = i + off, left to right within each row's window
        j = rows + off
        ok = (j >= 0) & (j < n)
        i, jj = rows[ok], j[ok]
        a = a0[jj, 2 * kl + (i - jj)]
        p = (a * xh[jj]).astype(f32)
        e = _fma32(a, xl[jj], _fma32(a, xh[jj], -p))
        t = (sh[i] + p).astype(f32)
        z = (t - sh[i]).astype(f32)
        corr = ((sh[i] - (t - z).astype(f32)).astype(f32) + (p - z).astype(f32)).astype(f32)
        sl[i] = (sl[i] + (corr + e).astype(f32)).astype(f32)
        sh[i] = t
    return b - (sh.astype(np.float64) + sl.astype(np.float64))


def coupled_runs(unk_node: np.ndarray, node_first: np.ndarray, num1np: int, num2np: int, rb: int, n: int,
                 kl: int) -> list[tuple[int, int]]:
    """The column runs [j0, j1) that the batched refinement residual walks for
    the 32 rows rb .. rb + 31 (patch_residual in band_lu_patch.cu), in
    increasing order: grid row g couples to points [s1a - 2, W) through the
    rows' points on grid row s2a, to [0, s1b + 2] through those on grid row
    s2b, and to the whole grid row through any grid row between them; each
    run clipped to the band window [rb - kl, rb + 32 + kl)."""
    W, H = num1np, num2np
    jlo, jhi = max(rb - kl, 0), min(n, rb + 32 + kl)
    na, nb = int(unk_node[rb]), int(unk_node[min(rb + 31, n - 1)])
    s1a, s2a, s1b, s2b = na % W, na // W, nb % W, nb // W
    runs = []
    for g in range(max(s2a - 2, 0), min(s2b + 2, H - 1) + 1):
        c0, c1, d0, d1 = 0, -1, 0, -1
        fa, fb = abs(g - s2a) <= 2, abs(g - s2b) <= 2
        fm = s2b - s2a >= 2 and s2a - 1 <= g <= s2b + 1
        if s2a == s2b:
            c0, c1 = max(s1a - 2, 0), min(s1b + 2, W - 1)
        elif fm or (fa and fb and s1b + 3 >= s1a - 2):
            c1 = W - 1
        else:
            if fb:
                c1 = min(s1b + 2, W - 1)
            if fa:
                d0, d1 = max(s1a - 2, 0), W - 1
        for e0, e1 in ((c0, c1), (d0, d1)):
            if e1 < e0:
                continue
            j0, j1 = max(int(node_first[g * W + e0]), jlo), min(int(node_first[g * W + e1 + 1]), jhi)
            if j0 < j1:
                runs.append((j0, j1))
    return runs
