"""The batched FP32 factorisation as a numpy model (oracle/patch_lu_model.py)
on the oracle's tangents: node-block pivoting with explicit inverses keeps the
growth moderate and the FP64 refinement contracting fast on the stiffest
tangents of the batched workload's parameter range (kb = 0.5, the low end of
its log-uniform [0.5, 2]).  Refined to 1e-8, the solution matches an FP64
band LU within five sweeps, each correction at most a twentieth of the last.  The CUDA kernels implement this
model (its results against the oracle: tests/test_batch.py, test_serving.py).
"""
import numpy as np
import pytest
import scipy.linalg.lapack as lapack

from _cases import M, O, params_pair, state
import patch_lu_model as PM

DT = 0.005


@pytest.mark.parametrize("motion,n", [(M.ALEVB, 12), (M.LAG, 12), (M.ALEVB, 24)])
def test_fp32_node_block_lu_refines_stiff_tangents(motion, n):
    p, q = params_pair(motion, M.F_PULL, n, n, kb=0.5, pull_speed=0.01)
    mesh, om = M.Mesh(p), O.Mesh(q)
    xms, cps = state(p, mesh, seed=3, amp=1e-4)
    om.update_xms(xms, cps, DT)
    r, ab = om.calc_r_K(xms, cps, DT, DT, nthreads=2)
    kl = om.half_bw
    ab0 = ab.astype(np.float32).astype(np.float64)  # the FP32 tangent the refinement solves
    lu = PM.PatchLU(ab0, kl, PM.node_blocks(om.ID_inv))
    assert lu.growth < 1e4
    x, hist = PM.refine(lu, ab0, kl, -r, tol=1e-8)
    assert len(hist) <= 5 and hist[-1] <= 1e-8
    ratios = np.array(hist[2:]) / np.array(hist[1:-1])
    assert len(ratios) >= 1 and np.all(ratios < 0.05), hist
    f, piv, info = lapack.dgbtrf(np.asfortranarray(ab0.T), kl, kl)
    assert info == 0
    x64, _ = lapack.dgbtrs(f, kl, kl, -r, piv)
    assert np.linalg.norm(x - x64) <= 1e-7 * np.linalg.norm(x64)


def test_double_float_residual_is_fp64_accurate():
    """The refinement's residual b - A0 x in double-float arithmetic on the FP32
    pipe (PM.double_float_residual, as the batched refinement forms it): each
    row within 2^-40 of its terms' magnitude sum Σ|a_ij x_j| (measured ≈ 2^-44 on
    the batch's stiffest tangents), against an extended-precision sum."""
    p, q = params_pair(M.ALEVB, M.F_PULL, 16, 16, kb=0.5, pull_speed=0.01)
    mesh, om = M.Mesh(p), O.Mesh(q)
    xms, cps = state(p, mesh, seed=4, amp=1e-4)
    om.update_xms(xms, cps, DT)
    r, ab = om.calc_r_K(xms, cps, DT, DT, nthreads=2)
    kl = om.half_bw
    ab0 = ab.astype(np.float32).astype(np.float64)
    lu = PM.PatchLU(ab0, kl, PM.node_blocks(om.ID_inv))
    x, _ = PM.refine(lu, ab0, kl, -r, tol=1e-6)
    b = -r
    df = PM.double_float_residual(ab0, kl, b, x)
    n = len(b)
    exact = np.zeros(n, dtype=np.longdouble)
    mag = np.zeros(n)
    rows = np.arange(n)
    for off in range(-kl, kl + 1):
        j = rows + off
        ok = (j >= 0) & (j < n)
        i, jj = rows[ok], j[ok]
        a = ab0[jj, 2 * kl + (i - jj)]
        exact[i] += a.astype(np.longdouble) * x[jj].astype(np.longdouble)
        mag[i] += np.abs(a * x[jj])
    err = np.abs(df.astype(np.longdouble) - (b.astype(np.longdouble) - exact)).astype(np.float64)
    assert np.all(err <= 2.0**-40 * mag)


@pytest.mark.parametrize("motion,n", [(M.ALEVB, 12), (M.LAG, 12), (M.ALEVB, 24)])
@pytest.mark.parametrize("tol", [1e-4, 1e-8])
def test_predicted_correction_stop_keeps_the_error_bound(motion, n, tol):
    """The batched refinement's stopping rule (stop once rho |d_k| <= tol |x|
    while the sweeps contract, rho = |d_k| / |d_k-1|): never more sweeps than
    the plain |d_k| <= tol |x| rule, and the forward error of x against an FP64
    band LU still within tol |x| (a factor 2 for the estimate of rho)."""
    p, q = params_pair(motion, M.F_PULL, n, n, kb=0.5, pull_speed=0.01)
    mesh, om = M.Mesh(p), O.Mesh(q)
    xms, cps = state(p, mesh, seed=3, amp=1e-4)
    om.update_xms(xms, cps, DT)
    r, ab = om.calc_r_K(xms, cps, DT, DT, nthreads=2)
    kl = om.half_bw
    ab0 = ab.astype(np.float32).astype(np.float64)
    lu = PM.PatchLU(ab0, kl, PM.node_blocks(om.ID_inv))
    x_plain, h_plain = PM.refine(lu, ab0, kl, -r, tol=tol)
    x_pred, h_pred = PM.refine(lu, ab0, kl, -r, tol=tol, predicted=True)
    assert len(h_pred) <= len(h_plain)
    f, piv, info = lapack.dgbtrf(np.asfortranarray(ab0.T), kl, kl)
    assert info == 0
    x64, _ = lapack.dgbtrs(f, kl, kl, -r, piv)
    assert np.linalg.norm(x_pred - x64) <= 2 * tol * np.linalg.norm(x64)


@pytest.mark.parametrize("motion,n1,n2", [(M.ALEVB, 12, 12), (M.LAG, 9, 9), (M.ALEVB, 16, 10), (M.LAG, 5, 7),
                                          (M.ALEV, 7, 7), (M.EUL, 6, 8)])
def test_refinement_residual_runs_cover_the_tangent(motion, n1, n2):
    """The batched refinement residual walks only the columns a warp's 32 rows
    couple to (patch_residual): on the oracle's assembled tangent every
    nonzero of those rows lies in one of the runs, and the runs are increasing,
    disjoint and inside the band window -- so the double-float sums equal the
    walk of the whole window, whose other entries are stored zeros."""
    p, q = params_pair(motion, M.F_PULL, n1, n2, pull_speed=0.3, pull_centre=1)
    mesh, om = M.Mesh(p), O.Mesh(q)
    xms, cps = state(p, mesh, seed=1, amp=1e-3)
    r, ab = om.calc_r_K(xms, cps, 0.01, 0.01, nthreads=2)
    kl = om.half_bw
    K = PM.dense_from_band(ab, kl, dtype=np.float64)
    n = K.shape[0]
    ID = np.asarray(mesh.ID)
    if ID.shape[0] != mesh.numnp:
        ID = ID.T
    unk_node = np.zeros(n, dtype=int)
    for nd in range(mesh.numnp):
        for d in range(mesh.ndf):
            if ID[nd, d] > 0:
                unk_node[ID[nd, d] - 1] = nd
    assert np.all(np.diff(unk_node) >= 0)  # the kernel's precondition (checked again at mafem_create)
    node_first = np.concatenate([[0], np.cumsum(np.bincount(unk_node, minlength=mesh.numnp))])
    walked = full = 0
    for rb in range(0, n, 32):
        runs = PM.coupled_runs(unk_node, node_first, mesh.num1np, mesh.num2np, rb, n, kl)
        jlo, jhi = max(rb - kl, 0), min(n, rb + 32 + kl)
        cover = np.zeros(n, dtype=bool)
        last = jlo
        for j0, j1 in runs:
            assert last <= j0 < j1 <= jhi
            last = j1
            cover[j0:j1] = True
            walked += j1 - j0
        full += jhi - jlo
        nz = np.nonzero(np.any(K[rb:min(rb + 32, n)] != 0, axis=0))[0]
        assert np.all(cover[nz])
    assert walked < full
