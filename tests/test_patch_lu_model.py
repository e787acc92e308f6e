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
