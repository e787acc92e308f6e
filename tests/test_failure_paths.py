"""Failure detection on the GPU path, every failure made on the host.

The reference stops on an @assert (src/analysis/FiniteElement.jl:61 for Newton;
Params.jl:70-125 for bad input).  The library returns a status instead, and
each status has a test here that provokes it from host-side data only:

* MAFEM_NAN_DETECTED: a NaN written into the uploaded state;
* MAFEM_ZERO_PIVOT and the full-pivoting fallback: small band systems built
  on the host and solved through the handle's own factorisation
  (mafem_solve_band) -- a node block without a usable pivot is solved by the
  fallback, a singular matrix is reported;
* MAFEM_REFINE_STALLED: the FP32 form with its refinement capped at one sweep;
* a bounded inter-CTA wait that runs out: the back substitution is told to
  withhold one panel's completion flag and to give up after a few polls
  (mafem_set_wait_test); the call returns MAFEM_ERR_CUDA, every CTA returns,
  the state is left as it was, and the next step on the same handle runs.

No kernel is made to fault, trap or hang.
"""
import numpy as np
import pytest

from _cases import M, O, params_pair, rel, state

pytestmark = pytest.mark.gpu


def _patch(motion=M.ALEVB, n=6, **kw):
    p, q = params_pair(motion, M.F_PULL, n, n, pull_speed=0.5, **kw)
    mesh = M.Mesh(p)
    xms, cps = state(p, mesh, seed=3, amp=1e-3)
    return p, q, mesh, xms, cps


@pytest.mark.parametrize("precision", [M.PLAIN_FP64, M.FP32_REFINE])
def test_nan_in_state_is_reported(precision):
    p, _, mesh, xms, cps = _patch()
    node = mesh.num1np * (mesh.num2np // 2) + mesh.num1np // 2  # an interior node
    cps[node, mesh.dofs[2] - 1] = np.nan  # vz
    with M.Solver(mesh, p, precision) as s:
        with pytest.raises(M.MafemError) as e:
            s.time_step(xms.copy(order="F"), cps.copy(order="F"), 0.01, 0.01)
        assert e.value.code == M.NAN_DETECTED


def test_nan_in_one_patch_of_a_batch():
    """The batched FP32 solve: the patch with the NaN reports it, the other
    patch's step completes and matches the oracle."""
    p, q, mesh, xms, cps = _patch()
    bad = cps.copy(order="F")
    bad[mesh.num1np * 3 + 3, mesh.dofs[0] - 1] = np.nan
    s1, s2 = M.Solver(mesh, p, M.FP32_REFINE), M.Solver(mesh, p, M.FP32_REFINE)
    try:
        s1.upload(xms, bad)
        s2.upload(xms, cps)
        with M.Batch([s1, s2]) as b:
            st, _ = b.step(0.01, 0.01)
        assert st == [M.NAN_DETECTED, M.OK]
        om = O.Mesh(q)
        xo, co = xms.copy(order="F"), cps.copy(order="F")
        om.update_xms(xo, co, 0.01)
        om.time_step(xo, co, 0.01, 0.01, nthreads=2)
        x2, c2 = s2.download()
        assert rel(x2, xo) < 1e-8 and rel(c2, co) < 1e-8
    finally:
        s1.close()
        s2.close()


def _random_band(mesh, kl, seed):
    """A diagonally dominant band matrix in calc_r_K's layout (row j = column j,
    A(i, j) at [j, 2 kl + i - j]) and its dense form."""
    n = mesh.nmdf
    rng = np.random.default_rng(seed)
    dense = np.zeros((n, n))
    for j in range(n):
        lo, hi = max(0, j - kl), min(n, j + kl + 1)
        dense[lo:hi, j] = rng.uniform(-1.0, 1.0, hi - lo)
    dense[np.arange(n), np.arange(n)] += 2.0 * kl
    return dense


def _to_band(dense, kl):
    n = dense.shape[0]
    ab = np.zeros((n, 3 * kl + 1))
    for j in range(n):
        for i in range(max(0, j - kl), min(n, j + kl + 1)):
            ab[j, 2 * kl + i - j] = dense[i, j]
    return ab


@pytest.mark.parametrize("precision", [M.PLAIN_FP64, M.FP32_REFINE])
def test_node_block_without_pivot_falls_back_to_full_pivoting(precision):
    p, _, mesh, _, _ = _patch()
    kl = mesh.half_bw
    dense = _random_band(mesh, kl, seed=5)
    # column 0's entries in its node block (the unknowns of the first node with
    # free unknowns) are zero: node-block pivoting has no pivot there, full
    # partial pivoting takes one from a later row
    nodes = mesh.ID_inv[:, 0]
    blk = int(np.argmax(nodes != nodes[0]))
    assert 1 <= blk <= kl
    dense[:blk, 0] = 0.0
    dense[blk, 0] = 3.0 * kl
    rhs = np.random.default_rng(6).uniform(-1, 1, mesh.nmdf)
    x_ref = np.linalg.solve(dense, rhs)
    with M.Solver(mesh, p, precision) as s:
        f0 = s.fallback_count()
        x = s.solve_band(_to_band(dense, kl), rhs)
        assert s.fallback_count() == f0 + 1
    # FP32 form: the refinement solves the FP32-rounded matrix
    tol = 1e-12 if precision == M.PLAIN_FP64 else 1e-6
    assert rel(x, x_ref) < tol


@pytest.mark.parametrize("precision", [M.PLAIN_FP64, M.FP32_REFINE])
def test_singular_band_reports_zero_pivot(precision):
    p, _, mesh, _, _ = _patch()
    kl = mesh.half_bw
    dense = _random_band(mesh, kl, seed=7)
    dense[:, 5] = 0.0  # an all-zero column
    rhs = np.ones(mesh.nmdf)
    with M.Solver(mesh, p, precision) as s:
        with pytest.raises(M.MafemError) as e:
            s.solve_band(_to_band(dense, kl), rhs)
        assert e.value.code == M.ZERO_PIVOT
        # the handle still works afterwards
        x = s.solve_band(_to_band(_random_band(mesh, kl, seed=8), kl), rhs)
        assert np.all(np.isfinite(x))


def test_refinement_cap_reports_stall():
    p, _, mesh, xms, cps = _patch()
    with M.Solver(mesh, p, M.FP32_REFINE) as s:
        s.set_refinement(1, 1e-14)
        with pytest.raises(M.MafemError) as e:
            s.time_step(xms.copy(order="F"), cps.copy(order="F"), 0.01, 0.01)
        assert e.value.code == M.REFINE_STALLED
    # the batched solve hands the stalled iteration to the handle's own solver,
    # which stalls too
    with M.Solver(mesh, p, M.FP32_REFINE) as s:
        s.set_refinement(1, 1e-14)
        s.upload(xms, cps)
        with M.Batch([s]) as b:
            st, _ = b.step(0.01, 0.01)
        assert st == [M.REFINE_STALLED]


def test_bounded_wait_runs_out_and_the_handle_recovers():
    p, q, mesh, xms, cps = _patch(n=8)
    dt = 0.01
    with M.Solver(mesh, p, M.PLAIN_FP64) as s:
        s.upload(xms, cps)
        s.predict(dt)
        x_pred, c_pred = s.download()
        s.set_wait_test(1 << 10, 0)  # withhold the last panel's flag, give up after 1024 polls
        with pytest.raises(M.MafemError) as e:
            s.time_step_resident(dt, dt)
        assert e.value.code == M.ERR_CUDA and "bounded wait" in str(e.value)
        x1, c1 = s.download()  # the failed iteration left the state alone
        assert np.array_equal(x1, x_pred) and np.array_equal(c1, c_pred)
        s.set_wait_test(0, -1)
        s.time_step_resident(dt, dt)  # the same handle and device run the step
        xg, cg = s.download()
    om = O.Mesh(q)
    xo, co = xms.copy(order="F"), cps.copy(order="F")
    om.update_xms(xo, co, dt)
    om.time_step(xo, co, dt, dt, nthreads=2)
    assert rel(xg, xo) < 1e-9 and rel(cg, co) < 1e-9
