"""The three banded LU paths against each other and against the oracle.

MAFEM_LU_AUTO (node-block pivoting in one persistent cooperative launch),
MAFEM_LU_PANELS (the same factorisation as per-panel launches, the fallback
when a cooperative launch is refused) and MAFEM_LU_FULL (LAPACK's partial
pivoting rule, the fallback when a node block has no usable pivot) must give
the same solve (1e-10 relative in FP64, the solve tolerance of the other
parity tests; 1e-8 for the FP32 LU with FP64 refinement) and the same Newton steps as the oracle (1e-9, identical iteration
counts).  Each path is selected through mafem_set_lu_path.
"""
import numpy as np
import pytest

from _cases import M, O, params_pair, rel, state

pytestmark = pytest.mark.gpu

PATHS = [M.LU_AUTO, M.LU_PANELS, M.LU_FULL]


@pytest.mark.parametrize("motion,n1,n2", [(M.ALEVB, 7, 7), (M.LAG, 8, 6), (M.ALEVB, 20, 18)])
@pytest.mark.parametrize("precision,tol", [(M.PLAIN_FP64, 1e-10), (M.FP32_REFINE, 1e-8)])
def test_lu_paths_solve_alike(motion, n1, n2, precision, tol):
    p, _ = params_pair(motion, M.F_PULL, n1, n2)
    mesh = M.Mesh(p)
    xms, cps = state(p, mesh, seed=4, amp=1e-2, vel_amp=0.02)
    sols = []
    with M.Solver(mesh, p, precision) as s:
        r, ab = s.calc_r_K(xms, cps, 0.01, 0.01)
        for path in PATHS:
            s.set_lu_path(path)
            s.calc_r_K(xms, cps, 0.01, 0.01)  # reassemble: the band is factorised in place
            sols.append(s.solve(r))
    A = O.band_to_dense(ab, mesh.half_bw, mesh.half_bw, mesh.nmdf)
    ref = -np.linalg.solve(A, r)
    for du in sols:
        assert rel(du, ref) < tol


@pytest.mark.parametrize("path", PATHS)
def test_lu_paths_time_steps_match_oracle(path):
    p, q = params_pair(M.ALEVB, M.F_PULL, 9, 9, pull_speed=1.0)
    mesh, om = M.Mesh(p), O.Mesh(q)
    xms, cps = state(p, mesh, seed=0, amp=1e-4)
    x2, c2 = xms.copy(order="F"), cps.copy(order="F")
    dt, t = 0.01, 0.0
    with M.Solver(mesh, p) as s:
        s.set_lu_path(path)
        for _ in range(2):
            t += dt
            om.update_xms(xms, cps, dt)
            stats = s.time_step(xms, cps, t, dt)
            om.update_xms(x2, c2, dt)
            eps = om.time_step(x2, c2, t, dt, nthreads=4)
            assert stats["newton_iters"] == len(eps)
    assert rel(xms, x2) < 1e-9
    assert rel(cps, c2) < 1e-9


def test_lu_path_rejects_unknown_values():
    p, _ = params_pair(M.LAG, M.F_PULL, 4, 4)
    mesh = M.Mesh(p)
    with M.Solver(mesh, p) as s:
        with pytest.raises(M.MafemError):
            s.set_lu_path(7)
