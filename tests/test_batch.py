"""Batching: many patches of different sizes, motions and precisions stepped
together (mafem_batch_step) must give each patch exactly what stepping it
alone gives (1e-13 relative: the same kernels on the same data; only the
persistent factorisation's CTA count and the interleaving differ), and the
plain FP64 patches must match the oracle (1e-9, the FP64 parity bar).  A patch
whose Newton iteration fails reports its status without disturbing the others.
"""
import numpy as np
import pytest

from _cases import M, O, params_pair, rel, state

pytestmark = pytest.mark.gpu

PATCHES = [  # (motion, n1, n2, precision)
    (M.ALEVB, 7, 7, M.PLAIN_FP64), (M.LAG, 8, 6, M.PLAIN_FP64), (M.ALEVB, 9, 9, M.PLAIN_FP64),
    (M.ALEVB, 12, 10, M.PLAIN_FP64), (M.ALEVB, 6, 8, M.FP32_REFINE), (M.LAG, 5, 7, M.FP32_REFINE),
]
DT, STEPS = 0.01, 2


def _setup(motion, n1, n2, seed):
    p, q = params_pair(motion, M.F_PULL, n1, n2, pull_speed=1.0)
    mesh = M.Mesh(p)
    xms, cps = state(p, mesh, seed=seed, amp=1e-4)
    return p, q, mesh, xms, cps


def test_batch_equals_patches_alone_and_oracle():
    alone = []
    for k, (motion, n1, n2, prec) in enumerate(PATCHES):
        p, _, mesh, xms, cps = _setup(motion, n1, n2, k)
        with M.Solver(mesh, p, prec) as s:
            s.upload(xms, cps)
            t = 0.0
            for _ in range(STEPS):
                t += DT
                s.predict(DT)
                s.time_step_resident(t, DT)
            alone.append(s.download())
    solvers, oracle_in = [], []
    try:
        for k, (motion, n1, n2, prec) in enumerate(PATCHES):
            p, q, mesh, xms, cps = _setup(motion, n1, n2, k)
            s = M.Solver(mesh, p, prec)
            s.upload(xms, cps)
            solvers.append(s)
            oracle_in.append((q, xms, cps))
        with M.Batch(solvers) as b:
            t = 0.0
            for _ in range(STEPS):
                t += DT
                status, stats = b.step(t, DT)
                assert status == [M.OK] * len(PATCHES)
                assert all(st["newton_iters"] >= 1 for st in stats)
        for k, s in enumerate(solvers):
            x, c = s.download()
            assert rel(x, alone[k][0]) < 1e-13
            assert rel(c, alone[k][1]) < 1e-13
        # the plain FP64 patches against the oracle
        for k, (motion, n1, n2, prec) in enumerate(PATCHES[:2]):
            q, xms, cps = oracle_in[k]
            om = O.Mesh(q)
            t = 0.0
            for _ in range(STEPS):
                t += DT
                om.update_xms(xms, cps, DT)
                om.time_step(xms, cps, t, DT, nthreads=4)
            x, c = solvers[k].download()
            assert rel(x, xms) < 1e-9 and rel(c, cps) < 1e-9
    finally:
        for s in solvers:
            s.close()


def test_batch_reports_a_failing_patch_without_disturbing_the_others():
    # a patch with an unreachable Newton tolerance (eps_nr = 0) must end with
    # NEWTON_NOT_CONVERGED after 14 iterations; its neighbour must still match
    # its run alone
    p_bad, _, mesh_bad, xb, cb = _setup(M.ALEVB, 6, 6, 0)
    p_bad.eps_nr = 0.0
    p_ok, _, mesh_ok, xo, co = _setup(M.LAG, 6, 6, 1)
    with M.Solver(mesh_ok, p_ok) as s:
        s.upload(xo, co)
        s.predict(DT)
        s.time_step_resident(DT, DT)
        ref = s.download()
    with M.Solver(mesh_bad, p_bad) as sb, M.Solver(mesh_ok, p_ok) as so:
        sb.upload(xb, cb)
        so.upload(xo, co)
        with M.Batch([sb, so]) as b:
            status, _ = b.step(DT, DT)
        assert status[0] == M.NEWTON_NOT_CONVERGED
        assert status[1] == M.OK
        x, c = so.download()
        assert rel(x, ref[0]) < 1e-13 and rel(c, ref[1]) < 1e-13
