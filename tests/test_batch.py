"""Batching: many patches of different sizes, motions and precisions stepped
together (mafem_batch_step).  With the batched FP32 solve off, each patch gets
exactly what stepping it alone gives (1e-13 relative: the same kernels on the
same data; only the persistent factorisation's CTA count and the interleaving
differ).  With it on (the default), the FP32 patches are factored and refined
one CTA per patch in two launches: a different FP32 factorisation, so they
are checked against the oracle at the FP32 form's bar (1e-8), and the FP64
patches must still equal their runs alone.  Every patch matches the oracle
(1e-9 plain FP64, 1e-8 FP32).  A patch whose Newton iteration fails reports its
status without disturbing the others.
"""
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


def _oracle_steps(q, xms, cps):
    om = O.Mesh(q)
    t = 0.0
    for _ in range(STEPS):
        t += DT
        om.update_xms(xms, cps, DT)
        om.time_step(xms, cps, t, DT, nthreads=4)
    return xms, cps


@pytest.mark.parametrize("patch_solve", [False, True])
def test_batch_equals_patches_alone_and_oracle(patch_solve):
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
            assert b.set_patch_solve(patch_solve) == patch_solve
            t = 0.0
            for _ in range(STEPS):
                t += DT
                status, stats = b.step(t, DT)
                assert status == [M.OK] * len(PATCHES)
                assert all(st["newton_iters"] >= 1 for st in stats)
                for st, pc in zip(stats, PATCHES):
                    if pc[3] == M.FP32_REFINE:
                        assert st["refine_iters"] >= st["newton_iters"]
        for k, s in enumerate(solvers):
            x, c = s.download()
            if patch_solve and PATCHES[k][3] == M.FP32_REFINE:
                assert rel(x, alone[k][0]) < 1e-8 and rel(c, alone[k][1]) < 1e-8
            else:
                assert rel(x, alone[k][0]) < 1e-13
                assert rel(c, alone[k][1]) < 1e-13
        # every patch against the oracle
        for k, (motion, n1, n2, prec) in enumerate(PATCHES):
            q, xms, cps = oracle_in[k]
            xo, co = _oracle_steps(q, xms.copy(order="F"), cps.copy(order="F"))
            x, c = solvers[k].download()
            tol = 1e-9 if prec == M.PLAIN_FP64 else 1e-8
            assert rel(x, xo) < tol and rel(c, co) < tol
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


def test_batched_fp32_solve_mixed_sizes_matches_oracle():
    """Only FP32 patches, eight sizes and both motions, batched solve on: every
    patch within 1e-8 of the oracle after two steps."""
    cases = [(M.LAG, 4, 4), (M.ALEVB, 5, 7), (M.LAG, 8, 8), (M.ALEVB, 9, 9), (M.LAG, 11, 6),
             (M.ALEVB, 12, 12), (M.LAG, 14, 10), (M.ALEVB, 16, 16)]
    solvers, inputs = [], []
    try:
        for k, (motion, n1, n2) in enumerate(cases):
            p, q, mesh, xms, cps = _setup(motion, n1, n2, 10 + k)
            s = M.Solver(mesh, p, M.FP32_REFINE)
            s.upload(xms, cps)
            solvers.append(s)
            inputs.append((q, xms, cps))
        with M.Batch(solvers) as b:
            assert b.set_patch_solve(True)
            t = 0.0
            for _ in range(STEPS):
                t += DT
                status, _ = b.step(t, DT)
                assert status == [M.OK] * len(cases)
        for s, (q, xms, cps) in zip(solvers, inputs):
            xo, co = _oracle_steps(q, xms.copy(order="F"), cps.copy(order="F"))
            x, c = s.download()
            assert rel(x, xo) < 1e-8 and rel(c, co) < 1e-8
    finally:
        for s in solvers:
            s.close()
