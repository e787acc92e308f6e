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


def _oracle_steps(q, xms, cps, ramp=0, steps=STEPS):
    """The oracle's steps; ramp > 0: before step k the pull's Dirichlet values are
    scaled by min(1, (k + 1) / ramp), the state edit mafem_set_dirichlet_scale makes."""
    om = O.Mesh(q)
    t = 0.0
    for k in range(steps):
        if ramp:
            for u, node, v in om.dirichlet():
                cps[node - 1, om.dofs[u - 1] - 1] = min(1.0, (k + 1) / ramp) * v
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


def test_48x48_patch_matches_oracle():
    """The largest patch size of the batching workload (48 x 48 elements, half
    bandwidth 799: a two-CTA cluster in the batched FP32 solve), with the
    workload's centre pull, a tension lambda0 other than kb / 4, a flat start
    and the pull speed ramped over 30 steps, two steps at dt 0.01: the batched
    FP32 form within 1e-8 and the plain FP64 form within 1e-9 of the oracle."""
    kw = dict(pull_speed=0.3, pull_centre=1, lambda0=0.7, kb=1.3)
    p, q = params_pair(M.ALEVB, M.F_PULL, 48, 48, **kw)
    mesh = M.Mesh(p)
    assert mesh.half_bw == 799
    xms, cps = state(p, mesh, seed=48, amp=0.0)
    xo, co = _oracle_steps(q, xms.copy(order="F"), cps.copy(order="F"), ramp=30)
    p8, _ = params_pair(M.LAG, M.F_PULL, 8, 8, **kw)  # a small patch beside it in the batch
    m8 = M.Mesh(p8)
    x8, c8 = state(p8, m8, seed=8, amp=0.0)
    s32, s8, s64 = M.Solver(mesh, p, M.FP32_REFINE), M.Solver(m8, p8, M.FP32_REFINE), M.Solver(mesh, p)
    try:
        s32.upload(xms, cps)
        s8.upload(x8, c8)
        s64.upload(xms, cps)
        with M.Batch([s32, s8]) as b:
            assert b.set_patch_solve(True)
            t = 0.0
            for k in range(STEPS):
                t += DT
                for s in (s32, s8, s64):
                    s.set_dirichlet_scale(min(1.0, (k + 1) / 30))
                status, _ = b.step(t, DT)
                assert status == [M.OK, M.OK]
                s64.predict(DT)
                s64.time_step_resident(t, DT)
        x, c = s32.download()
        assert rel(x, xo) < 1e-8 and rel(c, co) < 1e-8
        x, c = s64.download()
        assert rel(x, xo) < 1e-9 and rel(c, co) < 1e-9
    finally:
        for s in (s32, s8, s64):
            s.close()


def test_64x64_patch_in_the_batched_fp32_solve():
    """A 64 x 64 ALEVB patch (half bandwidth 1055) is factored by the batched
    one-patch-per-cluster FP32 solve (its panel and the tensor-core chunk
    buffers fit one CTA's shared memory); one ramped step of it within 1e-8,
    and of the plain FP64 path within 1e-9, of the oracle's step.  Pull speed
    0.1: at 0.3 this fine graded patch loses Newton convergence in its first
    step at dt 0.01 (plain FP64 as well)."""
    p, q = params_pair(M.ALEVB, M.F_PULL, 64, 64, pull_speed=0.1, pull_centre=1)
    mesh = M.Mesh(p)
    assert mesh.half_bw == 1055
    xms, cps = state(p, mesh, seed=64, amp=0.0)
    with M.Solver(mesh, p, M.FP32_REFINE) as s32, M.Solver(mesh, p) as s64:
        s32.upload(xms, cps)
        s64.upload(xms, cps)
        for s in (s32, s64):
            s.set_dirichlet_scale(1.0 / 30)
        with M.Batch([s32]) as b:
            assert b.set_patch_solve(True)  # the batched form is available for this size
            status, st = b.step(DT, DT)
            assert status == [M.OK]
            assert s32.fallback_count() == 0  # solved by the batched form, not handed back
        s64.predict(DT)
        s64.time_step_resident(DT, DT)
        x1, c1 = s32.download()
        x2, c2 = s64.download()
    xo, co = _oracle_steps(q, xms.copy(order="F"), cps.copy(order="F"), ramp=30, steps=1)
    assert rel(x1, xo) < 1e-8 and rel(c1, co) < 1e-8
    assert rel(x2, xo) < 1e-9 and rel(c2, co) < 1e-9


# the batching workload's kind of patch: centre pull at a moderate speed, ramped
# over 30 steps, from a flat start
ROUND_CASES = [(M.LAG, 6, 6), (M.ALEVB, 7, 5), (M.LAG, 9, 9), (M.ALEVB, 10, 10), (M.LAG, 12, 8), (M.ALEVB, 16, 16),
               (M.LAG, 5, 5), (M.ALEVB, 24, 24)]
ROUND_RAMP = 30


def _round_setup(motion, n1, n2):
    p, q = params_pair(motion, M.F_PULL, n1, n2, pull_speed=0.2, pull_centre=1)
    mesh = M.Mesh(p)
    xms, cps = state(p, mesh, amp=0.0)
    return p, q, mesh, xms, cps


def _run_rounds(batched_assembly, graphs, cases=ROUND_CASES, steps=3):
    solvers = []
    try:
        for motion, n1, n2 in cases:
            p, _, mesh, xms, cps = _round_setup(motion, n1, n2)
            s = M.Solver(mesh, p, M.FP32_REFINE)
            s.upload(xms, cps)
            solvers.append(s)
        with M.Batch(solvers) as b:
            assert b.set_patch_solve(True)
            b.set_rounds(batched_assembly, graphs)
            t, iters, launches = 0.0, [], 0
            for k in range(steps):
                t += DT
                for s in solvers:
                    s.set_dirichlet_scale(min(1.0, (k + 1) / ROUND_RAMP))
                l0 = b.stats()["kernel_launches"]
                status, st = b.step(t, DT)
                launches += b.stats()["kernel_launches"] - l0
                assert status == [M.OK] * len(cases)
                iters.append([x["newton_iters"] for x in st])
            stats = b.stats()
            stats["kernel_launches"] = launches
        return [s.download() for s in solvers], iters, stats
    finally:
        for s in solvers:
            s.close()


def test_batched_rounds_match_per_patch_kernels_and_replay_graphs():
    """The batched Newton round (assembly, update and norms of every patch in
    one launch per kernel) against the per-patch kernels: the same Newton
    iteration counts and states within 1e-10 (the element kernels are compiled
    separately, so a multiply-add may round differently); with CUDA-graph
    replay bit-identical to the same rounds launched on the stream; the graphs
    captured once per distinct round and replayed in later steps; every patch
    within 1e-8 of the oracle."""
    ref, it_ref, _ = _run_rounds(False, False)
    got, it_got, st_plain = _run_rounds(True, False)
    gra, it_gra, st_graph = _run_rounds(True, True)
    assert it_got == it_ref and it_gra == it_ref
    for (x0, c0), (x1, c1), (x2, c2) in zip(ref, got, gra):
        assert rel(x1, x0) < 1e-10 and rel(c1, c0) < 1e-10
        assert np.array_equal(x1, x2) and np.array_equal(c1, c2)
    assert st_plain["graph_launches"] == 0
    rounds = sum(max(r) for r in it_gra)
    assert st_graph["graph_launches"] == rounds
    assert 1 <= st_graph["graph_captures"] < rounds  # later steps replay the first step's rounds
    for k, (motion, n1, n2) in enumerate(ROUND_CASES):
        _, q, _, xms, cps = _round_setup(motion, n1, n2)
        xo, co = _oracle_steps(q, xms.copy(order="F"), cps.copy(order="F"), ramp=ROUND_RAMP, steps=3)
        assert rel(gra[k][0], xo) < 1e-8 and rel(gra[k][1], co) < 1e-8


def test_batched_round_launches_do_not_grow_with_the_patch_count():
    """Kernels enqueued per Newton round: a fixed number with batched rounds
    (twice as many patches, the same launches per round up to one more
    cluster-size group of the factorisation), one set per patch without them."""
    def per_round(cases, on):
        _, iters, st = _run_rounds(on, on, cases=cases, steps=1)
        return st["kernel_launches"] / max(iters[0])
    small = ROUND_CASES[:4]
    large = ROUND_CASES[:4] + [(m, n1 + 1, n2) for m, n1, n2 in ROUND_CASES[:4]]
    assert per_round(large, True) <= per_round(small, True) + 3
    assert per_round(large, False) > 1.5 * per_round(small, False)


def test_tangent_tile_autotuned_per_motion():
    """mafem_batch_create times the batched FP32 tangent kernel with 2 and 4
    elements per CTA for each kind of patch and keeps the faster; the choice
    and both times are reported per kind."""
    solvers = []
    try:
        for motion, n in ((M.LAG, 10), (M.ALEVB, 12)):
            p, _, mesh, xms, cps = _round_setup(motion, n, n)
            s = M.Solver(mesh, p, M.FP32_REFINE)
            s.upload(xms, cps)
            solvers.append(s)
        with M.Batch(solvers) as b:
            assert b.set_patch_solve(True)
            for s in solvers:
                epb, ms2, ms4 = s.tangent_tile()
                assert epb in (2, 4) and ms2 > 0 and ms4 > 0
                assert (ms2 if epb == 2 else ms4) == min(ms2, ms4)
    finally:
        for s in solvers:
            s.close()
