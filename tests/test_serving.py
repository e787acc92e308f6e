"""Serving (mafem_server_*): continuous batching of solves of different sizes,
motions and precisions.

A request's result must not depend on what runs beside it: each request is
served once alone and once in a mix where other requests arrive while it
runs, and the two results must be identical (the batched FP32 solve runs each
patch in its own CTA; the plain FP64 requests use their own handle's solver).
The FP32 results are also checked against the oracle at the FP32 form's bar
(1e-8) and the plain FP64 one against the same request stepped with
mafem_time_step (identical).  Admission follows the HBM budget: a request
that can never fit is refused, one that does not fit yet waits.
"""
import time

import numpy as np
import pytest

from _cases import M, O, params_pair, rel, state

pytestmark = pytest.mark.gpu

DT = 0.005
REQS = [  # (motion, n, precision, steps, seed)
    (M.ALEVB, 12, M.FP32_REFINE, 3, 1), (M.LAG, 9, M.FP32_REFINE, 4, 2), (M.ALEVB, 8, M.PLAIN_FP64, 3, 3),
    (M.LAG, 16, M.FP32_REFINE, 2, 4), (M.ALEVB, 7, M.FP32_REFINE, 5, 5),
]


def _req(motion, n, seed):
    p, q = params_pair(motion, M.F_PULL, n, n, pull_speed=0.5)
    mesh = M.Mesh(p)
    xms, cps = state(p, mesh, seed=seed, amp=1e-4)
    return p, q, mesh, xms, cps


def _drain(srv, ids, arrivals=()):
    """Run rounds until every id has a result; submit each (round, request) of
    `arrivals` when that round is reached.  Returns {id: (status, xms, cps)}."""
    out, pending, rnd = {}, list(arrivals), 0
    ids = list(ids)
    total = len(ids) + len(arrivals)
    t_end = time.monotonic() + 120.0  # rounds do not wait for the GPU: bound the loop by time
    while len(out) < total:
        for a in [a for a in pending if a[0] <= rnd]:
            ids.append(srv.submit(*a[1]))
            pending.remove(a)
        srv.round()
        rnd += 1
        for i in ids:
            if i not in out:
                r = srv.result(i)
                if r is not None:
                    out[i] = r
        assert time.monotonic() < t_end
    return [out[i] for i in ids]


def test_result_same_alone_and_in_mix_and_matches_oracle():
    built = [_req(m, n, seed) for (m, n, _, _, seed) in REQS]
    alone = []
    for (m, n, prec, steps, _), (p, _, mesh, xms, cps) in zip(REQS, built):
        with M.Server() as srv:
            rid = srv.submit(mesh, p, xms, cps, steps, DT, precision=prec)
            alone.append(_drain(srv, [rid])[0])
    # the mix: two requests at once, the others arriving in later rounds
    with M.Server() as srv:
        first = [srv.submit(built[k][2], built[k][0], built[k][3], built[k][4], REQS[k][3], DT,
                            precision=REQS[k][2]) for k in (0, 1)]
        arrivals = [(2 + 3 * j, (built[k][2], built[k][0], built[k][3], built[k][4], REQS[k][3], DT, 0.0,
                                 REQS[k][2])) for j, k in enumerate((2, 3, 4))]
        mixed = _drain(srv, first, arrivals)
        st = srv.stats()
    assert st["steps_done"] == sum(r[3] for r in REQS)
    assert 0 < st["p50_step_ms"] <= st["p99_step_ms"] <= st["max_step_ms"]
    for k, (a, b) in enumerate(zip(alone, mixed)):
        assert a[0] == M.OK and b[0] == M.OK
        assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2]), k
    for (m, n, prec, steps, _), (p, q, mesh, xms, cps), res in zip(REQS, built, mixed):
        if prec == M.PLAIN_FP64:
            with M.Solver(mesh, p) as s:
                s.upload(xms, cps)
                s.run_analysis([DT] * steps)
                x, c = s.download()
            assert np.array_equal(res[1], x) and np.array_equal(res[2], c)
        else:
            om = O.Mesh(q)
            x, c = xms.copy(order="F"), cps.copy(order="F")
            t = 0.0
            for _ in range(steps):
                t += DT
                om.update_xms(x, c, DT)
                om.time_step(x, c, t, DT, nthreads=4)
            assert rel(res[1], x) < 1e-8 and rel(res[2], c) < 1e-8


def test_admission_by_footprint():
    p, _, mesh, xms, cps = _req(M.ALEVB, 10, 7)
    need = M.footprint_bytes(mesh, M.FP32_REFINE)
    # a budget that holds one such request at a time
    with M.Server(hbm_budget_bytes=int(1.6 * need) + (16 << 20)) as srv:
        a = srv.submit(mesh, p, xms, cps, 2, DT)
        b = srv.submit(mesh, p, xms, cps, 2, DT)
        active, pending = srv.round()
        assert (active, pending) == (1, 1)  # b waits until a has finished and freed its memory
        ra = rb = None
        t_end = time.monotonic() + 60.0
        while time.monotonic() < t_end:
            srv.round()
            ra = ra or srv.result(a)
            rb = rb or srv.result(b)
            if ra and rb:
                break
        assert ra[0] == M.OK and rb[0] == M.OK
        assert np.array_equal(ra[1], rb[1]) and np.array_equal(ra[2], rb[2])
        assert srv.stats()["bytes_in_use"] == 0
    with M.Server(hbm_budget_bytes=need // 4) as srv:
        with pytest.raises(M.MafemError) as e:
            srv.submit(mesh, p, xms, cps, 2, DT)
        assert e.value.code == M.ERR_ADMISSION


def test_ramped_request_matches_the_oracle():
    """A request with ramp_steps: before its step k the server scales the pull's
    Dirichlet values by min(1, (k + 1) / ramp_steps) -- the state edit the
    oracle makes here by hand before each of its steps."""
    ramp, steps = 4, 3
    p, q, mesh, xms, cps = _req(M.ALEVB, 10, 11)
    with M.Server() as srv:
        rid = srv.submit(mesh, p, xms, cps, steps, DT, precision=M.FP32_REFINE, ramp_steps=ramp)
        res = _drain(srv, [rid])[0]
    assert res[0] == M.OK
    om = O.Mesh(q)
    x, c = xms.copy(order="F"), cps.copy(order="F")
    t = 0.0
    for k in range(steps):
        for u, node, v in om.dirichlet():
            c[node - 1, om.dofs[u - 1] - 1] = min(1.0, (k + 1) / ramp) * v
        t += DT
        om.update_xms(x, c, DT)
        om.time_step(x, c, t, DT, nthreads=4)
    assert rel(res[1], x) < 1e-8 and rel(res[2], c) < 1e-8
