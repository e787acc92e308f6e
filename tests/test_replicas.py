"""bench.py's N > 1 path on the CPU: two ranks over gloo, as torchrun launches
them (RANK / WORLD_SIZE / MASTER_* in the environment, 127.0.0.1).

The path shards into independent replicas (each rank its own patch, no
data-path collective): what the ranks share is the barrier around the timed
region and the max over ranks of the timed totals, and only rank 0 prints.
The reference arm runs on rank 0 alone; the other ranks exit without output.
The reference arm's CPU sample is replaced by a stub here (its own timing is
covered by the bench itself), so the test checks the plumbing, not the oracle.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import contextlib, io, json, os, sys
sys.path.insert(0, sys.argv[1])
import bench
rank, world, local, dist = bench.dist_init()
assert dist is not None and world == 2 and rank == int(os.environ["RANK"])
bench.barrier(dist)
m = bench.allmax(dist, 10.0 * (rank + 1))
bench.cpu_baseline = lambda **kw: {"value": 0.5, "unit": "time-steps/s", "cores": 1, "kind": "port",
                                   "sample": "stub", "steps_timed": 2, "first_timed_step": 4}
sys.argv = ["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "2", "--warmup", "3"]
buf = io.StringIO()
with contextlib.redirect_stdout(buf):
    bench.main()
bench.barrier(dist)
print(json.dumps({"rank": rank, "max": m, "out": buf.getvalue()}))
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_share_barrier_and_max_and_rank0_prints():
    pytest.importorskip("torch.distributed")
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", LOCAL_WORLD_SIZE="2",
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD, ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    try:
        for p in procs:
            out, err = p.communicate(timeout=240)
            assert p.returncode == 0, err[-2000:]
            outs.append(json.loads(out.strip().splitlines()[-1]))
    finally:
        for p in procs:
            if p.poll() is None:
                p.kill()
    by_rank = {o["rank"]: o for o in outs}
    assert sorted(by_rank) == [0, 1]
    assert by_rank[0]["max"] == by_rank[1]["max"] == 20.0
    assert by_rank[1]["out"] == ""
    lines = [ln for ln in by_rank[0]["out"].splitlines() if ln.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] == 0.5
    assert line["cpu_baseline"]["sample"] == "stub"
    assert line["e2e"] == {"value": 0.5, "unit": "time-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    for key in ("metric", "unit", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling", "vs_baseline",
                "dtype", "data", "config"):
        assert key in line
    assert line["config"]["parallelism"] == "replicas x2"


def test_cpu_baseline_times_the_oracle_on_a_small_patch():
    """The reference arm's measurement itself (the oracle's assembly + sparse
    LU on the host cores), on a 6 x 6 version of the workload."""
    import bench
    wl = dict(bench.WORKLOAD, n=6)
    cb = bench.cpu_baseline(wl=wl, warmup=1, max_seconds=10.0, max_steps=2)
    assert cb["kind"] == "port" and cb["unit"] == "time-steps/s"
    assert cb["value"] > 0 and cb["cores"] >= 1
    assert cb["steps_timed"] == 2 and cb["first_timed_step"] == 2
    assert cb["sample"].startswith("time steps 2..3")


def test_reference_arm_loads_only_the_oracle():
    """The CPU baseline builds its mesh and seeded initial state with the oracle:
    the product library is never loaded into that process."""
    code = ("import sys; sys.path.insert(0, sys.argv[1]); import bench; "
            "bench.cpu_baseline(wl=dict(bench.WORKLOAD, n=6), warmup=1, max_steps=1); "
            "maps = open('/proc/self/maps').read(); "
            "print(int('libmafem' in maps), int('liboracle' in maps))")
    out = subprocess.run([sys.executable, "-c", code, ROOT], capture_output=True, text=True, check=True)
    assert out.stdout.split() == ["0", "1"], out.stdout + out.stderr


def test_rel_err_vs_oracle_report():
    """The bench's accuracy report against the oracle sample: same initial state,
    same steps.  The device solver is replaced by the oracle's own band-LU
    stepping, so the report compares two CPU solvers and must sit far below
    the 1e-9 bar."""
    import dataclasses
    import types

    import bench
    from _cases import M, O

    wl = dict(bench.WORKLOAD, n=6)
    ref = {}
    bench.cpu_baseline(wl=wl, warmup=1, max_seconds=10.0, max_steps=2, state_out=ref)
    assert ref["steps"] == 3

    fields = {f.name for f in dataclasses.fields(O.Params)}

    class OracleSolver:
        def __init__(self, mesh, p, precision):
            d = dataclasses.asdict(p)
            d["zv"] = d.pop("zeta_v")
            self.om = O.Mesh(O.Params(**{k: v for k, v in d.items() if k in fields}))

        def __enter__(self):
            return self

        def __exit__(self, *a):
            pass

        def upload(self, x, c):
            self.x, self.c = x.copy(order="F"), c.copy(order="F")

        def predict(self, dt):
            self.om.update_xms(self.x, self.c, dt)

        def time_step_resident(self, t, dt):
            self.om.time_step(self.x, self.c, t, dt, nthreads=2)

        def download(self):
            return self.x, self.c

    fake = types.SimpleNamespace(**{k: getattr(M, k) for k in dir(M) if not k.startswith("__")})
    fake.Solver = OracleSolver
    rep = bench.rel_err_vs_oracle(fake, ref, wl)
    assert rep["steps"] == 3 and rep["bar"] == 1e-9
    assert max(rep["xms"], rep["velocities"], rep["lambda"]) < 1e-11, rep


def test_stratified_baseline_sample_covers_every_class():
    """The bounded bench's plain FP64 baseline on the batching workload: the
    first patches of every (size, motion) class, weighted so that the weights
    add up to each class's patch count (and to every patch with no sampling)."""
    sys.path.insert(0, ROOT)
    import bench
    import mafem as M
    patches = bench.batch_patches(M, dict(bench.BATCH, patches=40))
    classes = {}
    for k, (p, _, _, _) in enumerate(patches):
        classes.setdefault((p.num1el, p.motion), []).append(k)
    idx, w = bench._baseline_sample(patches, 2)
    assert sorted(idx) == idx and set(idx) == set(w)
    for key, ks in classes.items():
        picked = [k for k in idx if k in ks]
        assert picked == ks[:2]
        assert abs(sum(w[k] for k in picked) - len(ks)) < 1e-12
    assert abs(sum(w.values()) - len(patches)) < 1e-9
    idx_all, w_all = bench._baseline_sample(patches, 0)
    assert idx_all == list(range(len(patches))) and all(v == 1.0 for v in w_all.values())
