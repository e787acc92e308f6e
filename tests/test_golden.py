"""Committed golden fixtures (tests/golden/, made by tests/golden/make_golden.py
from the CPU oracle).

CPU: the oracle still reproduces every fixture (a change to the oracle that
moves a result shows here before it can move a parity bar), the product's host
mesh has the fixture's sizes, and the product's state-file writer and reader
give the committed t3-*.txt files byte for byte.

GPU: the CUDA path against the fixtures on their stored inputs, with the
tolerances of the parity tests: residual 1e-12 of its largest entry; tangent
through its diagonal, K·v and Kᵀ·v, each entry i within
tol·max|K|·Σ_{|i-q|<=kl} |v_q| — what an entrywise error of tol·max|K| allows —
with tol 1e-11 (plain FP64, dual numbers against the oracle's complex step) or
2e-5 (all-FP32 tangent); states after the time steps 1e-9 (plain FP64, with
the oracle's Newton iteration counts) and 1e-8 (FP32 + FP64 refinement).
"""
import os
import sys

import numpy as np
import pytest

from _cases import M, O, rel

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden as G  # noqa: E402

ARRAYS, META = G.load()
N_ASM, N_STEP = len(META["assembly"]), len(META["steps"])


def _product_params(kw):
    """The fixture's Params keywords (the oracle's spelling) for the product's Params."""
    names = {"zv": "zeta_v", "adb": "alpha_db", "am": "alpha_m"}
    return M.Params(**{names.get(k, k): v for k, v in kw.items()})


def _assembly_inputs(k):
    c = META["assembly"][k]
    return c, ARRAYS[f"a{k}_xms"], ARRAYS[f"a{k}_cps"], ARRAYS[f"a{k}_v"]


def _tangent_views(ab, kl, v):
    return ab[:, 2 * kl], G.band_matvec(ab, kl, v), G.band_matvec(ab, kl, v, transpose=True)


def _band_sum_abs(v, kl):
    """Σ_{|i-q|<=kl} |v_q| for every i (a sliding window sum)."""
    c = np.concatenate(([0.0], np.cumsum(np.abs(v))))
    i = np.arange(len(v))
    return c[np.minimum(i + kl + 1, len(v))] - c[np.maximum(i - kl, 0)]


# ---- CPU ---------------------------------------------------------------------
@pytest.mark.parametrize("k", range(N_ASM))
def test_oracle_reproduces_assembly_fixture(k):
    c, xms, cps, v = _assembly_inputs(k)
    om = O.Mesh(O.Params(**c["params"]))
    assert (om.nmdf, om.half_bw, om.numnp, om.ndf) == (c["nmdf"], c["half_bw"], c["numnp"], c["ndf"])
    r, ab = om.calc_r_K(xms, cps, META["assembly_time"], META["assembly_dt"], nthreads=1)
    diag, Kv, KTv = _tangent_views(ab, om.half_bw, v)
    assert rel(r, ARRAYS[f"a{k}_r"]) < 1e-13
    assert rel(diag, ARRAYS[f"a{k}_Kdiag"]) < 1e-13
    assert rel(Kv, ARRAYS[f"a{k}_Kv"]) < 1e-13
    assert rel(KTv, ARRAYS[f"a{k}_KTv"]) < 1e-13


@pytest.mark.parametrize("k", range(N_STEP))
def test_oracle_reproduces_step_fixture(k):
    c = META["steps"][k]
    om = O.Mesh(O.Params(**c["params"]))
    xms, cps = ARRAYS[f"s{k}_xms0"].copy(order="F"), ARRAYS[f"s{k}_cps0"].copy(order="F")
    dt, t, iters = META["step_dt"], 0.0, []
    for _ in range(c["steps"]):
        t += dt
        om.update_xms(xms, cps, dt)
        iters.append(len(om.time_step(xms, cps, t, dt, nthreads=1)))
    assert iters == ARRAYS[f"s{k}_iters"].tolist()
    assert rel(xms, ARRAYS[f"s{k}_xms"]) < 1e-12
    assert rel(cps, ARRAYS[f"s{k}_cps"]) < 1e-12


@pytest.mark.parametrize("k", range(N_ASM))
def test_product_mesh_has_the_fixture_sizes(k):
    c = META["assembly"][k]
    mesh = M.Mesh(_product_params(c["params"]))
    assert (mesh.nmdf, mesh.half_bw, mesh.numnp, mesh.ndf) == (c["nmdf"], c["half_bw"], c["numnp"], c["ndf"])


def test_state_files_byte_exact(tmp_path):
    step = META["state_files_step"]
    for name in ("xms", "cps"):
        a = ARRAYS[f"s0_{name}"]
        with open(os.path.join(HERE, "golden", f"t{step}-{name}.txt"), "rb") as f:
            golden = f.read()
        assert O.writedlm_text(a).encode() == golden
        out = str(tmp_path / f"t{step}-{name}.txt")
        M.writedlm(out, a)
        with open(out, "rb") as f:
            assert f.read() == golden
        back = M.readdlm(os.path.join(HERE, "golden", f"t{step}-{name}.txt"), *a.shape)
        assert np.array_equal(back, a)


# ---- GPU ---------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(M.PLAIN_FP64, 1e-11), (M.FP32_REFINE, 2e-5)])
@pytest.mark.parametrize("k", range(N_ASM))
def test_gpu_assembly_matches_fixture(k, precision, tol):
    c, xms, cps, v = _assembly_inputs(k)
    p = _product_params(c["params"])
    mesh = M.Mesh(p)
    with M.Solver(mesh, p, precision) as s:
        r, ab = s.calc_r_K(xms, cps, META["assembly_time"], META["assembly_dt"])
    kl = mesh.half_bw
    assert np.all(ab[:, :kl] == 0.0)
    diag, Kv, KTv = _tangent_views(ab, kl, v)
    assert rel(r, ARRAYS[f"a{k}_r"]) < 1e-12
    kmax = float(np.abs(ab).max())
    bound = tol * kmax * _band_sum_abs(v, kl)
    for got, key in ((Kv, "Kv"), (KTv, "KTv")):
        assert np.all(np.abs(got - ARRAYS[f"a{k}_{key}"]) <= bound), key
    assert np.abs(diag - ARRAYS[f"a{k}_Kdiag"]).max() <= tol * kmax


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(M.PLAIN_FP64, 1e-9), (M.FP32_REFINE, 1e-8)])
@pytest.mark.parametrize("k", range(N_STEP))
def test_gpu_steps_match_fixture(k, precision, tol):
    c = META["steps"][k]
    p = _product_params(c["params"])
    mesh = M.Mesh(p)
    dt, t = META["step_dt"], 0.0
    with M.Solver(mesh, p, precision) as s:
        s.upload(ARRAYS[f"s{k}_xms0"], ARRAYS[f"s{k}_cps0"])
        for j in range(c["steps"]):
            t += dt
            s.predict(dt)
            st = s.time_step_resident(t, dt)
            if precision == M.PLAIN_FP64:
                assert st["newton_iters"] == ARRAYS[f"s{k}_iters"][j]
        xms, cps = s.download()
    assert rel(xms, ARRAYS[f"s{k}_xms"]) < tol
    assert rel(cps, ARRAYS[f"s{k}_cps"]) < tol
