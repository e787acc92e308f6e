"""Generate the golden fixtures of the parity tests from the CPU oracle.

    python tests/golden/make_golden.py        # rewrites oracle_cases.npz and t*-xms/cps.txt

The oracle (oracle/, a C++ restatement of MembraneAleFem.jl pinned by the
reference's own known-answer tests) computes, on seeded small meshes of every
motion and scenario:

* assembly cases: the residual r of ``calc_r_K`` (src/analysis/FiniteElement.jl:
  120-200) and three size-independent views of the band tangent K: its
  diagonal, K·v and Kᵀ·v for a seeded v;
* step cases: the state after ``update_xms!`` + ``time_step!``
  (src/analysis/FiniteElement.jl:11-63, src/analysis/Analysis.jl:60-78) for a
  few steps, and the Newton iteration count of each step;
* the state files ``run_analysis!`` writes after the last step of step case 0
  (t3-xms.txt / t3-cps.txt, src/analysis/Analysis.jl:75-78), in Julia's
  print(::Float64) format.

Every input is stored beside its outputs, so a test needs nothing but the
fixture and the parameters stored with it.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402

NPZ = os.path.join(HERE, "oracle_cases.npz")

_COMMON = dict(length=1.0, pull_speed=0.5, bend_mf=0.5, bend_tm=2.0)
# (motion, scenario, num1el, num2el, seed[, parameter overrides])
ASSEMBLY = [
    (O.ALEVB, O.F_PULL, 4, 5, 1), (O.ALEV, O.F_PULL, 3, 3, 2), (O.LAG, O.F_PULL, 3, 4, 3),
    (O.EUL, O.F_PULL, 3, 3, 4), (O.LAG, O.F_PULL, 1, 1, 5), (O.STATIC, O.F_CAVI, 3, 3, 6),
    (O.STATIC, O.F_COUE, 4, 3, 7), (O.STATIC, O.F_POIS, 3, 4, 8), (O.LAG, O.F_BEND, 3, 4, 9),
    (O.ALEV, O.F_BEND, 4, 3, 10),
    # non-default moduli, viscosity and size (a normal pressure is rejected for
    # F_PULL and F_BEND, Bc.jl:266 and Params.jl:103, and has no z unknowns to
    # act on in the flat flows)
    (O.ALEVB, O.F_PULL, 5, 4, 14, dict(kb=1.7, kg=-0.3, zv=0.6)),
    (O.LAG, O.F_PULL, 4, 4, 15, dict(kb=0.6, zv=1.8)),
    (O.EUL, O.F_PULL, 4, 3, 16, dict(kg=-0.8, length=2.0)),
    (O.ALEV, O.F_BEND, 3, 3, 17, dict(kb=1.4, kg=-0.7, bend_mf=0.7, zv=0.5)),
    (O.EUL, O.F_BEND, 4, 3, 18),
]
ASSEMBLY_TIME, ASSEMBLY_DT = 0.37, 0.01
# (motion, num1el, num2el, steps, seed): tether pull at pull speed 1.0
STEPS = [(O.LAG, 5, 5, 3, 11), (O.ALEVB, 7, 7, 3, 12), (O.ALEVB, 9, 9, 2, 13)]
STEP_DT = 0.01


def case_params(motion, scenario, n1, n2, **over) -> dict:
    """Keyword arguments of Params (oracle and product spell them alike, zv aside)."""
    kw = dict(_COMMON, motion=int(motion), scenario=int(scenario), num1el=int(n1), num2el=int(n2))
    kw.update(over)
    return kw


def initial_state(mesh: "O.Mesh", p: dict, seed: int, amp: float, vel_amp: float):
    """prepare_input's state (a flat sheet with lambda 0.25 for F_BEND) plus a
    seeded z perturbation of the interior nodes and seeded velocities on the
    free unknowns, so every physics term is exercised."""
    rng = np.random.default_rng(seed)
    if p["scenario"] == O.F_BEND:
        xms = np.zeros((mesh.numnp, 3), order="F")
        s1 = np.arange(mesh.numnp) % mesh.num1np
        s2 = np.arange(mesh.numnp) // mesh.num1np
        L = p["length"]
        xms[:, 0] = L * np.clip((s1 - 0.5) / (mesh.num1np - 2), 0, 1)
        xms[:, 1] = L * np.clip((s2 - 0.5) / (mesh.num2np - 2), 0, 1)
        cps = np.zeros((mesh.numnp, mesh.ndf), order="F")
        cps[:, mesh.dofs[6] - 1] = 0.25
    else:
        xms, cps = mesh.prepare_input()
    s1 = np.arange(mesh.numnp) % mesh.num1np
    s2 = np.arange(mesh.numnp) // mesh.num1np
    interior = (s1 > 0) & (s1 < mesh.num1np - 1) & (s2 > 0) & (s2 < mesh.num2np - 1)
    xms[:, 2] += np.where(interior, amp * rng.uniform(-1.0, 1.0, mesh.numnp), 0.0)
    if vel_amp:
        free = mesh.ID.T > 0  # numnp x ndf
        cps = cps + np.where(free, vel_amp * rng.uniform(-1.0, 1.0, free.shape), 0.0)
    return np.asfortranarray(xms), np.asfortranarray(cps)


def band_matvec(ab: np.ndarray, kl: int, v: np.ndarray, transpose: bool = False) -> np.ndarray:
    """K·v (or Kᵀ·v) of a LAPACK band (row q holds column q, K[i, q] at
    ab[q, 2kl + i - q], kl = ku), summed in a fixed order."""
    n = ab.shape[0]
    y = np.zeros(n)
    q = np.arange(n)
    for off in range(-kl, kl + 1):  # i - q
        i = q + off
        ok = (i >= 0) & (i < n)
        a = ab[q[ok], 2 * kl + off]
        if transpose:
            y[q[ok]] += a * v[i[ok]]
        else:
            np.add.at(y, i[ok], a * v[q[ok]])
    return y


def generate() -> dict:
    out, meta = {}, {"assembly": [], "steps": [], "assembly_time": ASSEMBLY_TIME,
                     "assembly_dt": ASSEMBLY_DT, "step_dt": STEP_DT}
    for k, (motion, scen, n1, n2, seed, *over) in enumerate(ASSEMBLY):
        kw = case_params(motion, scen, n1, n2, **(over[0] if over else {}))
        mesh = O.Mesh(O.Params(**kw))
        xms, cps = initial_state(mesh, kw, seed, amp=2e-2, vel_amp=0.05)
        r, ab = mesh.calc_r_K(xms, cps, ASSEMBLY_TIME, ASSEMBLY_DT, nthreads=1)
        kl = mesh.half_bw
        v = np.random.default_rng(1000 + seed).uniform(-1.0, 1.0, mesh.nmdf)
        out.update({f"a{k}_xms": xms, f"a{k}_cps": cps, f"a{k}_v": v, f"a{k}_r": r,
                    f"a{k}_Kdiag": ab[:, 2 * kl].copy(), f"a{k}_Kv": band_matvec(ab, kl, v),
                    f"a{k}_KTv": band_matvec(ab, kl, v, transpose=True)})
        meta["assembly"].append({"params": kw, "nmdf": mesh.nmdf, "half_bw": kl,
                                 "numnp": mesh.numnp, "ndf": mesh.ndf})
    for k, (motion, n1, n2, steps, seed) in enumerate(STEPS):
        kw = case_params(motion, O.F_PULL, n1, n2, pull_speed=1.0)
        mesh = O.Mesh(O.Params(**kw))
        xms, cps = initial_state(mesh, kw, seed, amp=1e-4, vel_amp=0.0)
        out[f"s{k}_xms0"], out[f"s{k}_cps0"] = xms.copy(order="F"), cps.copy(order="F")
        iters, t = [], 0.0
        for _ in range(steps):
            t += STEP_DT
            mesh.update_xms(xms, cps, STEP_DT)
            iters.append(len(mesh.time_step(xms, cps, t, STEP_DT, nthreads=1)))
        out[f"s{k}_xms"], out[f"s{k}_cps"] = xms, cps
        out[f"s{k}_iters"] = np.array(iters, dtype=np.int32)
        meta["steps"].append({"params": kw, "steps": steps, "numnp": mesh.numnp, "ndf": mesh.ndf})
        if k == 0:
            for name, a in (("xms", xms), ("cps", cps)):
                with open(os.path.join(HERE, f"t{steps}-{name}.txt"), "w", newline="\n") as f:
                    f.write(O.writedlm_text(a))
            meta["state_files_step"] = steps
    out["meta"] = np.array(json.dumps(meta))
    return out


def load() -> tuple[dict, dict]:
    """(arrays, meta) of the committed fixture."""
    z = np.load(NPZ)
    arrays = {k: z[k] for k in z.files if k != "meta"}
    return arrays, json.loads(str(z["meta"]))


if __name__ == "__main__":
    data = generate()
    np.savez_compressed(NPZ, **data)
    print(f"wrote {NPZ} ({os.path.getsize(NPZ)} bytes)")
