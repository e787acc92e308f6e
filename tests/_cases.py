"""Shared helpers for the parity tests: build matching product/oracle meshes and
seeded states."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "membranealefem.jl_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import mafem as M  # noqa: E402
import oracle as O  # noqa: E402


def params_pair(motion, scenario, n1, n2, **kw):
    kw.setdefault("length", 1.0)
    kw.setdefault("pull_speed", 0.5)
    p = M.Params(motion=motion, scenario=scenario, num1el=n1, num2el=n2,
                 **{k: v for k, v in kw.items() if k != "zv"})
    q = O.Params(motion=motion, scenario=scenario, num1el=n1, num2el=n2,
                 **{("zv" if k == "zeta_v" else k): v for k, v in kw.items()})
    return p, q


def state(p, mesh, seed=0, amp=1e-2, vel_amp=0.0):
    """Flat initial state with seeded z perturbation (and optional seeded
    velocities on the free unknowns) so every physics term is exercised."""
    if p.scenario == M.F_BEND:
        xms = np.zeros((mesh.numnp, 3), order="F")
        s1 = np.arange(mesh.numnp) % mesh.num1np
        s2 = np.arange(mesh.numnp) // mesh.num1np
        xms[:, 0] = p.length * np.maximum(0, np.minimum(1, (s1 - 0.5) / (mesh.num1np - 2)))
        xms[:, 1] = p.length * np.maximum(0, np.minimum(1, (s2 - 0.5) / (mesh.num2np - 2)))
        cps = np.zeros((mesh.numnp, mesh.ndf), order="F")
        cps[:, mesh.dofs[6] - 1] = 0.25
    else:
        _, xms, cps = M.prepare_input(p, mesh)
    M.perturb_interior_z(mesh, xms, seed=seed, amp=amp)
    if vel_amp:
        u = M.splitmix64(seed + 17, mesh.numnp * mesh.ndf).reshape(mesh.ndf, mesh.numnp).T
        ID = mesh.ID.T  # numnp x ndf
        cps = np.asfortranarray(cps + np.where(ID > 0, vel_amp * (2 * u - 1), 0.0))
    return np.asfortranarray(xms), np.asfortranarray(cps)


def rel(a, b):
    s = np.abs(b).max()
    return float(np.abs(a - b).max() / (s if s > 0 else 1.0))
