"""All four moving-mesh motions on the tether pull: Lagrangian, Eulerian, ALE
and ALE-viscous-bending (src/input/Enums.jl:56-73) describe the same
membrane, so the physical response must not depend on the motion.

CPU: on a 7 x 7 patch pulled at 0.05 from flat, the oracle's pull force
(calc_pull_force, src/analysis/PullForce.jl:61-80) agrees across the four
motions to within 3e-6 k² (relative) after k steps: the motions discretise
the mesh's movement differently, and that difference accumulates as the
surface moves.  Its in-plane components vanish by symmetry (odd n: the pull
element is central).  A wrong mesh-motion coupling term would break both.

GPU: the CUDA path steps every motion in both precisions, and each trajectory
and pull force matches the oracle's (1e-9 plain FP64, 1e-8 FP32 +
refinement), which extends the time-step parity of the Lagrangian and ALEVB
motions to the Eulerian and ALE ones.
"""
import numpy as np
import pytest

from _cases import M, O, params_pair, rel, state

MOTIONS = [M.LAG, M.EUL, M.ALEV, M.ALEVB]
N, SPEED, DT, STEPS = 7, 0.05, 0.01, 10


def _setup(motion):
    p, q = params_pair(motion, M.F_PULL, N, N, pull_speed=SPEED)
    mesh = M.Mesh(p)
    xms, cps = state(p, mesh, amp=0.0)
    return p, q, mesh, xms, cps


def _oracle_run(q, xms, cps):
    om = O.Mesh(q)
    xms, cps = xms.copy(order="F"), cps.copy(order="F")
    t, forces = 0.0, []
    for _ in range(STEPS):
        t += DT
        om.update_xms(xms, cps, DT)
        om.time_step(xms, cps, t, DT, nthreads=2)
        forces.append(om.pull_force(xms, cps))
    return xms, cps, np.array(forces)


def test_oracle_pull_force_does_not_depend_on_the_motion():
    forces = np.array([_oracle_run(q, x, c)[2] for (_, q, _, x, c) in map(_setup, MOTIONS)])
    fz = forces[:, :, 2]
    assert np.all(fz > 0)
    spread = (fz.max(axis=0) - fz.min(axis=0)) / fz.max(axis=0)
    k = np.arange(1, STEPS + 1)
    assert np.all(spread < 3e-6 * k * k), spread
    assert np.abs(forces[:, :, :2]).max() < 1e-12 * fz.max()


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(M.PLAIN_FP64, 1e-9), (M.FP32_REFINE, 1e-8)])
@pytest.mark.parametrize("motion", MOTIONS)
def test_gpu_motion_steps_and_pull_force_match_oracle(motion, precision, tol):
    p, q, mesh, xms, cps = _setup(motion)
    xo, co, fo = _oracle_run(q, xms, cps)
    forces = []
    with M.Solver(mesh, p, precision) as s:
        s.upload(xms, cps)
        t = 0.0
        for _ in range(STEPS):
            t += DT
            s.predict(DT)
            s.time_step_resident(t, DT)
            forces.append(s.pull_force())
        x, c = s.download()
    assert rel(x, xo) < tol and rel(c, co) < tol
    assert rel(np.array(forces), fo) < tol
