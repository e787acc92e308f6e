"""calc_pull_force (PullForce.jl:61-80) on the GPU against the oracle.

The pull force is the area-integral velocity residual of the 5x5 elements
around element ceil(numel/2) at that element's nodes, summed (a 3-vector).  It
is checked at the state after Newton steps (where the reference evaluates it,
Analysis.jl:81-91) on an odd mesh (pull element in the centre) and an even
mesh (ceil(numel/2) lies on the right edge, as in the reference), to 1e-11
relative to its largest component (FP64 residual arithmetic on both sides; the
GPU sums in a different order).
"""
import numpy as np
import pytest

from _cases import M, O, params_pair, rel, state

pytestmark = pytest.mark.gpu


# (the 32x32 benchmark mesh with the benchmark's step: larger pull speeds lose
# Newton convergence on it, in the oracle as on the GPU)
# The last two cases use the F_PULL extensions: the centre element of an even
# patch and a tension lambda0 other than kb / 4.
@pytest.mark.parametrize("motion,n,speed,dt,ext", [(M.ALEVB, 9, 1.0, 0.01, {}), (M.ALEVB, 8, 1.0, 0.01, {}),
                                                   (M.LAG, 7, 1.0, 0.01, {}), (M.ALEVB, 32, 0.02, 0.005, {}),
                                                   (M.ALEVB, 8, 1.0, 0.01, dict(pull_centre=1, lambda0=2.0)),
                                                   (M.LAG, 10, 0.5, 0.01, dict(pull_centre=1, lambda0=0.3))])
def test_pull_force_matches_oracle(motion, n, speed, dt, ext):
    p, q = params_pair(motion, M.F_PULL, n, n, pull_speed=speed, **ext)
    mesh, om = M.Mesh(p), O.Mesh(q)
    xms, cps = state(p, mesh, seed=2, amp=1e-4)
    t = 0.0
    with M.Solver(mesh, p) as s:
        for _ in range(2):
            t += dt
            om.update_xms(xms, cps, dt)
            s.time_step(xms, cps, t, dt)
        s.upload(xms, cps)
        f_gpu = s.pull_force()
    f_ref = om.pull_force(xms, cps)
    assert np.all(np.isfinite(f_ref)) and np.abs(f_ref).max() > 0
    assert rel(f_gpu, f_ref) < 1e-11
