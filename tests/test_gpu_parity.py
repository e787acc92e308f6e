"""GPU parity: the CUDA path against the CPU oracle on the same seeded inputs.

Tolerances (FP64 path): element residual / global residual 1e-12 and tangent
1e-11 relative to the largest entry (forward-mode duals vs the reference's
complex step differ only by rounding); state after Newton steps 1e-9 relative
(the stated parity bar of the plain FP64 form).  FP32 tangent + FP32 LU + FP64
refinement: Newton converges to the same FP64 solution, checked at 1e-8.
"""
import numpy as np
import pytest

from _cases import M, O, params_pair, rel, state

pytestmark = pytest.mark.gpu

ASSEMBLY_CASES = [
    (M.ALEVB, M.F_PULL, 4, 5), (M.ALEVB, M.F_PULL, 7, 6), (M.ALEV, M.F_PULL, 5, 5),
    (M.LAG, M.F_PULL, 6, 6), (M.EUL, M.F_PULL, 4, 4), (M.LAG, M.F_PULL, 1, 1),
    (M.STATIC, M.F_CAVI, 3, 3), (M.STATIC, M.F_COUE, 4, 3), (M.STATIC, M.F_POIS, 3, 4),
    (M.LAG, M.F_BEND, 3, 4), (M.ALEV, M.F_BEND, 4, 3), (M.ALEVB, M.F_PULL, 20, 19),
]


@pytest.mark.parametrize("motion,scenario,n1,n2", ASSEMBLY_CASES)
def test_calc_r_K_matches_oracle(motion, scenario, n1, n2):
    p, q = params_pair(motion, scenario, n1, n2, bend_mf=0.5, bend_tm=2.0)
    mesh, om = M.Mesh(p), O.Mesh(q)
    xms, cps = state(p, mesh, seed=3, amp=2e-2, vel_amp=0.05)
    time, dt = 0.37, 0.01
    with M.Solver(mesh, p) as s:
        r, ab = s.calc_r_K(xms, cps, time, dt)
    r0, ab0 = om.calc_r_K(xms, cps, time, dt, nthreads=4)
    kl = mesh.half_bw
    assert rel(r, r0) < 1e-12
    assert rel(ab[:, kl:], ab0[:, kl:]) < 1e-11
    assert np.all(ab[:, :kl] == 0.0)  # pivoting-fill rows start empty


@pytest.mark.parametrize("motion,scenario,n1,n2", ASSEMBLY_CASES)
def test_fp32_form_assembly_matches_oracle(motion, scenario, n1, n2):
    """FP32 form: the FP64 residual kernel (one thread per element and Gauss
    point) to the plain form's 1e-12; the all-FP32 tangent to 2e-5 of the
    largest entry (FP32 rounding of primal and tangent arithmetic)."""
    p, q = params_pair(motion, scenario, n1, n2, bend_mf=0.5, bend_tm=2.0)
    mesh, om = M.Mesh(p), O.Mesh(q)
    xms, cps = state(p, mesh, seed=3, amp=2e-2, vel_amp=0.05)
    time, dt = 0.37, 0.01
    with M.Solver(mesh, p, M.FP32_REFINE) as s:
        r, ab = s.calc_r_K(xms, cps, time, dt)
    r0, ab0 = om.calc_r_K(xms, cps, time, dt, nthreads=4)
    kl = mesh.half_bw
    assert rel(r, r0) < 1e-12
    assert rel(ab[:, kl:], ab0[:, kl:]) < 2e-5
    assert np.all(ab[:, :kl] == 0.0)


def test_tangent_is_the_derivative_of_the_residual():
    """Central differences of the GPU residual against the GPU tangent."""
    p, _ = params_pair(M.ALEVB, M.F_PULL, 5, 4)
    mesh = M.Mesh(p)
    xms, cps = state(p, mesh, seed=5, amp=2e-2, vel_amp=0.05)
    dt, h = 0.01, 1e-6
    mmo = [4, 5, 6]
    with M.Solver(mesh, p) as s:
        _, ab = s.calc_r_K(xms, cps, 0.0, dt)
        A = O.band_to_dense(ab, mesh.half_bw, mesh.half_bw, mesh.nmdf)
        J = np.zeros_like(A)
        for q, (node, d) in enumerate(mesh.ID_inv):
            cp, cm = cps.copy(order="F"), cps.copy(order="F")
            xp, xm = xms.copy(order="F"), xms.copy(order="F")
            cp[node - 1, d - 1] += h
            cm[node - 1, d - 1] -= h
            if d in mmo:
                xp[node - 1, mmo.index(d)] += h * dt
                xm[node - 1, mmo.index(d)] -= h * dt
            rp, _ = s.calc_r_K(xp, cp, 0.0, dt, tangent=False)
            rm, _ = s.calc_r_K(xm, cm, 0.0, dt, tangent=False)
            J[:, q] = (rp - rm) / (2 * h)
    # differs from the reference tangent only by the |τ| derivative the reference drops
    assert rel(J, A) < 1e-4


@pytest.mark.parametrize("motion,n", [(M.LAG, 6), (M.ALEVB, 7)])
def test_solve_matches_dense(motion, n):
    p, _ = params_pair(motion, M.F_PULL, n, n)
    mesh = M.Mesh(p)
    xms, cps = state(p, mesh, seed=1, amp=1e-2, vel_amp=0.02)
    with M.Solver(mesh, p) as s:
        r, ab = s.calc_r_K(xms, cps, 0.01, 0.01)
        A = O.band_to_dense(ab, mesh.half_bw, mesh.half_bw, mesh.nmdf)
        du = s.solve(r)
        du2 = s.solve(2.0 * r)  # re-solve with the stored factors
    ref = -np.linalg.solve(A, r)
    assert rel(du, ref) < 1e-10
    assert rel(du2, 2 * ref) < 1e-10


@pytest.mark.parametrize("precision,tol", [(M.PLAIN_FP64, 1e-9), (M.FP32_REFINE, 1e-8)])
@pytest.mark.parametrize("motion,n1,n2,steps", [(M.LAG, 8, 8, 3), (M.ALEVB, 9, 9, 3), (M.ALEVB, 20, 18, 2)])
def test_time_steps_match_oracle(precision, tol, motion, n1, n2, steps):
    p, q = params_pair(motion, M.F_PULL, n1, n2, pull_speed=1.0)
    mesh, om = M.Mesh(p), O.Mesh(q)
    xms, cps = state(p, mesh, seed=0, amp=1e-4)
    x2, c2 = xms.copy(order="F"), cps.copy(order="F")
    dt, t = 0.01, 0.0
    with M.Solver(mesh, p, precision) as s:
        for _ in range(steps):
            t += dt
            om.update_xms(xms, cps, dt)  # predictor on the host, as in run_analysis!
            stats = s.time_step(xms, cps, t, dt)
            om.update_xms(x2, c2, dt)
            eps = om.time_step(x2, c2, t, dt, nthreads=4)
            assert stats["eps"][-1] < p.eps_nr
            if precision == M.PLAIN_FP64:
                assert stats["newton_iters"] == len(eps)
    assert rel(xms, x2) < tol
    ndf = mesh.ndf
    lam = mesh.dofs[6] - 1
    vel = [d for d in range(ndf) if d != lam]
    assert rel(cps[:, vel], c2[:, vel]) < tol
    assert rel(cps[:, lam], c2[:, lam]) < tol


def test_resident_run_matches_host_steps():
    p, _ = params_pair(M.ALEVB, M.F_PULL, 8, 8, pull_speed=1.0)
    mesh = M.Mesh(p)
    xms, cps = state(p, mesh, seed=0, amp=1e-4)
    dts = [0.01] * 3
    with M.Solver(mesh, p) as s:
        s.upload(xms, cps)
        s.run_analysis(dts)
        xa, ca = s.download()
        s.upload(xms, cps)
        t = 0.0
        for dt in dts:
            t += dt
            s.predict(dt)
            s.time_step_resident(t, dt)
        xb, cb = s.download()
    assert np.array_equal(xa, xb) and np.array_equal(ca, cb)


def test_deterministic():
    p, _ = params_pair(M.ALEVB, M.F_PULL, 6, 6)
    mesh = M.Mesh(p)
    xms, cps = state(p, mesh, seed=2, amp=1e-2, vel_amp=0.02)
    with M.Solver(mesh, p) as s:
        r1, a1 = s.calc_r_K(xms, cps, 0.0, 0.01)
        r2, a2 = s.calc_r_K(xms, cps, 0.0, 0.01)
    assert np.array_equal(r1, r2) and np.array_equal(a1, a2)


def test_newton_failure_is_reported_not_hung():
    """A time step that cannot converge in 14 iterations returns the reference's
    assertion as NewtonNotConverged (FiniteElement.jl:61)."""
    p, _ = params_pair(M.LAG, M.F_PULL, 4, 4, eps_nr=1e-300)
    mesh = M.Mesh(p)
    xms, cps = state(p, mesh)
    with M.Solver(mesh, p) as s:
        with pytest.raises(M.NewtonNotConverged):
            s.time_step(xms, cps, 0.01, 0.01)
        assert s.last_stats["newton_iters"] == 14


def _config1():
    p, q = params_pair(M.ALEVB, M.F_PULL, 32, 32, pull_speed=0.1)
    mesh, om = M.Mesh(p), O.Mesh(q)
    _, xms, cps = M.prepare_input(p, mesh)
    M.perturb_interior_z(mesh, xms, seed=0, amp=1e-4)
    return p, mesh, om, xms, cps


def test_config1_assembly_and_solve():
    """Full benchmark size (8430 unknowns, half bandwidth 543)."""
    import scipy.sparse.linalg as sla
    p, mesh, om, xms, cps = _config1()
    dt = 0.005
    om.update_xms(xms, cps, dt)
    with M.Solver(mesh, p) as s:
        r, ab = s.calc_r_K(xms, cps, dt, dt)
        du = s.solve(r)
    r0, ab0 = om.calc_r_K(xms, cps, dt, dt)
    kl = mesh.half_bw
    assert rel(r, r0) < 1e-12
    assert rel(ab[:, kl:], ab0[:, kl:]) < 1e-11
    K = O.band_to_csr(ab0, kl, kl, mesh.nmdf).tocsc()
    ref = -sla.spsolve(K, r0)
    assert rel(du, ref) < 1e-9


def test_config1_steps_match_oracle():
    p, mesh, om, xms, cps = _config1()
    x2, c2 = xms.copy(order="F"), cps.copy(order="F")
    dt, t = 0.005, 0.0
    with M.Solver(mesh, p) as s:
        for _ in range(4):
            t += dt
            om.update_xms(xms, cps, dt)
            st = s.time_step(xms, cps, t, dt)
            om.update_xms(x2, c2, dt)
            eps = O.time_step_sparse(om, x2, c2, t, dt)
            assert st["newton_iters"] == len(eps), (st["eps"], eps)
    assert rel(xms, x2) < 1e-9
    assert rel(cps, c2) < 1e-9
