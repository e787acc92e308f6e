"""Closed-form solutions: an independent pin of the assembly, the boundary
conditions, Newton and the solve.

The reference's own tests stop at the Gauss-point geometry (GeoDynStress).
Three of its scenarios have closed-form steady states, which pin what those
tests do not.  Each state is evaluated at every Gauss point through the
oracle's Gauss-point evaluation (GeoDynStress) and compared with its formula.
The checks run on the oracle (CPU) and on the CUDA path (GPU, its state read
back and evaluated the same way).

Flows.  The flat static scenarios' steady solutions lie in the biquadratic
B-spline space, so the discrete solution must equal them to rounding.  Take
the in-plane stress σ = λ 1 + ζ (∇v + ∇vᵀ) on the square [-L/2, L/2]²
(src/input/Bc.jl:110-157 and 273-316 give the conditions):

* Couette (F_COUE): vx = 0 on the bottom edge, 3 on the top, vy = 0 on every
  edge, normal traction 4 on the left and right edges:
  vx = 3 (y + L/2) / L, vy = 0, λ = 4.
* Poiseuille (F_POIS): vx = 0 on the top and bottom edges, vy = 0 on every
  edge, normal traction 4 on the left edge and 8 on the right:
  λ = 6 + 4 x / L, vx = (4 / L) / (2 ζ) · (L² / 4 - y²), vy = 0.

One time step of the static mesh reaches the steady state (no inertia).

Bending (F_BEND, Lagrangian).  The patch [0, L]² gets the moment kb / (2L) on
its left and right edges, ramped up over bend_tm (src/input/Bc.jl:319-393,
Params.jl:97-100).  It settles into a cylinder of half-angle 1/2:
H = 1 / (2L), K = 0, and λ = kb / (4L²), the analytical values with which
src/Input.jl:68-69 initialises λ and src/Output.jl:142 measures the error.
Both ends stay at z = 0 (v = 0 on the left edge, vz = 0 on the right,
src/input/Bc.jl:369-386), so the section is the arc of radius L about
(L sin 1/2, L cos 1/2) in the x-z plane.  (analyze_output's position error Er,
src/Output.jl:163, measures the distance from (sin 1, cos 1) instead, the
centre of an arc whose left end stays horizontal; with these boundary
conditions it does not tend to zero, so only its Eλ and EH are checked.)  The
top and bottom edges are moment-free, which a cylinder satisfies only with
kg = -kb / 2 (the reference's defaults kb = 1, kg = -0.5).  The B-spline
surface approximates the circle: on 8 x 2 elements the mean of H is within
1e-3 of 1/(2L), every point within 1e-2 and within 2e-3 L of the arc (under
refinement the error of the mean falls as h², the pointwise one as h); K
vanishes to rounding.  The Eulerian mesh (its nodes move only along the
normal) settles into the same cylinder.  It has the same mean H and the mean
of λ within 2e-3, and its pointwise errors are larger: H within 5e-2, the arc
within 1e-2 L.  The ALE mesh is still relaxing long after the membrane has
settled and is not checked here.
"""
import numpy as np
import pytest

from _cases import M, O, params_pair, state

FLOWS = [  # (scenario, num1el, num2el, length, zeta_v)
    (M.F_COUE, 4, 5, 2.0, 1.5), (M.F_COUE, 6, 4, 1.0, 0.7), (M.F_POIS, 4, 5, 2.0, 1.5),
    (M.F_POIS, 6, 4, 1.0, 0.7), (M.F_POIS, 5, 5, 3.0, 2.0),
]
FLOW_DT = 0.01
BENDS = [  # (motion, num1el, num2el, length, kb, zeta_v)
    (M.LAG, 8, 2, 1.0, 1.0, 1.0), (M.LAG, 8, 2, 1.0, 2.0, 1.0), (M.LAG, 8, 2, 2.0, 4.0, 1.0),
    (M.LAG, 8, 3, 1.0, 0.5, 0.5), (M.EUL, 8, 2, 1.0, 1.0, 1.0), (M.EUL, 8, 2, 2.0, 3.0, 1.5),
]
BEND_DT, BEND_STEPS = 0.05, 40  # the moment reaches its final value at t = 1, the state settles by t = 1.5


def _gauss_points(om, xms, cps, fields):
    out = []
    for e in range(1, om.numel + 1):
        for g in range(1, 10):
            d = om.gds(xms, cps, e, g)
            out.append([d[f] if np.isscalar(d[f]) else d[f][k] for f, k in fields])
    return np.array(out).T


def _flow_exact(scenario, L, zv, X, Y):
    if scenario == M.F_COUE:
        return 3.0 * (Y + L / 2) / L, np.zeros_like(Y), np.full_like(X, 4.0)
    dlam = 4.0 / L
    return dlam / (2.0 * zv) * (L * L / 4 - Y * Y), np.zeros_like(Y), 6.0 + dlam * X


def _check_flow(om, scenario, L, zv, xms, cps, tol):
    X, Y, vx, vy, lam = _gauss_points(om, xms, cps, [("x", 0), ("x", 1), ("v", 0), ("v", 1), ("lam", 0)])
    ex, ey, el = _flow_exact(scenario, L, zv, X, Y)
    vs = max(np.abs(ex).max(), 1.0)
    assert np.abs(vx - ex).max() < tol * vs
    assert np.abs(vy - ey).max() < tol * vs
    assert np.abs(lam - el).max() < tol * np.abs(el).max()


def _flow_setup(scenario, n1, n2, L, zv):
    p, q = params_pair(M.STATIC, scenario, n1, n2, length=L, zeta_v=zv)
    return p, q, O.Mesh(q)


def _bend_setup(motion, n1, n2, L, kb, zv):
    p, q = params_pair(motion, M.F_BEND, n1, n2, length=L, kb=kb, kg=-kb / 2, zeta_v=zv,
                       bend_mf=kb / 2 / L, bend_tm=1.0)
    om = O.Mesh(q)
    mesh = M.Mesh(p)
    xms, cps = state(p, mesh, amp=0.0)
    cps[:, mesh.dofs[6] - 1] = kb / 4 / L**2 * (BEND_DT / 1.0) ** 2  # src/Input.jl:69
    return p, mesh, om, xms, cps


def _check_bend(om, motion, L, kb, xms, cps):
    H, K, lam, X, Z = _gauss_points(om, xms, cps, [("H", 0), ("K", 0), ("lam", 0), ("x", 0), ("x", 2)])
    r = np.hypot(X - L * np.sin(0.5), Z - L * np.cos(0.5))
    lag = motion == M.LAG
    assert np.abs(r / L - 1.0).max() < (2e-3 if lag else 1e-2)
    assert abs(H.mean() * 2 * L - 1.0) < 1e-3
    assert np.abs(H * 2 * L - 1.0).max() < (1e-2 if lag else 5e-2)
    assert np.abs(K).max() * L * L < 1e-12
    lam_n = lam * 4 * L * L / kb
    assert abs(lam_n.mean() - 1.0) < 2e-3
    if lag:
        assert np.abs(lam_n - 1.0).max() < 2e-2


@pytest.mark.parametrize("scenario,n1,n2,L,zv", FLOWS)
def test_oracle_reaches_the_closed_form_flow(scenario, n1, n2, L, zv):
    _, _, om = _flow_setup(scenario, n1, n2, L, zv)
    xms, cps = om.prepare_input()
    eps = om.time_step(xms, cps, FLOW_DT, FLOW_DT, nthreads=2)
    assert len(eps) <= 3  # a linear problem: one correction, then the check
    _check_flow(om, scenario, L, zv, xms, cps, 1e-12)


@pytest.mark.parametrize("motion,n1,n2,L,kb,zv", BENDS)
def test_oracle_bends_into_the_cylinder(motion, n1, n2, L, kb, zv):
    _, _, om, xms, cps = _bend_setup(motion, n1, n2, L, kb, zv)
    t = 0.0
    for _ in range(BEND_STEPS):
        t += BEND_DT
        om.update_xms(xms, cps, BEND_DT)
        om.time_step(xms, cps, t, BEND_DT, nthreads=2)
    _check_bend(om, motion, L, kb, xms, cps)


def test_oracle_bending_error_falls_under_refinement():
    """The mean of H, and analyze_output's Eλ and EH (src/Output.jl:129-180)."""
    errs, norms = [], []
    for n1 in (4, 8, 16):
        _, _, om, xms, cps = _bend_setup(M.LAG, n1, 2, 1.0, 1.0, 1.0)
        t = 0.0
        for _ in range(BEND_STEPS):
            t += BEND_DT
            om.update_xms(xms, cps, BEND_DT)
            om.time_step(xms, cps, t, BEND_DT, nthreads=2)
        (H,) = _gauss_points(om, xms, cps, [("H", 0)])
        errs.append(abs(H.mean() * 2 - 1.0))
        norms.append(O.bend_errors(om, xms, cps)[1:])
    assert errs[0] > 3.5 * errs[1] > 12.0 * errs[2]  # the mean's error: about h^2 each halving
    (el4, eh4), (el8, eh8), (el16, eh16) = norms
    assert el8 < 2e-3 and eh8 < 2e-3
    assert el4 > 2.0 * el8 > 4.0 * el16 and eh4 > 2.0 * eh8 > 4.0 * eh16


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [M.PLAIN_FP64, M.FP32_REFINE])
@pytest.mark.parametrize("scenario,n1,n2,L,zv", FLOWS)
def test_gpu_reaches_the_closed_form_flow(scenario, n1, n2, L, zv, precision):
    p, _, om = _flow_setup(scenario, n1, n2, L, zv)
    mesh = M.Mesh(p)
    _, xms, cps = M.prepare_input(p, mesh)
    with M.Solver(mesh, p, precision) as s:
        s.time_step(xms, cps, FLOW_DT, FLOW_DT)
    _check_flow(om, scenario, L, zv, xms, cps, 1e-12 if precision == M.PLAIN_FP64 else 1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("motion,n1,n2,L,kb,zv", BENDS)
def test_gpu_bends_into_the_cylinder(motion, n1, n2, L, kb, zv):
    p, mesh, om, xms, cps = _bend_setup(motion, n1, n2, L, kb, zv)
    with M.Solver(mesh, p) as s:
        s.upload(xms, cps)
        t = 0.0
        for _ in range(BEND_STEPS):
            t += BEND_DT
            s.predict(BEND_DT)
            s.time_step_resident(t, BEND_DT)
        xms, cps = s.download()
    _check_bend(om, motion, L, kb, xms, cps)
