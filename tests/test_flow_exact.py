"""Closed-form flows: an independent pin of the assembly, the boundary
conditions, Newton and the solve.

The reference's own tests stop at the Gauss-point geometry (GeoDynStress); its
flat, static scenarios have closed-form steady solutions, and both lie in the
biquadratic B-spline space, so the discrete solution must equal them to
rounding.  With the in-plane stress σ = λ 1 + ζ (∇v + ∇vᵀ) on the square
[-L/2, L/2]² (src/input/Bc.jl:109-153 and 273-310 give the conditions):

* Couette (F_COUE): vx = 0 on the bottom edge, 3 on the top, vy = 0 on every
  edge, normal traction 4 on the left and right edges:
  vx = 3 (y + L/2) / L, vy = 0, λ = 4.
* Poiseuille (F_POIS): vx = 0 on the top and bottom edges, vy = 0 on every
  edge, normal traction 4 on the left edge and 8 on the right:
  λ = 6 + 4 x / L, vx = (4 / L) / (2 ζ) · (L² / 4 - y²), vy = 0.

One time step of the static mesh reaches the steady state (no inertia); the
velocity and λ are then evaluated at every Gauss point through the oracle's
Gauss-point evaluation (GeoDynStress) and compared with the formulas.  CPU: the
oracle; GPU: the CUDA path in both precisions, its state read back and
evaluated the same way.
"""
import numpy as np
import pytest

from _cases import M, O, params_pair

CASES = [  # (scenario, num1el, num2el, length, zeta_v)
    (M.F_COUE, 4, 5, 2.0, 1.5), (M.F_COUE, 6, 4, 1.0, 0.7), (M.F_POIS, 4, 5, 2.0, 1.5),
    (M.F_POIS, 6, 4, 1.0, 0.7), (M.F_POIS, 5, 5, 3.0, 2.0),
]
DT = 0.01


def _exact(scenario, L, zv, X, Y):
    if scenario == M.F_COUE:
        return 3.0 * (Y + L / 2) / L, np.zeros_like(Y), np.full_like(X, 4.0)
    dlam = 4.0 / L
    return dlam / (2.0 * zv) * (L * L / 4 - Y * Y), np.zeros_like(Y), 6.0 + dlam * X


def _check(om, scenario, L, zv, xms, cps, tol):
    pts = []
    for e in range(1, om.numel + 1):
        for g in range(1, 10):
            d = om.gds(xms, cps, e, g)
            pts.append((d["x"][0], d["x"][1], d["v"][0], d["v"][1], d["lam"]))
    X, Y, vx, vy, lam = np.array(pts).T
    ex, ey, el = _exact(scenario, L, zv, X, Y)
    vs = max(np.abs(ex).max(), 1.0)
    assert np.abs(vx - ex).max() < tol * vs
    assert np.abs(vy - ey).max() < tol * vs
    assert np.abs(lam - el).max() < tol * np.abs(el).max()


def _setup(scenario, n1, n2, L, zv):
    p, q = params_pair(M.STATIC, scenario, n1, n2, length=L, zeta_v=zv)
    return p, q, O.Mesh(q)


@pytest.mark.parametrize("scenario,n1,n2,L,zv", CASES)
def test_oracle_reaches_the_closed_form_flow(scenario, n1, n2, L, zv):
    _, _, om = _setup(scenario, n1, n2, L, zv)
    xms, cps = om.prepare_input()
    eps = om.time_step(xms, cps, DT, DT, nthreads=2)
    assert len(eps) <= 3  # a linear problem: one correction, then the check
    _check(om, scenario, L, zv, xms, cps, 1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [M.PLAIN_FP64, M.FP32_REFINE])
@pytest.mark.parametrize("scenario,n1,n2,L,zv", CASES)
def test_gpu_reaches_the_closed_form_flow(scenario, n1, n2, L, zv, precision):
    p, _, om = _setup(scenario, n1, n2, L, zv)
    mesh = M.Mesh(p)
    _, xms, cps = M.prepare_input(p, mesh)
    with M.Solver(mesh, p, precision) as s:
        s.time_step(xms, cps, DT, DT)
    _check(om, scenario, L, zv, xms, cps, 1e-12 if precision == M.PLAIN_FP64 else 1e-9)
