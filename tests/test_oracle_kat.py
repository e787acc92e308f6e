"""Pin the CPU oracle against every known-answer test of the reference's own suite.

Each test restates one block of the reference's tests (test/input/spline_tests.jl,
test/input/gauss_pt_tests.jl, test/input/gp_basis_fn_tests.jl,
test/analysis/geo_dyn_stress_tests.jl) with the same inputs, expected values and
tolerances (``eps(x)`` is the spacing of doubles at x, i.e. ``np.spacing(x)``).
"""
import math

import numpy as np
import pytest

import oracle as O
from oracle import AssertionFailed, CLAMPED, CLOSED, KnotVector

eps = np.spacing  # Julia eps(x)
norm = np.linalg.norm


# ---- test/input/spline_tests.jl:3-46 (knot span) -----------------------------
def test_knot_span():
    kv0 = KnotVector([0., 0., 0., 0.3, 0.5, 0.5, 0.6, 1., 1., 1.], 0, CLAMPED)
    assert O.get_knot_span_index(kv0, 0.0) == 3
    assert O.get_knot_span_index(kv0, 0.5) == 6
    assert O.get_knot_span_index(kv0, 1.0) == 7

    kv1 = KnotVector([0., 0., 0., 1., 2., 3., 4., 4., 4.], 2, CLAMPED)
    for z, s in [(0.0, 3), (0.7, 3), (1.0, 4), (1.3, 4), (2.0, 5), (2.1, 5), (3.0, 6),
                 (3.9, 6), (4.0, 6)]:
        assert O.get_knot_span_index(kv1, z) == s
    with pytest.raises(AssertionFailed):
        O.get_knot_span_index(kv1, -0.1)
    with pytest.raises(AssertionFailed):
        O.get_knot_span_index(kv1, 4.1)

    kv1_dup = KnotVector([0., 0., 0., 1., 2., 3., 4., 4., 4.], 2, CLAMPED)
    assert kv1 == kv1_dup and hash(kv1) == hash(kv1_dup)
    kv1_nz = KnotVector([0., 0., 0., 1.0001, 2., 3., 4., 4., 4.], 2, CLAMPED)
    assert kv1 != kv1_nz and hash(kv1) != hash(kv1_nz)

    for zs, poly, curve in [([2., 2., 2., 3., 4., 4., 4.], 3, CLAMPED),
                            ([2., 2., 2., 3., 4., 4.], 2, CLAMPED),
                            ([2., 2., 2., 3., 2.5, 4., 4., 4.], 2, CLAMPED),
                            ([2., 2., 2., 3., 4., 4., 4.], 2, CLOSED)]:
        with pytest.raises(AssertionFailed):
            KnotVector(zs, poly, curve)

    kv2 = KnotVector.uniform(4, 3, CLOSED)
    for z in (-0.75, 1.1, 1.75):
        with pytest.raises(AssertionFailed):
            O.get_knot_span_index(kv2, z)
    for z, s in [(0.0, 4), (0.2, 4), (0.4, 5), (0.5, 6), (0.75, 7), (1.0, 7)]:
        assert O.get_knot_span_index(kv2, z) == s


# ---- spline_tests.jl:48-71 (B-spline values) ---------------------------------
def test_bspline_vals():
    kv1 = KnotVector([0., 0., 0., 1., 2., 3., 4., 4., 5., 5., 5.], 2, CLAMPED)
    assert norm(O.get_bspline_vals(kv1, 2.5) - [1 / 8, 6 / 8, 1 / 8]) < eps(8.)
    kv2 = KnotVector([0., 0., 0., 1 / 3, 2 / 3, 1., 1., 1.], 2, CLAMPED)
    assert norm(O.get_bspline_vals(kv2, 0.0) - [1., 0., 0.]) < eps(8.)
    assert norm(O.get_bspline_vals(kv2, 1 / 3 - eps(1.0)) - [0., 1 / 2, 1 / 2]) < eps(8.)
    assert norm(O.get_bspline_vals(kv2, 1 / 3) - [1 / 2, 1 / 2, 0.]) < eps(8.)
    assert kv2 == KnotVector.uniform(3, 2, CLAMPED)
    assert hash(kv2) == hash(KnotVector.uniform(3, 2, CLAMPED))
    zs3 = [0., 0., 0., 0.3, 0.5, 0.5, 0.6, 1., 1., 1.]
    kv3 = KnotVector(zs3, 1, CLAMPED)
    for z, v in [(0.00, [1.00, 0.00]), (0.15, [0.50, 0.50]), (0.35, [0.75, 0.25]),
                 (0.53, [0.70, 0.30]), (0.60, [1.00, 0.00]), (0.90, [0.25, 0.75])]:
        assert norm(O.get_bspline_vals(kv3, z) - v) < eps(8.)


# ---- spline_tests.jl:73-114 (B-spline derivatives) ---------------------------
def test_bspline_ders():
    kv1 = KnotVector([0., 0., 0., 1., 2., 3., 4., 4., 5., 5., 5.], 2, CLAMPED)
    assert norm(O.get_bspline_ders(kv1, 2.5, 2)[:, 0] - [1 / 8, 6 / 8, 1 / 8]) < eps(8.)
    kv2 = KnotVector([0., 0., 0., 1 / 3, 2 / 3, 1., 1., 1.], 2, CLAMPED)
    assert norm(O.get_bspline_ders(kv2, 0.0, 0)[:, 0] - [1., 0., 0.]) < eps(8.)
    assert norm(O.get_bspline_ders(kv2, 1 / 3 - eps(1.0), 0)[:, 0] - [0., 1 / 2, 1 / 2]) < eps(8.)
    assert norm(O.get_bspline_ders(kv2, 1 / 3, 1)[:, 0] - [1 / 2, 1 / 2, 0.]) < eps(8.)
    assert norm(O.get_bspline_ders(kv2, 1 / 2, 1) - np.array([[0.125, -1.5], [0.75, 0], [0.125, 1.5]])) < eps(8.)
    zs3 = [0., 0., 0., 0.3, 0.5, 0.5, 0.6, 1., 1., 1.]
    kv3 = KnotVector(zs3, 1, CLAMPED)
    for z, d, tol in [(0.00, [-10 / 3, 10 / 3], 8.), (0.15, [-10 / 3, 10 / 3], 8.), (0.35, [-5, 5], 8.),
                      (0.53, [-10, 10], 16.), (0.60, [-2.5, 2.5], 8.), (0.90, [-2.5, 2.5], 8.)]:
        assert norm(O.get_bspline_ders(kv3, z, 1)[:, 1] - d) < eps(tol)
    kv4 = KnotVector(zs3, 2, CLAMPED)
    for z, d, tol in [(0.00, [200 / 9, -320 / 9, 40 / 3], 64.), (0.15, [200 / 9, -320 / 9, 40 / 3], 64.),
                      (0.35, [20, -70, 50], 64.), (0.53, [200, -240, 40], 2e3),
                      (0.60, [10, -22.5, 12.5], 128.), (0.90, [10, -22.5, 12.5], 128.),
                      (1.00, [10, -22.5, 12.5], 128.)]:
        assert norm(O.get_bspline_ders(kv4, z, 2)[:, 2] - d) < eps(tol)
    for z, nd in [(0.50, -1), (0.50, 3), (-0.01, 2), (1.01, 2)]:
        with pytest.raises(AssertionFailed):
            O.get_bspline_ders(kv4, z, nd)


# ---- spline_tests.jl:116-144 (global indices) --------------------------------
def test_bspline_indices():
    zs1 = [0., 0., 0., 0.3, 0.5, 0.5, 0.6, 1., 1., 1.]
    kv1 = KnotVector(zs1, 2, CLAMPED)
    for z, ids in [(0.00, [1, 2, 3]), (0.29, [1, 2, 3]), (0.30, [2, 3, 4]), (0.49, [2, 3, 4]),
                   (0.50, [4, 5, 6]), (0.59, [4, 5, 6]), (0.60, [5, 6, 7]), (0.69, [5, 6, 7]),
                   (1.00, [5, 6, 7])]:
        assert O.get_bspline_indices(kv1, z) == ids
    kv2 = KnotVector(zs1, 1, CLAMPED)
    for z, ids in [(0.00, [2, 3]), (0.29, [2, 3]), (0.30, [3, 4]), (0.49, [3, 4]), (0.50, [5, 6]),
                   (0.59, [5, 6]), (0.60, [6, 7]), (0.69, [6, 7]), (1.00, [6, 7])]:
        assert O.get_bspline_indices(kv2, z) == ids


# ---- spline_tests.jl:146-162 (control points reproduce polynomials) ----------
def test_control_points():
    kvs = [KnotVector([0., 0., 0., 1 / 3, 2 / 3, 1., 1., 1.], 2, CLAMPED),
           KnotVector([0., 0., 0., 0., 1 / 3, 2 / 3, 1., 1., 1., 1.], 3, CLAMPED)]
    for kv in kvs:
        for f in (lambda x: x, lambda x: 3 * x + 1, lambda x: 1 - 4 * (x - 0.5) ** 2):
            cps = O.get_1d_bspline_cps(kv, f)
            for z in np.arange(0.0, 1.0 + 1e-12, 0.1):
                z = min(z, 1.0)
                val = np.dot(O.get_bspline_vals(kv, z), cps[np.array(O.get_bspline_indices(kv, z)) - 1])
                assert math.isclose(val, f(z), rel_tol=math.sqrt(np.finfo(float).eps))
    for zs, poly in [([1., 1., 2., 3., 3.], 1), ([1., 1., 1., 1., 1., 2., 3., 3., 3., 3., 3.], 4),
                     ([1., 1., 1., 2., 2., 3., 3., 3.], 2)]:
        with pytest.raises(AssertionFailed):
            O.get_1d_bspline_cps(KnotVector(zs, poly, CLAMPED), lambda x: x)


# ---- spline_tests.jl:164-220 (unique 1-D elements) ---------------------------
def test_unique_1d_elements():
    cases = [
        (KnotVector.uniform(2, 2, CLAMPED), 2, 2, [1, 2], [(0.0, 1 / 2), (1 / 2, 1.0)]),
        (KnotVector.uniform(5, 2, CLAMPED), 5, 5, [1, 2, 3, 4, 5],
         [(0.0, 1 / 5), (1 / 5, 2 / 5), (2 / 5, 3 / 5), (3 / 5, 4 / 5), (4 / 5, 1.0)]),
        (KnotVector.uniform(8, 2, CLAMPED), 5, 8, [1, 2, 3, 3, 3, 3, 4, 5],
         [(0.0, 1 / 8), (1 / 8, 2 / 8), (2 / 8, 3 / 8), (6 / 8, 7 / 8), (7 / 8, 1.0)]),
        (KnotVector([0., 0., 0., 1., 2., 3., 4., 5., 6., 7., 8., 8.1, 8.2, 8.3, 8.4, 8.5, 8.6, 8.7,
                     8.8, 8.9, 9., 10., 11., 12., 13., 14., 15., 16., 17., 17., 17.], 2, CLAMPED),
         15, 26, [1, 2, 3, 3, 3, 3, 4, 5, 6, 7, 8, 8, 8, 8, 8, 8, 9, 10, 11, 12, 13, 13, 13, 13, 14, 15],
         [(0., 1.), (1., 2.), (2., 3.), (6., 7.), (7., 8.), (8., 8.1), (8.1, 8.2), (8.2, 8.3),
          (8.8, 8.9), (8.9, 9.), (9., 10.), (10., 11.), (11., 12.), (15., 16.), (16., 17.)]),
        (KnotVector.uniform(3, 3, CLAMPED), 3, 3, [1, 2, 3], [(0.0, 1 / 3), (1 / 3, 2 / 3), (2 / 3, 1.0)]),
        (KnotVector.uniform(6, 3, CLAMPED), 6, 6, [1, 2, 3, 4, 5, 6],
         [(0.0, 1 / 6), (1 / 6, 2 / 6), (2 / 6, 3 / 6), (3 / 6, 4 / 6), (4 / 6, 5 / 6), (5 / 6, 1.0)]),
        (KnotVector.uniform(9, 3, CLAMPED), 7, 9, [1, 2, 3, 4, 4, 4, 5, 6, 7],
         [(0.0, 1 / 9), (1 / 9, 2 / 9), (2 / 9, 3 / 9), (3 / 9, 4 / 9), (6 / 9, 7 / 9), (7 / 9, 8 / 9),
          (8 / 9, 1.0)]),
        (KnotVector([0., 0., 0., 0., 1., 2., 3., 4., 5., 6., 7., 8., 8.1, 8.2, 8.3, 8.4, 8.5, 8.6, 8.7,
                     8.8, 8.9, 9., 10., 11., 12., 13., 14., 15., 16., 17., 17., 17., 17.], 3, CLAMPED),
         21, 26, [1, 2, 3, 4, 4, 5, 6, 7, 8, 9, 10, 11, 11, 11, 11, 12, 13, 14, 15, 16, 17, 18, 18, 19, 20, 21],
         [(0., 1.), (1., 2.), (2., 3.), (3., 4.), (5., 6.), (6., 7.), (7., 8.), (8., 8.1), (8.1, 8.2),
          (8.2, 8.3), (8.3, 8.4), (8.7, 8.8), (8.8, 8.9), (8.9, 9.), (9., 10.), (10., 11.), (11., 12.),
          (12., 13.), (14., 15.), (15., 16.), (16., 17.)]),
        (KnotVector.uniform(5, 2, CLOSED), 1, 5, [1, 1, 1, 1, 1], [(0, 0.2)]),
    ]
    for kv, un, ne, ids, lst in cases:
        u, n, i, l = O.get_unique_1d_elements(kv)
        assert (u, n, i) == (un, ne, ids)
        assert l == [(float(a), float(b)) for a, b in lst]


# ---- spline_tests.jl:222-225 (collocation) -----------------------------------
def test_collocate():
    for poly in (2, 3):
        np.testing.assert_allclose(O.collocate_z(KnotVector.uniform(5, poly, CLOSED)),
                                   [0.1, 0.3, 0.5, 0.7, 0.9], rtol=math.sqrt(np.finfo(float).eps))


# ---- test/input/gauss_pt_tests.jl:3-23 ---------------------------------------
def test_gauss_points():
    xs, ws = O.gauss_xi(3)
    assert list(xs) == [-math.sqrt(3 / 5), 0, math.sqrt(3 / 5)]
    assert list(ws) == [5 / 9, 8 / 9, 5 / 9]
    xs4, ws4 = O.gauss_xi(4)
    assert norm(xs4 - [-math.sqrt(3 / 7 + 2 / 7 * math.sqrt(6 / 5)), -math.sqrt(3 / 7 - 2 / 7 * math.sqrt(6 / 5)),
                       math.sqrt(3 / 7 - 2 / 7 * math.sqrt(6 / 5)), math.sqrt(3 / 7 + 2 / 7 * math.sqrt(6 / 5))]) < eps(1.)
    assert list(ws4) == [(18 - math.sqrt(30)) / 36, (18 + math.sqrt(30)) / 36, (18 + math.sqrt(30)) / 36,
                         (18 - math.sqrt(30)) / 36]
    zs, wz = O.gauss_zeta(3, 0.5, 3.5)
    assert norm(zs - (xs * 1.5 + 2.0)) < eps(1.)
    assert norm(wz - ws * 1.5) < eps(1.)
    zs, wz = O.gauss_zeta(4, 1.0, 6.0)
    assert norm(zs - (xs4 * 2.5 + 3.5)) < eps(1.)
    assert norm(wz - ws4 * 2.5) < eps(1.)


# ---- test/input/gp_basis_fn_tests.jl:4-14 ------------------------------------
def test_gp_basis_fns_z():
    kv1 = KnotVector.uniform(4, 2, CLAMPED)
    f = O.gp_basis_fns_z(0.1, 0.4, kv1)
    D = O.get_bspline_ders(kv1, 0.4, 2)
    assert f.w == 0.1
    assert np.array_equal(f.N, D[:, 0]) and np.array_equal(f.dN, D[:, 1]) and np.array_equal(f.ddN, D[:, 2])
    for z in (-0.1, 1.1):
        with pytest.raises(AssertionFailed):
            O.gp_basis_fns_z(0.1, z, kv1)


# ---- gp_basis_fn_tests.jl:17-37 (tensor products) ----------------------------
def test_gp_basis_fns_za():
    kv3 = KnotVector([0., 0., 0., 1., 3., 3.5, 6., 6., 6.], 2, CLAMPED)
    kv4 = KnotVector([2., 2., 2., 4., 5., 5., 5.], 2, CLAMPED)
    rng = np.random.default_rng(7)  # the reference draws these weights unseeded
    for z1 in np.arange(0.0, 6.0 + 1e-9, 1.5):
        for z2 in np.arange(2.0, 5.0 + 1e-9, 1.5):
            w1, w2 = rng.random(), rng.random()
            f1 = O.gp_basis_fns_z(w1, z1, kv3)
            f2 = O.gp_basis_fns_z(w2, z2, kv4)
            g = O.gp_basis_fns_za(f1, f2)
            assert g.w == f1.w * f2.w
            for i1 in range(3):
                for i2 in range(3):
                    a = i1 + 3 * i2
                    assert g.N[a] == f1.N[i1] * f2.N[i2]
                    assert g.dN[a, 0] == f1.dN[i1] * f2.N[i2]
                    assert g.dN[a, 1] == f1.N[i1] * f2.dN[i2]
                    assert g.ddN[a, 0] == f1.ddN[i1] * f2.N[i2]
                    assert g.ddN[a, 1] == f1.N[i1] * f2.ddN[i2]
                    assert g.ddN[a, 2] == f1.dN[i1] * f2.dN[i2]


# ---- gp_basis_fn_tests.jl:40-74 (line basis functions) -----------------------
def test_line_gp_basis_fns():
    kv3s = KnotVector([1., 1., 1., 2., 3., 4., 5., 6., 7., 8., 8., 8.], 2, CLAMPED)
    kv3l = KnotVector([1., 1., 1., 2., 3., 4., 5., 6., 7., 8., 9., 10., 11., 12., 12., 12.], 2, CLAMPED)
    fs = O.LineGpBasisFns(kv3s, 3)
    fl = O.LineGpBasisFns(kv3l, 3)
    assert fs.nel == 7 and fl.nel == 11
    assert max(fs.uel_ids) == 5 and max(fl.uel_ids) == 5
    for i in range(5):
        for j in range(3):
            assert fs.ufns[i][j] == fl.ufns[i][j]
    z01, _ = O.gauss_zeta(3, 0.0, 1.0)
    assert np.array_equal(fs.ufns[0][0].N, O.get_bspline_ders(kv3s, z01[0] + 1, 0)[:, 0])
    assert np.array_equal(fs.ufns[1][1].dN, O.get_bspline_ders(kv3l, z01[1] + 2, 1)[:, 1])
    assert np.array_equal(fs.ufns[3][2].N, O.get_bspline_ders(kv3l, z01[2] + 8, 0)[:, 0])
    assert np.array_equal(fs.ufns[3][2].ddN, O.get_bspline_ders(kv3l, z01[2] + 8, 2)[:, 2])
    assert np.array_equal(fs.ufns[4][0].N, O.get_bspline_ders(kv3l, z01[0] + 11, 0)[:, 0])
    kv2 = KnotVector([0., 0., 0., 3., 4., 4.5, 6.5, 9., 9.6, 10.1, 10.1, 10.1], 2, CLAMPED)
    f2 = O.LineGpBasisFns(kv2, 3)
    assert max(f2.uel_ids) == 7
    assert not np.array_equal(f2.ufns[0][0].N, f2.ufns[6][2].N)
    assert not np.array_equal(f2.ufns[0][0].N, f2.ufns[6][0].N)
    z03, _ = O.gauss_zeta(3, 0.0, 3.0)
    assert np.array_equal(f2.ufns[0][0].N, O.get_bspline_ders(kv2, z03[0], 0)[:, 0])
    z96, _ = O.gauss_zeta(3, 9.0, 9.6)
    assert np.array_equal(f2.ufns[5][1].N, O.get_bspline_ders(kv2, z96[1], 0)[:, 0])


# ---- test/analysis/geo_dyn_stress_tests.jl:5-55 (curved patch) ---------------
def _cavi_mesh(n1, n2):
    return O.Mesh(O.Params(motion=O.STATIC, scenario=O.F_CAVI, num1el=n1, num2el=n2))


def test_geo_dyn_stress_curved_patch():
    m = _cavi_mesh(2, 3)
    k1, k2 = m.knots()
    kv1, kv2 = KnotVector(k1, 2), KnotVector(k2, 2)
    xms = np.zeros((m.numnp, 3), order="F")
    cps = np.zeros((m.numnp, m.ndf), order="F")
    A, B = 2.2, 1.7
    xc = O.get_1d_bspline_cps(kv1, lambda z1: 4 * z1 + 2)
    yc = O.get_1d_bspline_cps(kv2, lambda z2: 2 * z2 - 3)
    zc = O.get_2d_bspline_cps(kv1, kv2, lambda z1, z2: A * (4 * z1 - 2) ** 2 + B * (2 * z2 - 1) ** 2)
    for node in range(1, m.numnp + 1):
        xms[node - 1, 0] = xc[(node - 1) % m.num1np]
        xms[node - 1, 1] = yc[(node - 1) // m.num1np]
        xms[node - 1, 2] = zc[node - 1]
    for e in range(1, m.numel + 1):
        for gp in range(1, 10):
            g = m.gds(xms, cps, e, gp)
            x, y, z = g["x"]
            assert math.isclose(z, A * (x - 4) ** 2 + B * (y + 2) ** 2, rel_tol=math.sqrt(np.finfo(float).eps))
            assert norm(g["a"] - np.array([[4., 0.], [0., 2.], [8 * A * (x - 4), 4 * B * (y + 2)]])) < eps(4e2)
            a_ab = g["a"].T @ g["a"]
            ainv = g["ainv"]
            assert norm(ainv @ a_ab - np.eye(2)) < eps(1e2)
            assert norm(a_ab @ ainv - np.eye(2)) < eps(1e2)
            assert abs(np.trace(ainv @ g["b"]) / 2 - g["H"]) < eps(1e1)
            assert abs(np.linalg.det(ainv @ g["b"]) - g["K"]) < eps(1e1)


# ---- geo_dyn_stress_tests.jl:57-119 (flat patch, Couette / Poiseuille) -------
def test_geo_dyn_stress_flat_patch():
    m = _cavi_mesh(3, 2)
    k1, k2 = m.knots()
    kv1, kv2 = KnotVector(k1, 2), KnotVector(k2, 2)
    xms = np.zeros((m.numnp, 3), order="F")
    cc = np.zeros((m.numnp, m.ndf), order="F")
    cp = np.zeros((m.numnp, m.ndf), order="F")
    xc = O.get_1d_bspline_cps(kv1, lambda z1: 4 * z1 + 2)
    yc = O.get_1d_bspline_cps(kv2, lambda z2: 2 * z2 - 3)
    w, U = 12., 16.
    cv = O.get_1d_bspline_cps(kv2, lambda z2: 2 * w * z2)
    pv = O.get_1d_bspline_cps(kv1, lambda z1: -4 * U * (z1 ** 2 - z1))
    for node in range(1, m.numnp + 1):
        xms[node - 1, 0] = xc[(node - 1) % m.num1np]
        xms[node - 1, 1] = yc[(node - 1) // m.num1np]
        cc[node - 1, 0] = cv[(node - 1) // m.num1np]   # Dof.vx
        cp[node - 1, 1] = pv[(node - 1) % m.num1np]    # Dof.vy
    area = 0.0
    _, ufns = m.area_tables()
    uel, _ = m.area_tables()
    zv = m.p.zv
    for e in range(1, m.numel + 1):
        for gp in range(1, 10):
            gc = m.gds(xms, cc, e, gp)
            gpp = m.gds(xms, cp, e, gp)
            area += gpp["J"] * ufns[uel[e - 1] - 1, gp - 1, 0]
            x = gc["x"][0]
            assert norm(gc["sig"] - zv * np.array([0., 0., 2 * w / 8])) < eps(2e2)
            assert norm(gpp["sig"] - zv * np.array([0., 0., U * (4 - x) / 8])) < eps(3e2)
    assert math.isclose(area, 8.0, rel_tol=math.sqrt(np.finfo(float).eps))
