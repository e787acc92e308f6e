"""Host-side parity (CPU): the library's Mesh / prepare_input against the oracle.

The integer maps (IX, ID, LM, ID_inv: Mesh.jl:276-299, 574-593), the Dirichlet
and Neumann lists (Bc.jl) and the GP tables (GpBasisFn.jl) must be bit-exact.
"""
import numpy as np
import pytest

from _cases import M, O, params_pair

CASES = [(M.LAG, M.F_PULL, 8, 8), (M.ALEVB, M.F_PULL, 32, 32), (M.ALEVB, M.F_PULL, 19, 21),
         (M.ALEVB, M.F_PULL, 64, 64), (M.EUL, M.F_PULL, 5, 6), (M.ALEV, M.F_PULL, 4, 7),
         (M.LAG, M.F_PULL, 1, 1), (M.STATIC, M.F_CAVI, 2, 3), (M.STATIC, M.F_COUE, 3, 4),
         (M.STATIC, M.F_POIS, 5, 4), (M.LAG, M.F_BEND, 3, 3), (M.ALEV, M.F_BEND, 2, 5),
         (M.EUL, M.F_BEND, 8, 2)]


@pytest.mark.parametrize("motion,scenario,n1,n2", CASES)
def test_mesh_bit_exact(motion, scenario, n1, n2):
    p, q = params_pair(motion, scenario, n1, n2, bend_mf=0.5)
    m, o = M.Mesh(p), O.Mesh(q)
    assert (m.numel, m.numnp, m.ndf, m.nmdf) == (o.numel, o.numnp, o.ndf, o.nmdf)
    assert m.dofs == o.dofs
    assert np.array_equal(m.IX, o.IX)
    assert np.array_equal(m.ID, o.ID)
    assert np.array_equal(m.LM, o.LM)
    assert np.array_equal(m.ID_inv, o.ID_inv)
    assert m.half_bw == o.half_bw
    u1, t1 = m.area_tables()
    u2, t2 = o.area_tables()
    assert np.array_equal(u1, u2) and np.array_equal(t1, t2)
    for b in (M.BOTTOM, M.RIGHT, M.TOP, M.LEFT):
        a1, b1 = m.bdry_tables(b)
        a2, b2 = o.bdry_tables(b)
        assert np.array_equal(a1, a2) and np.array_equal(b1, b2)
    assert m.neumann() == o.neumann()
    assert m.dirichlet() == o.dirichlet()


@pytest.mark.parametrize("motion,scenario,n1,n2", [c for c in CASES if c[1] != M.F_BEND and c[2] * c[3] <= 1024])
def test_prepare_input(motion, scenario, n1, n2):
    p, q = params_pair(motion, scenario, n1, n2)
    m, o = M.Mesh(p), O.Mesh(q)
    _, x1, c1 = M.prepare_input(p, m)
    x2, c2 = o.prepare_input()
    # the library solves the separable collocation system per direction, the
    # reference (and oracle) the dense tensor-product system: same values to rounding
    assert np.abs(x1 - x2).max() <= 1e-14 * p.length
    assert np.array_equal(c1, c2)


def test_band_sizes_of_the_configs():
    """Half bandwidths and unknown counts of the benchmark meshes."""
    expect = {(M.LAG, 8): (309, 80), (M.ALEVB, 32): (8430, 543), (M.ALEVB, 64): (33262, 1055)}
    for (mot, n), (nmdf, b) in expect.items():
        m = M.Mesh(M.Params(motion=mot, scenario=M.F_PULL, num1el=n, num2el=n, length=1.0))
        assert (m.nmdf, m.half_bw) == (nmdf, b)


def test_errors_like_the_reference():
    with pytest.raises(M.MafemError):  # Params.jl:93-95
        M.Mesh(M.Params(poly=3))
    with pytest.raises(M.MafemError):  # Bc.jl:266
        M.Mesh(M.Params(scenario=M.F_PULL, pn=1.0))
    with pytest.raises(M.MafemError):  # Params.jl:108-115
        M.Mesh(M.Params(scenario=M.F_CAVI, motion=M.LAG))
    # F_BEND's conditions (Params.jl:100-103), on the library and on the oracle
    bad = [dict(bend_mf=0.4), dict(bend_mf=0.5, motion=M.ALEVB), dict(bend_mf=0.5, motion=M.STATIC),
           dict(bend_mf=0.5, pn=0.1)]
    for over in bad:
        kw = dict(dict(motion=M.LAG), **over)
        p, q = params_pair(kw.pop("motion"), M.F_BEND, 3, 3, **kw)
        with pytest.raises(M.MafemError):
            M.Mesh(p)
        with pytest.raises(O.AssertionFailed):
            O.Mesh(q)
    p, q = params_pair(M.LAG, M.F_BEND, 3, 3, kb=1.4, length=2.0, bend_mf=1.4 / 2 / 2.0)
    assert M.Mesh(p).numnp == O.Mesh(q).numnp == 25
    with pytest.raises(O.AssertionFailed):  # Params.jl:108-115
        O.Mesh(O.Params(scenario=O.F_POIS, motion=O.LAG, num1el=3, num2el=3))


# The two F_PULL extensions (no reference keyword): lambda0 (edge tension and
# initial λ instead of kb / 4, Bc.jl:259, Input.jl:85) and pull_centre (the
# element (floor(n1/2) + 1, floor(n2/2) + 1) instead of ceil(numel / 2),
# PullForce.jl:8-13).  Library and oracle must agree bit for bit.
EXT_CASES = [(M.LAG, 8, 8, 0.0, 1), (M.ALEVB, 12, 12, 2.5, 1), (M.ALEVB, 48, 48, 0.1, 1),
             (M.LAG, 9, 9, 10.0, 0), (M.ALEV, 6, 7, 0.7, 1), (M.ALEVB, 16, 16, 0.0, 0)]


@pytest.mark.parametrize("motion,n1,n2,lam0,centre", EXT_CASES)
def test_pull_extensions_bit_exact(motion, n1, n2, lam0, centre):
    p, q = params_pair(motion, M.F_PULL, n1, n2, kb=1.3, lambda0=lam0, pull_centre=centre)
    m, o = M.Mesh(p), O.Mesh(q)
    assert np.array_equal(m.ID, o.ID) and np.array_equal(m.LM, o.LM) and m.half_bw == o.half_bw
    assert m.neumann() == o.neumann() and m.dirichlet() == o.dirichlet()
    lv = lam0 if lam0 > 0 else 1.3 / 4
    assert [v for _, _, v in m.neumann()] == [lv] * 4
    _, x1, c1 = M.prepare_input(p, m)
    x2, c2 = o.prepare_input()
    assert np.array_equal(c1, c2)
    assert np.all(c1[:, m.dofs[6] - 1] == lv)
    # the pulled nodes: the nine nodes of the chosen element carry the pull speed
    e = (n1 // 2 + 1) + n1 * (n2 // 2) if centre else (n1 * n2 + 1) // 2
    pulled = sorted({nd for u, nd, v in m.dirichlet() if u == 3})
    assert pulled == sorted(m.IX[:, e - 1].tolist())


def test_centre_rule_is_the_reference_rule_for_odd_square_patches():
    for n in (5, 9, 17, 49):
        a = M.Mesh(M.Params(motion=M.LAG, scenario=M.F_PULL, num1el=n, num2el=n, length=1.0, pull_speed=0.1))
        b = M.Mesh(M.Params(motion=M.LAG, scenario=M.F_PULL, num1el=n, num2el=n, length=1.0, pull_speed=0.1,
                            pull_centre=1))
        assert np.array_equal(a.ID, b.ID) and a.dirichlet() == b.dirichlet()


def test_pull_extension_arguments_rejected():
    for kw in (dict(lambda0=-1.0), dict(lambda0=float("nan")), dict(pull_centre=2)):
        p, q = params_pair(M.LAG, M.F_PULL, 4, 4, **kw)
        with pytest.raises(M.MafemError):
            M.Mesh(p)
        if "lambda0" in kw:
            with pytest.raises(O.AssertionFailed):
                O.Mesh(q)
    p, q = params_pair(M.STATIC, M.F_COUE, 3, 3, lambda0=1.0)  # F_PULL only
    with pytest.raises(M.MafemError):
        M.Mesh(p)
    with pytest.raises(O.AssertionFailed):
        O.Mesh(q)
