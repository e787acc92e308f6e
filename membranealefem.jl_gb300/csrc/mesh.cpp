// mesh.cpp -- host-side construction of the reference's Mesh and initial state.
//
// Restates Mesh(p; args...) (src/input/Mesh.jl:94-302), the scenario boundary
// conditions (src/input/Bc.jl) and prepare_input's default initial state
// (src/Input.jl:40-108) in the layout the C ABI uses (mafem_mesh_desc: the
// reference's own 1-based, column-major arrays).  A Julia caller does not need
// this file: it passes its own `mesh` through mafem_mesh_desc.  The Python
// host API and the benchmarks use it to build meshes without Julia.
//
// Implementation choices (same results, different structure from the
// reference): elements are knot spans, so basis functions are evaluated with
// the element's span known in closed form instead of a binary search; IX uses
// the tensor-product formula IX[n1 + 3(n2-1), e1 + nel1(e2-1)] =
// (e1+n1-1) + num1np (e2+n2-2) (Mesh.jl:582-589); the flat-patch collocation
// solve is done per direction because the target functions are separable.

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "mafem.h"
#include "mafem_internal.h"

namespace mafem {

namespace {

constexpr int P = 2;  // POLY (Params.jl:161)

// Clamped uniform knots (Spline.jl:76-96).
std::vector<double> uniform_knots(int nel) {
  std::vector<double> z(nel + 2 * P + 1, 0.0);
  for (int k = 1; k < nel; ++k) z[P + k] = (double)k / nel;
  for (int k = nel + P; k < (int)z.size(); ++k) z[k] = 1.0;
  return z;
}

// Knots concentrated at the centre for F_PULL with >= 18 elements
// (Spline.jl:122-183), written with 0-based knot positions.
std::vector<double> graded_knots(int nel) {
  const int num = nel + 2 * P + 1;
  std::vector<double> z(num, 0.0);
  const int w1 = 6, f1 = nel - 2 * w1 - 1;
  const double zw1 = 1.0 / 3.0, zf1 = 1.0 - 2 * zw1;
  const double d1 = zw1 / w1;
  for (int k = 1; k <= w1; ++k) z[P + k] = k * d1;  // level 1, left: ζ = k Δζ
  // level 1, right: ζs[idx] = 1 - ζw1 + (idx - num + poly + w1) Δζ for the
  // 1-based idx = num-poly-w1 .. num-poly-1, i.e. 0-based num-P-w1-1+k, k = 0..w1-1
  for (int k = 0; k < w1; ++k) z[num - P - w1 - 1 + k] = 1.0 - zw1 + (double)k * d1;
  const int w2 = f1 / 4, f2 = f1 - 2 * w2;
  const double zw2 = 1.0 / 9.0, zf2 = zf1 - 2 * zw2;
  if (2 * w2 <= w1) {
    const double d = zf1 / (f1 + 1);
    for (int idx = P + w1 + 2; idx <= num - P - w1 - 1; ++idx) z[idx - 1] = zw1 + (idx - P - w1 - 1) * d;
  } else {
    double d = zw2 / w2;
    for (int idx = w1 + P + 2; idx <= w1 + P + 1 + w2; ++idx) z[idx - 1] = zw1 + (idx - w1 - P - 1) * d;
    for (int idx = num - P - w1 - w2; idx <= num - P - w1 - 1; ++idx)
      z[idx - 1] = 1.0 - zw1 - zw2 + (idx - num + P + w1 + w2) * d;
    d = zf2 / (f2 + 1);
    for (int idx = w1 + P + 2 + w2; idx <= num - P - w1 - w2 - 1; ++idx)
      z[idx - 1] = zw1 + zw2 + (idx - w1 - P - 1 - w2) * d;
  }
  for (int k = num - P - 1; k < num; ++k) z[k] = 1.0;
  return z;
}

// Values and first/second derivatives of the P+1 non-zero B-splines of knot
// span `s` (0-based index of the knot that starts the span) at u; the
// Piegl-Tiller algorithm A2.3 (The NURBS Book, 2nd ed., section 2.5).
void basis_ders(const std::vector<double>& U, int s, double u, double N[3], double dN[3], double ddN[3]) {
  double ndu[P + 1][P + 1], left[P + 1], right[P + 1];
  ndu[0][0] = 1.0;
  for (int j = 1; j <= P; ++j) {
    left[j] = u - U[s + 1 - j];
    right[j] = U[s + j] - u;
    double saved = 0.0;
    for (int r = 0; r < j; ++r) {
      ndu[j][r] = right[r + 1] + left[j - r];
      double t = ndu[r][j - 1] / ndu[j][r];
      ndu[r][j] = saved + right[r + 1] * t;
      saved = left[j - r] * t;
    }
    ndu[j][j] = saved;
  }
  double ders[3][P + 1];
  for (int j = 0; j <= P; ++j) ders[0][j] = ndu[j][P];
  double a[2][P + 1];
  for (int r = 0; r <= P; ++r) {
    int s1 = 0, s2 = 1;
    a[0][0] = 1.0;
    for (int k = 1; k <= 2; ++k) {
      double d = 0.0;
      int rk = r - k, pk = P - k;
      if (r >= k) {
        a[s2][0] = a[s1][0] / ndu[pk + 1][rk];
        d = a[s2][0] * ndu[rk][pk];
      }
      int j1 = (rk >= -1) ? 1 : -rk;
      int j2 = (r - 1 <= pk) ? k - 1 : P - r;
      for (int j = j1; j <= j2; ++j) {
        a[s2][j] = (a[s1][j] - a[s1][j - 1]) / ndu[pk + 1][rk + j];
        d += a[s2][j] * ndu[rk + j][pk];
      }
      if (r <= pk) {
        a[s2][k] = -a[s1][k - 1] / ndu[pk + 1][r];
        d += a[s2][k] * ndu[r][pk];
      }
      ders[k][r] = d;
      std::swap(s1, s2);
    }
  }
  for (int j = 0; j <= P; ++j) {
    N[j] = ders[0][j];
    dN[j] = ders[1][j] * P;
    ddN[j] = ders[2][j] * (P * (P - 1));
  }
}

struct Line {  // per-direction tables (LineGpBasisFns, GpBasisFn.jl:143-202)
  int nel = 0;
  std::vector<int> uel;                 // element -> unique element (0-based)
  std::vector<std::array<double, 10>> ufns;  // [uel*3 + gp] -> w, N[3], dN[3], ddN[3]
  std::array<double, 10> zmin{}, zmax{};
};

std::array<double, 10> pack1(double w, const double N[3], const double dN[3], const double ddN[3]) {
  std::array<double, 10> f{};
  f[0] = w;
  for (int i = 0; i < 3; ++i) { f[1 + i] = N[i]; f[4 + i] = dN[i]; f[7 + i] = ddN[i]; }
  return f;
}

bool close_rel(double x, double y) {  // Julia isapprox, rtol = sqrt(eps)
  return x == y || std::fabs(x - y) <= 1.4901161193847656e-08 * std::max(std::fabs(x), std::fabs(y));
}

Line line_tables(const std::vector<double>& U) {
  Line L;
  const int num = (int)U.size();
  L.nel = num - 2 * P - 1;
  L.uel.resize(L.nel);
  // element e (0-based) is knot span s = e + P; it is "unique" when the knot
  // spacings around it differ from the previous element's (Spline.jl:640-671)
  std::array<double, 2 * P + 1> prev{}, ctx{};
  const double xi[3] = {-std::sqrt(3.0 / 5), 0.0, std::sqrt(3.0 / 5)};
  const double wx[3] = {5.0 / 9, 8.0 / 9, 5.0 / 9};
  int nu = 0;
  for (int e = 0; e < L.nel; ++e) {
    int s = e + P;
    for (int q = 0; q < 2 * P + 1; ++q) ctx[q] = U[s - P + 1 + q] - U[s - P + q];
    bool same = true;
    for (int q = 0; q < 2 * P + 1; ++q) same = same && close_rel(ctx[q], prev[q]);
    if (!same) {
      ++nu;
      double lo = U[s], hi = U[s + 1];
      for (int g = 0; g < 3; ++g) {  // GaussPointsζ (GaussPoint.jl:72-77)
        double u = xi[g] * (hi - lo) / 2 + (hi + lo) / 2;
        double w = wx[g] * (hi - lo) / 2;
        double N[3], dN[3], ddN[3];
        basis_ders(U, s, u, N, dN, ddN);
        L.ufns.push_back(pack1(w, N, dN, ddN));
      }
    }
    L.uel[e] = nu - 1;
    prev = ctx;
  }
  double N[3], dN[3], ddN[3];
  basis_ders(U, P, U[0], N, dN, ddN);
  L.zmin = pack1(1.0, N, dN, ddN);
  basis_ders(U, num - P - 2, U[num - 1], N, dN, ddN);
  L.zmax = pack1(1.0, N, dN, ddN);
  return L;
}

// Tensor product of two 1-D GP basis records (GpBasisFnsζα, GpBasisFn.jl:102-110),
// packed as 55 doubles: w, N[9], dN 9x2, ddN 9x3 (column-major).
void tensor55(const std::array<double, 10>& f1, const std::array<double, 10>& f2, double* o) {
  o[0] = f1[0] * f2[0];
  for (int i2 = 0; i2 < 3; ++i2)
    for (int i1 = 0; i1 < 3; ++i1) {
      int a = i1 + 3 * i2;
      o[1 + a] = f1[1 + i1] * f2[1 + i2];
      o[10 + a] = f1[4 + i1] * f2[1 + i2];
      o[19 + a] = f1[1 + i1] * f2[4 + i2];
      o[28 + a] = f1[7 + i1] * f2[1 + i2];
      o[37 + a] = f1[1 + i1] * f2[7 + i2];
      o[46 + a] = f1[4 + i1] * f2[4 + i2];
    }
}

}  // namespace

// ---------------------------------------------------------------------------
int build_mesh(const mafem_params& p, const mafem_args& args, HostMesh& M, std::string& err) {
  if (p.poly != 2 || p.nen != 9 || p.nders != 2 || p.gp1d != 3) {
    err = "only poly = 2, nen = 9, nders = 2, gp1d = 3 are supported (Params.jl:93-95)";
    return MAFEM_ERR_UNSUPPORTED;
  }
  if (p.num1el < 1 || p.num2el < 1) { err = "num1el/num2el must be >= 1"; return MAFEM_ERR_ARG; }
  if (p.scenario < MAFEM_F_CAVI || p.scenario > MAFEM_F_BEND) { err = "unknown scenario"; return MAFEM_ERR_ARG; }
  if (p.motion < MAFEM_STATIC || p.motion > MAFEM_ALEVB) { err = "unknown motion"; return MAFEM_ERR_ARG; }
  if (!(args.lambda0 >= 0.0) || !std::isfinite(args.lambda0)) { err = "lambda0 must be finite and >= 0 (0: kb / 4)"; return MAFEM_ERR_ARG; }
  if (args.pull_centre != 0 && args.pull_centre != 1) { err = "pull_centre must be 0 or 1"; return MAFEM_ERR_ARG; }
  if (args.lambda0 > 0.0 && p.scenario != MAFEM_F_PULL) { err = "lambda0 is an F_PULL extension"; return MAFEM_ERR_ARG; }
  M.lambda0 = pull_tension(p, args);  // kb / 4 for every scenario but a F_PULL run given lambda0
  const int n1 = p.num1el, n2 = p.num2el, numel = n1 * n2;
  const int n1np = n1 + P, n2np = n2 + P, numnp = n1np * n2np;
  M.num1el = n1; M.num2el = n2; M.numel = numel; M.num1np = n1np; M.num2np = n2np; M.numnp = numnp;

  const bool fine = p.scenario == MAFEM_F_PULL && n1 >= 18 && n2 >= 18;  // Mesh.jl:176-185
  M.kv1 = fine ? graded_knots(n1) : uniform_knots(n1);
  M.kv2 = fine ? graded_knots(n2) : uniform_knots(n2);
  Line l1 = line_tables(M.kv1), l2 = line_tables(M.kv2);
  const int nu1 = (int)l1.ufns.size() / 3, nu2 = (int)l2.ufns.size() / 3;

  // area tables (AreaGpBasisFns, GpBasisFn.jl:325-356)
  M.n_uel = nu1 * nu2;
  M.uel_ids.resize(numel);
  for (int e2 = 0; e2 < n2; ++e2)
    for (int e1 = 0; e1 < n1; ++e1) M.uel_ids[e1 + n1 * e2] = 1 + l1.uel[e1] + nu1 * l2.uel[e2];
  M.ufns.assign((size_t)M.n_uel * 9 * 55, 0.0);
  for (int u2 = 0; u2 < nu2; ++u2)
    for (int u1 = 0; u1 < nu1; ++u1)
      for (int g2 = 0; g2 < 3; ++g2)
        for (int g1 = 0; g1 < 3; ++g1)
          tensor55(l1.ufns[u1 * 3 + g1], l2.ufns[u2 * 3 + g2],
                   &M.ufns[((size_t)(u1 + nu1 * u2) * 9 + g1 + 3 * g2) * 55]);

  // boundary tables (BdryGpBasisFns, Mesh.jl:220-225); BOTTOM/TOP run along ζ¹
  for (int b = 0; b < 4; ++b) {
    const Line& ln = (b == 0 || b == 2) ? l1 : l2;
    const auto& perp = b == 0 ? l2.zmin : b == 1 ? l1.zmax : b == 2 ? l2.zmax : l1.zmin;
    int nu = (int)ln.ufns.size() / 3;
    M.bdry_n_uel[b] = nu;
    M.bdry_uel_ids[b].resize(ln.nel);
    for (int e = 0; e < ln.nel; ++e) M.bdry_uel_ids[b][e] = ln.uel[e] + 1;
    M.bdry_ufns[b].assign((size_t)nu * 3 * 55, 0.0);
    for (int u = 0; u < nu; ++u)
      for (int g = 0; g < 3; ++g) {
        double* o = &M.bdry_ufns[b][((size_t)u * 3 + g) * 55];
        if (b == 0 || b == 2) tensor55(ln.ufns[u * 3 + g], perp, o);
        else tensor55(perp, ln.ufns[u * 3 + g], o);
      }
  }

  // IX (Mesh.jl:574-593) in closed form
  M.IX.resize((size_t)9 * numel);
  for (int e2 = 0; e2 < n2; ++e2)
    for (int e1 = 0; e1 < n1; ++e1)
      for (int a2 = 0; a2 < 3; ++a2)
        for (int a1 = 0; a1 < 3; ++a1)
          M.IX[(size_t)(a1 + 3 * a2) + 9 * (size_t)(e1 + n1 * e2)] = 1 + (e1 + a1) + (int64_t)n1np * (e2 + a2);

  // node sets (Mesh.jl:144-173); 1-based node numbers
  auto node = [&](int s1, int s2) { return (int64_t)1 + s1 + (int64_t)n1np * s2; };
  std::vector<int64_t> bn[4], bin[4];
  for (int s = 0; s < n1np; ++s) {
    bn[0].push_back(node(s, 0)); bin[0].push_back(node(s, 1));
    bn[2].push_back(node(s, n2np - 1)); bin[2].push_back(node(s, n2np - 2));
  }
  for (int s = 0; s < n2np; ++s) {
    bn[1].push_back(node(n1np - 1, s)); bin[1].push_back(node(n1np - 2, s));
    bn[3].push_back(node(0, s)); bin[3].push_back(node(1, s));
  }

  // scenario dofs and Dirichlet set (Bc.jl)
  std::fill(std::begin(M.dofs), std::end(M.dofs), 0);
  enum { VX = 0, VY, VZ, VMX, VMY, VMZ, LAM, PM };
  bool three = p.scenario == MAFEM_F_CAVI || p.scenario == MAFEM_F_COUE || p.scenario == MAFEM_F_POIS;
  if (three) {
    if (p.motion != MAFEM_STATIC) { err = "flat 2-D scenarios need STATIC motion (Params.jl:108-115)"; return MAFEM_ERR_ARG; }
    M.dofs[VX] = 1; M.dofs[VY] = 2; M.dofs[LAM] = 3; M.ndf = 3;
  } else if (p.motion == MAFEM_LAG || p.motion == MAFEM_STATIC) {  // Bc.jl:414-431
    M.dofs[VX] = 1; M.dofs[VY] = 2; M.dofs[VZ] = 3; M.dofs[LAM] = 4; M.ndf = 4;
  } else if (p.motion == MAFEM_EUL) {
    for (int u = 0; u < 6; ++u) M.dofs[u] = u + 1;
    M.dofs[LAM] = 7; M.ndf = 7;
  } else {
    for (int u = 0; u < 8; ++u) M.dofs[u] = u + 1;
    M.ndf = 8;
  }
  const int ndf = M.ndf;
  std::vector<char> fixed((size_t)ndf * numnp, 0);
  auto fix = [&](int u, int64_t nd) {
    if (M.dofs[u]) fixed[(size_t)(M.dofs[u] - 1) + (size_t)ndf * (nd - 1)] = 1;
  };
  M.dir_unknown.clear(); M.dir_node.clear(); M.dir_val.clear();
  M.neu_bdry.clear(); M.neu_type.clear(); M.neu_val.clear();
  auto dir = [&](int u1, int64_t nd, double v) { M.dir_unknown.push_back(u1); M.dir_node.push_back(nd); M.dir_val.push_back(v); };
  auto neu = [&](int b, int t, double v) { M.neu_bdry.push_back(b); M.neu_type.push_back(t); M.neu_val.push_back(v); };
  const bool ale = p.motion == MAFEM_ALEV || p.motion == MAFEM_ALEVB;
  switch (p.scenario) {
    case MAFEM_F_CAVI:  // Bc.jl:58-106
      for (int b = 0; b < 4; ++b) for (auto nd : bn[b]) { fix(VX, nd); fix(VY, nd); }
      for (auto nd : bn[2]) if (nd != node(0, n2np - 1) && nd != node(n1np - 1, n2np - 1)) dir(1, nd, 1.0);
      { int64_t c = numnp / 2 + 1; fix(LAM, c); dir(7, c, 0.0); }
      break;
    case MAFEM_F_COUE:  // Bc.jl:122-157
      for (int b : {0, 2}) for (auto nd : bn[b]) { fix(VX, nd); fix(VY, nd); }
      for (auto nd : bn[2]) dir(1, nd, 3.0);
      for (int b : {1, 3}) for (auto nd : bn[b]) fix(VY, nd);
      neu(MAFEM_LEFT, MAFEM_STRETCH, 4.0); neu(MAFEM_RIGHT, MAFEM_STRETCH, 4.0);
      break;
    case MAFEM_F_POIS:  // Bc.jl:286-316
      for (int b : {0, 2}) for (auto nd : bn[b]) { fix(VX, nd); fix(VY, nd); }
      for (int b : {1, 3}) for (auto nd : bn[b]) fix(VY, nd);
      neu(MAFEM_LEFT, MAFEM_STRETCH, 4.0); neu(MAFEM_RIGHT, MAFEM_STRETCH, 8.0);
      break;
    case MAFEM_F_BEND:  // Bc.jl:347-393
      if (p.motion == MAFEM_STATIC || p.motion == MAFEM_ALEVB) { err = "F_BEND needs LAG, EUL or ALEV motion (Params.jl:101-102)"; return MAFEM_ERR_ARG; }
      // Params.jl:100 and 103, the same exact comparison: (kb / 2) / length
      if (args.bend_mf != p.kb / 2 / p.length) { err = "F_BEND needs bend_mf == kb / 2 / length: the half-angle is 1/2 (Params.jl:100)"; return MAFEM_ERR_ARG; }
      if (p.pn != 0.0) { err = "F_BEND with a normal pressure is not implemented (Params.jl:103)"; return MAFEM_ERR_ARG; }
      for (int b : {0, 2}) for (auto nd : bn[b]) { fix(VY, nd); if (ale) fix(VMY, nd); }
      for (auto nd : bn[3]) { fix(VX, nd); fix(VY, nd); fix(VZ, nd); if (ale) { fix(VMX, nd); fix(VMY, nd); fix(VMZ, nd); } }
      for (auto nd : bn[1]) { fix(VZ, nd); if (ale) fix(VMZ, nd); }
      neu(MAFEM_LEFT, MAFEM_MOMENT, args.bend_mf); neu(MAFEM_RIGHT, MAFEM_MOMENT, args.bend_mf);
      break;
    case MAFEM_F_PULL: {  // Bc.jl:188-269
      if (p.pn != 0.0) { err = "F_PULL with a normal pressure is not implemented (Bc.jl:266)"; return MAFEM_ERR_ARG; }
      for (int b = 0; b < 4; ++b) for (auto nd : bn[b]) { fix(VZ, nd); if (ale) { fix(VMX, nd); fix(VMY, nd); fix(VMZ, nd); } }
      for (int b = 0; b < 4; ++b) for (auto nd : bin[b]) { fix(VZ, nd); if (p.motion == MAFEM_ALEVB) fix(VMZ, nd); }
      const int ce = pull_element(n1, n2, args);  // get_pull_el_id (PullForce.jl:8-13), or the centre element
      for (int a = 0; a < 9; ++a) {
        int64_t nd = M.IX[(size_t)a + 9 * (size_t)(ce - 1)];
        fix(VX, nd); fix(VY, nd); fix(VZ, nd); dir(3, nd, args.pull_speed);
        if (p.motion != MAFEM_LAG) { fix(VMX, nd); fix(VMY, nd); fix(VMZ, nd); dir(6, nd, args.pull_speed); }
      }
      for (int b = 0; b < 4; ++b) {  // rigid-body constraints at the middle of each edge
        int64_t c = bn[b][bn[b].size() / 2];
        fix(VX, c); fix(VY, c);
        if (p.motion != MAFEM_LAG) { fix(VMX, c); fix(VMY, c); }
      }
      const double lv = pull_tension(p, args);  // kb / 4 (Bc.jl:259) unless lambda0 is given
      neu(MAFEM_LEFT, MAFEM_STRETCH, lv); neu(MAFEM_RIGHT, MAFEM_STRETCH, lv);
      neu(MAFEM_TOP, MAFEM_STRETCH, lv); neu(MAFEM_BOTTOM, MAFEM_STRETCH, lv);
      break;
    }
  }
  // ID, node-major / dof-minor numbering (Mesh.jl:276-284)
  M.ID.assign((size_t)ndf * numnp, 0);
  int64_t next = 1;
  for (int nd = 0; nd < numnp; ++nd)
    for (int d = 0; d < ndf; ++d)
      if (!fixed[(size_t)d + (size_t)ndf * nd]) M.ID[(size_t)d + (size_t)ndf * nd] = next++;
  M.nmdf = next - 1;
  return MAFEM_OK;
}

void mesh_desc(const HostMesh& M, mafem_mesh_desc& d) {
  std::memset(&d, 0, sizeof d);
  d.num1el = M.num1el; d.num2el = M.num2el; d.numel = M.numel;
  d.num1np = M.num1np; d.num2np = M.num2np; d.numnp = M.numnp;
  d.ndf = M.ndf; d.nmdf = M.nmdf;
  for (int u = 0; u < 8; ++u) d.dofs[u] = M.dofs[u];
  d.IX = M.IX.data(); d.ID = M.ID.data();
  d.n_uel = M.n_uel; d.uel_ids = M.uel_ids.data(); d.ufns = M.ufns.data();
  for (int b = 0; b < 4; ++b) {
    d.bdry_n_uel[b] = M.bdry_n_uel[b];
    d.bdry_uel_ids[b] = M.bdry_uel_ids[b].data();
    d.bdry_ufns[b] = M.bdry_ufns[b].data();
  }
  d.n_neu = (int64_t)M.neu_bdry.size();
  d.neu_bdry = M.neu_bdry.data(); d.neu_type = M.neu_type.data(); d.neu_val = M.neu_val.data();
  d.n_dir = (int64_t)M.dir_node.size();
  d.dir_unknown = M.dir_unknown.data(); d.dir_node = M.dir_node.data(); d.dir_val = M.dir_val.data();
}

// Solve the 1-D collocation system (Spline.jl:510-528) for f at the
// collocation points (Spline.jl:589-620, poly = 2): the matrix is tridiagonal.
static std::vector<double> collocate_1d(const std::vector<double>& U, double (*f)(double, double), double L) {
  const int num = (int)U.size(), nb = num - P - 1, nel = num - 2 * P - 1;
  std::vector<double> zc(nb);
  zc[0] = U[0];
  zc[nb - 1] = U[num - 1];
  for (int i = 1; i < nb - 1; ++i) zc[i] = (U[P + i - 1] + U[P + i]) / 2;  // midpoints of unique knots
  std::vector<double> A((size_t)nb * nb, 0.0), b(nb);
  for (int j = 0; j < nb; ++j) {
    int e = 0;  // span containing zc[j]
    while (e < nel - 1 && zc[j] >= U[P + e + 1]) ++e;
    double N[3], dN[3], ddN[3];
    basis_ders(U, P + e, zc[j], N, dN, ddN);
    for (int q = 0; q < 3; ++q) A[(size_t)j * nb + e + q] = N[q];
    b[j] = f(zc[j], L);
  }
  // dense Gaussian elimination with partial pivoting (nb is small)
  for (int k = 0; k < nb; ++k) {
    int pv = k;
    for (int i = k + 1; i < nb; ++i)
      if (std::fabs(A[(size_t)i * nb + k]) > std::fabs(A[(size_t)pv * nb + k])) pv = i;
    if (pv != k) {
      for (int c = 0; c < nb; ++c) std::swap(A[(size_t)k * nb + c], A[(size_t)pv * nb + c]);
      std::swap(b[k], b[pv]);
    }
    for (int i = k + 1; i < nb; ++i) {
      double m = A[(size_t)i * nb + k] / A[(size_t)k * nb + k];
      if (m == 0.0) continue;
      for (int c = k; c < nb; ++c) A[(size_t)i * nb + c] -= m * A[(size_t)k * nb + c];
      b[i] -= m * b[k];
    }
  }
  for (int k = nb - 1; k >= 0; --k) {
    double s = b[k];
    for (int c = k + 1; c < nb; ++c) s -= A[(size_t)k * nb + c] * b[c];
    b[k] = s / A[(size_t)k * nb + k];
  }
  return b;
}

int prepare_input(const HostMesh& M, const mafem_params& p, double* xms, double* cps, std::string& err) {
  if (p.scenario == MAFEM_F_BEND) {
    err = "F_BEND's initial state draws from the unseeded global RNG (Input.jl:53-60); pass xms/cps explicitly";
    return MAFEM_ERR_UNSUPPORTED;
  }
  const int np = M.numnp, ndf = M.ndf;
  std::fill(xms, xms + (size_t)np * 3, 0.0);
  std::fill(cps, cps + (size_t)np * ndf, 0.0);
  // x = L(ζ¹ - 1/2), y = L(ζ² - 1/2): the tensor-product collocation system
  // (Spline.jl:540-567) separates, and partition of unity makes the other
  // direction's factor exactly 1.
  auto fx = [](double z, double L) { return L * (z - 0.5); };
  std::vector<double> cx = collocate_1d(M.kv1, fx, p.length), cy = collocate_1d(M.kv2, fx, p.length);
  for (int s2 = 0; s2 < M.num2np; ++s2)
    for (int s1 = 0; s1 < M.num1np; ++s1) {
      xms[s1 + (size_t)M.num1np * s2] = cx[s1];
      xms[(size_t)np + s1 + (size_t)M.num1np * s2] = cy[s2];
    }
  const double lv = M.lambda0;  // Input.jl:85-86: kb / 4 unless lambda0 is given
  for (int i = 0; i < np; ++i) cps[i + (size_t)np * (M.dofs[6] - 1)] = lv;
  for (size_t q = 0; q < M.dir_node.size(); ++q) {  // Input.jl:103-108
    int u = (int)M.dir_unknown[q];
    cps[(M.dir_node[q] - 1) + (size_t)np * (M.dofs[u - 1] - 1)] = M.dir_val[q];
    if (p.scenario == MAFEM_F_PULL && p.motion == MAFEM_EUL)
      cps[(M.dir_node[q] - 1) + (size_t)np * (M.dofs[5] - 1)] = M.dir_val[q];
  }
  return MAFEM_OK;
}

}  // namespace mafem

// ---- C ABI -------------------------------------------------------------------
struct mafem_mesh {
  mafem::HostMesh m;
};

extern "C" int mafem_mesh_build(const mafem_params* p, const mafem_args* a, mafem_mesh** out) {
  if (!p || !a || !out) return MAFEM_ERR_ARG;
  auto mm = std::make_unique<mafem_mesh>();
  std::string err;
  int rc = mafem::build_mesh(*p, *a, mm->m, err);
  if (rc != MAFEM_OK) {
    mafem::set_global_error(err);
    return rc;
  }
  *out = mm.release();
  return MAFEM_OK;
}
extern "C" int mafem_mesh_view(const mafem_mesh* m, mafem_mesh_desc* out) {
  if (!m || !out) return MAFEM_ERR_ARG;
  mafem::mesh_desc(m->m, *out);
  return MAFEM_OK;
}
extern "C" void mafem_mesh_free(mafem_mesh* m) { delete m; }
extern "C" int mafem_prepare_input(const mafem_mesh* m, const mafem_params* p, double* xms, double* cps) {
  if (!m || !p || !xms || !cps) return MAFEM_ERR_ARG;
  std::string err;
  int rc = mafem::prepare_input(m->m, *p, xms, cps, err);
  if (rc != MAFEM_OK) mafem::set_global_error(err);
  return rc;
}
