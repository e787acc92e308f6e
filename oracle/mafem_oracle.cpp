// mafem_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A plain CPU restatement of MembraneAleFem.jl (Julia) used as the parity oracle
// for the GPU library.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline leg load it.  Nothing in the product links, loads or calls this file.
//
// Pinning: the spline / Gauss-point / GP-basis / GeoDynStress layers are checked
// against every known-answer test of the reference's own test suite
// (test/input/*.jl, test/analysis/geo_dyn_stress_tests.jl), restated in
// tests/test_oracle_kat.py.  The reference's tests do not cover calc_r_K,
// time_step!, the connectivity or the solve, so those layers are pinned only by
// this restatement (plus internal consistency checks: complex-step tangent vs
// central differences, Newton convergence, scipy's sparse LU as a second solver).
//
// Faithfulness notes
//  * Every function follows the reference file:line named in its comment, with
//    the reference's 1-based index conventions kept (helper Mat1/Vec1 below).
//  * The tangent is computed exactly like the reference: complex-step
//    differentiation with std::complex<double> and eps_k = 1e-15
//    (src/analysis/FiniteElement.jl:100-126, 151-197), including the
//    conjugating norm of tau in calc_tau_nu (FiniteElement.jl:448).
//  * Julia's dense `\` (LAPACK getrf/getrs, partial pivoting) is restated for
//    the collocation solves; the sparse `K \ r` (UMFPACK) is replaced by a
//    banded LU with partial pivoting (the LAPACK gbtf2 algorithm description).

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace orc {

using cd = std::complex<double>;

// ---- enums (src/input/Enums.jl:24-157, src/input/Dof.jl:29-34) -------------
enum Scenario { F_CAVI = 1, F_COUE = 2, F_POIS = 3, F_PULL = 4, F_BEND = 5 };
enum Topology { FLAT = 1, CYLINDER = 2 };
enum Motion { STATIC = 1, EUL = 2, LAG = 3, ALEV = 4, ALEVB = 5 };
enum Boundary { BOTTOM = 1, RIGHT = 2, TOP = 3, LEFT = 4 };
enum Neumann { SHEAR = 1, STRETCH = 2, MOMENT = 3 };
enum Curve { CLAMPED = 1, CLOSED = 2 };
enum Unknown { vx = 1, vy = 2, vz = 3, vmx = 4, vmy = 5, vmz = 6, lam = 7, pm = 8 };

// compile-time constants (src/input/Params.jl:161-179)
constexpr int POLY = 2, GP1D = 3, NDERS = 2, ZDIM = 2, XDIM = 3, NEN = 9, VOIGT = 3,
              NEDBDF = 3;

struct AssertionError : std::runtime_error {
  explicit AssertionError(const std::string& s) : std::runtime_error(s) {}
};
#define ORC_ASSERT(c, msg) \
  do {                     \
    if (!(c)) throw AssertionError(msg); \
  } while (0)

// 1-based column-major matrix, as in Julia.
template <class T>
struct Mat1 {
  int m = 0, n = 0;
  std::vector<T> d;
  Mat1() = default;
  Mat1(int m_, int n_) : m(m_), n(n_), d((size_t)m_ * n_, T(0)) {}
  T& operator()(int i, int j) { return d[(size_t)(i - 1) + (size_t)m * (j - 1)]; }
  const T& operator()(int i, int j) const { return d[(size_t)(i - 1) + (size_t)m * (j - 1)]; }
};
template <class T>
struct Vec1 {
  std::vector<T> d;
  Vec1() = default;
  explicit Vec1(int n, T v = T(0)) : d(n, v) {}
  T& operator[](int i) { return d[i - 1]; }
  const T& operator[](int i) const { return d[i - 1]; }
  int size() const { return (int)d.size(); }
};

// ---- Params (src/input/Params.jl:36-55) ------------------------------------
struct Params {
  int motion = ALEVB, scenario = F_PULL, num1el = 17, num2el = 17;
  double length = 64.0, kb = 1.0, kg = -0.5, zv = 1.0, pn = 0.0;
  int poly = 2, gp1d = 3, nders = 2, nen = 9;
  double adb = 64.0 * 64.0, am = 1.0, eps_k = 1e-15, eps_nr = 1e-12;
};
// keyword arguments used on the hot path (pull_speed: Bc.jl:234,240;
// bend_tm / bend_mf: FiniteElement.jl:379, Bc.jl:389-390)
// Two F_PULL extensions with no reference keyword (their zero values are the
// reference's behaviour): lambda0 > 0 replaces the edge tension and initial λ
// kb / 4 (Bc.jl:259, Input.jl:85); pull_centre = 1 pulls element
// (floor(n1/2) + 1, floor(n2/2) + 1) instead of ceil(numel / 2).
struct Args {
  double pull_speed = 0.0, bend_tm = 1.0, bend_mf = 0.0;
  double lambda0 = 0.0;
  int pull_centre = 0;
};

// ---- KnotVector (src/input/Spline.jl:20-96) --------------------------------
struct KnotVector {
  std::vector<double> zs;  // 0-based storage; zs1(i) gives the 1-based view
  int nel = 0, poly = 0;
  int curve = CLAMPED;
  double zs1(int i) const { return zs[i - 1]; }
  int len() const { return (int)zs.size(); }
};

static bool approx_eq(double x, double y) {
  // Julia isapprox with default rtol = sqrt(eps), atol = 0
  if (x == y) return true;
  double rtol = std::sqrt(2.220446049250313e-16);
  return std::fabs(x - y) <= rtol * std::max(std::fabs(x), std::fabs(y));
}

// Spline.jl:46-61
KnotVector knot_vector(const std::vector<double>& zs, int poly, int curve) {
  int L = (int)zs.size();
  if (curve == CLAMPED) {
    for (int i = 0; i + 1 < L; ++i) ORC_ASSERT(zs[i] <= zs[i + 1], "knots must be non-decreasing");
    ORC_ASSERT(L >= poly + 1, "need poly+1 repeated knots at start");
    for (int i = 0; i < poly + 1; ++i) ORC_ASSERT(zs[i] == zs[0], "need poly+1 repeated knots at start");
    for (int i = L - poly - 1; i < L; ++i) ORC_ASSERT(zs[i] == zs[L - 1], "need poly+1 repeated knots at end");
  } else if (curve == CLOSED) {
    // ζs[2:end] - ζs[1:end-1] ≈ (ζs[2]-ζs[1]) * ones: isapprox on the vectors (norm-based)
    double h = zs[1] - zs[0];
    double dn = 0, xn = 0, yn = 0;
    for (int i = 0; i + 1 < L; ++i) {
      double a = zs[i + 1] - zs[i];
      dn += (a - h) * (a - h);
      xn += a * a;
      yn += h * h;
    }
    ORC_ASSERT(std::sqrt(dn) <= std::sqrt(2.220446049250313e-16) * std::max(std::sqrt(xn), std::sqrt(yn)),
               "closed knots must be uniform");
  } else {
    ORC_ASSERT(false, "knot vector curve not implemented");
  }
  KnotVector kv;
  kv.zs = zs;
  kv.nel = L - 2 * poly - 1;
  kv.poly = poly;
  kv.curve = curve;
  return kv;
}

// Spline.jl:76-96
KnotVector knot_vector_uniform(int nel, int poly, int curve) {
  int num = nel + 2 * poly + 1;
  std::vector<double> zs(num, 0.0);
  if (curve == CLAMPED) {
    for (int idx = poly + 2; idx <= num - poly - 1; ++idx) zs[idx - 1] = (double)(idx - poly - 1) / nel;
    for (int idx = num - poly; idx <= num; ++idx) zs[idx - 1] = 1.0;
  } else if (curve == CLOSED) {
    for (int idx = 1; idx <= num; ++idx) zs[idx - 1] = (double)(idx - poly - 1) / nel;
  }
  return knot_vector(zs, poly, curve);
}

// Spline.jl:122-183
std::vector<double> get_fine_zs(int nel, int poly) {
  ORC_ASSERT(nel >= 18, "fine mesh requires at least 18 1-D elements");
  int num = nel + 2 * poly + 1;
  Vec1<double> zs(num, 0.0);
  int num_wide_l1 = 6;
  int num_fine_l1 = nel - 2 * num_wide_l1 - 1;
  double z_wide_l1 = 1.0 / 3.0;
  double z_fine_l1 = 1.0 - 2 * z_wide_l1;
  for (int idx = poly + 2; idx <= poly + num_wide_l1 + 1; ++idx) {
    double dz = z_wide_l1 / num_wide_l1;
    zs[idx] = (idx - poly - 1) * dz;
  }
  for (int idx = num - poly - num_wide_l1; idx <= num - poly - 1; ++idx) {
    double dz = z_wide_l1 / num_wide_l1;
    zs[idx] = 1.0 - z_wide_l1 + (idx - num + poly + num_wide_l1) * dz;
  }
  int num_wide_l2 = (int)std::floor(num_fine_l1 / 4.0);
  int num_fine_l2 = num_fine_l1 - 2 * num_wide_l2;
  double z_wide_l2 = 1.0 / 9.0;
  double z_fine_l2 = z_fine_l1 - 2 * z_wide_l2;
  if (2 * num_wide_l2 <= num_wide_l1) {
    double dz = z_fine_l1 / (num_fine_l1 + 1);
    for (int idx = poly + num_wide_l1 + 2; idx <= num - poly - num_wide_l1 - 1; ++idx)
      zs[idx] = z_wide_l1 + (idx - poly - num_wide_l1 - 1) * dz;
  } else {
    double dz = z_wide_l2 / num_wide_l2;
    for (int idx = num_wide_l1 + poly + 2; idx <= num_wide_l1 + poly + 1 + num_wide_l2; ++idx)
      zs[idx] = z_wide_l1 + (idx - num_wide_l1 - poly - 1) * dz;
    for (int idx = num - poly - num_wide_l1 - num_wide_l2; idx <= num - poly - num_wide_l1 - 1; ++idx)
      zs[idx] = 1.0 - z_wide_l1 - z_wide_l2 + (idx - num + poly + num_wide_l1 + num_wide_l2) * dz;
    dz = z_fine_l2 / (num_fine_l2 + 1);
    for (int idx = num_wide_l1 + poly + 2 + num_wide_l2; idx <= num - poly - num_wide_l1 - num_wide_l2 - 1; ++idx)
      zs[idx] = z_wide_l1 + z_wide_l2 + (idx - num_wide_l1 - poly - 1 - num_wide_l2) * dz;
  }
  for (int idx = num - poly; idx <= num; ++idx) zs[idx] = 1.0;
  return zs.d;
}

// Spline.jl:198-248 (Piegl-Tiller A2.1, extended to CLOSED knots)
int get_knot_span_index(const KnotVector& kv, double z) {
  std::vector<double> zs = kv.zs;
  int L = (int)zs.size();
  if (kv.curve == CLOSED) {
    for (int i = 0; i < kv.poly; ++i) zs[i] = zs[kv.poly];
    for (int i = L - kv.poly; i < L; ++i) zs[i] = zs[L - kv.poly - 1];
  }
  ORC_ASSERT(z >= zs[0], "ζ smaller than first active knot");
  ORC_ASSERT(z <= zs[L - 1], "ζ larger than last active knot");
  auto Z = [&](int i) { return zs[i - 1]; };
  int m = 1;
  while (Z(m) == Z(1)) m = m + 1;
  int n = L;
  while (Z(n) == Z(L)) n = n - 1;
  if (z == Z(n + 1)) return n;
  int low = m - 1, high = n + 1;
  int mid = (int)std::floor((low + high) / 2.0);
  while (z < Z(mid) || z >= Z(mid + 1)) {
    if (z < Z(mid)) high = mid;
    else low = mid;
    mid = (int)std::floor((low + high) / 2.0);
  }
  return mid;
}

// Spline.jl:264-296 (Piegl-Tiller A2.2)
std::vector<double> get_bspline_vals(const KnotVector& kv, double z) {
  ORC_ASSERT(z >= kv.zs.front(), "ζ is less than smallest knot");
  ORC_ASSERT(z <= kv.zs.back(), "ζ is greater than largest knot");
  int poly = kv.poly;
  Vec1<double> left(poly + 1), right(poly + 1), bf(poly + 1);
  int span = get_knot_span_index(kv, z);
  bf[1] = 1.0;
  for (int j = 1; j <= poly; ++j) {
    left[j + 1] = z - kv.zs1(span + 1 - j);
    right[j + 1] = kv.zs1(span + j) - z;
    double saved = 0.0;
    for (int r = 1; r <= j; ++r) {
      double temp = bf[r] / (right[r + 1] + left[j + 2 - r]);
      bf[r] = saved + right[r + 1] * temp;
      saved = left[j + 2 - r] * temp;
    }
    bf[j + 1] = saved;
  }
  return bf.d;
}

// Spline.jl:319-422 (Piegl-Tiller A2.3); returns (poly+1) x (num_ders+1)
Mat1<double> get_bspline_ders(const KnotVector& kv, double z, int num_ders) {
  ORC_ASSERT(z >= kv.zs.front(), "ζ is less than smallest knot");
  ORC_ASSERT(z <= kv.zs.back(), "ζ is greater than largest knot");
  int poly = kv.poly;
  Vec1<double> left(poly + 1), right(poly + 1);
  ORC_ASSERT(num_ders >= 0, "cannot have fewer than zero derivatives");
  ORC_ASSERT(num_ders <= poly, "basis functions have only `poly` derivatives");
  int span = get_knot_span_index(kv, z);
  Mat1<double> ders(poly + 1, num_ders + 1);
  Mat1<double> ndu(poly + 1, poly + 1);
  Mat1<double> a(2, poly + 1);
  ndu(1, 1) = 1.0;
  for (int j = 1; j <= poly; ++j) {
    left[j + 1] = z - kv.zs1(span + 1 - j);
    right[j + 1] = kv.zs1(span + j) - z;
    double saved = 0.0;
    for (int r = 1; r <= j; ++r) {
      ndu(j + 1, r) = right[r + 1] + left[j + 2 - r];
      double temp = ndu(r, j) / ndu(j + 1, r);
      ndu(r, j + 1) = saved + right[r + 1] * temp;
      saved = left[j + 2 - r] * temp;
    }
    ndu(j + 1, j + 1) = saved;
  }
  for (int j = 1; j <= poly + 1; ++j) ders(j, 1) = ndu(j, poly + 1);
  for (int r = 1; r <= poly + 1; ++r) {
    int s1 = 1, s2 = 2;
    a(1, 1) = 1.0;
    for (int k = 1; k <= num_ders; ++k) {
      double d = 0.0;
      int rk = r - k, pk = poly - k;
      if (r > k) {
        a(s2, 1) = a(s1, 1) / ndu(pk + 2, rk);
        d = a(s2, 1) * ndu(rk, pk + 1);
      }
      int j1 = rk >= 0 ? 1 : -rk + 1;
      int j2 = (r - 2 <= pk) ? k - 1 : poly - r + 1;
      for (int j = j1; j <= j2; ++j) {
        a(s2, j + 1) = (a(s1, j + 1) - a(s1, j)) / ndu(pk + 2, rk + j);
        d += a(s2, j + 1) * ndu(rk + j, pk + 1);
      }
      if (r - 1 <= pk) {
        a(s2, k + 1) = -a(s1, k) / ndu(pk + 2, r);
        d += a(s2, k + 1) * ndu(r, pk + 1);
      }
      ders(r, k + 1) = d;
      std::swap(s1, s2);
    }
  }
  int r = poly;
  for (int k = 1; k <= num_ders; ++k) {
    for (int j = 1; j <= poly + 1; ++j) ders(j, k + 1) *= r;
    r *= (poly - k);
  }
  return ders;
}

// Spline.jl:465-481
std::vector<int> get_bspline_indices_span(const KnotVector& kv, int ks_id) {
  std::vector<int> ids(kv.poly + 1);
  for (int i = 1; i <= kv.poly + 1; ++i) ids[i - 1] = i + (ks_id - kv.poly - 1);
  if (kv.curve == CLOSED)
    for (auto& v : ids) v = ((v - 1) % kv.nel) + 1;  // Julia % keeps the dividend's sign
  return ids;
}
// Spline.jl:441-449
std::vector<int> get_bspline_indices(const KnotVector& kv, double z) {
  return get_bspline_indices_span(kv, get_knot_span_index(kv, z));
}

// Spline.jl:580-626
std::vector<double> collocate_z(const KnotVector& kv) {
  int L = kv.len();
  if (kv.curve == CLOSED) {
    std::vector<double> out;
    for (int i = kv.poly + 1; i <= L - kv.poly - 1; ++i) out.push_back((kv.zs1(i) + kv.zs1(i + 1)) / 2);
    return out;
  }
  ORC_ASSERT(kv.curve == CLAMPED, "interpolation curve not implemented");
  int poly = kv.poly;
  std::vector<double> u;  // unique(kv.ζs), in order of first appearance
  for (double z : kv.zs)
    if (std::find(u.begin(), u.end(), z) == u.end()) u.push_back(z);
  ORC_ASSERT(poly > 1, "interpolation for poly ≥ 2 only when clamped");
  ORC_ASSERT(poly < 4, "interpolation for poly ≤ 3 only when clamped");
  ORC_ASSERT((int)u.size() == L - 2 * poly, "no repeated interior knots");
  int nb = L - poly - 1;
  Vec1<double> zl(nb, 0.0);
  auto U = [&](int i) { return u[i - 1]; };
  zl[1] = U(1);
  zl[nb] = U((int)u.size());
  if (poly == 2) {
    for (int i = 2; i <= nb - 1; ++i) zl[i] = (U(i - 1) + U(i)) / 2;
  } else if (poly == 3) {
    zl[2] = (U(1) + U(2)) / 2;
    zl[nb - 1] = (U((int)u.size() - 1) + U((int)u.size())) / 2;
    for (int i = 3; i <= nb - 2; ++i) zl[i] = U(i - 1);
  }
  return zl.d;
}

// Julia's dense `A \ b` for square A: LU with partial pivoting (getrf), then getrs.
std::vector<double> dense_solve(Mat1<double> A, std::vector<double> b) {
  int n = A.m;
  std::vector<int> piv(n + 1);
  for (int k = 1; k <= n; ++k) {
    int p = k;
    double mx = std::fabs(A(k, k));
    for (int i = k + 1; i <= n; ++i)
      if (std::fabs(A(i, k)) > mx) { mx = std::fabs(A(i, k)); p = i; }
    piv[k] = p;
    ORC_ASSERT(A(p, k) != 0.0, "singular matrix in dense solve");
    if (p != k)
      for (int j = 1; j <= n; ++j) std::swap(A(k, j), A(p, j));
    for (int i = k + 1; i <= n; ++i) A(i, k) /= A(k, k);
    for (int j = k + 1; j <= n; ++j) {
      double akj = A(k, j);
      if (akj != 0.0)
        for (int i = k + 1; i <= n; ++i) A(i, j) -= A(i, k) * akj;
    }
  }
  for (int k = 1; k <= n; ++k)
    if (piv[k] != k) std::swap(b[k - 1], b[piv[k] - 1]);
  for (int j = 1; j <= n; ++j)
    for (int i = j + 1; i <= n; ++i) b[i - 1] -= A(i, j) * b[j - 1];
  for (int j = n; j >= 1; --j) {
    b[j - 1] /= A(j, j);
    for (int i = 1; i < j; ++i) b[i - 1] -= A(i, j) * b[j - 1];
  }
  return b;
}

// Spline.jl:510-528
std::vector<double> get_1d_bspline_cps(const KnotVector& kv, const std::function<double(double)>& f) {
  std::vector<double> zl = collocate_z(kv);
  int nb = (int)zl.size();
  Mat1<double> M(nb, nb);
  for (int j = 1; j <= nb; ++j) {
    auto ids = get_bspline_indices(kv, zl[j - 1]);
    auto vals = get_bspline_vals(kv, zl[j - 1]);
    for (size_t q = 0; q < ids.size(); ++q) M(j, ids[q]) = vals[q];
  }
  std::vector<double> rhs(nb);
  for (int j = 0; j < nb; ++j) rhs[j] = f(zl[j]);
  return dense_solve(M, rhs);
}

// Spline.jl:540-567: the dense (B2 ⊗ B1) collocation solve, as written.
std::vector<double> get_2d_bspline_cps(const KnotVector& kv1, const KnotVector& kv2,
                                       const std::function<double(double, double)>& f) {
  std::vector<double> z1 = collocate_z(kv1), z2 = collocate_z(kv2);
  int n1 = (int)z1.size(), n2 = (int)z2.size(), nb = n1 * n2;
  Mat1<double> M(nb, nb);
  for (int k = 1; k <= n2; ++k)
    for (int j = 1; j <= n1; ++j) {
      auto i2s = get_bspline_indices(kv2, z2[k - 1]);
      auto i1s = get_bspline_indices(kv1, z1[j - 1]);
      auto v2s = get_bspline_vals(kv2, z2[k - 1]);
      auto v1s = get_bspline_vals(kv1, z1[j - 1]);
      for (size_t b = 0; b < i2s.size(); ++b)
        for (size_t a = 0; a < i1s.size(); ++a)
          M(j + (k - 1) * n1, i1s[a] + (i2s[b] - 1) * n1) = v1s[a] * v2s[b];
    }
  std::vector<double> rhs(nb);
  for (int k = 1; k <= n2; ++k)
    for (int j = 1; j <= n1; ++j) rhs[(j - 1) + (size_t)(k - 1) * n1] = f(z1[j - 1], z2[k - 1]);
  return dense_solve(M, rhs);
}

// Spline.jl:640-671
struct Unique1D {
  int uel_num = 0, num_el = 0;
  std::vector<int> uel_ids;                      // 1-based ids
  std::vector<std::pair<double, double>> uel_list;
};
Unique1D get_unique_1d_elements(const KnotVector& kv) {
  int poly = kv.poly, L = kv.len();
  std::vector<double> prev(2 * poly + 1, 0.0);
  Unique1D u;
  u.num_el = L - 2 * poly - 1;
  u.uel_ids.assign(u.num_el, 0);
  for (int k = poly + 1; k <= L - poly - 1; ++k) {
    int el = k - poly;
    std::vector<double> ctx(2 * poly + 1);
    for (int q = 0; q < 2 * poly + 1; ++q) ctx[q] = kv.zs1(k - poly + 1 + q) - kv.zs1(k - poly + q);
    bool same = true;
    for (int q = 0; q < 2 * poly + 1; ++q) same = same && approx_eq(ctx[q], prev[q]);
    if (!same) {
      u.uel_num += 1;
      u.uel_list.push_back({kv.zs1(k), kv.zs1(k + 1)});
    }
    u.uel_ids[el - 1] = u.uel_num;
    prev = ctx;
  }
  return u;
}

// ---- Gauss points (src/input/GaussPoint.jl:67-171) -------------------------
std::vector<double> get_xis(int ngp) {
  ORC_ASSERT(ngp <= 4, "have at most 4 1-D Gauss points");
  if (ngp == 1) return {-1.0};
  if (ngp == 3) return {-std::sqrt(3.0 / 5), 0.0, std::sqrt(3.0 / 5)};
  if (ngp == 4)
    return {-std::sqrt(3.0 / 7 + std::sqrt(6.0 / 5) * 2 / 7), -std::sqrt(3.0 / 7 - std::sqrt(6.0 / 5) * 2 / 7),
            std::sqrt(3.0 / 7 - std::sqrt(6.0 / 5) * 2 / 7), std::sqrt(3.0 / 7 + std::sqrt(6.0 / 5) * 2 / 7)};
  ORC_ASSERT(false, "ξs for this number of Gauss points not implemented");
  return {};
}
std::vector<double> get_xi_weights(int ngp) {
  ORC_ASSERT(ngp <= 4, "have at most 4 1-D Gauss points");
  if (ngp == 1) return {0.0};
  if (ngp == 3) return {5.0 / 9, 8.0 / 9, 5.0 / 9};
  if (ngp == 4)
    return {(18 - std::sqrt(30.0)) / 36, (18 + std::sqrt(30.0)) / 36, (18 + std::sqrt(30.0)) / 36,
            (18 - std::sqrt(30.0)) / 36};
  ORC_ASSERT(false, "weights for this number of Gauss points not implemented");
  return {};
}
// GaussPoint.jl:72-77: ζ = ξ (hi-lo)/2 + (hi+lo)/2,  w = ŵ (hi-lo)/2
void gauss_zeta(int ngp, double lo, double hi, std::vector<double>& zs, std::vector<double>& ws) {
  auto xs = get_xis(ngp);
  auto wx = get_xi_weights(ngp);
  zs.resize(ngp);
  ws.resize(ngp);
  for (int i = 0; i < ngp; ++i) {
    zs[i] = xs[i] * (hi - lo) / 2 + (hi + lo) / 2;
    ws[i] = wx[i] * (hi - lo) / 2;
  }
}

// ---- GP basis functions (src/input/GpBasisFn.jl) ---------------------------
struct Fz {  // GpBasisFnsζ (GpBasisFn.jl:20-55)
  double w = 0, N[3] = {0, 0, 0}, dN[3] = {0, 0, 0}, ddN[3] = {0, 0, 0};
};
Fz gp_basis_fns_z(double w, double z, const KnotVector& kv) {
  Mat1<double> D = get_bspline_ders(kv, z, NDERS);
  Fz f;
  f.w = w;
  for (int i = 0; i < 3; ++i) {
    f.N[i] = D(i + 1, 1);
    f.dN[i] = D(i + 1, 2);
    f.ddN[i] = D(i + 1, 3);
  }
  return f;
}
struct Fza {  // GpBasisFnsζα (GpBasisFn.jl:96-112); node index a = id1 + 3(id2-1)
  double w = 0, N[9] = {}, dN[9][2] = {}, ddN[9][3] = {};
};
Fza gp_basis_fns_za(const Fz& f1, const Fz& f2) {
  Fza g;
  g.w = f1.w * f2.w;
  for (int i2 = 0; i2 < 3; ++i2)
    for (int i1 = 0; i1 < 3; ++i1) {
      int a = i1 + 3 * i2;
      g.N[a] = f1.N[i1] * f2.N[i2];
      g.dN[a][0] = f1.dN[i1] * f2.N[i2];
      g.dN[a][1] = f1.N[i1] * f2.dN[i2];
      g.ddN[a][0] = f1.ddN[i1] * f2.N[i2];
      g.ddN[a][1] = f1.N[i1] * f2.ddN[i2];
      g.ddN[a][2] = f1.dN[i1] * f2.dN[i2];
    }
  return g;
}
struct LineFns {  // LineGpBasisFns (GpBasisFn.jl:143-202)
  int nel = 0;
  std::vector<int> uel_ids;         // 1-based
  std::vector<std::vector<Fz>> ufns;  // [uel][gp]
  Fz zmin, zmax;
};
LineFns line_gp_basis_fns(const KnotVector& kv, int ngp) {
  Unique1D u = get_unique_1d_elements(kv);
  LineFns L;
  L.nel = u.num_el;
  L.uel_ids = u.uel_ids;
  L.ufns.resize(u.uel_num);
  for (int q = 0; q < u.uel_num; ++q) {
    std::vector<double> zs, ws;
    gauss_zeta(ngp, u.uel_list[q].first, u.uel_list[q].second, zs, ws);
    for (int g = 0; g < ngp; ++g) L.ufns[q].push_back(gp_basis_fns_z(ws[g], zs[g], kv));
  }
  if (kv.curve == CLAMPED) {
    L.zmin = gp_basis_fns_z(1.0, kv.zs.front(), kv);
    L.zmax = gp_basis_fns_z(1.0, kv.zs.back(), kv);
  } else {
    L.zmin = gp_basis_fns_z(1.0, kv.zs1(kv.poly + 1), kv);
    L.zmax = gp_basis_fns_z(1.0, kv.zs1(kv.len() - kv.poly), kv);
  }
  return L;
}
struct BdryFns {  // BdryGpBasisFns (GpBasisFn.jl:231-277)
  int nel = 0;
  std::vector<int> uel_ids;
  std::vector<std::vector<Fza>> ufns;
};
BdryFns bdry_gp_basis_fns(const LineFns& line, const Fz& perp, int bdry) {
  BdryFns B;
  B.nel = line.nel;
  B.uel_ids = line.uel_ids;
  B.ufns.resize(line.ufns.size());
  for (size_t q = 0; q < line.ufns.size(); ++q)
    for (size_t g = 0; g < line.ufns[q].size(); ++g)
      B.ufns[q].push_back((bdry == BOTTOM || bdry == TOP) ? gp_basis_fns_za(line.ufns[q][g], perp)
                                                           : gp_basis_fns_za(perp, line.ufns[q][g]));
  return B;
}
struct AreaFns {  // AreaGpBasisFns (GpBasisFn.jl:300-356)
  int nel = 0;
  std::vector<int> uel_ids;               // 1-based
  std::vector<std::vector<Fza>> ufns;     // [uel][gp], gp = gp1 + 3(gp2-1)
};
AreaFns area_gp_basis_fns(const LineFns& l1, const LineFns& l2) {
  AreaFns A;
  int ne1 = l1.nel, ne2 = l2.nel;
  int nu1 = (int)l1.ufns.size(), nu2 = (int)l2.ufns.size();
  int ng1 = nu1 ? (int)l1.ufns[0].size() : 0, ng2 = nu2 ? (int)l2.ufns[0].size() : 0;
  A.nel = ne1 * ne2;
  A.uel_ids.assign(A.nel, 0);
  for (int i1 = 1; i1 <= ne1; ++i1)
    for (int i2 = 1; i2 <= ne2; ++i2)
      A.uel_ids[(i1 + (i2 - 1) * ne1) - 1] = l1.uel_ids[i1 - 1] + (l2.uel_ids[i2 - 1] - 1) * nu1;
  A.ufns.assign(nu1 * nu2, std::vector<Fza>(ng1 * ng2));
  for (int i1 = 1; i1 <= nu1; ++i1)
    for (int i2 = 1; i2 <= nu2; ++i2)
      for (int g1 = 1; g1 <= ng1; ++g1)
        for (int g2 = 1; g2 <= ng2; ++g2)
          A.ufns[(i1 + (i2 - 1) * nu1) - 1][(g1 + (g2 - 1) * ng1) - 1] =
              gp_basis_fns_za(l1.ufns[i1 - 1][g1 - 1], l2.ufns[i2 - 1][g2 - 1]);
  return A;
}

// ---- Mesh (src/input/Mesh.jl, src/input/Bc.jl) ------------------------------
struct DirBC { int unknown, node; double value; };
struct NeuBC { int bdry, ntype; double value; };

struct Mesh {
  int num1el, num2el, numel, num1np, num2np, numnp;
  Mat1<int> IX;                            // NEN x numel, 1-based nodes
  std::map<int, std::vector<int>> bdry_elems, bdry_nodes, bdry_inner_nodes;
  std::map<int, int> crnr_nodes;
  KnotVector kv1, kv2;
  AreaFns area;
  std::map<int, BdryFns> bdry_fns;
  int topology;
  int dofs[9];                             // dofs[Unknown] -> 1-based dof index, 0 if absent
  int ndf;
  Mat1<int> ID;                            // ndf x numnp, 1-based, 0 = Dirichlet
  std::vector<std::pair<int, int>> ID_inv; // (node, dof), 1-based
  int nmdf;
  Mat1<int> LM;                            // (ndf*NEN) x numel
  std::vector<DirBC> inh_dir_bcs;
  std::vector<NeuBC> inh_neu_bcs;
  Params p;
  Args args;
};

// Mesh.jl:477-542
static std::vector<int> get_v_order(const Mesh& m) { return {m.dofs[vx], m.dofs[vy], m.dofs[vz]}; }
static std::vector<int> get_m_order(const Mesh& m) { return {m.dofs[vmx], m.dofs[vmy], m.dofs[vmz]}; }
static int get_lam_order(const Mesh& m) { return m.dofs[lam]; }
static int get_p_order(const Mesh& m) { return m.dofs[pm]; }
static std::vector<int> get_m_motion_order(int motion, const Mesh& m) {
  if (motion == STATIC) return {0, 0, 0};
  if (motion == LAG) return get_v_order(m);
  return get_m_order(m);
}

// Bc.jl:414-431
static void get_dofs(int motion, int* dofs, int& ndf) {
  for (int i = 0; i < 9; ++i) dofs[i] = 0;
  if (motion == LAG || motion == STATIC) {
    dofs[vx] = 1; dofs[vy] = 2; dofs[vz] = 3; dofs[lam] = 4; ndf = 4;
  } else if (motion == EUL) {
    dofs[vx] = 1; dofs[vy] = 2; dofs[vz] = 3; dofs[vmx] = 4; dofs[vmy] = 5; dofs[vmz] = 6; dofs[lam] = 7; ndf = 7;
  } else if (motion == ALEV || motion == ALEVB) {
    dofs[vx] = 1; dofs[vy] = 2; dofs[vz] = 3; dofs[vmx] = 4; dofs[vmy] = 5; dofs[vmz] = 6; dofs[lam] = 7;
    dofs[pm] = 8; ndf = 8;
  } else {
    ORC_ASSERT(false, "motion degrees of freedom not provided");
  }
}

// get_pull_el_id, src/analysis/PullForce.jl:8-13
int get_pull_el_id(int numel) { return (int)std::ceil(numel / 2.0); }
// the pulled element: get_pull_el_id, or with the centre extension the element
// at (floor(n1/2) + 1, floor(n2/2) + 1), numbered e1 + n1 (e2 - 1) (Mesh.jl:582-589)
int pull_el_id(const Params& p, const Args& a) {
  if (a.pull_centre) return (p.num1el / 2 + 1) + p.num1el * (p.num2el / 2);
  return get_pull_el_id(p.num1el * p.num2el);
}
// F_PULL's tension: kb / 4 (Bc.jl:259, Input.jl:85) unless lambda0 > 0
double pull_lambda(const Params& p, const Args& a) { return a.lambda0 > 0 ? a.lambda0 : p.kb / 4; }

// Bc.jl:15-40 and the per-scenario helpers
static void scenario_bc_info(Mesh& M) {
  const Params& p = M.p;
  int numnp = M.numnp;
  auto set_dofs3 = [&]() {
    for (int i = 0; i < 9; ++i) M.dofs[i] = 0;
    M.dofs[vx] = 1; M.dofs[vy] = 2; M.dofs[lam] = 3; M.ndf = 3;
  };
  M.inh_dir_bcs.clear();
  M.inh_neu_bcs.clear();
  if (p.scenario == F_CAVI) {  // Bc.jl:58-106
    set_dofs3();
    M.ID = Mat1<int>(M.ndf, numnp);
    for (int i : M.bdry_nodes[BOTTOM]) { M.ID(M.dofs[vx], i) = -1; M.ID(M.dofs[vy], i) = -1; }
    for (int i : M.bdry_nodes[TOP]) {
      M.ID(M.dofs[vx], i) = -1; M.ID(M.dofs[vy], i) = -1;
      if (i != M.crnr_nodes[3] && i != M.crnr_nodes[4]) M.inh_dir_bcs.push_back({vx, i, 1.0});
    }
    for (int i : M.bdry_nodes[LEFT]) { M.ID(M.dofs[vx], i) = -1; M.ID(M.dofs[vy], i) = -1; }
    for (int i : M.bdry_nodes[RIGHT]) { M.ID(M.dofs[vx], i) = -1; M.ID(M.dofs[vy], i) = -1; }
    int c = (int)std::floor(numnp / 2.0) + 1;
    M.ID(M.dofs[lam], c) = -1;
    M.inh_dir_bcs.push_back({lam, c, 0.0});
  } else if (p.scenario == F_COUE) {  // Bc.jl:122-157
    set_dofs3();
    M.ID = Mat1<int>(M.ndf, numnp);
    for (int i : M.bdry_nodes[BOTTOM]) { M.ID(M.dofs[vx], i) = -1; M.ID(M.dofs[vy], i) = -1; }
    for (int i : M.bdry_nodes[TOP]) {
      M.ID(M.dofs[vx], i) = -1; M.ID(M.dofs[vy], i) = -1;
      M.inh_dir_bcs.push_back({vx, i, 3.0});
    }
    for (int i : M.bdry_nodes[LEFT]) M.ID(M.dofs[vy], i) = -1;
    for (int i : M.bdry_nodes[RIGHT]) M.ID(M.dofs[vy], i) = -1;
    M.inh_neu_bcs = {{LEFT, STRETCH, 4.0}, {RIGHT, STRETCH, 4.0}};
  } else if (p.scenario == F_POIS) {  // Bc.jl:286-316
    set_dofs3();
    M.ID = Mat1<int>(M.ndf, numnp);
    for (int b : {TOP, BOTTOM})
      for (int i : M.bdry_nodes[b]) { M.ID(M.dofs[vx], i) = -1; M.ID(M.dofs[vy], i) = -1; }
    for (int b : {LEFT, RIGHT})
      for (int i : M.bdry_nodes[b]) M.ID(M.dofs[vy], i) = -1;
    M.inh_neu_bcs = {{LEFT, STRETCH, 4.0}, {RIGHT, STRETCH, 8.0}};
  } else if (p.scenario == F_BEND) {  // Bc.jl:347-393
    get_dofs(p.motion, M.dofs, M.ndf);
    M.ID = Mat1<int>(M.ndf, numnp);
    bool ale = p.motion == ALEV || p.motion == ALEVB;
    for (int b : {TOP, BOTTOM})
      for (int i : M.bdry_nodes[b]) {
        M.ID(M.dofs[vy], i) = -1;
        if (ale) M.ID(M.dofs[vmy], i) = -1;
      }
    for (int i : M.bdry_nodes[LEFT]) {
      M.ID(M.dofs[vx], i) = -1; M.ID(M.dofs[vy], i) = -1; M.ID(M.dofs[vz], i) = -1;
      if (ale) { M.ID(M.dofs[vmx], i) = -1; M.ID(M.dofs[vmy], i) = -1; M.ID(M.dofs[vmz], i) = -1; }
    }
    for (int i : M.bdry_nodes[RIGHT]) {
      M.ID(M.dofs[vz], i) = -1;
      if (ale) M.ID(M.dofs[vmz], i) = -1;
    }
    M.inh_neu_bcs = {{LEFT, MOMENT, M.args.bend_mf}, {RIGHT, MOMENT, M.args.bend_mf}};
  } else if (p.scenario == F_PULL) {  // Bc.jl:188-269
    get_dofs(p.motion, M.dofs, M.ndf);
    M.ID = Mat1<int>(M.ndf, numnp);
    bool ale = p.motion == ALEV || p.motion == ALEVB;
    for (auto& kvp : M.bdry_nodes)
      for (int i : kvp.second) {
        M.ID(M.dofs[vz], i) = -1;
        if (ale) { M.ID(M.dofs[vmx], i) = -1; M.ID(M.dofs[vmy], i) = -1; M.ID(M.dofs[vmz], i) = -1; }
      }
    for (auto& kvp : M.bdry_inner_nodes)
      for (int i : kvp.second) {
        M.ID(M.dofs[vz], i) = -1;
        if (p.motion == ALEVB) M.ID(M.dofs[vmz], i) = -1;
      }
    int ce = pull_el_id(p, M.args);
    for (int a = 1; a <= NEN; ++a) {
      int node = M.IX(a, ce);
      M.ID(M.dofs[vx], node) = -1; M.ID(M.dofs[vy], node) = -1; M.ID(M.dofs[vz], node) = -1;
      M.inh_dir_bcs.push_back({vz, node, M.args.pull_speed});
      if (p.motion != LAG) {
        M.ID(M.dofs[vmx], node) = -1; M.ID(M.dofs[vmy], node) = -1; M.ID(M.dofs[vmz], node) = -1;
        M.inh_dir_bcs.push_back({vmz, node, M.args.pull_speed});
      }
    }
    for (auto& kvp : M.bdry_nodes) {
      const auto& lst = kvp.second;
      int c = lst[(int)std::floor(lst.size() / 2.0)];  // lst[floor(end/2)+1], 1-based
      M.ID(M.dofs[vx], c) = -1; M.ID(M.dofs[vy], c) = -1;
      if (p.motion != LAG) { M.ID(M.dofs[vmx], c) = -1; M.ID(M.dofs[vmy], c) = -1; }
    }
    double lv = pull_lambda(p, M.args);  // kb / 4 unless lambda0 is given
    M.inh_neu_bcs = {{LEFT, STRETCH, lv}, {RIGHT, STRETCH, lv}, {TOP, STRETCH, lv}, {BOTTOM, STRETCH, lv}};
    ORC_ASSERT(p.pn == 0.0, "F_PULL with a normal pressure is not implemented");
  } else {
    ORC_ASSERT(false, "need boundary conditions for scenario");
  }
}

// Mesh.jl:574-593
static Mat1<int> construct_IX(const KnotVector& kv1, const KnotVector& kv2, int num1np) {
  Mat1<int> IX(NEN, kv1.nel * kv2.nel);
  for (int e2 = 1; e2 <= kv2.nel; ++e2)
    for (int e1 = 1; e1 <= kv1.nel; ++e1) {
      auto s2 = get_bspline_indices_span(kv2, e2 + POLY);
      auto s1 = get_bspline_indices_span(kv1, e1 + POLY);
      for (int n2 = 1; n2 <= POLY + 1; ++n2)
        for (int n1 = 1; n1 <= POLY + 1; ++n1)
          IX(n1 + (n2 - 1) * (POLY + 1), e1 + (e2 - 1) * kv1.nel) = s1[n1 - 1] + num1np * (s2[n2 - 1] - 1);
    }
  return IX;
}

// Mesh.jl:94-302 (FLAT topology; every scenario of the reference is FLAT)
std::unique_ptr<Mesh> generate_mesh(const Params& p, const Args& a) {
  auto M = std::make_unique<Mesh>();
  M->p = p;
  M->args = a;
  ORC_ASSERT(p.scenario >= F_CAVI && p.scenario <= F_BEND, "topology not specified");
  M->topology = FLAT;
  M->num1el = p.num1el; M->num2el = p.num2el;
  M->numel = p.num1el * p.num2el;
  M->num1np = p.num1el + p.poly; M->num2np = p.num2el + p.poly;
  M->numnp = M->num1np * M->num2np;
  int n1 = p.num1el, numel = M->numel, n1np = M->num1np, numnp = M->numnp;
  for (int i = 1; i <= n1; ++i) M->bdry_elems[BOTTOM].push_back(i);
  for (int i = n1; i <= numel; i += n1) M->bdry_elems[RIGHT].push_back(i);
  for (int i = numel - n1 + 1; i <= numel; ++i) M->bdry_elems[TOP].push_back(i);
  for (int i = 1; i <= numel - n1 + 1; i += n1) M->bdry_elems[LEFT].push_back(i);
  for (int i = 1; i <= n1np; ++i) M->bdry_nodes[BOTTOM].push_back(i);
  for (int i = n1np; i <= numnp; i += n1np) M->bdry_nodes[RIGHT].push_back(i);
  for (int i = numnp - n1np + 1; i <= numnp; ++i) M->bdry_nodes[TOP].push_back(i);
  for (int i = 1; i <= numnp - n1np + 1; i += n1np) M->bdry_nodes[LEFT].push_back(i);
  for (int i = 1; i <= n1np; ++i) M->bdry_inner_nodes[BOTTOM].push_back(i + n1np);
  for (int i = n1np; i <= numnp; i += n1np) M->bdry_inner_nodes[RIGHT].push_back(i - 1);
  for (int i = numnp - n1np + 1; i <= numnp; ++i) M->bdry_inner_nodes[TOP].push_back(i - n1np);
  for (int i = 1; i <= numnp - n1np + 1; i += n1np) M->bdry_inner_nodes[LEFT].push_back(i + 1);
  M->crnr_nodes[1] = 1; M->crnr_nodes[2] = n1np; M->crnr_nodes[3] = numnp - n1np + 1; M->crnr_nodes[4] = numnp;
  if (p.scenario == F_PULL && p.num1el >= 18 && p.num2el >= 18) {
    M->kv1 = knot_vector(get_fine_zs(p.num1el, p.poly), p.poly, CLAMPED);
    M->kv2 = knot_vector(get_fine_zs(p.num2el, p.poly), p.poly, CLAMPED);
  } else {
    M->kv1 = knot_vector_uniform(p.num1el, p.poly, CLAMPED);
    M->kv2 = knot_vector_uniform(p.num2el, p.poly, CLAMPED);
  }
  LineFns l1 = line_gp_basis_fns(M->kv1, p.gp1d);
  LineFns l2 = line_gp_basis_fns(M->kv2, p.gp1d);
  M->area = area_gp_basis_fns(l1, l2);
  M->bdry_fns[BOTTOM] = bdry_gp_basis_fns(l1, l2.zmin, BOTTOM);
  M->bdry_fns[RIGHT] = bdry_gp_basis_fns(l2, l1.zmax, RIGHT);
  M->bdry_fns[TOP] = bdry_gp_basis_fns(l1, l2.zmax, TOP);
  M->bdry_fns[LEFT] = bdry_gp_basis_fns(l2, l1.zmin, LEFT);
  M->IX = construct_IX(M->kv1, M->kv2, n1np);
  // generate_scenario, Mesh.jl:262-302
  scenario_bc_info(*M);
  int idx = 1;
  for (int node = 1; node <= numnp; ++node)
    for (int d = 1; d <= M->ndf; ++d) {
      if (M->ID(d, node) != -1) M->ID(d, node) = idx++;
      else M->ID(d, node) = 0;
    }
  M->nmdf = idx - 1;
  for (int node = 1; node <= numnp; ++node)
    for (int d = 1; d <= M->ndf; ++d)
      if (M->ID(d, node) != 0) M->ID_inv.push_back({node, d});
  M->LM = Mat1<int>(M->ndf * NEN, numel);
  for (int e = 1; e <= numel; ++e)
    for (int a = 1; a <= NEN; ++a)
      for (int d = 1; d <= M->ndf; ++d) M->LM(d + M->ndf * (a - 1), e) = M->ID(d, M->IX(a, e));
  return M;
}

// ---- GeoDynStress (src/analysis/GeoDynStress.jl:91-205), complex ------------
struct GDS {
  cd x[3], a[3][2], xab[3][3], aab[2][2], ainv[2][2], aup[3][2], J, Gam[3][2], n[3], b[2][2], H, K;
  cd v[3], dv[3][2], ddv[3][3], lam, pm, vm[3], dvm[3][2], ddvm[3][3];
  cd sig[3], sigm[3], M[3];
  cd Ba[3][27], Bb[3][27];
};

static cd det2(const cd A[2][2]) { return A[0][0] * A[1][1] - A[0][1] * A[1][0]; }

// get_dof_cps (GeoDynStress.jl:190-205): value of unknown u at element node a, 0 if absent
static inline cd dof_cp(const Mat1<cd>& cps, const Mesh& m, int u, int a) {
  int d = m.dofs[u];
  return d ? cps(a, d) : cd(0.0);
}

GDS geo_dyn_stress(const Mat1<cd>& xms, const Mat1<cd>& cps, const Mesh& m, const Fza& f, const Params& p) {
  GDS g;
  // geometry
  for (int i = 0; i < 3; ++i) {
    cd s = 0, s1 = 0, s2 = 0, t0 = 0, t1 = 0, t2 = 0;
    for (int a = 0; a < 9; ++a) {
      cd xa = xms(a + 1, i + 1);
      s += xa * f.N[a];
      s1 += xa * f.dN[a][0];
      s2 += xa * f.dN[a][1];
      t0 += xa * f.ddN[a][0];
      t1 += xa * f.ddN[a][1];
      t2 += xa * f.ddN[a][2];
    }
    g.x[i] = s; g.a[i][0] = s1; g.a[i][1] = s2; g.xab[i][0] = t0; g.xab[i][1] = t1; g.xab[i][2] = t2;
  }
  for (int al = 0; al < 2; ++al)
    for (int be = 0; be < 2; ++be) {
      cd s = 0;
      for (int i = 0; i < 3; ++i) s += g.a[i][al] * g.a[i][be];
      g.aab[al][be] = s;
    }
  cd da = det2(g.aab);
  g.ainv[0][0] = g.aab[1][1] / da; g.ainv[0][1] = -g.aab[0][1] / da;
  g.ainv[1][0] = -g.aab[1][0] / da; g.ainv[1][1] = g.aab[0][0] / da;
  for (int i = 0; i < 3; ++i)
    for (int al = 0; al < 2; ++al) g.aup[i][al] = g.a[i][0] * g.ainv[0][al] + g.a[i][1] * g.ainv[1][al];
  g.J = std::sqrt(da);
  for (int k = 0; k < 3; ++k)
    for (int mu = 0; mu < 2; ++mu) {
      cd s = 0;
      for (int i = 0; i < 3; ++i) s += g.xab[i][k] * g.aup[i][mu];
      g.Gam[k][mu] = s;
    }
  cd c0 = g.a[1][0] * g.a[2][1] - g.a[2][0] * g.a[1][1];
  cd c1 = g.a[2][0] * g.a[0][1] - g.a[0][0] * g.a[2][1];
  cd c2 = g.a[0][0] * g.a[1][1] - g.a[1][0] * g.a[0][1];
  g.n[0] = c0 / g.J; g.n[1] = c1 / g.J; g.n[2] = c2 / g.J;
  cd bf[3];
  for (int k = 0; k < 3; ++k) bf[k] = g.xab[0][k] * g.n[0] + g.xab[1][k] * g.n[1] + g.xab[2][k] * g.n[2];
  g.b[0][0] = bf[0]; g.b[0][1] = bf[2]; g.b[1][0] = bf[2]; g.b[1][1] = bf[1];
  cd bup[2][2], tmp[2][2];
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) tmp[i][j] = g.ainv[i][0] * g.b[0][j] + g.ainv[i][1] * g.b[1][j];
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) bup[i][j] = tmp[i][0] * g.ainv[0][j] + tmp[i][1] * g.ainv[1][j];
  g.H = (g.ainv[0][0] * g.b[0][0] + g.ainv[1][0] * g.b[1][0] + g.ainv[0][1] * g.b[0][1] + g.ainv[1][1] * g.b[1][1]) / 2.0;
  g.K = det2(g.b) / da;
  // dynamics
  const int vu[3] = {vx, vy, vz}, mu_[3] = {vmx, vmy, vmz};
  for (int i = 0; i < 3; ++i) {
    cd s = 0, s1 = 0, s2 = 0, t0 = 0, t1 = 0, t2 = 0;
    cd q = 0, q1 = 0, q2 = 0, r0 = 0, r1 = 0, r2 = 0;
    for (int a = 0; a < 9; ++a) {
      cd va = dof_cp(cps, m, vu[i], a + 1), wa = dof_cp(cps, m, mu_[i], a + 1);
      s += va * f.N[a]; s1 += va * f.dN[a][0]; s2 += va * f.dN[a][1];
      t0 += va * f.ddN[a][0]; t1 += va * f.ddN[a][1]; t2 += va * f.ddN[a][2];
      q += wa * f.N[a]; q1 += wa * f.dN[a][0]; q2 += wa * f.dN[a][1];
      r0 += wa * f.ddN[a][0]; r1 += wa * f.ddN[a][1]; r2 += wa * f.ddN[a][2];
    }
    g.v[i] = s; g.dv[i][0] = s1; g.dv[i][1] = s2; g.ddv[i][0] = t0; g.ddv[i][1] = t1; g.ddv[i][2] = t2;
    g.vm[i] = q; g.dvm[i][0] = q1; g.dvm[i][1] = q2; g.ddvm[i][0] = r0; g.ddvm[i][1] = r1; g.ddvm[i][2] = r2;
  }
  {
    cd s = 0, q = 0;
    for (int a = 0; a < 9; ++a) {
      s += dof_cp(cps, m, lam, a + 1) * f.N[a];
      q += dof_cp(cps, m, pm, a + 1) * f.N[a];
    }
    g.lam = s; g.pm = q;
  }
  // stresses
  auto visc = [&](const cd dvv[3][2], cd out[2][2]) {
    cd t[3][2];
    for (int i = 0; i < 3; ++i)
      for (int be = 0; be < 2; ++be) t[i][be] = dvv[i][0] * g.ainv[0][be] + dvv[i][1] * g.ainv[1][be];
    cd P[2][2];
    for (int al = 0; al < 2; ++al)
      for (int be = 0; be < 2; ++be) P[al][be] = g.aup[0][al] * t[0][be] + g.aup[1][al] * t[1][be] + g.aup[2][al] * t[2][be];
    for (int al = 0; al < 2; ++al)
      for (int be = 0; be < 2; ++be) out[al][be] = (P[al][be] + P[be][al]) * p.zv;
  };
  cd pi[2][2], sg[2][2], Mm[2][2], sm[2][2];
  visc(g.dv, pi);
  cd c_s = p.kb * g.H * g.H - p.kg * g.K + g.lam;
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) sg[i][j] = g.ainv[i][j] * c_s - bup[i][j] * 2.0 * p.kb * g.H + pi[i][j];
  g.sig[0] = sg[0][0]; g.sig[1] = sg[1][1]; g.sig[2] = 2.0 * sg[0][1];
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) Mm[i][j] = g.ainv[i][j] * g.H * (p.kb + 2 * p.kg) - bup[i][j] * p.kg;
  g.M[0] = Mm[0][0]; g.M[1] = Mm[1][1]; g.M[2] = Mm[0][1] + Mm[1][0];
  visc(g.dvm, sm);
  cd c_m = p.kb * g.H * g.H - p.kg * g.K;
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) sm[i][j] = g.ainv[i][j] * c_m - bup[i][j] * 2.0 * p.kb * g.H + sm[i][j];
  g.sigm[0] = sm[0][0]; g.sigm[1] = sm[1][1]; g.sigm[2] = 2.0 * sm[0][1];
  // shape function matrices; column i + 3(a-1)
  for (int a = 0; a < 9; ++a)
    for (int i = 0; i < 3; ++i) {
      int c = i + 3 * a;
      g.Ba[0][c] = g.a[i][0] * f.dN[a][0];
      g.Ba[1][c] = g.a[i][1] * f.dN[a][1];
      g.Ba[2][c] = (g.a[i][0] * f.dN[a][1] + g.a[i][1] * f.dN[a][0]) * 0.5;
    }
  for (int a = 0; a < 9; ++a) {
    cd nn[3];
    for (int k = 0; k < 3; ++k) nn[k] = f.ddN[a][k] - (f.dN[a][0] * g.Gam[k][0] + f.dN[a][1] * g.Gam[k][1]);
    for (int k = 0; k < 3; ++k)
      for (int i = 0; i < 3; ++i) g.Bb[k][i + 3 * a] = g.n[i] * nn[k];
  }
  return g;
}

// ---- element residuals (src/analysis/FiniteElement.jl) ----------------------
// Dohrmann-Bochev constant Gᵀ H⁻¹ G of a unique element (FiniteElement.jl:279-323),
// state-independent.
static void db_matrix(const std::vector<Fza>& fns, double out[9][9]) {
  auto xi = get_xis(GP1D);
  double G[3][9] = {}, Hm[3][3] = {};
  for (int gp = 1; gp <= GP1D * GP1D; ++gp) {
    const Fza& f = fns[gp - 1];
    double NDB[3] = {xi[(gp - 1) % GP1D], xi[(int)std::floor((gp - 1) / (double)GP1D)], 1.0};
    for (int r = 0; r < 3; ++r) {
      for (int a = 0; a < 9; ++a) G[r][a] += NDB[r] * f.N[a] * f.w;
      for (int c = 0; c < 3; ++c) Hm[r][c] += NDB[r] * NDB[c] * f.w;
    }
  }
  // inv(H) via Gauss-Jordan with partial pivoting
  double A[3][6];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 6; ++c) A[r][c] = c < 3 ? Hm[r][c] : (c - 3 == r ? 1.0 : 0.0);
  for (int k = 0; k < 3; ++k) {
    int pv = k;
    for (int r = k + 1; r < 3; ++r)
      if (std::fabs(A[r][k]) > std::fabs(A[pv][k])) pv = r;
    for (int c = 0; c < 6; ++c) std::swap(A[k][c], A[pv][c]);
    double d = A[k][k];
    for (int c = 0; c < 6; ++c) A[k][c] /= d;
    for (int r = 0; r < 3; ++r)
      if (r != k) {
        double fct = A[r][k];
        for (int c = 0; c < 6; ++c) A[r][c] -= fct * A[k][c];
      }
  }
  double Hi[3][3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) Hi[r][c] = A[r][c + 3];
  double HG[3][9];
  for (int r = 0; r < 3; ++r)
    for (int a = 0; a < 9; ++a) HG[r][a] = Hi[r][0] * G[0][a] + Hi[r][1] * G[1][a] + Hi[r][2] * G[2][a];
  for (int a = 0; a < 9; ++a)
    for (int b = 0; b < 9; ++b) out[a][b] = G[0][a] * HG[0][b] + G[1][a] * HG[1][b] + G[2][a] * HG[2][b];
}

struct DofRes { std::vector<cd> rv, rm, rl, rp; };

// FiniteElement.jl:253-330
DofRes calc_elem_dof_residuals(const Mesh& m, int el_id, const Mat1<cd>& xms, const Mat1<cd>& cps) {
  const Params& p = m.p;
  int lo = get_lam_order(m), po = get_p_order(m);
  DofRes R;
  R.rv.assign(27, 0.0); R.rm.assign(27, 0.0); R.rl.assign(9, 0.0); R.rp.assign(po ? 9 : 0, 0.0);
  const auto& fns = m.area.ufns[m.area.uel_ids[el_id - 1] - 1];
  for (int gp = 1; gp <= GP1D * GP1D; ++gp) {
    const Fza& f = fns[gp - 1];
    double w = f.w;
    GDS g = geo_dyn_stress(xms, cps, m, f, p);
    for (int c = 0; c < 27; ++c) {
      cd s = g.Ba[0][c] * g.sig[0] + g.Ba[1][c] * g.sig[1] + g.Ba[2][c] * g.sig[2] + g.Bb[0][c] * g.M[0] +
             g.Bb[1][c] * g.M[1] + g.Bb[2][c] * g.M[2];
      R.rv[c] += s * g.J * w;
    }
    if (p.pn != 0.0)
      for (int a = 0; a < 9; ++a)
        for (int i = 0; i < 3; ++i) R.rv[i + 3 * a] -= g.n[i] * f.N[a] * p.pn * g.J * w;
    cd tr = 0;
    for (int al = 0; al < 2; ++al)
      for (int i = 0; i < 3; ++i) tr += g.aup[i][al] * g.dv[i][al];
    for (int a = 0; a < 9; ++a) R.rl[a] += f.N[a] * w * (g.J * tr - p.adb * g.lam / p.zv);
    if (p.motion == EUL) {
      cd nv = g.n[0] * g.v[0] + g.n[1] * g.v[1] + g.n[2] * g.v[2];
      for (int a = 0; a < 9; ++a)
        for (int i = 0; i < 3; ++i) R.rm[i + 3 * a] += (g.vm[i] - g.n[i] * nv) * f.N[a] * p.am * g.J * w;
    } else if (p.motion == ALEV || p.motion == ALEVB) {
      for (int c = 0; c < 27; ++c) {
        cd s = g.Ba[0][c] * g.sigm[0] + g.Ba[1][c] * g.sigm[1] + g.Ba[2][c] * g.sigm[2];
        R.rm[c] += s * g.J * w;
      }
      if (p.motion == ALEVB)
        for (int c = 0; c < 27; ++c) {
          cd s = g.Bb[0][c] * g.M[0] + g.Bb[1][c] * g.M[1] + g.Bb[2][c] * g.M[2];
          R.rm[c] += s * g.J * w;
        }
      for (int a = 0; a < 9; ++a)
        for (int i = 0; i < 3; ++i) R.rm[i + 3 * a] -= g.n[i] * f.N[a] * g.pm * g.J * w;
      cd nd = g.n[0] * (g.vm[0] - g.v[0]) + g.n[1] * (g.vm[1] - g.v[1]) + g.n[2] * (g.vm[2] - g.v[2]);
      for (int a = 0; a < 9; ++a) R.rp[a] -= f.N[a] * w * g.J * nd;
      for (int a = 0; a < 9; ++a) R.rp[a] -= f.N[a] * w * p.adb * g.pm / p.zv;
    }
  }
  double T[9][9];
  db_matrix(fns, T);
  for (int a = 0; a < 9; ++a) {
    cd s = 0;
    for (int b = 0; b < 9; ++b) s += T[a][b] * cps(b + 1, lo);
    R.rl[a] += s * p.adb / p.zv;
  }
  if (p.motion == ALEV || p.motion == ALEVB)
    for (int a = 0; a < 9; ++a) {
      cd s = 0;
      for (int b = 0; b < 9; ++b) s += T[a][b] * cps(b + 1, po);
      R.rp[a] += s * p.adb / p.zv;
    }
  return R;
}

// FiniteElement.jl:208-242
std::vector<cd> calc_elem_residual(const Mesh& m, int el_id, const Mat1<cd>& xms, const Mat1<cd>& cps) {
  DofRes R = calc_elem_dof_residuals(m, el_id, xms, cps);
  auto vo = get_v_order(m), mo = get_m_order(m);
  int lo = get_lam_order(m), po = get_p_order(m);
  std::vector<cd> r(NEN * m.ndf, 0.0);
  for (int node = 1; node <= NEN; ++node) {
    for (int j = 1; j <= 3; ++j)
      if (vo[j - 1]) r[(vo[j - 1] + m.ndf * (node - 1)) - 1] = R.rv[(j + 3 * (node - 1)) - 1];
    for (int j = 1; j <= 3; ++j)
      if (mo[j - 1]) r[(mo[j - 1] + m.ndf * (node - 1)) - 1] = R.rm[(j + 3 * (node - 1)) - 1];
    r[(lo + m.ndf * (node - 1)) - 1] = R.rl[node - 1];
    if (po != 0) r[(po + m.ndf * (node - 1)) - 1] = R.rp[node - 1];
  }
  return r;
}

// FiniteElement.jl:431-452 (τ normalised with the conjugating dot product)
static void calc_tau_nu(int bdry, const cd a[3][2], const cd n[3], cd tau[3], cd nu[3]) {
  for (int i = 0; i < 3; ++i) {
    if (bdry == BOTTOM) tau[i] = a[i][0];
    else if (bdry == RIGHT) tau[i] = a[i][1];
    else if (bdry == TOP) tau[i] = -a[i][0];
    else tau[i] = -a[i][1];
  }
  cd dd = std::conj(tau[0]) * tau[0] + std::conj(tau[1]) * tau[1] + std::conj(tau[2]) * tau[2];
  cd s = std::sqrt(dd);
  for (int i = 0; i < 3; ++i) tau[i] /= s;
  nu[0] = tau[1] * n[2] - tau[2] * n[1];
  nu[1] = tau[2] * n[0] - tau[0] * n[2];
  nu[2] = tau[0] * n[1] - tau[1] * n[0];
}

// FiniteElement.jl:338-400
std::vector<cd> calc_bdry_element_residual(const Mesh& m, int bdry, int ntype, double nval, int el_id,
                                           const Mat1<cd>& xms, const Mat1<cd>& cps, double time) {
  const Params& p = m.p;
  auto vo = get_v_order(m), mo = get_m_order(m);
  std::vector<cd> rv(27, 0.0), rm(27, 0.0);
  const BdryFns& B = m.bdry_fns.at(bdry);
  const auto& bel = m.bdry_elems.at(bdry);
  int bel_id = (int)(std::find(bel.begin(), bel.end(), el_id) - bel.begin()) + 1;
  ORC_ASSERT(bel_id <= (int)bel.size(), "element id not found on boundary");
  for (int gp = 1; gp <= GP1D; ++gp) {
    const Fza& f = B.ufns[B.uel_ids[bel_id - 1] - 1][gp - 1];
    GDS g = geo_dyn_stress(xms, cps, m, f, p);
    cd tau[3], nu[3];
    calc_tau_nu(bdry, g.a, g.n, tau, nu);
    cd t0 = g.aup[0][0] * tau[0] + g.aup[1][0] * tau[1] + g.aup[2][0] * tau[2];
    cd t1 = g.aup[0][1] * tau[0] + g.aup[1][1] * tau[1] + g.aup[2][1] * tau[2];
    cd JG = 1.0 / std::sqrt(t0 * t0 + t1 * t1);
    if (ntype == STRETCH || ntype == SHEAR) {
      cd fv[3];
      for (int i = 0; i < 3; ++i) fv[i] = ntype == STRETCH ? nval * nu[i] : nval * tau[i];
      for (int a = 0; a < 9; ++a)
        for (int i = 0; i < 3; ++i) rv[i + 3 * a] -= fv[i] * f.N[a] * JG * f.w;
    } else if (ntype == MOMENT && p.scenario == F_BEND) {
      cd nu_up[2];
      for (int al = 0; al < 2; ++al) nu_up[al] = g.aup[0][al] * nu[0] + g.aup[1][al] * nu[1] + g.aup[2][al] * nu[2];
      double Mval = nval * std::min(time / m.args.bend_tm, 1.0);
      for (int a = 0; a < 9; ++a) {
        cd dn = f.dN[a][0] * nu_up[0] + f.dN[a][1] * nu_up[1];
        for (int i = 0; i < 3; ++i) rv[i + 3 * a] -= g.n[i] * dn * Mval * JG * f.w;
      }
    } else {
      ORC_ASSERT(false, "Neumann boundary condition not implemented");
    }
  }
  std::vector<cd> r(NEN * m.ndf, 0.0);
  for (int node = 1; node <= NEN; ++node) {
    for (int j = 1; j <= 3; ++j)
      if (vo[j - 1]) r[(vo[j - 1] + m.ndf * (node - 1)) - 1] = rv[(j + 3 * (node - 1)) - 1];
    for (int j = 1; j <= 3; ++j)
      if (mo[j - 1]) r[(mo[j - 1] + m.ndf * (node - 1)) - 1] = rm[(j + 3 * (node - 1)) - 1];
  }
  return r;
}

// complex-step element tangent (FiniteElement.jl:104-126 / 161-184); the
// residual functor r(xms_el, cps_el) is either the area or the boundary residual.
static void complex_step_tangent(const Mesh& m, int el_id, const Mat1<cd>& xel, const Mat1<cd>& cel, double dt,
                                 const std::function<std::vector<cd>(const Mat1<cd>&, const Mat1<cd>&)>& res,
                                 std::vector<double>& K) {
  int nd = NEN * m.ndf;
  K.assign((size_t)nd * nd, 0.0);  // column-major nd x nd
  auto mmo = get_m_motion_order(m.p.motion, m);
  double ek = m.p.eps_k;
  for (int a = 1; a <= NEN; ++a) {
    int gnode = m.IX(a, el_id);
    for (int d = 1; d <= m.ndf; ++d) {
      if (m.ID(d, gnode) == 0) continue;
      int col = d + m.ndf * (a - 1);
      Mat1<cd> dc = cel;
      dc(a, d) += cd(0.0, ek);
      auto r1 = res(xel, dc);
      for (int i = 0; i < nd; ++i) K[(size_t)i + (size_t)nd * (col - 1)] += std::imag(r1[i]) / ek;
      auto it = std::find(mmo.begin(), mmo.end(), d);
      if (it != mmo.end()) {
        int j = (int)(it - mmo.begin()) + 1;
        Mat1<cd> dx = xel;
        dx(a, j) += cd(0.0, ek);
        auto r2 = res(dx, cel);
        for (int i = 0; i < nd; ++i) K[(size_t)i + (size_t)nd * (col - 1)] += (std::imag(r2[i]) / ek) * dt;
      }
    }
  }
}

static void gather_el(const Mesh& m, int el_id, const double* xms, const double* cps, Mat1<cd>& xel, Mat1<cd>& cel) {
  xel = Mat1<cd>(NEN, 3);
  cel = Mat1<cd>(NEN, m.ndf);
  for (int a = 1; a <= NEN; ++a) {
    int node = m.IX(a, el_id);
    for (int i = 1; i <= 3; ++i) xel(a, i) = xms[(node - 1) + (size_t)m.numnp * (i - 1)];
    for (int d = 1; d <= m.ndf; ++d) cel(a, d) = cps[(node - 1) + (size_t)m.numnp * (d - 1)];
  }
}

// Element residual / tangent of area element el_id (1-based), plus the Neumann
// boundary element contributions of that element when `with_bdry` is set.
void elem_r_K(const Mesh& m, int el_id, const double* xms, const double* cps, double time, double dt,
              bool area, bool bdry_terms, std::vector<double>& r, std::vector<double>& K) {
  int nd = NEN * m.ndf;
  Mat1<cd> xel, cel;
  gather_el(m, el_id, xms, cps, xel, cel);
  r.assign(nd, 0.0);
  K.assign((size_t)nd * nd, 0.0);
  if (area) {
    auto res = [&](const Mat1<cd>& X, const Mat1<cd>& C) { return calc_elem_residual(m, el_id, X, C); };
    auto r0 = res(xel, cel);
    for (int i = 0; i < nd; ++i) r[i] = std::real(r0[i]);
    complex_step_tangent(m, el_id, xel, cel, dt, res, K);
  }
  if (bdry_terms) {
    for (const auto& nb : m.inh_neu_bcs) {
      const auto& bel = m.bdry_elems.at(nb.bdry);
      if (std::find(bel.begin(), bel.end(), el_id) == bel.end()) continue;
      auto res = [&](const Mat1<cd>& X, const Mat1<cd>& C) {
        return calc_bdry_element_residual(m, nb.bdry, nb.ntype, nb.value, el_id, X, C, time);
      };
      auto r0 = res(xel, cel);
      for (int i = 0; i < nd; ++i) r[i] += std::real(r0[i]);
      std::vector<double> Kb;
      complex_step_tangent(m, el_id, xel, cel, dt, res, Kb);
      for (size_t q = 0; q < K.size(); ++q) K[q] += Kb[q];
    }
  }
}

// ---- banded matrix (LAPACK layout, 1-based (i,j) -> ab[kl+ku+i-j + ldab*(j-1)]) ----
struct Band {
  int n, kl, ku, ldab;
  double* ab;
  double& at(int i, int j) { return ab[(size_t)(kl + ku + i - j) + (size_t)ldab * (j - 1)]; }
};

// calc_r_K (FiniteElement.jl:75-200): residual r (nmdf) and tangent K scattered
// into band storage (K must have kl, ku >= the mesh half bandwidth).  Area
// elements are processed by colour (e1 mod 3, e2 mod 3) so that threads of one
// colour touch disjoint rows; the Neumann loop runs after it, serially.
void calc_r_K(const Mesh& m, const double* xms, const double* cps, double time, double dt, int nthreads,
              double* r, Band* K) {
  int nd = NEN * m.ndf;
  std::fill(r, r + m.nmdf, 0.0);
  auto scatter = [&](int e, const std::vector<double>& re, const std::vector<double>& Ke) {
    for (int a = 1; a <= nd; ++a) {
      int ga = m.LM(a, e);
      if (!ga) continue;
      r[ga - 1] += re[a - 1];
      if (K)
        for (int b = 1; b <= nd; ++b) {
          int gb = m.LM(b, e);
          if (!gb) continue;
          K->at(ga, gb) += Ke[(size_t)(a - 1) + (size_t)nd * (b - 1)];
        }
    }
  };
  nthreads = std::max(1, nthreads);
  for (int c2 = 0; c2 < 3; ++c2)
    for (int c1 = 0; c1 < 3; ++c1) {
      std::vector<int> els;
      for (int e2 = 1 + c2; e2 <= m.num2el; e2 += 3)
        for (int e1 = 1 + c1; e1 <= m.num1el; e1 += 3) els.push_back(e1 + (e2 - 1) * m.num1el);
      auto work = [&](int t) {
        std::vector<double> re, Ke;
        for (size_t q = t; q < els.size(); q += nthreads) {
          elem_r_K(m, els[q], xms, cps, time, dt, true, false, re, Ke);
          scatter(els[q], re, Ke);
        }
      };
      if (nthreads == 1) work(0);
      else {
        std::vector<std::thread> th;
        for (int t = 0; t < nthreads; ++t) th.emplace_back(work, t);
        for (auto& t : th) t.join();
      }
    }
  for (const auto& nb : m.inh_neu_bcs)
    for (int e : m.bdry_elems.at(nb.bdry)) {
      Mat1<cd> xel, cel;
      gather_el(m, e, xms, cps, xel, cel);
      auto res = [&](const Mat1<cd>& X, const Mat1<cd>& C) {
        return calc_bdry_element_residual(m, nb.bdry, nb.ntype, nb.value, e, X, C, time);
      };
      auto r0 = res(xel, cel);
      std::vector<double> re(nd), Ke;
      for (int i = 0; i < nd; ++i) re[i] = std::real(r0[i]);
      if (K) complex_step_tangent(m, e, xel, cel, dt, res, Ke);
      else Ke.assign((size_t)nd * nd, 0.0);
      scatter(e, re, Ke);
    }
}

// half bandwidth of K in the reference's ID ordering
int half_bandwidth(const Mesh& m) {
  int b = 0, nd = NEN * m.ndf;
  for (int e = 1; e <= m.numel; ++e) {
    int lo = 1 << 30, hi = 0;
    for (int a = 1; a <= nd; ++a) {
      int g = m.LM(a, e);
      if (g) { lo = std::min(lo, g); hi = std::max(hi, g); }
    }
    if (hi) b = std::max(b, hi - lo);
  }
  return b;
}

// Banded LU with partial pivoting, unblocked (LAPACK gbtf2 algorithm; band has
// 2kl+ku+1 rows, the top kl rows hold the fill).  Returns 0 or the 1-based
// column of an exactly-zero pivot.
int band_lu(Band& A, int* ipiv) {
  int n = A.n, kl = A.kl, ku = A.ku;
  int kv = ku + kl;
  // zero the fill rows
  for (int j = 1; j <= n; ++j)
    for (int r = 0; r < kl; ++r) A.ab[(size_t)r + (size_t)A.ldab * (j - 1)] = 0.0;
  int ju = 1, info = 0;
  for (int j = 1; j <= n; ++j) {
    int km = std::min(kl, n - j);
    int p = j;
    double mx = std::fabs(A.at(j, j));
    for (int i = j + 1; i <= j + km; ++i)
      if (std::fabs(A.at(i, j)) > mx) { mx = std::fabs(A.at(i, j)); p = i; }
    ipiv[j - 1] = p;
    if (A.at(p, j) != 0.0) {
      ju = std::max(ju, std::min(j + ku + (p - j), n));
      if (p != j)
        for (int c = j; c <= ju; ++c) std::swap(A.at(j, c), A.at(p, c));
      double inv = 1.0 / A.at(j, j);
      for (int i = j + 1; i <= j + km; ++i) A.at(i, j) *= inv;
      for (int c = j + 1; c <= ju; ++c) {
        double u = A.at(j, c);
        if (u != 0.0)
          for (int i = j + 1; i <= j + km; ++i) A.at(i, c) -= A.at(i, j) * u;
      }
    } else if (info == 0) {
      info = j;
    }
    (void)kv;
  }
  return info;
}
void band_solve(Band& A, const int* ipiv, double* b) {
  int n = A.n, kl = A.kl, ku = A.ku;
  for (int j = 1; j <= n; ++j) {
    int km = std::min(kl, n - j);
    int p = ipiv[j - 1];
    if (p != j) std::swap(b[p - 1], b[j - 1]);
    for (int i = j + 1; i <= j + km; ++i) b[i - 1] -= A.at(i, j) * b[j - 1];
  }
  for (int j = n; j >= 1; --j) {
    b[j - 1] /= A.at(j, j);
    int top = std::max(1, j - (kl + ku));
    for (int i = top; i < j; ++i) b[i - 1] -= A.at(i, j) * b[j - 1];
  }
}

// update_xms! (FiniteElement.jl:408-423); xms, cps column-major numnp x {3, ndf}
void update_xms(const Mesh& m, double* xms, const double* c, double dt) {
  auto mmo = get_m_motion_order(m.p.motion, m);
  for (int j = 1; j <= 3; ++j) {
    if (!mmo[j - 1]) continue;
    for (int node = 0; node < m.numnp; ++node)
      xms[node + (size_t)m.numnp * (j - 1)] += dt * c[node + (size_t)m.numnp * (mmo[j - 1] - 1)];
  }
}

}  // namespace orc

// ============================================================================
// C ABI for the tests (ctypes).  Return codes: 0 ok, 1 reference assertion
// failed (message in orc_last_error), 2 other error.
// ============================================================================
using namespace orc;

static thread_local std::string g_err;
#define ORC_TRY(...)                                \
  try {                                             \
    __VA_ARGS__;                                    \
    return 0;                                       \
  } catch (const AssertionError& e) {               \
    g_err = e.what();                               \
    return 1;                                       \
  } catch (const std::exception& e) {               \
    g_err = e.what();                               \
    return 2;                                       \
  }

extern "C" {

typedef struct orc_params {
  int motion, scenario, num1el, num2el;
  double length, kb, kg, zv, pn;
  int poly, gp1d, nders, nen;
  double adb, am, eps_k, eps_nr;
  double pull_speed, bend_tm, bend_mf;
  double lambda0;
  int pull_centre;
} orc_params;

const char* orc_last_error() { return g_err.c_str(); }

static KnotVector mk_kv(const double* zs, int nz, int poly, int curve) {
  return knot_vector(std::vector<double>(zs, zs + nz), poly, curve);
}

int orc_knot_vector_check(const double* zs, int nz, int poly, int curve, int* nel) {
  ORC_TRY(*nel = mk_kv(zs, nz, poly, curve).nel)
}
int orc_knot_vector_uniform(int nel, int poly, int curve, double* out) {
  ORC_TRY({
    auto kv = knot_vector_uniform(nel, poly, curve);
    std::copy(kv.zs.begin(), kv.zs.end(), out);
  })
}
int orc_fine_zs(int nel, int poly, double* out) {
  ORC_TRY({
    auto v = get_fine_zs(nel, poly);
    std::copy(v.begin(), v.end(), out);
  })
}
int orc_knot_span(const double* zs, int nz, int poly, int curve, double z, int* out) {
  ORC_TRY(*out = get_knot_span_index(mk_kv(zs, nz, poly, curve), z))
}
int orc_bspline_vals(const double* zs, int nz, int poly, int curve, double z, double* out) {
  ORC_TRY({
    auto v = get_bspline_vals(mk_kv(zs, nz, poly, curve), z);
    std::copy(v.begin(), v.end(), out);
  })
}
int orc_bspline_ders(const double* zs, int nz, int poly, int curve, double z, int nders, double* out) {
  ORC_TRY({
    auto D = get_bspline_ders(mk_kv(zs, nz, poly, curve), z, nders);
    std::copy(D.d.begin(), D.d.end(), out);
  })
}
int orc_bspline_indices(const double* zs, int nz, int poly, int curve, double z, int* out) {
  ORC_TRY({
    auto v = get_bspline_indices(mk_kv(zs, nz, poly, curve), z);
    std::copy(v.begin(), v.end(), out);
  })
}
int orc_collocate(const double* zs, int nz, int poly, int curve, double* out, int* nout) {
  ORC_TRY({
    auto v = collocate_z(mk_kv(zs, nz, poly, curve));
    std::copy(v.begin(), v.end(), out);
    *nout = (int)v.size();
  })
}
typedef double (*orc_fn1)(double);
typedef double (*orc_fn2)(double, double);
int orc_1d_cps(const double* zs, int nz, int poly, int curve, orc_fn1 f, double* out, int* nout) {
  ORC_TRY({
    auto v = get_1d_bspline_cps(mk_kv(zs, nz, poly, curve), [&](double z) { return f(z); });
    std::copy(v.begin(), v.end(), out);
    *nout = (int)v.size();
  })
}
int orc_2d_cps(const double* zs1, int nz1, const double* zs2, int nz2, int poly, orc_fn2 f, double* out) {
  ORC_TRY({
    auto v = get_2d_bspline_cps(mk_kv(zs1, nz1, poly, CLAMPED), mk_kv(zs2, nz2, poly, CLAMPED),
                                [&](double a, double b) { return f(a, b); });
    std::copy(v.begin(), v.end(), out);
  })
}
int orc_unique_1d(const double* zs, int nz, int poly, int curve, int* uel_num, int* num_el, int* uel_ids,
                  double* uel_list) {
  ORC_TRY({
    auto u = get_unique_1d_elements(mk_kv(zs, nz, poly, curve));
    *uel_num = u.uel_num;
    *num_el = u.num_el;
    std::copy(u.uel_ids.begin(), u.uel_ids.end(), uel_ids);
    for (size_t q = 0; q < u.uel_list.size(); ++q) {
      uel_list[2 * q] = u.uel_list[q].first;
      uel_list[2 * q + 1] = u.uel_list[q].second;
    }
  })
}
int orc_gauss_xi(int ngp, double* xs, double* ws) {
  ORC_TRY({
    auto a = get_xis(ngp);
    auto b = get_xi_weights(ngp);
    std::copy(a.begin(), a.end(), xs);
    std::copy(b.begin(), b.end(), ws);
  })
}
int orc_gauss_zeta(int ngp, double lo, double hi, double* zs, double* ws) {
  ORC_TRY({
    std::vector<double> a, b;
    gauss_zeta(ngp, lo, hi, a, b);
    std::copy(a.begin(), a.end(), zs);
    std::copy(b.begin(), b.end(), ws);
  })
}
// GpBasisFnsζ packed as (w, N[3], dN[3], ddN[3])
int orc_gp_fns_z(double w, double z, const double* zs, int nz, int poly, int curve, double* out) {
  ORC_TRY({
    Fz f = gp_basis_fns_z(w, z, mk_kv(zs, nz, poly, curve));
    out[0] = f.w;
    for (int i = 0; i < 3; ++i) { out[1 + i] = f.N[i]; out[4 + i] = f.dN[i]; out[7 + i] = f.ddN[i]; }
  })
}
static Fz unpack_fz(const double* in) {
  Fz f;
  f.w = in[0];
  for (int i = 0; i < 3; ++i) { f.N[i] = in[1 + i]; f.dN[i] = in[4 + i]; f.ddN[i] = in[7 + i]; }
  return f;
}
// GpBasisFnsζα packed as (w, N[9], dN[9][2] (column-major 9x2), ddN[9][3] (column-major 9x3))
static void pack_fza(const Fza& g, double* out) {
  out[0] = g.w;
  for (int a = 0; a < 9; ++a) {
    out[1 + a] = g.N[a];
    for (int k = 0; k < 2; ++k) out[10 + a + 9 * k] = g.dN[a][k];
    for (int k = 0; k < 3; ++k) out[28 + a + 9 * k] = g.ddN[a][k];
  }
}
int orc_gp_fns_za(const double* f1, const double* f2, double* out) {
  ORC_TRY(pack_fza(gp_basis_fns_za(unpack_fz(f1), unpack_fz(f2)), out))
}
// LineGpBasisFns: uel_ids (nel), ufns packed [uel][gp] x 10 doubles, zmin/zmax 10 each
int orc_line_gp_fns(const double* zs, int nz, int poly, int curve, int ngp, int* nel, int* n_uel, int* uel_ids,
                    double* ufns, double* zmin, double* zmax) {
  ORC_TRY({
    LineFns L = line_gp_basis_fns(mk_kv(zs, nz, poly, curve), ngp);
    *nel = L.nel;
    *n_uel = (int)L.ufns.size();
    std::copy(L.uel_ids.begin(), L.uel_ids.end(), uel_ids);
    auto pk = [](const Fz& f, double* o) {
      o[0] = f.w;
      for (int i = 0; i < 3; ++i) { o[1 + i] = f.N[i]; o[4 + i] = f.dN[i]; o[7 + i] = f.ddN[i]; }
    };
    for (size_t q = 0; q < L.ufns.size(); ++q)
      for (int g = 0; g < ngp; ++g) pk(L.ufns[q][g], ufns + 10 * (q * ngp + g));
    pk(L.zmin, zmin);
    pk(L.zmax, zmax);
  })
}

// ---- mesh handle --------------------------------------------------------------
static Params to_params(const orc_params* q) {
  Params p;
  p.motion = q->motion; p.scenario = q->scenario; p.num1el = q->num1el; p.num2el = q->num2el;
  p.length = q->length; p.kb = q->kb; p.kg = q->kg; p.zv = q->zv; p.pn = q->pn;
  p.poly = q->poly; p.gp1d = q->gp1d; p.nders = q->nders; p.nen = q->nen;
  p.adb = q->adb; p.am = q->am; p.eps_k = q->eps_k; p.eps_nr = q->eps_nr;
  return p;
}
int orc_mesh_create(const orc_params* q, void** out) {
  ORC_TRY({
    Params p = to_params(q);
    ORC_ASSERT(p.nen == (p.poly + 1) * (p.poly + 1), "incorrect number of element nodes");
    ORC_ASSERT(p.nen == NEN && p.poly == POLY && p.nders == NDERS, "compile-time constants mismatch");
    Args a;
    a.pull_speed = q->pull_speed; a.bend_tm = q->bend_tm; a.bend_mf = q->bend_mf;
    a.lambda0 = q->lambda0; a.pull_centre = q->pull_centre;
    ORC_ASSERT(a.lambda0 >= 0.0 && std::isfinite(a.lambda0), "lambda0 must be finite and >= 0");
    ORC_ASSERT(a.lambda0 == 0.0 || p.scenario == F_PULL, "lambda0 is an F_PULL extension");
    // check_params' scenario conditions (Params.jl:97-119)
    if (p.scenario == F_BEND) {
      ORC_ASSERT(a.bend_mf == p.kb / 2 / p.length, "α = 1/2 is the half-angle");
      ORC_ASSERT(p.motion != STATIC, "mesh cannot be static for F_BEND scenario");
      ORC_ASSERT(p.motion != ALEVB, "F_BEND not implemented for ALEVB motion");
      ORC_ASSERT(p.pn == 0.0, "F_BEND with normal pressure not implemented");
    } else if (p.scenario == F_CAVI || p.scenario == F_COUE || p.scenario == F_POIS) {
      ORC_ASSERT(p.motion == STATIC, "need static motion for the flat flow scenarios");
    }
    *out = generate_mesh(p, a).release();
  })
}
void orc_mesh_destroy(void* h) { delete (Mesh*)h; }
// sizes: num1el num2el numel num1np num2np numnp ndf nmdf n_uel half_bw n_neu n_dir
void orc_mesh_sizes(void* h, int* s) {
  Mesh* m = (Mesh*)h;
  s[0] = m->num1el; s[1] = m->num2el; s[2] = m->numel; s[3] = m->num1np; s[4] = m->num2np; s[5] = m->numnp;
  s[6] = m->ndf; s[7] = m->nmdf; s[8] = (int)m->area.ufns.size(); s[9] = half_bandwidth(*m);
  s[10] = (int)m->inh_neu_bcs.size(); s[11] = (int)m->inh_dir_bcs.size();
}
void orc_mesh_dofs(void* h, int* dofs8) {
  Mesh* m = (Mesh*)h;
  for (int u = 1; u <= 8; ++u) dofs8[u - 1] = m->dofs[u];
}
void orc_mesh_IX(void* h, int* out) { Mesh* m = (Mesh*)h; std::copy(m->IX.d.begin(), m->IX.d.end(), out); }
void orc_mesh_ID(void* h, int* out) { Mesh* m = (Mesh*)h; std::copy(m->ID.d.begin(), m->ID.d.end(), out); }
void orc_mesh_LM(void* h, int* out) { Mesh* m = (Mesh*)h; std::copy(m->LM.d.begin(), m->LM.d.end(), out); }
void orc_mesh_ID_inv(void* h, int* out) {
  Mesh* m = (Mesh*)h;
  for (size_t q = 0; q < m->ID_inv.size(); ++q) { out[2 * q] = m->ID_inv[q].first; out[2 * q + 1] = m->ID_inv[q].second; }
}
void orc_mesh_knots(void* h, double* kv1, double* kv2) {
  Mesh* m = (Mesh*)h;
  std::copy(m->kv1.zs.begin(), m->kv1.zs.end(), kv1);
  std::copy(m->kv2.zs.begin(), m->kv2.zs.end(), kv2);
}
// area tables: uel_ids (numel, 1-based), ufns [uel][gp] x 55 doubles
void orc_mesh_area(void* h, int* uel_ids, double* ufns) {
  Mesh* m = (Mesh*)h;
  std::copy(m->area.uel_ids.begin(), m->area.uel_ids.end(), uel_ids);
  for (size_t q = 0; q < m->area.ufns.size(); ++q)
    for (int g = 0; g < 9; ++g) pack_fza(m->area.ufns[q][g], ufns + 55 * (q * 9 + g));
}
// boundary tables of boundary b: n_uel, uel_ids (len nel), ufns [uel][gp] x 55
void orc_mesh_bdry(void* h, int b, int* nel, int* n_uel, int* uel_ids, double* ufns) {
  Mesh* m = (Mesh*)h;
  const BdryFns& B = m->bdry_fns.at(b);
  *nel = B.nel;
  *n_uel = (int)B.ufns.size();
  if (uel_ids) std::copy(B.uel_ids.begin(), B.uel_ids.end(), uel_ids);
  if (ufns)
    for (size_t q = 0; q < B.ufns.size(); ++q)
      for (size_t g = 0; g < B.ufns[q].size(); ++g) pack_fza(B.ufns[q][g], ufns + 55 * (q * 3 + g));
}
void orc_mesh_bdry_elems(void* h, int b, int* out) {
  Mesh* m = (Mesh*)h;
  const auto& v = m->bdry_elems.at(b);
  std::copy(v.begin(), v.end(), out);
}
void orc_mesh_bdry_nodes(void* h, int b, int inner, int* out) {
  Mesh* m = (Mesh*)h;
  const auto& v = inner ? m->bdry_inner_nodes.at(b) : m->bdry_nodes.at(b);
  std::copy(v.begin(), v.end(), out);
}
void orc_mesh_neu(void* h, int* bdry, int* ntype, double* val) {
  Mesh* m = (Mesh*)h;
  for (size_t q = 0; q < m->inh_neu_bcs.size(); ++q) {
    bdry[q] = m->inh_neu_bcs[q].bdry; ntype[q] = m->inh_neu_bcs[q].ntype; val[q] = m->inh_neu_bcs[q].value;
  }
}
void orc_mesh_dir(void* h, int* unknown, int* node, double* val) {
  Mesh* m = (Mesh*)h;
  for (size_t q = 0; q < m->inh_dir_bcs.size(); ++q) {
    unknown[q] = m->inh_dir_bcs[q].unknown; node[q] = m->inh_dir_bcs[q].node; val[q] = m->inh_dir_bcs[q].value;
  }
}
// prepare_input (src/Input.jl:22-121), default (non-file) initial state for the
// non-F_BEND scenarios; xms numnp x 3, cps numnp x ndf column-major.
int orc_prepare_input(void* h, double* xms, double* cps) {
  ORC_TRY({
    Mesh* m = (Mesh*)h;
    const Params& p = m->p;
    ORC_ASSERT(p.scenario != F_BEND, "F_BEND initial state uses the unseeded global RNG");
    int np = m->numnp;
    std::fill(xms, xms + (size_t)np * 3, 0.0);
    std::fill(cps, cps + (size_t)np * m->ndf, 0.0);
    auto X = get_2d_bspline_cps(m->kv1, m->kv2, [&](double z1, double) { return p.length * (z1 - 0.5); });
    auto Y = get_2d_bspline_cps(m->kv1, m->kv2, [&](double, double z2) { return p.length * (z2 - 0.5); });
    for (int i = 0; i < np; ++i) { xms[i] = X[i]; xms[i + np] = Y[i]; }
    double lv = p.scenario == F_PULL ? pull_lambda(p, m->args) : p.kb / 4;  // Input.jl:85 (kb / 4)
    for (int i = 0; i < np; ++i) cps[i + (size_t)np * (m->dofs[lam] - 1)] = lv;
    for (const auto& bc : m->inh_dir_bcs) {
      cps[(bc.node - 1) + (size_t)np * (m->dofs[bc.unknown] - 1)] = bc.value;
      if (p.scenario == F_PULL && p.motion == EUL) cps[(bc.node - 1) + (size_t)np * (m->dofs[vmz] - 1)] = bc.value;
    }
  })
}
// GeoDynStress fields at (element, area GP) [or boundary GP when bdry > 0]:
// x[3] a[3x2] aup[3x2] J n[3] b[2x2] H K v[3] dv[3x2] lam pm vm[3] sig[3] sigm[3] M[3] Gam[3x2]
// ainv[2x2] (real parts; 58 doubles, matrices column-major)
int orc_gds(void* h, const double* xms, const double* cps, int el_id, int gp_id, int bdry, double* out) {
  ORC_TRY({
    Mesh* m = (Mesh*)h;
    Mat1<cd> xel, cel;
    gather_el(*m, el_id, xms, cps, xel, cel);
    const Fza* f;
    if (bdry > 0) {
      const BdryFns& B = m->bdry_fns.at(bdry);
      const auto& bel = m->bdry_elems.at(bdry);
      int bel_id = (int)(std::find(bel.begin(), bel.end(), el_id) - bel.begin()) + 1;
      f = &B.ufns[B.uel_ids[bel_id - 1] - 1][gp_id - 1];
    } else {
      f = &m->area.ufns[m->area.uel_ids[el_id - 1] - 1][gp_id - 1];
    }
    GDS g = geo_dyn_stress(xel, cel, *m, *f, m->p);
    int o = 0;
    for (int i = 0; i < 3; ++i) out[o++] = g.x[i].real();
    for (int al = 0; al < 2; ++al) for (int i = 0; i < 3; ++i) out[o++] = g.a[i][al].real();
    for (int al = 0; al < 2; ++al) for (int i = 0; i < 3; ++i) out[o++] = g.aup[i][al].real();
    out[o++] = g.J.real();
    for (int i = 0; i < 3; ++i) out[o++] = g.n[i].real();
    for (int j = 0; j < 2; ++j) for (int i = 0; i < 2; ++i) out[o++] = g.b[i][j].real();
    out[o++] = g.H.real();
    out[o++] = g.K.real();
    for (int i = 0; i < 3; ++i) out[o++] = g.v[i].real();
    for (int al = 0; al < 2; ++al) for (int i = 0; i < 3; ++i) out[o++] = g.dv[i][al].real();
    out[o++] = g.lam.real();
    out[o++] = g.pm.real();
    for (int i = 0; i < 3; ++i) out[o++] = g.vm[i].real();
    for (int i = 0; i < 3; ++i) out[o++] = g.sig[i].real();
    for (int i = 0; i < 3; ++i) out[o++] = g.sigm[i].real();
    for (int i = 0; i < 3; ++i) out[o++] = g.M[i].real();
    for (int mu = 0; mu < 2; ++mu) for (int k = 0; k < 3; ++k) out[o++] = g.Gam[k][mu].real();
    for (int j = 0; j < 2; ++j) for (int i = 0; i < 2; ++i) out[o++] = g.ainv[i][j].real();
  })
}
// element residual (nd) and tangent (nd x nd column-major); area and/or boundary terms
int orc_elem_r_K(void* h, const double* xms, const double* cps, int el_id, double time, double dt, int area,
                 int bdry_terms, double* r, double* K) {
  ORC_TRY({
    Mesh* m = (Mesh*)h;
    std::vector<double> re, Ke;
    elem_r_K(*m, el_id, xms, cps, time, dt, area != 0, bdry_terms != 0, re, Ke);
    std::copy(re.begin(), re.end(), r);
    if (K) std::copy(Ke.begin(), Ke.end(), K);
  })
}
// calc_r_K into LAPACK band storage (ldab >= 2kl+ku+1, kl/ku >= half bandwidth); K may be null
int orc_calc_r_K(void* h, const double* xms, const double* cps, double time, double dt, int nthreads, double* r,
                 double* ab, int kl, int ku, int ldab) {
  ORC_TRY({
    Mesh* m = (Mesh*)h;
    if (ab) {
      std::fill(ab, ab + (size_t)ldab * m->nmdf, 0.0);
      Band B{m->nmdf, kl, ku, ldab, ab};
      calc_r_K(*m, xms, cps, time, dt, nthreads, r, &B);
    } else {
      calc_r_K(*m, xms, cps, time, dt, nthreads, r, nullptr);
    }
  })
}
int orc_band_lu(int n, int kl, int ku, double* ab, int ldab, int* ipiv, int* info) {
  ORC_TRY({
    Band B{n, kl, ku, ldab, ab};
    *info = band_lu(B, ipiv);
  })
}
int orc_band_solve(int n, int kl, int ku, double* ab, int ldab, const int* ipiv, double* b) {
  ORC_TRY({
    Band B{n, kl, ku, ldab, ab};
    band_solve(B, ipiv, b);
  })
}
void orc_update_xms(void* h, double* xms, const double* c, double dt) { update_xms(*(Mesh*)h, xms, c, dt); }

// calc_pull_force (PullForce.jl:61-80) with get_pull_el_id (:8-13) and
// get_adj_maps (:25-53): real(rv) of calc_elem_dof_residuals of each element
// adjacent to the pulled element (ceil(numel/2), or the centre element), at the nodes it shares with that element,
// summed over the pulled element's nodes -> f[3].  Ids outside 1..numel are an
// error (the reference would raise a BoundsError).
int orc_pull_force(void* h, const double* xms, const double* cps, double* f) {
  ORC_TRY({
    Mesh* m = (Mesh*)h;
    const int poly = m->p.poly, numel = m->numel, n1 = m->p.num1el;
    const int pull = pull_el_id(m->p, m->args);  // ceil(numel / 2) or the centre element, 1-based
    std::vector<int> pull_nodes;
    for (int a = 1; a <= NEN; ++a) pull_nodes.push_back(m->IX(a, pull));
    std::vector<double> rv_pull((size_t)3 * NEN, 0.0);
    for (int i = -poly; i <= poly; ++i)
      for (int j = -poly; j <= poly; ++j) {
        const int adj = pull + i * n1 + j;
        ORC_ASSERT(adj >= 1 && adj <= numel, "pull-force neighbourhood leaves the patch");
        Mat1<cd> xel, cel;
        gather_el(*m, adj, xms, cps, xel, cel);
        DofRes R = calc_elem_dof_residuals(*m, adj, xel, cel);
        // (pull-local node, adj-local node) pairs in increasing local order on both sides
        std::vector<int> pl, al;
        for (int a = 1; a <= NEN; ++a) {
          for (int b = 1; b <= NEN; ++b)
            if (m->IX(b, adj) == pull_nodes[a - 1]) { pl.push_back(a); break; }
        }
        for (int b = 1; b <= NEN; ++b)
          if (std::find(pull_nodes.begin(), pull_nodes.end(), m->IX(b, adj)) != pull_nodes.end()) al.push_back(b);
        for (size_t t = 0; t < pl.size(); ++t)
          for (int k = 0; k < 3; ++k) rv_pull[(size_t)3 * (pl[t] - 1) + k] += R.rv[(size_t)3 * (al[t] - 1) + k].real();
      }
    for (int k = 0; k < 3; ++k) {
      double s = 0.0;
      for (int a = 0; a < NEN; ++a) s += rv_pull[(size_t)3 * a + k];
      f[k] = s;
    }
  })
}

// time_step! (FiniteElement.jl:11-63) with the banded LU as the linear solver.
// eps_out receives up to 14 values; returns 1 (assertion) if not converged.
int orc_time_step(void* h, double* xms, double* cps, double time, double dt, int nthreads, int* iters,
                  double* eps_out) {
  ORC_TRY({
    Mesh* m = (Mesh*)h;
    int n = m->nmdf, b = half_bandwidth(*m);
    int ldab = 2 * b + b + 1;
    std::vector<double> ab((size_t)ldab * n), r(n), dcps((size_t)m->numnp * m->ndf);
    std::vector<int> ipiv(n);
    int iter = 1;
    double eps = 1e300;
    *iters = 0;
    while (iter < 15) {
      std::fill(ab.begin(), ab.end(), 0.0);
      Band B{n, b, b, ldab, ab.data()};
      calc_r_K(*m, xms, cps, time, dt, nthreads, r.data(), &B);
      int info = band_lu(B, ipiv.data());
      ORC_ASSERT(info == 0, "singular tangent");
      band_solve(B, ipiv.data(), r.data());
      std::fill(dcps.begin(), dcps.end(), 0.0);
      double nrm = 0;
      for (int q = 0; q < n; ++q) {
        double du = -r[q];
        auto nd = m->ID_inv[q];
        dcps[(nd.first - 1) + (size_t)m->numnp * (nd.second - 1)] = du;
        nrm += du * du;
      }
      for (size_t q = 0; q < dcps.size(); ++q) cps[q] += dcps[q];
      update_xms(*m, xms, dcps.data(), dt);
      eps = std::sqrt(nrm) / n;
      eps_out[iter - 1] = eps;
      *iters = iter;
      iter += 1;
      if (eps < m->p.eps_nr) break;
    }
    ORC_ASSERT(eps < m->p.eps_nr, "did not reach Newton--Raphson tolerance");
  })
}

}  // extern "C"
