// elem.cu -- element residual + tangent (calc_r_K's element loop) and the
// atomics-free gather of element blocks into the banded global tangent.
//
// Reference: src/analysis/FiniteElement.jl:75-200 (calc_r_K), :208-242
// (calc_elem_residual), :253-330 (calc_elem_dof_residuals), :338-400
// (calc_bdry_element_residual), :431-452 (calc_τ_ν); GP kinematics and
// stresses from src/analysis/GeoDynStress.jl:91-178.
//
// The reference differentiates the element residual by complex steps, one
// residual evaluation per active element dof (FiniteElement.jl:109-126).  Here
// the same derivative is computed in forward mode: each thread of an element
// owns one element dof q = (node a*, dof d*) and evaluates the residual on dual
// numbers (primal FP64, tangent T = double or float) seeded with
// ∂cps[a*, d*] = 1 and, when d* is a mesh-motion dof of component j,
// ∂xms[a*, j] = Δt -- the reference's two complex steps of one column merged by
// linearity (FiniteElement.jl:113-122).  The derivative of |τ| is dropped in
// the boundary term, exactly as the reference's conjugating `dot` drops it
// (FiniteElement.jl:448).
//
// Two precisions.  The plain FP64 form evaluates primal and tangent in FP64
// (P = T = double) and takes the residual from the same pass (each thread keeps
// the primal value of its own row).  The FP32 form splits the work by pipe:
// elem_tan_kernel evaluates primal and tangent in FP32 (P = T = float, staged
// inputs converted once per element), and elem_resid_kernel evaluates the
// primal alone in FP64, one thread per (element, Gauss point), so that the
// FP64 pipe -- 1/64 of the FP32 rate on this GPU -- does 1/72 of the plain
// form's FP64 work.  The residual's summation order (Gauss points 0..8, the
// Dohrmann-Bochev term, then the Neumann points) is the plain form's.
//
// Layout: elements are independent, so one CTA processes EPB elements with
// nq = 9*ndf threads each; the element's tangent columns accumulate in shared
// memory ([row][q], conflict-free) and are written once, column-major, to a
// staging buffer K_el[e][q][row].  A second kernel gathers, for every band
// entry, the <= 9 element contributions that land on it (a biquadratic node
// lies in up to 3 x 3 elements; no atomics: each
// output is written by exactly one thread), zero-filling the rest of the band.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "batch_common.cuh"
#include "mafem_internal.h"

namespace mafem {

// ---- dual numbers ------------------------------------------------------------
// primal P, tangent T (Nil: primal only)
struct Nil {
  __device__ __forceinline__ Nil() {}
  __device__ __forceinline__ explicit Nil(double) {}
  __device__ __forceinline__ explicit Nil(float) {}
  __device__ __forceinline__ explicit Nil(int) {}
};
__device__ __forceinline__ Nil operator+(Nil, Nil) { return Nil(); }
__device__ __forceinline__ Nil operator-(Nil, Nil) { return Nil(); }
__device__ __forceinline__ Nil operator-(Nil) { return Nil(); }
__device__ __forceinline__ Nil operator*(Nil, Nil) { return Nil(); }

template <class P, class T>
struct Dual {
  P v;
  T d;
};
template <class P, class T>
__device__ __forceinline__ Dual<P, T> mk(P v, T d) { return Dual<P, T>{v, d}; }
template <class P, class T>
__device__ __forceinline__ Dual<P, T> cst(P v) { return Dual<P, T>{v, T(0.0)}; }
template <class P, class T>
__device__ __forceinline__ Dual<P, T> operator+(Dual<P, T> a, Dual<P, T> b) { return {a.v + b.v, a.d + b.d}; }
template <class P, class T>
__device__ __forceinline__ Dual<P, T> operator-(Dual<P, T> a, Dual<P, T> b) { return {a.v - b.v, a.d - b.d}; }
template <class P, class T>
__device__ __forceinline__ Dual<P, T> operator-(Dual<P, T> a) { return {-a.v, -a.d}; }
template <class P, class T>
__device__ __forceinline__ Dual<P, T> operator*(Dual<P, T> a, Dual<P, T> b) {
  return {a.v * b.v, a.d * T(b.v) + T(a.v) * b.d};
}
// scalars are converted to the primal type (constants fold at compile time;
// runtime parameters are converted once, in Coef)
template <class P, class T>
__device__ __forceinline__ Dual<P, T> operator*(Dual<P, T> a, P c) { return {a.v * c, a.d * T(c)}; }
template <class P, class T>
__device__ __forceinline__ Dual<P, T> operator*(P c, Dual<P, T> a) { return {a.v * c, a.d * T(c)}; }
template <class P, class T>
__device__ __forceinline__ Dual<P, T> operator+(Dual<P, T> a, P c) { return {a.v + c, a.d}; }
template <class P, class T>
__device__ __forceinline__ Dual<P, T> operator-(Dual<P, T> a, P c) { return {a.v - c, a.d}; }
template <class P, class T>
__device__ __forceinline__ Dual<P, T> inv(Dual<P, T> a) {
  P r = P(1) / a.v;
  return {r, -a.d * T(r * r)};
}
template <class P, class T>
__device__ __forceinline__ Dual<P, T> dsqrt(Dual<P, T> a) {
  P s = sqrt(a.v);
  return {s, a.d * T(P(0.5) / s)};
}

// material coefficients in the primal type (PhysParams holds doubles)
template <class P>
struct Coef {
  P kb, kg, zv, pn, adb_zv, am;
  __device__ __forceinline__ explicit Coef(const PhysParams& pp)
      : kb(P(pp.kb)), kg(P(pp.kg)), zv(P(pp.zv)), pn(P(pp.pn)), adb_zv(P(pp.adb / pp.zv)), am(P(pp.am)) {}
};

// Row accumulators.  A residual row at one Gauss point is linear in node b's
// basis values (N, N_,α, N_,αβ): lin() receives the row's coefficient duals
// c[s] and the basis values phi[s] of node b and adds sum_s phi[s] c[s].  The
// tangent pass adds the tangent part to column q of the element block (and, in
// the plain form, the primal of row q alone); the residual pass adds the
// primal of every row into a per-task array.
template <class P, class T, bool WANT_R>
struct AccTan {
  T* Ks;
  int ldk, q;
  P rsum;
  __device__ __forceinline__ void operator()(int row, Dual<P, T> val) {
    if (WANT_R && row == q) rsum += val.v;
    Ks[row * ldk + q] += val.d;
  }
  template <int NS>
  __device__ __forceinline__ void lin(int row, const Dual<P, T> (&c)[NS], const P (&phi)[NS]) {
    T d = T(phi[0]) * c[0].d;
#pragma unroll
    for (int s = 1; s < NS; ++s) d += T(phi[s]) * c[s].d;
    Ks[row * ldk + q] += d;
    if (WANT_R && row == q) {
      P v = phi[0] * c[0].v;
#pragma unroll
      for (int s = 1; s < NS; ++s) v += phi[s] * c[s].v;
      rsum += v;
    }
  }
};
struct AccRes {
  double* R;  // [row]
  template <int NS>
  __device__ __forceinline__ void lin(int row, const Dual<double, Nil> (&c)[NS], const double (&phi)[NS]) {
    double v = phi[0] * c[0].v;
#pragma unroll
    for (int s = 1; s < NS; ++s) v += phi[s] * c[s].v;
    R[row] += v;
  }
};
// boundary rows are velocity rows only: R[b*3 + i] for row vd[i] + ndf*b
struct AccResV {
  double* R;
  int ndf, vd0, vd1;
  __device__ __forceinline__ void operator()(int row, Dual<double, Nil> val) {
    const int b = row / ndf, d = row - b * ndf;
    R[b * 3 + (d == vd0 ? 0 : d == vd1 ? 1 : 2)] += val.v;
  }
};

// Primal values of one (element, area Gauss point) that every tangent
// direction shares, formed once: a_α and x_,αβ (sums over the 9 nodes of the
// mesh positions) and the interpolants of the 8 unknowns -- u N for u = 0..7,
// u N_,1 and u N_,2 for u = 0..5 (zero for an unknown the motion lacks).
constexpr int kPreA = 0, kPreX = 6, kPreN = 15, kPreD0 = 23, kPreD1 = 29, kPre = 35;
template <class P>
__device__ __forceinline__ P gp_pre_value(int j, const PhysParams& pp, const P* X, const P* C, const P* f) {
  const P* wts;
  const P* src;
  int stride;
  if (j < kPreX) {  // a[i][α] = sum_b N_,α[b] x[b][i]
    wts = f + 10 + 9 * (j & 1);
    src = X + (j >> 1);
    stride = 3;
  } else if (j < kPreN) {  // xab[i][k] = sum_b N_,k[b] x[b][i]
    const int i = (j - kPreX) / 3, k = j - kPreX - 3 * i;
    wts = f + 28 + 9 * k;
    src = X + i;
    stride = 3;
  } else {
    const int u = j < kPreD0 ? j - kPreN : j < kPreD1 ? j - kPreD0 : j - kPreD1;
    const int d = pp.dof_of[u];
    if (d < 0) return P(0);  // get_dof_cps zero-fills absent unknowns (GeoDynStress.jl:190-205)
    wts = f + (j < kPreD0 ? 1 : j < kPreD1 ? 10 : 19);
    src = C + d;
    stride = 8;
  }
  P s = 0;
#pragma unroll
  for (int b = 0; b < 9; ++b) s += wts[b] * src[b * stride];
  return s;
}

// ---- element kernel --------------------------------------------------------------
// motion is a template parameter; the dof maps are runtime (PhysParams).
enum { STATIC_ = 1, EUL_ = 2, LAG_ = 3, ALEV_ = 4, ALEVB_ = 5 };

// One area Gauss point: calc_elem_dof_residuals' GP body (FiniteElement.jl:284-321)
// with geo_dyn_stress (GeoDynStress.jl:91-178) inlined, on dual numbers.
template <class P, class T, int MOTION, class Acc>
__device__ __forceinline__ void area_gp(const PhysParams& pp, const Coef<P>& cf, const P* pre, const P* f, int as,
                                        int js, int us, P dt, Acc& acc) {
  const int ndf = pp.ndf;
  const P w = f[0];
  const P* N = f + 1;
  const P* dN0 = f + 10;
  const P* dN1 = f + 19;
  const P* dd[3] = {f + 28, f + 37, f + 46};
  const T sN = T(N[as]), sd0 = T(dN0[as]), sd1 = T(dN1[as]);

  // geometry: a_α, x_,αβ (x itself is not used by the residual); the seed of a
  // mesh-motion direction is ∂xms[as, js] = Δt
  Dual<P, T> a[3][2], xab[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    T g = (i == js) ? T(dt) : T(0);
    a[i][0] = mk<P, T>(pre[kPreA + 2 * i], g * sd0);
    a[i][1] = mk<P, T>(pre[kPreA + 2 * i + 1], g * sd1);
#pragma unroll
    for (int k = 0; k < 3; ++k) xab[i][k] = mk<P, T>(pre[kPreX + 3 * i + k], g * T(dd[k][as]));
  }
  Dual<P, T> a11 = a[0][0] * a[0][0] + a[1][0] * a[1][0] + a[2][0] * a[2][0];
  Dual<P, T> a12 = a[0][0] * a[0][1] + a[1][0] * a[1][1] + a[2][0] * a[2][1];
  Dual<P, T> a22 = a[0][1] * a[0][1] + a[1][1] * a[1][1] + a[2][1] * a[2][1];
  Dual<P, T> det = a11 * a22 - a12 * a12;
  Dual<P, T> idet = inv(det);
  Dual<P, T> i11 = a22 * idet, i12 = -(a12 * idet), i22 = a11 * idet;  // a^αβ
  Dual<P, T> aup[3][2];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    aup[i][0] = a[i][0] * i11 + a[i][1] * i12;
    aup[i][1] = a[i][0] * i12 + a[i][1] * i22;
  }
  Dual<P, T> J = dsqrt(det);
  Dual<P, T> iJ = inv(J);
  Dual<P, T> n[3];
  n[0] = (a[1][0] * a[2][1] - a[2][0] * a[1][1]) * iJ;
  n[1] = (a[2][0] * a[0][1] - a[0][0] * a[2][1]) * iJ;
  n[2] = (a[0][0] * a[1][1] - a[1][0] * a[0][1]) * iJ;
  Dual<P, T> Gam[3][2], bf[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    Gam[k][0] = xab[0][k] * aup[0][0] + xab[1][k] * aup[1][0] + xab[2][k] * aup[2][0];
    Gam[k][1] = xab[0][k] * aup[0][1] + xab[1][k] * aup[1][1] + xab[2][k] * aup[2][1];
    bf[k] = xab[0][k] * n[0] + xab[1][k] * n[1] + xab[2][k] * n[2];
  }
  // b^αβ = a⁻¹ b a⁻¹ (symmetric)
  Dual<P, T> t11 = i11 * bf[0] + i12 * bf[2], t12 = i11 * bf[2] + i12 * bf[1];
  Dual<P, T> t21 = i12 * bf[0] + i22 * bf[2], t22 = i12 * bf[2] + i22 * bf[1];
  Dual<P, T> bu11 = t11 * i11 + t12 * i12, bu12 = t11 * i12 + t12 * i22, bu22 = t21 * i12 + t22 * i22;
  Dual<P, T> H = (i11 * bf[0] + i12 * bf[2] + i12 * bf[2] + i22 * bf[1]) * P(0.5);
  Dual<P, T> K = (bf[0] * bf[1] - bf[2] * bf[2]) * idet;

  // dynamics: interpolants of unknown u (pre-formed), seeded when u is this
  // direction's unknown; kind 0: N, 1: N_,1, 2: N_,2
  auto interp = [&](int u, int kind, T swt) -> Dual<P, T> {
    const P s = pre[(kind == 0 ? kPreN : kind == 1 ? kPreD0 : kPreD1) + u];
    return mk<P, T>(s, (u == us) ? swt : T(0));
  };
  Dual<P, T> dv[3][2];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    dv[i][0] = interp(i, 1, sd0);
    dv[i][1] = interp(i, 2, sd1);
  }
  Dual<P, T> lam = interp(6, 0, sN);

  // π^αβ = ζv sym(a^αᵀ v_,α a⁻¹)  (GeoDynStress.jl:148-149)
  auto visc = [&](Dual<P, T> g[3][2], Dual<P, T>& p11, Dual<P, T>& p12, Dual<P, T>& p22) {
    Dual<P, T> u[3][2];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      u[i][0] = g[i][0] * i11 + g[i][1] * i12;
      u[i][1] = g[i][0] * i12 + g[i][1] * i22;
    }
    Dual<P, T> P11 = aup[0][0] * u[0][0] + aup[1][0] * u[1][0] + aup[2][0] * u[2][0];
    Dual<P, T> P12 = aup[0][0] * u[0][1] + aup[1][0] * u[1][1] + aup[2][0] * u[2][1];
    Dual<P, T> P21 = aup[0][1] * u[0][0] + aup[1][1] * u[1][0] + aup[2][1] * u[2][0];
    Dual<P, T> P22 = aup[0][1] * u[0][1] + aup[1][1] * u[1][1] + aup[2][1] * u[2][1];
    p11 = (P11 + P11) * cf.zv;
    p12 = (P12 + P21) * cf.zv;
    p22 = (P22 + P22) * cf.zv;
  };
  Dual<P, T> p11, p12, p22;
  visc(dv, p11, p12, p22);
  // tr(a^αᵀ v_,α) for rλ (FiniteElement.jl:298)
  Dual<P, T> tr = aup[0][0] * dv[0][0] + aup[1][0] * dv[1][0] + aup[2][0] * dv[2][0] + aup[0][1] * dv[0][1] +
               aup[1][1] * dv[1][1] + aup[2][1] * dv[2][1];
  // σ, M in Voigt form (GeoDynStress.jl:150-154)
  Dual<P, T> cb = cf.kb * (H * H) - cf.kg * K;
  Dual<P, T> cs = cb + lam;
  Dual<P, T> hb = H * (P(2) * cf.kb);
  Dual<P, T> sg0 = i11 * cs - bu11 * hb + p11;
  Dual<P, T> sg1 = i22 * cs - bu22 * hb + p22;
  Dual<P, T> sg2 = (i12 * cs - bu12 * hb + p12) * P(2);
  Dual<P, T> hm = H * (cf.kb + P(2) * cf.kg);
  Dual<P, T> M0 = i11 * hm - bu11 * cf.kg;
  Dual<P, T> M1 = i22 * hm - bu22 * cf.kg;
  Dual<P, T> M2 = (i12 * hm - bu12 * cf.kg) * P(2);
  Dual<P, T> JW = J * w;

  // mesh-motion quantities
  Dual<P, T> sm0, sm1, sm2, pm_, vmv[3], nd_;
  if (MOTION == ALEV_ || MOTION == ALEVB_) {
    Dual<P, T> dvm[3][2];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      dvm[i][0] = interp(3 + i, 1, sd0);
      dvm[i][1] = interp(3 + i, 2, sd1);
    }
    Dual<P, T> m11, m12, m22;
    visc(dvm, m11, m12, m22);
    sm0 = i11 * cb - bu11 * hb + m11;  // GeoDynStress.jl:156-159
    sm1 = i22 * cb - bu22 * hb + m22;
    sm2 = (i12 * cb - bu12 * hb + m12) * P(2);
    pm_ = interp(7, 0, sN);
    Dual<P, T> nd = cst<P, T>(P(0));
#pragma unroll
    for (int i = 0; i < 3; ++i) nd = nd + n[i] * (interp(3 + i, 0, sN) - interp(i, 0, sN));
    nd_ = nd;
  }
  Dual<P, T> nv;
  if (MOTION == EUL_) {
    Dual<P, T> v[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      v[i] = interp(i, 0, sN);
      vmv[i] = interp(3 + i, 0, sN);
    }
    nv = n[0] * v[0] + n[1] * v[1] + n[2] * v[2];
  }

  // Residual rows (node-major packing of calc_elem_residual,
  // FiniteElement.jl:225-239).  Row (node b, dof) of this point is linear in
  // node b's basis values -- with nn_k(b) = N_,k[b] - Γ^α_k N_,α[b],
  //   r_v,i = a_i,1 c1 + a_i,2 c2 + n_i (nn·M) J w - n_i pn N J w,
  //   c1 = (σ11 N_,1 + σ12 N_,2) J w, c2 = (σ22 N_,2 + σ12 N_,1) J w,
  // and likewise for the mesh, pressure and λ rows -- so each row's
  // coefficients of (N_,1, N_,2, N_,11, N_,22, N_,12, N) are formed once per
  // point and the node loop is a 6-term sum per row.
  const int vd[3] = {pp.dof_of[0], pp.dof_of[1], pp.dof_of[2]};
  const int mo[3] = {pp.dof_of[3], pp.dof_of[4], pp.dof_of[5]};
  const int lo = pp.dof_of[6], po = pp.dof_of[7];
  auto phi6 = [&](int b, P (&ph)[6]) {
    ph[0] = dN0[b];
    ph[1] = dN1[b];
    ph[2] = dd[0][b];
    ph[3] = dd[1][b];
    ph[4] = dd[2][b];
    ph[5] = N[b];
  };
  const Dual<P, T> JWh = JW * P(0.5);
  const Dual<P, T> MJ[3] = {M0 * JW, M1 * JW, M2 * JW};  // bending: nn·M J w = sum_k N_,k MJ_k - N_,α GM_α
  const Dual<P, T> GM0 = Gam[0][0] * MJ[0] + Gam[1][0] * MJ[1] + Gam[2][0] * MJ[2];
  const Dual<P, T> GM1 = Gam[0][1] * MJ[0] + Gam[1][1] * MJ[1] + Gam[2][1] * MJ[2];
  {
    const Dual<P, T> S0 = sg0 * JW, S1 = sg1 * JW, S2 = sg2 * JWh, PN = JW * cf.pn;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      if (vd[i] < 0) continue;
      const Dual<P, T> c[6] = {a[i][0] * S0 + a[i][1] * S2 - n[i] * GM0, a[i][0] * S2 + a[i][1] * S1 - n[i] * GM1,
                               n[i] * MJ[0], n[i] * MJ[1], n[i] * MJ[2], -(n[i] * PN)};
#pragma unroll 1
      for (int b = 0; b < 9; ++b) {
        P ph[6];
        phi6(b, ph);
        acc.lin(vd[i] + ndf * b, c, ph);
      }
    }
  }
  if (MOTION == ALEV_ || MOTION == ALEVB_) {
    const Dual<P, T> E0 = sm0 * JW, E1 = sm1 * JW, E2 = sm2 * JWh, PJ = pm_ * JW;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      if (MOTION == ALEVB_) {  // the mesh rows carry the bending term too
        const Dual<P, T> c[6] = {a[i][0] * E0 + a[i][1] * E2 - n[i] * GM0, a[i][0] * E2 + a[i][1] * E1 - n[i] * GM1,
                                 n[i] * MJ[0], n[i] * MJ[1], n[i] * MJ[2], -(n[i] * PJ)};
#pragma unroll 1
        for (int b = 0; b < 9; ++b) {
          P ph[6];
          phi6(b, ph);
          acc.lin(mo[i] + ndf * b, c, ph);
        }
      } else {
        const Dual<P, T> c[3] = {a[i][0] * E0 + a[i][1] * E2, a[i][0] * E2 + a[i][1] * E1, -(n[i] * PJ)};
#pragma unroll 1
        for (int b = 0; b < 9; ++b) {
          const P ph[3] = {dN0[b], dN1[b], N[b]};
          acc.lin(mo[i] + ndf * b, c, ph);
        }
      }
    }
    const Dual<P, T> c[1] = {-(JW * nd_) - pm_ * (w * cf.adb_zv)};
#pragma unroll 1
    for (int b = 0; b < 9; ++b) {
      const P ph[1] = {N[b]};
      acc.lin(po + ndf * b, c, ph);
    }
  }
  if (MOTION == EUL_) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const Dual<P, T> c[1] = {(vmv[i] - n[i] * nv) * JW * cf.am};
#pragma unroll 1
      for (int b = 0; b < 9; ++b) {
        const P ph[1] = {N[b]};
        acc.lin(mo[i] + ndf * b, c, ph);
      }
    }
  }
  {
    const Dual<P, T> c[1] = {(J * tr - cf.adb_zv * lam) * w};
#pragma unroll 1
    for (int b = 0; b < 9; ++b) {
      const P ph[1] = {N[b]};
      acc.lin(lo + ndf * b, c, ph);
    }
  }
}

// One boundary Gauss point of calc_bdry_element_residual (FiniteElement.jl:363-384).
template <class P, class T, class Acc>
__device__ __forceinline__ void bdry_gp(const PhysParams& pp, const P* X, const P* f, int bdry, int ntype, P nval,
                                        P mscale, int as, int js, P dt, Acc& acc) {
  const int ndf = pp.ndf;
  const P w = f[0];
  const P* N = f + 1;
  const P* dN0 = f + 10;
  const P* dN1 = f + 19;
  const T sd0 = T(dN0[as]), sd1 = T(dN1[as]);
  Dual<P, T> a[3][2];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    P s0 = 0, s1 = 0;
#pragma unroll
    for (int b = 0; b < 9; ++b) {
      s0 += dN0[b] * X[b * 3 + i];
      s1 += dN1[b] * X[b * 3 + i];
    }
    T g = (i == js) ? T(dt) : T(0);
    a[i][0] = mk<P, T>(s0, g * sd0);
    a[i][1] = mk<P, T>(s1, g * sd1);
  }
  Dual<P, T> a11 = a[0][0] * a[0][0] + a[1][0] * a[1][0] + a[2][0] * a[2][0];
  Dual<P, T> a12 = a[0][0] * a[0][1] + a[1][0] * a[1][1] + a[2][0] * a[2][1];
  Dual<P, T> a22 = a[0][1] * a[0][1] + a[1][1] * a[1][1] + a[2][1] * a[2][1];
  Dual<P, T> det = a11 * a22 - a12 * a12;
  Dual<P, T> idet = inv(det);
  Dual<P, T> i11 = a22 * idet, i12 = -(a12 * idet), i22 = a11 * idet;
  Dual<P, T> aup[3][2];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    aup[i][0] = a[i][0] * i11 + a[i][1] * i12;
    aup[i][1] = a[i][0] * i12 + a[i][1] * i22;
  }
  Dual<P, T> iJ = inv(dsqrt(det));
  Dual<P, T> n[3];
  n[0] = (a[1][0] * a[2][1] - a[2][0] * a[1][1]) * iJ;
  n[1] = (a[2][0] * a[0][1] - a[0][0] * a[2][1]) * iJ;
  n[2] = (a[0][0] * a[1][1] - a[1][0] * a[0][1]) * iJ;
  // τ = ±a_α / |a_α|; the norm is a primal constant (conjugating dot, FiniteElement.jl:448)
  int col = (bdry == 0 || bdry == 2) ? 0 : 1;
  const float sgn = (bdry == 0 || bdry == 1) ? 1.0f : -1.0f;
  P nrm = sqrt(a[0][col].v * a[0][col].v + a[1][col].v * a[1][col].v + a[2][col].v * a[2][col].v);
  P sc = P(sgn) / nrm;
  Dual<P, T> tau[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) tau[i] = a[i][col] * sc;
  Dual<P, T> nu[3];
  nu[0] = tau[1] * n[2] - tau[2] * n[1];
  nu[1] = tau[2] * n[0] - tau[0] * n[2];
  nu[2] = tau[0] * n[1] - tau[1] * n[0];
  Dual<P, T> t0 = aup[0][0] * tau[0] + aup[1][0] * tau[1] + aup[2][0] * tau[2];
  Dual<P, T> t1 = aup[0][1] * tau[0] + aup[1][1] * tau[1] + aup[2][1] * tau[2];
  Dual<P, T> JG = inv(dsqrt(t0 * t0 + t1 * t1));
  const int vd[3] = {pp.dof_of[0], pp.dof_of[1], pp.dof_of[2]};
  if (ntype == MAFEM_STRETCH || ntype == MAFEM_SHEAR) {
    Dual<P, T> fv[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) fv[i] = (ntype == MAFEM_STRETCH ? nu[i] : tau[i]) * (nval * w);
    Dual<P, T> fj[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) fj[i] = fv[i] * JG;
#pragma unroll 1
    for (int b = 0; b < 9; ++b)
#pragma unroll
      for (int i = 0; i < 3; ++i)
        if (vd[i] >= 0) acc(vd[i] + ndf * b, -(fj[i] * N[b]));
  } else {  // MOMENT (F_BEND only; other types are rejected on the host)
    Dual<P, T> nu0 = aup[0][0] * nu[0] + aup[1][0] * nu[1] + aup[2][0] * nu[2];
    Dual<P, T> nu1 = aup[0][1] * nu[0] + aup[1][1] * nu[1] + aup[2][1] * nu[2];
    Dual<P, T> s = JG * (nval * mscale * w);
#pragma unroll 1
    for (int b = 0; b < 9; ++b) {
      Dual<P, T> dn = (nu0 * dN0[b] + nu1 * dN1[b]) * s;
#pragma unroll
      for (int i = 0; i < 3; ++i)
        if (vd[i] >= 0) acc(vd[i] + ndf * b, -(n[i] * dn));
    }
  }
}

// Plain form (P = T = double, WANT_R): primal and tangent of every element dof
// in one pass.  FP32 form (P = T = float, !WANT_R): the tangent alone.
// elist (optional): evaluate only elements elist[0 .. nlist) and write their
// rows to r_el[k][q]; area_only: the area Gauss points alone
// (calc_elem_dof_residuals without the Dohrmann-Bochev projection or boundary
// terms, as PullForce.jl uses it); K_el may be null (no tangent written).
// The element loop of one CTA (CTA number blk of the patch), shared by the
// single-patch kernel and the batched kernel, which reads Pt / pp from a job
// table into shared memory.
template <class P, class T, bool WANT_R, int MOTION, int EPB>
__device__ __forceinline__ void elem_body(const DevPatch& Pt, const PhysParams& pp, double time, double dt,
                                          double* __restrict__ r_el, T* __restrict__ K_el,
                                          const int* __restrict__ elist, int nlist, int area_only, int blk,
                                          unsigned char* smem_raw) {
  const int nq = pp.nq, ndf = pp.ndf;
  const int ldk = nq + 1;
  const int slot = threadIdx.x / nq;
  const int q = threadIdx.x - slot * nq;
  const int kk = blk * EPB + slot;  // element (or list) index of this slot
  const int e = elist ? (kk < nlist ? elist[kk] : 0) : kk;
  // per-slot shared memory: X[27], C[72], GP tables [9][kTab], the points'
  // shared primal values [9][kPre] in P; then the blocks
  const size_t per_slot = 27 + 72 + 9 * kTab + 9 * kPre;
  P* base = reinterpret_cast<P*>(smem_raw);
  P* X = base + slot * per_slot;
  P* C = X + 27;
  P* tab = C + 72;
  P* pre = tab + 9 * kTab;
  T* Ks = reinterpret_cast<T*>(base + EPB * per_slot) + (size_t)slot * nq * ldk;
  const bool live = (slot < EPB) && (elist ? kk < nlist : e < Pt.numel);

  if (live) {
    const int u = Pt.uel[e];
    for (int k = q; k < 9 * kTab; k += nq) tab[k] = P(Pt.tab[(size_t)u * 9 * kTab + k]);
    for (int k = q; k < 27; k += nq) {
      int b = k / 3, i = k - 3 * (k / 3);
      X[k] = P(Pt.xms[(size_t)i * Pt.numnp + Pt.ix[e * 9 + b]]);
    }
    for (int k = q; k < 72; k += nq) {
      int b = k / 8, d = k - 8 * (k / 8);
      C[k] = d < ndf ? P(Pt.cps[(size_t)d * Pt.numnp + Pt.ix[e * 9 + b]]) : P(0);
    }
    for (int k = q; k < nq * ldk; k += nq) Ks[k] = T(0.0);
  }
  __syncthreads();
  if (live)
    for (int k = q; k < 9 * kPre; k += nq) {
      const int gp = k / kPre;
      pre[k] = gp_pre_value<P>(k - gp * kPre, pp, X, C, tab + gp * kTab);
    }
  __syncthreads();
  if (live) {
    const int as = q / ndf, ds = q - as * ndf;
    const int us = pp.unk_of[ds];
    const int js = (pp.mmo[0] == ds) ? 0 : (pp.mmo[1] == ds) ? 1 : (pp.mmo[2] == ds) ? 2 : -1;
    const Coef<P> cf(pp);
    const P pdt = P(dt);
    AccTan<P, T, WANT_R> acc{Ks, ldk, q, P(0)};

#pragma unroll 1
    for (int gp = 0; gp < 9; ++gp)
      area_gp<P, T, MOTION>(pp, cf, pre + gp * kPre, tab + gp * kTab, as, js, us, pdt, acc);

    // Dohrmann-Bochev projection (FiniteElement.jl:323-327): rλ += Gᵀ H⁻¹ G λ αdb/ζv,
    // and for ALEV/ALEVB rp += Gᵀ H⁻¹ G p αdb/ζv.  Linear in λ / p.
    if (!area_only) {
      const double* T81 = Pt.db + (size_t)Pt.uel[e] * 81;
      const double s = pp.adb / pp.zv;
      const int lo = pp.dof_of[6], po = pp.dof_of[7];
      const bool alep = (MOTION == ALEV_ || MOTION == ALEVB_);
      for (int b = 0; b < 9; ++b) {
        const int rowl = lo + ndf * b;
        if (us == 6) Ks[rowl * ldk + q] += T(T81[b * 9 + as] * s);
        if (alep && us == 7) Ks[(po + ndf * b) * ldk + q] += T(T81[b * 9 + as] * s);
        if (WANT_R) {
          double sl = 0, sp = 0;
          for (int c = 0; c < 9; ++c) {
            sl += T81[b * 9 + c] * C[c * 8 + lo];
            if (alep) sp += T81[b * 9 + c] * C[c * 8 + po];
          }
          if (rowl == q) acc.rsum += sl * s;
          if (alep && po + ndf * b == q) acc.rsum += sp * s;
        }
      }
    }

    // Neumann boundary terms of this element (calc_r_K's boundary loop,
    // FiniteElement.jl:150-197): same LM, so they add into the same block.
    for (int k = 0; k < (area_only ? 0 : pp.n_neu); ++k) {
      const int b = pp.neu_bdry[k];
      const int row = Pt.bref[e * 4 + b];
      if (row < 0) continue;
      const P mscale = P(pp.neu_type[k] == MAFEM_MOMENT ? fmin(time / pp.bend_tm, 1.0) : 1.0);
      for (int g = 0; g < 3; ++g) {
        const double* src = Pt.btab + ((size_t)row * 3 + g) * kTab;
        if constexpr (sizeof(P) == sizeof(double)) {
          bdry_gp<P, T>(pp, X, src, b, pp.neu_type[k], P(pp.neu_val[k]), mscale, as, js, pdt, acc);
        } else {
          P fb[28];  // w, N, dN: the boundary term uses no second derivatives
          for (int t = 0; t < 28; ++t) fb[t] = P(src[t]);
          bdry_gp<P, T>(pp, X, fb, b, pp.neu_type[k], P(pp.neu_val[k]), mscale, as, js, pdt, acc);
        }
      }
    }
    if (WANT_R) r_el[(size_t)(elist ? kk : e) * nq + q] = acc.rsum;
  }
  __syncthreads();
  if (live && K_el) {
    // column-major element block K_el[e][col][row] (coalesced stores)
    T* dst = K_el + (size_t)e * nq * nq;
    for (int idx = q; idx < nq * nq; idx += nq) {
      int c = idx / nq, r = idx - c * nq;
      dst[idx] = Ks[r * ldk + c];
    }
  }
}

template <class P, class T, bool WANT_R, int MOTION, int EPB>
__global__ void elem_kernel(DevPatch Pt, PhysParams pp, double time, double dt, double* __restrict__ r_el,
                            T* __restrict__ K_el, const int* __restrict__ elist, int nlist, int area_only) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  elem_body<P, T, WANT_R, MOTION, EPB>(Pt, pp, time, dt, r_el, K_el, elist, nlist, area_only, blockIdx.x, smem_raw);
}

// FP64 residual of the FP32 form: primal only, one thread per (element, area
// Gauss point).  Phase 1: each task adds its point's contribution to every
// element row into its own shared array; phase 2: one thread per (element,
// row) sums them in Gauss-point order and adds the Dohrmann-Bochev term;
// phase 3: the Neumann points (task = element, bc, point; velocity rows only)
// likewise, summed in (bc, point) order -- the plain form's order.
constexpr int kResEPB = 16;  // elements per CTA: 144 threads
template <int MOTION>
__device__ __forceinline__ void resid_body(const DevPatch& Pt, const PhysParams& pp, double time, double dt,
                                           double* __restrict__ r_el, int blk, unsigned char* smem_raw) {
  const int nq = pp.nq, ndf = pp.ndf;
  double* X = reinterpret_cast<double*>(smem_raw);  // [kResEPB][27]
  double* C = X + kResEPB * 27;                       // [kResEPB][72]
  double* R = C + kResEPB * 72;                       // [kResEPB*9][nq], reused as [kResEPB*24][27]
  const int tid = threadIdx.x;
  const int e0 = blk * kResEPB;
  const int ne = min(kResEPB, Pt.numel - e0);
  for (int k = tid; k < ne * 27; k += blockDim.x) {
    const int el = k / 27, r = k - 27 * el, b = r / 3, i = r - 3 * b;
    X[k] = Pt.xms[(size_t)i * Pt.numnp + Pt.ix[(e0 + el) * 9 + b]];
  }
  for (int k = tid; k < ne * 72; k += blockDim.x) {
    const int el = k / 72, r = k - 72 * el, b = r / 8, d = r - 8 * b;
    C[k] = d < ndf ? Pt.cps[(size_t)d * Pt.numnp + Pt.ix[(e0 + el) * 9 + b]] : 0.0;
  }
  for (int k = tid; k < kResEPB * 9 * nq; k += blockDim.x) R[k] = 0.0;
  __syncthreads();
  const Coef<double> cf(pp);
  {
    const int el = tid / 9, gp = tid - 9 * el;
    if (el < ne) {
      const double* f = Pt.tab + ((size_t)Pt.uel[e0 + el] * 9 + gp) * kTab;
      double pre[kPre];
#pragma unroll
      for (int j = 0; j < kPre; ++j) pre[j] = gp_pre_value<double>(j, pp, X + el * 27, C + el * 72, f);
      AccRes acc{R + (size_t)tid * nq};
      area_gp<double, Nil, MOTION>(pp, cf, pre, f, 0, -1, -1, dt, acc);
    }
  }
  __syncthreads();
  // phase 2: rows (each thread keeps its sums for phase 3)
  constexpr int kMaxOwn = (kResEPB * 72 + kResEPB * 9 - 1) / (kResEPB * 9);  // 8
  double own[kMaxOwn];
  const double s = pp.adb / pp.zv;
  const int lo = pp.dof_of[6], po = pp.dof_of[7];
  const bool alep = (MOTION == ALEV_ || MOTION == ALEVB_);
#pragma unroll
  for (int j = 0; j < kMaxOwn; ++j) {
    const int pr = tid + j * kResEPB * 9;
    const int el = pr / nq, row = pr - el * nq;
    own[j] = 0.0;
    if (el < ne) {
      double r = 0.0;
      for (int gp = 0; gp < 9; ++gp) r += R[(size_t)(el * 9 + gp) * nq + row];
      const int b = row / ndf, d = row - b * ndf;
      if (d == lo || (alep && d == po)) {
        const double* T81 = Pt.db + (size_t)Pt.uel[e0 + el] * 81;
        double sv = 0;
        for (int c = 0; c < 9; ++c) sv += T81[b * 9 + c] * C[el * 72 + c * 8 + d];
        r += sv * s;
      }
      own[j] = r;
    }
  }
  // phase 3: Neumann points
  const int nn = pp.n_neu;
  if (nn > 0) {
    __syncthreads();
    const int ntask = ne * nn * 3;
    for (int k = tid; k < kResEPB * 24 * 27; k += blockDim.x) R[k] = 0.0;
    __syncthreads();
    for (int t = tid; t < ntask; t += blockDim.x) {
      const int el = t / (nn * 3), r = t - el * nn * 3, k = r / 3, g = r - 3 * k;
      const int bd = pp.neu_bdry[k];
      const int row = Pt.bref[(e0 + el) * 4 + bd];
      if (row < 0) continue;
      const double mscale = pp.neu_type[k] == MAFEM_MOMENT ? fmin(time / pp.bend_tm, 1.0) : 1.0;
      AccResV acc{R + (size_t)t * 27, ndf, pp.dof_of[0], pp.dof_of[1]};
      bdry_gp<double, Nil>(pp, X + el * 27, Pt.btab + ((size_t)row * 3 + g) * kTab, bd, pp.neu_type[k],
                           pp.neu_val[k], mscale, 0, -1, dt, acc);
    }
    __syncthreads();
    const int vd0 = pp.dof_of[0], vd1 = pp.dof_of[1], vd2 = pp.dof_of[2];
#pragma unroll
    for (int j = 0; j < kMaxOwn; ++j) {
      const int pr = tid + j * kResEPB * 9;
      const int el = pr / nq, row = pr - el * nq;
      if (el >= ne) continue;
      const int b = row / ndf, d = row - b * ndf;
      const int i = d == vd0 ? 0 : d == vd1 ? 1 : d == vd2 ? 2 : -1;
      if (i < 0) continue;
      for (int k = 0; k < nn; ++k) {
        if (Pt.bref[(e0 + el) * 4 + pp.neu_bdry[k]] < 0) continue;
        for (int g = 0; g < 3; ++g) own[j] += R[(size_t)((el * nn + k) * 3 + g) * 27 + b * 3 + i];
      }
    }
  }
#pragma unroll
  for (int j = 0; j < kMaxOwn; ++j) {
    const int pr = tid + j * kResEPB * 9;
    const int el = pr / nq, row = pr - el * nq;
    if (el < ne) r_el[(size_t)(e0 + el) * nq + row] = own[j];
  }
}

template <int MOTION>
__global__ void __launch_bounds__(kResEPB * 9) elem_resid_kernel(DevPatch Pt, PhysParams pp, double time, double dt,
                                                                double* __restrict__ r_el) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  resid_body<MOTION>(Pt, pp, time, dt, r_el, blockIdx.x, smem_raw);
}

// ---- batched element kernels of the FP32 form: every patch of a round in one launch per motion ----
// The CTA reads its patch's tables and parameters into shared memory, then runs
// the single-patch kernel's body on its CTA number within the patch.
// elements per CTA of the FP32 tangent kernel: 2 or 4, chosen per motion by
// the batch's autotuner (fewer elements per CTA, more CTAs per SM)
template <int MOTION>
__global__ void __launch_bounds__(kResEPB * 9) batch_resid_kernel(const AsmJob* __restrict__ jobs,
                                                                 const AsmItem* __restrict__ items,
                                                                 const int* __restrict__ off, int m) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_k;
  __shared__ __align__(16) DevPatch sP;
  __shared__ __align__(16) PhysParams spp;
  const int k = batch_item(off, m, &s_k);
  const AsmItem it = items[k];
  const AsmJob* J = jobs + it.job;
  batch_copy(&sP, &J->P, (int)sizeof(DevPatch));
  batch_copy(&spp, &J->pp, (int)sizeof(PhysParams));
  __syncthreads();
  resid_body<MOTION>(sP, spp, it.time, it.dt, J->r_el, off[0] + (int)blockIdx.x - off[k], smem_raw);
}
template <int MOTION, int EPB>
__global__ void batch_tan_kernel(const AsmJob* __restrict__ jobs, const AsmItem* __restrict__ items,
                                 const int* __restrict__ off, int m) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_k;
  __shared__ __align__(16) DevPatch sP;
  __shared__ __align__(16) PhysParams spp;
  const int k = batch_item(off, m, &s_k);
  const AsmItem it = items[k];
  const AsmJob* J = jobs + it.job;
  batch_copy(&sP, &J->P, (int)sizeof(DevPatch));
  batch_copy(&spp, &J->pp, (int)sizeof(PhysParams));
  __syncthreads();
  elem_body<float, float, false, MOTION, EPB>(sP, spp, it.time, it.dt, nullptr, J->K_el, nullptr, 0, 0,
                                                  off[0] + (int)blockIdx.x - off[k], smem_raw);
}

// ---- launchers -----------------------------------------------------------------------
template <class P, class T>
static size_t elem_smem(int nq, int epb) {
  return (size_t)epb * (27 + 72 + 9 * kTab + 9 * kPre) * sizeof(P) + (size_t)epb * nq * (nq + 1) * sizeof(T);
}
template <class T>
size_t elem_smem_bytes(int nq, int epb) {
  return elem_smem<T, T>(nq, epb);
}
static size_t resid_smem(int nq) {
  return (size_t)kResEPB * (27 + 72) * 8 + (size_t)std::max(kResEPB * 9 * nq, kResEPB * 24 * 27) * 8;
}

template <class P, class T, bool WANT_R, int MOTION, int EPB>
static cudaError_t launch_elem_t(const DevPatch& Pt, const PhysParams& pp, double time, double dt, double* r_el,
                                 T* K_el, cudaStream_t st, const int* elist, int nlist, int area_only) {
  // the cap is the size needed by the largest element (nq = 72), identical for every caller
  auto kern = elem_kernel<P, T, WANT_R, MOTION, EPB>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)elem_smem<P, T>(72, EPB));
  if (e != cudaSuccess) return e;
  const int blocks = ((elist ? nlist : Pt.numel) + EPB - 1) / EPB;
  kern<<<blocks, EPB * pp.nq, elem_smem<P, T>(pp.nq, EPB), st>>>(Pt, pp, time, dt, r_el, K_el, elist, nlist,
                                                                   area_only);
  return cudaGetLastError();
}

template <int MOTION>
static cudaError_t launch_resid_t(const DevPatch& Pt, const PhysParams& pp, double time, double dt, double* r_el,
                                  cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(elem_resid_kernel<MOTION>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)resid_smem(72));
  if (e != cudaSuccess) return e;
  elem_resid_kernel<MOTION><<<(Pt.numel + kResEPB - 1) / kResEPB, kResEPB * 9, resid_smem(pp.nq), st>>>(Pt, pp, time,
                                                                                                     dt, r_el);
  return cudaGetLastError();
}

template <>
cudaError_t launch_elem<double>(const DevPatch& Pt, const PhysParams& pp, double time, double dt, double* r_el,
                                double* K_el, cudaStream_t st, const int* elist, int nlist, int area_only) {
  switch (pp.motion) {
    case MAFEM_STATIC:
      return launch_elem_t<double, double, true, STATIC_, 4>(Pt, pp, time, dt, r_el, K_el, st, elist, nlist, area_only);
    case MAFEM_EUL:
      return launch_elem_t<double, double, true, EUL_, 2>(Pt, pp, time, dt, r_el, K_el, st, elist, nlist, area_only);
    case MAFEM_LAG:
      return launch_elem_t<double, double, true, LAG_, 4>(Pt, pp, time, dt, r_el, K_el, st, elist, nlist, area_only);
    case MAFEM_ALEV:
      return launch_elem_t<double, double, true, ALEV_, 2>(Pt, pp, time, dt, r_el, K_el, st, elist, nlist, area_only);
    default:
      return launch_elem_t<double, double, true, ALEVB_, 2>(Pt, pp, time, dt, r_el, K_el, st, elist, nlist,
                                                            area_only);
  }
}

// FP32 form: the FP64 residual kernel, then the FP32 tangent (whole patch only)
template <>
cudaError_t launch_elem<float>(const DevPatch& Pt, const PhysParams& pp, double time, double dt, double* r_el,
                               float* K_el, cudaStream_t st, const int* elist, int nlist, int area_only) {
  if (elist || nlist || area_only) return cudaErrorInvalidValue;
  cudaError_t e;
  switch (pp.motion) {
    case MAFEM_STATIC:
      e = launch_resid_t<STATIC_>(Pt, pp, time, dt, r_el, st);
      return e ? e : launch_elem_t<float, float, false, STATIC_, 4>(Pt, pp, time, dt, r_el, K_el, st, nullptr, 0, 0);
    case MAFEM_EUL:
      e = launch_resid_t<EUL_>(Pt, pp, time, dt, r_el, st);
      return e ? e : launch_elem_t<float, float, false, EUL_, 4>(Pt, pp, time, dt, r_el, K_el, st, nullptr, 0, 0);
    case MAFEM_LAG:
      e = launch_resid_t<LAG_>(Pt, pp, time, dt, r_el, st);
      return e ? e : launch_elem_t<float, float, false, LAG_, 4>(Pt, pp, time, dt, r_el, K_el, st, nullptr, 0, 0);
    case MAFEM_ALEV:
      e = launch_resid_t<ALEV_>(Pt, pp, time, dt, r_el, st);
      return e ? e : launch_elem_t<float, float, false, ALEV_, 4>(Pt, pp, time, dt, r_el, K_el, st, nullptr, 0, 0);
    default:
      e = launch_resid_t<ALEVB_>(Pt, pp, time, dt, r_el, st);
      return e ? e : launch_elem_t<float, float, false, ALEVB_, 4>(Pt, pp, time, dt, r_el, K_el, st, nullptr, 0, 0);
  }
}

int batch_resid_ctas(int numel) { return (numel + kResEPB - 1) / kResEPB; }
int batch_tan_ctas(int numel, int epb) { return (numel + epb - 1) / epb; }

template <int MOTION>
static cudaError_t batch_setup_t() {
  cudaError_t e = cudaFuncSetAttribute(batch_resid_kernel<MOTION>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)resid_smem(72));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(batch_tan_kernel<MOTION, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)elem_smem<float, float>(72, 2));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(batch_tan_kernel<MOTION, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)elem_smem<float, float>(72, 4));
  return e;
}
cudaError_t batch_asm_setup() {
  cudaError_t e = batch_setup_t<STATIC_>();
  if (e == cudaSuccess) e = batch_setup_t<EUL_>();
  if (e == cudaSuccess) e = batch_setup_t<LAG_>();
  if (e == cudaSuccess) e = batch_setup_t<ALEV_>();
  if (e == cudaSuccess) e = batch_setup_t<ALEVB_>();
  return e;
}

cudaError_t launch_batch_resid(int motion, const AsmJob* jobs, const AsmItem* items, const int* off, int m, int ctas,
                               int nq, cudaStream_t st) {
  if (ctas <= 0) return cudaSuccess;
  const size_t sm = resid_smem(nq);
  switch (motion) {
    case MAFEM_STATIC: batch_resid_kernel<STATIC_><<<ctas, kResEPB * 9, sm, st>>>(jobs, items, off, m); break;
    case MAFEM_EUL: batch_resid_kernel<EUL_><<<ctas, kResEPB * 9, sm, st>>>(jobs, items, off, m); break;
    case MAFEM_LAG: batch_resid_kernel<LAG_><<<ctas, kResEPB * 9, sm, st>>>(jobs, items, off, m); break;
    case MAFEM_ALEV: batch_resid_kernel<ALEV_><<<ctas, kResEPB * 9, sm, st>>>(jobs, items, off, m); break;
    default: batch_resid_kernel<ALEVB_><<<ctas, kResEPB * 9, sm, st>>>(jobs, items, off, m); break;
  }
  return cudaGetLastError();
}
template <int EPB>
static cudaError_t launch_batch_tan_t(int motion, const AsmJob* jobs, const AsmItem* items, const int* off, int m,
                                      int ctas, int nq, cudaStream_t st) {
  const size_t sm = elem_smem<float, float>(nq, EPB);
  const int thr = EPB * nq;
  switch (motion) {
    case MAFEM_STATIC: batch_tan_kernel<STATIC_, EPB><<<ctas, thr, sm, st>>>(jobs, items, off, m); break;
    case MAFEM_EUL: batch_tan_kernel<EUL_, EPB><<<ctas, thr, sm, st>>>(jobs, items, off, m); break;
    case MAFEM_LAG: batch_tan_kernel<LAG_, EPB><<<ctas, thr, sm, st>>>(jobs, items, off, m); break;
    case MAFEM_ALEV: batch_tan_kernel<ALEV_, EPB><<<ctas, thr, sm, st>>>(jobs, items, off, m); break;
    default: batch_tan_kernel<ALEVB_, EPB><<<ctas, thr, sm, st>>>(jobs, items, off, m); break;
  }
  return cudaGetLastError();
}
cudaError_t launch_batch_tan(int motion, int epb, const AsmJob* jobs, const AsmItem* items, const int* off, int m,
                             int ctas, int nq, cudaStream_t st) {
  if (ctas <= 0) return cudaSuccess;
  if (epb == 2) return launch_batch_tan_t<2>(motion, jobs, items, off, m, ctas, nq, st);
  if (epb == 4) return launch_batch_tan_t<4>(motion, jobs, items, off, m, ctas, nq, st);
  return cudaErrorInvalidValue;
}

template size_t elem_smem_bytes<double>(int, int);
template size_t elem_smem_bytes<float>(int, int);

}  // namespace mafem
