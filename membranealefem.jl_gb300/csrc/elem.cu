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
// Layout: elements are independent, so one CTA processes EPB elements with
// nq = 9*ndf threads each; the element's tangent columns accumulate in shared
// memory ([row][q], conflict-free) and are written once, column-major, to a
// staging buffer K_el[e][q][row].  A second kernel gathers, for every band
// entry, the <= 4 element contributions that land on it (no atomics: each
// output is written by exactly one thread), zero-filling the rest of the band.

#include <cuda_runtime.h>

#include <cstdint>

#include "mafem_internal.h"

namespace mafem {

// ---- dual numbers ------------------------------------------------------------
template <class T>
struct Dual {
  double v;
  T d;
};
template <class T>
__device__ __forceinline__ Dual<T> mk(double v, T d) { return Dual<T>{v, d}; }
template <class T>
__device__ __forceinline__ Dual<T> cst(double v) { return Dual<T>{v, T(0)}; }
template <class T>
__device__ __forceinline__ Dual<T> operator+(Dual<T> a, Dual<T> b) { return {a.v + b.v, a.d + b.d}; }
template <class T>
__device__ __forceinline__ Dual<T> operator-(Dual<T> a, Dual<T> b) { return {a.v - b.v, a.d - b.d}; }
template <class T>
__device__ __forceinline__ Dual<T> operator-(Dual<T> a) { return {-a.v, -a.d}; }
template <class T>
__device__ __forceinline__ Dual<T> operator*(Dual<T> a, Dual<T> b) {
  return {a.v * b.v, a.d * T(b.v) + T(a.v) * b.d};
}
template <class T>
__device__ __forceinline__ Dual<T> operator*(Dual<T> a, double c) { return {a.v * c, a.d * T(c)}; }
template <class T>
__device__ __forceinline__ Dual<T> operator*(double c, Dual<T> a) { return {a.v * c, a.d * T(c)}; }
template <class T>
__device__ __forceinline__ Dual<T> operator+(Dual<T> a, double c) { return {a.v + c, a.d}; }
template <class T>
__device__ __forceinline__ Dual<T> operator-(Dual<T> a, double c) { return {a.v - c, a.d}; }
template <class T>
__device__ __forceinline__ Dual<T> inv(Dual<T> a) {
  double r = 1.0 / a.v;
  return {r, -a.d * T(r * r)};
}
template <class T>
__device__ __forceinline__ Dual<T> dsqrt(Dual<T> a) {
  double s = sqrt(a.v);
  return {s, a.d * T(0.5 / s)};
}

// ---- element kernel --------------------------------------------------------------
// motion is a template parameter; the dof maps are runtime (PhysParams).
enum { STATIC_ = 1, EUL_ = 2, LAG_ = 3, ALEV_ = 4, ALEVB_ = 5 };

template <class T>
__device__ __forceinline__ void acc_row(int row, int q, Dual<T> val, double& rsum, T* Ks, int ldk) {
  if (row == q) rsum += val.v;
  Ks[row * ldk + q] += val.d;
}

// One area Gauss point: calc_elem_dof_residuals' GP body (FiniteElement.jl:284-321)
// with geo_dyn_stress (GeoDynStress.jl:91-178) inlined, on dual numbers.
template <class T, int MOTION>
__device__ __forceinline__ void area_gp(const PhysParams& pp, const double* X, const double* C, const double* f,
                                        int q, int as, int js, int us, double dt, double& rsum, T* Ks, int ldk) {
  const int ndf = pp.ndf;
  const double w = f[0];
  const double* N = f + 1;
  const double* dN0 = f + 10;
  const double* dN1 = f + 19;
  const double* dd[3] = {f + 28, f + 37, f + 46};
  const T sN = T(N[as]), sd0 = T(dN0[as]), sd1 = T(dN1[as]);

  // geometry: a_α, x_,αβ (x itself is not used by the residual)
  Dual<T> a[3][2], xab[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double s0 = 0, s1 = 0, t0 = 0, t1 = 0, t2 = 0;
#pragma unroll
    for (int b = 0; b < 9; ++b) {
      double xb = X[b * 3 + i];
      s0 += dN0[b] * xb; s1 += dN1[b] * xb;
      t0 += dd[0][b] * xb; t1 += dd[1][b] * xb; t2 += dd[2][b] * xb;
    }
    T g = (i == js) ? T(dt) : T(0);
    a[i][0] = mk<T>(s0, g * sd0);
    a[i][1] = mk<T>(s1, g * sd1);
    xab[i][0] = mk<T>(t0, g * T(dd[0][as]));
    xab[i][1] = mk<T>(t1, g * T(dd[1][as]));
    xab[i][2] = mk<T>(t2, g * T(dd[2][as]));
  }
  Dual<T> a11 = a[0][0] * a[0][0] + a[1][0] * a[1][0] + a[2][0] * a[2][0];
  Dual<T> a12 = a[0][0] * a[0][1] + a[1][0] * a[1][1] + a[2][0] * a[2][1];
  Dual<T> a22 = a[0][1] * a[0][1] + a[1][1] * a[1][1] + a[2][1] * a[2][1];
  Dual<T> det = a11 * a22 - a12 * a12;
  Dual<T> idet = inv(det);
  Dual<T> i11 = a22 * idet, i12 = -(a12 * idet), i22 = a11 * idet;  // a^αβ
  Dual<T> aup[3][2];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    aup[i][0] = a[i][0] * i11 + a[i][1] * i12;
    aup[i][1] = a[i][0] * i12 + a[i][1] * i22;
  }
  Dual<T> J = dsqrt(det);
  Dual<T> iJ = inv(J);
  Dual<T> n[3];
  n[0] = (a[1][0] * a[2][1] - a[2][0] * a[1][1]) * iJ;
  n[1] = (a[2][0] * a[0][1] - a[0][0] * a[2][1]) * iJ;
  n[2] = (a[0][0] * a[1][1] - a[1][0] * a[0][1]) * iJ;
  Dual<T> Gam[3][2], bf[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    Gam[k][0] = xab[0][k] * aup[0][0] + xab[1][k] * aup[1][0] + xab[2][k] * aup[2][0];
    Gam[k][1] = xab[0][k] * aup[0][1] + xab[1][k] * aup[1][1] + xab[2][k] * aup[2][1];
    bf[k] = xab[0][k] * n[0] + xab[1][k] * n[1] + xab[2][k] * n[2];
  }
  // b^αβ = a⁻¹ b a⁻¹ (symmetric)
  Dual<T> t11 = i11 * bf[0] + i12 * bf[2], t12 = i11 * bf[2] + i12 * bf[1];
  Dual<T> t21 = i12 * bf[0] + i22 * bf[2], t22 = i12 * bf[2] + i22 * bf[1];
  Dual<T> bu11 = t11 * i11 + t12 * i12, bu12 = t11 * i12 + t12 * i22, bu22 = t21 * i12 + t22 * i22;
  Dual<T> H = (i11 * bf[0] + i12 * bf[2] + i12 * bf[2] + i22 * bf[1]) * 0.5;
  Dual<T> K = (bf[0] * bf[1] - bf[2] * bf[2]) * idet;

  // dynamics (get_dof_cps zero-fills absent unknowns, GeoDynStress.jl:190-205)
  auto interp = [&](int u, const double* wts, T swt) -> Dual<T> {
    int d = pp.dof_of[u];
    double s = 0;
    if (d >= 0) {
#pragma unroll
      for (int b = 0; b < 9; ++b) s += wts[b] * C[b * 8 + d];
    }
    return mk<T>(s, (u == us) ? swt : T(0));
  };
  Dual<T> dv[3][2];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    dv[i][0] = interp(i, dN0, sd0);
    dv[i][1] = interp(i, dN1, sd1);
  }
  Dual<T> lam = interp(6, N, sN);

  // π^αβ = ζv sym(a^αᵀ v_,α a⁻¹)  (GeoDynStress.jl:148-149)
  auto visc = [&](Dual<T> g[3][2], Dual<T>& p11, Dual<T>& p12, Dual<T>& p22) {
    Dual<T> u[3][2];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      u[i][0] = g[i][0] * i11 + g[i][1] * i12;
      u[i][1] = g[i][0] * i12 + g[i][1] * i22;
    }
    Dual<T> P11 = aup[0][0] * u[0][0] + aup[1][0] * u[1][0] + aup[2][0] * u[2][0];
    Dual<T> P12 = aup[0][0] * u[0][1] + aup[1][0] * u[1][1] + aup[2][0] * u[2][1];
    Dual<T> P21 = aup[0][1] * u[0][0] + aup[1][1] * u[1][0] + aup[2][1] * u[2][0];
    Dual<T> P22 = aup[0][1] * u[0][1] + aup[1][1] * u[1][1] + aup[2][1] * u[2][1];
    p11 = (P11 + P11) * pp.zv;
    p12 = (P12 + P21) * pp.zv;
    p22 = (P22 + P22) * pp.zv;
  };
  Dual<T> p11, p12, p22;
  visc(dv, p11, p12, p22);
  // tr(a^αᵀ v_,α) for rλ (FiniteElement.jl:298)
  Dual<T> tr = aup[0][0] * dv[0][0] + aup[1][0] * dv[1][0] + aup[2][0] * dv[2][0] + aup[0][1] * dv[0][1] +
               aup[1][1] * dv[1][1] + aup[2][1] * dv[2][1];
  // σ, M in Voigt form (GeoDynStress.jl:150-154)
  Dual<T> cb = pp.kb * (H * H) - pp.kg * K;
  Dual<T> cs = cb + lam;
  Dual<T> hb = H * (2.0 * pp.kb);
  Dual<T> sg0 = i11 * cs - bu11 * hb + p11;
  Dual<T> sg1 = i22 * cs - bu22 * hb + p22;
  Dual<T> sg2 = (i12 * cs - bu12 * hb + p12) * 2.0;
  Dual<T> hm = H * (pp.kb + 2.0 * pp.kg);
  Dual<T> M0 = i11 * hm - bu11 * pp.kg;
  Dual<T> M1 = i22 * hm - bu22 * pp.kg;
  Dual<T> M2 = (i12 * hm - bu12 * pp.kg) * 2.0;
  Dual<T> JW = J * w;

  // mesh-motion quantities
  Dual<T> sm0, sm1, sm2, pm_, vmv[3], nd_;
  if (MOTION == ALEV_ || MOTION == ALEVB_) {
    Dual<T> dvm[3][2];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      dvm[i][0] = interp(3 + i, dN0, sd0);
      dvm[i][1] = interp(3 + i, dN1, sd1);
    }
    Dual<T> m11, m12, m22;
    visc(dvm, m11, m12, m22);
    sm0 = i11 * cb - bu11 * hb + m11;  // GeoDynStress.jl:156-159
    sm1 = i22 * cb - bu22 * hb + m22;
    sm2 = (i12 * cb - bu12 * hb + m12) * 2.0;
    pm_ = interp(7, N, sN);
    Dual<T> nd = cst<T>(0.0);
#pragma unroll
    for (int i = 0; i < 3; ++i) nd = nd + n[i] * (interp(3 + i, N, sN) - interp(i, N, sN));
    nd_ = nd;
  }
  Dual<T> nv;
  if (MOTION == EUL_) {
    Dual<T> v[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      v[i] = interp(i, N, sN);
      vmv[i] = interp(3 + i, N, sN);
    }
    nv = n[0] * v[0] + n[1] * v[1] + n[2] * v[2];
  }

  // residual rows (node-major packing of calc_elem_residual, FiniteElement.jl:225-239)
  const int vo0 = pp.dof_of[0], vo1 = pp.dof_of[1], vo2 = pp.dof_of[2];
  const int vd[3] = {vo0, vo1, vo2};
  const int mo[3] = {pp.dof_of[3], pp.dof_of[4], pp.dof_of[5]};
  const int lo = pp.dof_of[6], po = pp.dof_of[7];
  Dual<T> rl_c = J * tr - (pp.adb / pp.zv) * lam;
#pragma unroll 1
  for (int b = 0; b < 9; ++b) {
    Dual<T> nn0 = cst<T>(dd[0][b]) - (Gam[0][0] * dN0[b] + Gam[0][1] * dN1[b]);
    Dual<T> nn1 = cst<T>(dd[1][b]) - (Gam[1][0] * dN0[b] + Gam[1][1] * dN1[b]);
    Dual<T> nn2 = cst<T>(dd[2][b]) - (Gam[2][0] * dN0[b] + Gam[2][1] * dN1[b]);
    Dual<T> cbm = (nn0 * M0 + nn1 * M1 + nn2 * M2) * JW;  // Bbᵀ𝗠 coefficient of n_i
    Dual<T> c1 = (sg0 * dN0[b] + sg2 * (0.5 * dN1[b])) * JW;
    Dual<T> c2 = (sg1 * dN1[b] + sg2 * (0.5 * dN0[b])) * JW;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      if (vd[i] >= 0) {
        Dual<T> rv = a[i][0] * c1 + a[i][1] * c2 + n[i] * cbm;
        if (pp.pn != 0.0) rv = rv - n[i] * (N[b] * pp.pn) * JW;
        acc_row<T>(vd[i] + ndf * b, q, rv, rsum, Ks, ldk);
      }
    }
    if (MOTION == ALEV_ || MOTION == ALEVB_) {
      Dual<T> e1 = (sm0 * dN0[b] + sm2 * (0.5 * dN1[b])) * JW;
      Dual<T> e2 = (sm1 * dN1[b] + sm2 * (0.5 * dN0[b])) * JW;
      Dual<T> pnj = pm_ * JW * N[b];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        Dual<T> rm = a[i][0] * e1 + a[i][1] * e2;
        if (MOTION == ALEVB_) rm = rm + n[i] * cbm;
        rm = rm - n[i] * pnj;
        acc_row<T>(mo[i] + ndf * b, q, rm, rsum, Ks, ldk);
      }
      Dual<T> rp = -((JW * nd_) * N[b]) - pm_ * (N[b] * w * pp.adb / pp.zv);
      acc_row<T>(po + ndf * b, q, rp, rsum, Ks, ldk);
    }
    if (MOTION == EUL_) {
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        Dual<T> rm = (vmv[i] - n[i] * nv) * JW * (N[b] * pp.am);
        acc_row<T>(mo[i] + ndf * b, q, rm, rsum, Ks, ldk);
      }
    }
    acc_row<T>(lo + ndf * b, q, rl_c * (N[b] * w), rsum, Ks, ldk);
  }
}

// One boundary Gauss point of calc_bdry_element_residual (FiniteElement.jl:363-384).
template <class T>
__device__ __forceinline__ void bdry_gp(const PhysParams& pp, const double* X, const double* f, int bdry, int ntype,
                                        double nval, double time, int q, int as, int js, double dt, double& rsum,
                                        T* Ks, int ldk) {
  const int ndf = pp.ndf;
  const double w = f[0];
  const double* N = f + 1;
  const double* dN0 = f + 10;
  const double* dN1 = f + 19;
  const T sd0 = T(dN0[as]), sd1 = T(dN1[as]);
  Dual<T> a[3][2];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double s0 = 0, s1 = 0;
#pragma unroll
    for (int b = 0; b < 9; ++b) {
      s0 += dN0[b] * X[b * 3 + i];
      s1 += dN1[b] * X[b * 3 + i];
    }
    T g = (i == js) ? T(dt) : T(0);
    a[i][0] = mk<T>(s0, g * sd0);
    a[i][1] = mk<T>(s1, g * sd1);
  }
  Dual<T> a11 = a[0][0] * a[0][0] + a[1][0] * a[1][0] + a[2][0] * a[2][0];
  Dual<T> a12 = a[0][0] * a[0][1] + a[1][0] * a[1][1] + a[2][0] * a[2][1];
  Dual<T> a22 = a[0][1] * a[0][1] + a[1][1] * a[1][1] + a[2][1] * a[2][1];
  Dual<T> det = a11 * a22 - a12 * a12;
  Dual<T> idet = inv(det);
  Dual<T> i11 = a22 * idet, i12 = -(a12 * idet), i22 = a11 * idet;
  Dual<T> aup[3][2];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    aup[i][0] = a[i][0] * i11 + a[i][1] * i12;
    aup[i][1] = a[i][0] * i12 + a[i][1] * i22;
  }
  Dual<T> iJ = inv(dsqrt(det));
  Dual<T> n[3];
  n[0] = (a[1][0] * a[2][1] - a[2][0] * a[1][1]) * iJ;
  n[1] = (a[2][0] * a[0][1] - a[0][0] * a[2][1]) * iJ;
  n[2] = (a[0][0] * a[1][1] - a[1][0] * a[0][1]) * iJ;
  // τ = ±a_α / |a_α|; the norm is a primal constant (conjugating dot, FiniteElement.jl:448)
  int col = (bdry == 0 || bdry == 2) ? 0 : 1;
  double sgn = (bdry == 0 || bdry == 1) ? 1.0 : -1.0;
  double nrm = sqrt(a[0][col].v * a[0][col].v + a[1][col].v * a[1][col].v + a[2][col].v * a[2][col].v);
  double sc = sgn / nrm;
  Dual<T> tau[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) tau[i] = a[i][col] * sc;
  Dual<T> nu[3];
  nu[0] = tau[1] * n[2] - tau[2] * n[1];
  nu[1] = tau[2] * n[0] - tau[0] * n[2];
  nu[2] = tau[0] * n[1] - tau[1] * n[0];
  Dual<T> t0 = aup[0][0] * tau[0] + aup[1][0] * tau[1] + aup[2][0] * tau[2];
  Dual<T> t1 = aup[0][1] * tau[0] + aup[1][1] * tau[1] + aup[2][1] * tau[2];
  Dual<T> JG = inv(dsqrt(t0 * t0 + t1 * t1));
  const int vd[3] = {pp.dof_of[0], pp.dof_of[1], pp.dof_of[2]};
  if (ntype == MAFEM_STRETCH || ntype == MAFEM_SHEAR) {
    Dual<T> fv[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) fv[i] = (ntype == MAFEM_STRETCH ? nu[i] : tau[i]) * (nval * w);
    Dual<T> fj[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) fj[i] = fv[i] * JG;
#pragma unroll 1
    for (int b = 0; b < 9; ++b)
#pragma unroll
      for (int i = 0; i < 3; ++i)
        if (vd[i] >= 0) acc_row<T>(vd[i] + ndf * b, q, -(fj[i] * N[b]), rsum, Ks, ldk);
  } else {  // MOMENT (F_BEND only; other types are rejected on the host)
    Dual<T> nu0 = aup[0][0] * nu[0] + aup[1][0] * nu[1] + aup[2][0] * nu[2];
    Dual<T> nu1 = aup[0][1] * nu[0] + aup[1][1] * nu[1] + aup[2][1] * nu[2];
    double Mval = nval * fmin(time / pp.bend_tm, 1.0);
    Dual<T> s = JG * (Mval * w);
#pragma unroll 1
    for (int b = 0; b < 9; ++b) {
      Dual<T> dn = (nu0 * dN0[b] + nu1 * dN1[b]) * s;
#pragma unroll
      for (int i = 0; i < 3; ++i)
        if (vd[i] >= 0) acc_row<T>(vd[i] + ndf * b, q, -(n[i] * dn), rsum, Ks, ldk);
    }
  }
}

// elist (optional): evaluate only elements elist[0 .. nlist) and write their rows
// to r_el[k][q]; area_only: the area Gauss points alone (calc_elem_dof_residuals
// without the Dohrmann-Bochev projection or boundary terms, as PullForce.jl uses
// it); K_el may be null (no tangent written).
template <class T, int MOTION, int EPB>
__global__ void elem_kernel(DevPatch P, PhysParams pp, double time, double dt, double* __restrict__ r_el,
                            T* __restrict__ K_el, const int* __restrict__ elist, int nlist, int area_only) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nq = pp.nq, ndf = pp.ndf;
  const int ldk = nq + 1;
  const int slot = threadIdx.x / nq;
  const int q = threadIdx.x - slot * nq;
  const int kk = blockIdx.x * EPB + slot;  // element (or list) index of this slot
  const int e = elist ? (kk < nlist ? elist[kk] : 0) : kk;
  // per-slot shared memory
  const size_t dbl_per_slot = 27 + 72 + 9 * kTab;
  double* base = reinterpret_cast<double*>(smem_raw);
  double* X = base + slot * dbl_per_slot;
  double* C = X + 27;
  double* tab = C + 72;
  T* Ks = reinterpret_cast<T*>(base + EPB * dbl_per_slot) + (size_t)slot * nq * ldk;
  const bool live = (slot < EPB) && (elist ? kk < nlist : e < P.numel);

  if (live) {
    const int u = P.uel[e];
    for (int k = q; k < 9 * kTab; k += nq) tab[k] = P.tab[(size_t)u * 9 * kTab + k];
    for (int k = q; k < 27; k += nq) {
      int b = k / 3, i = k - 3 * (k / 3);
      X[k] = P.xms[(size_t)i * P.numnp + P.ix[e * 9 + b]];
    }
    for (int k = q; k < 72; k += nq) {
      int b = k / 8, d = k - 8 * (k / 8);
      C[k] = d < ndf ? P.cps[(size_t)d * P.numnp + P.ix[e * 9 + b]] : 0.0;
    }
    for (int k = q; k < nq * ldk; k += nq) Ks[k] = T(0);
  }
  __syncthreads();
  if (live) {

  const int as = q / ndf, ds = q - as * ndf;
  const int us = pp.unk_of[ds];
  const int js = (pp.mmo[0] == ds) ? 0 : (pp.mmo[1] == ds) ? 1 : (pp.mmo[2] == ds) ? 2 : -1;
  double rsum = 0.0;

#pragma unroll 1
  for (int gp = 0; gp < 9; ++gp)
    area_gp<T, MOTION>(pp, X, C, tab + gp * kTab, q, as, js, us, dt, rsum, Ks, ldk);

  // Dohrmann-Bochev projection (FiniteElement.jl:323-327): rλ += Gᵀ H⁻¹ G λ αdb/ζv,
  // and for ALEV/ALEVB rp += Gᵀ H⁻¹ G p αdb/ζv.  Linear in λ / p.
  if (!area_only) {
    const double* T81 = P.db + (size_t)P.uel[e] * 81;
    const double s = pp.adb / pp.zv;
    const int lo = pp.dof_of[6], po = pp.dof_of[7];
    const bool alep = (MOTION == ALEV_ || MOTION == ALEVB_);
    for (int b = 0; b < 9; ++b) {
      double sl = 0, sp = 0;
      for (int c = 0; c < 9; ++c) {
        sl += T81[b * 9 + c] * C[c * 8 + lo];
        if (alep) sp += T81[b * 9 + c] * C[c * 8 + po];
      }
      int rowl = lo + ndf * b;
      if (rowl == q) rsum += sl * s;
      if (us == 6) Ks[rowl * ldk + q] += T(T81[b * 9 + as] * s);
      if (alep) {
        int rowp = po + ndf * b;
        if (rowp == q) rsum += sp * s;
        if (us == 7) Ks[rowp * ldk + q] += T(T81[b * 9 + as] * s);
      }
    }
  }

  // Neumann boundary terms of this element (calc_r_K's boundary loop,
  // FiniteElement.jl:150-197): same LM, so they add into the same block.
  for (int k = 0; k < (area_only ? 0 : pp.n_neu); ++k) {
    int b = pp.neu_bdry[k];
    int row = P.bref[e * 4 + b];
    if (row < 0) continue;
    for (int g = 0; g < 3; ++g)
      bdry_gp<T>(pp, X, P.btab + ((size_t)row * 3 + g) * kTab, b, pp.neu_type[k], pp.neu_val[k], time, q, as, js, dt,
                 rsum, Ks, ldk);
  }

  r_el[(size_t)(elist ? kk : e) * nq + q] = rsum;
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

// ---- launcher ----------------------------------------------------------------------
template <class T>
size_t elem_smem_bytes(int nq, int epb) {
  return (size_t)epb * (27 + 72 + 9 * kTab) * sizeof(double) + (size_t)epb * nq * (nq + 1) * sizeof(T);
}

template <class T, int MOTION, int EPB>
static cudaError_t launch_elem_t(const DevPatch& P, const PhysParams& pp, double time, double dt, double* r_el,
                                 T* K_el, cudaStream_t st, const int* elist, int nlist, int area_only) {
  // the cap is the size needed by the largest element (nq = 72), identical for every caller
  cudaError_t e = cudaFuncSetAttribute(elem_kernel<T, MOTION, EPB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)elem_smem_bytes<T>(72, EPB));
  if (e != cudaSuccess) return e;
  const int blocks = ((elist ? nlist : P.numel) + EPB - 1) / EPB;
  elem_kernel<T, MOTION, EPB><<<blocks, EPB * pp.nq, elem_smem_bytes<T>(pp.nq, EPB), st>>>(P, pp, time, dt, r_el,
                                                                                         K_el, elist, nlist,
                                                                                         area_only);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_elem(const DevPatch& P, const PhysParams& pp, double time, double dt, double* r_el, T* K_el,
                        cudaStream_t st, const int* elist, int nlist, int area_only) {
  switch (pp.motion) {
    case MAFEM_STATIC: return launch_elem_t<T, STATIC_, 4>(P, pp, time, dt, r_el, K_el, st, elist, nlist, area_only);
    case MAFEM_EUL: return launch_elem_t<T, EUL_, 2>(P, pp, time, dt, r_el, K_el, st, elist, nlist, area_only);
    case MAFEM_LAG: return launch_elem_t<T, LAG_, 4>(P, pp, time, dt, r_el, K_el, st, elist, nlist, area_only);
    case MAFEM_ALEV: return launch_elem_t<T, ALEV_, 2>(P, pp, time, dt, r_el, K_el, st, elist, nlist, area_only);
    default: return launch_elem_t<T, ALEVB_, 2>(P, pp, time, dt, r_el, K_el, st, elist, nlist, area_only);
  }
}

template cudaError_t launch_elem<double>(const DevPatch&, const PhysParams&, double, double, double*, double*,
                                         cudaStream_t, const int*, int, int);
template cudaError_t launch_elem<float>(const DevPatch&, const PhysParams&, double, double, double*, float*,
                                        cudaStream_t, const int*, int, int);
template size_t elem_smem_bytes<double>(int, int);
template size_t elem_smem_bytes<float>(int, int);

}  // namespace mafem
