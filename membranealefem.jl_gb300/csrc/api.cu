// api.cu -- device handle, Newton driver and the C ABI of include/mafem.h.
//
// time_step! (src/analysis/FiniteElement.jl:11-63) runs on the device: per
// Newton iteration the element kernel, the band/residual gathers, the banded
// LU (FP64, or FP32 + FP64 refinement), the back substitution and the state
// update are stream-ordered launches; the host reads back three doubles per
// iteration (ε, ‖r‖, a NaN flag) to apply the reference's stopping rule
// (`iter < 15`, `ε < εnr`).

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <thread>
#include <vector>

#include "mafem.h"
#include "mafem_internal.h"

namespace mafem {

static std::mutex g_err_mu;
static std::string g_err;
void set_global_error(const std::string& s) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_err = s;
}

int64_t half_bandwidth(const mafem_mesh_desc& d) {
  int64_t b = 0;
  for (int64_t e = 0; e < d.numel; ++e) {
    int64_t lo = INT64_MAX, hi = -1;
    for (int a = 0; a < 9; ++a) {
      int64_t node = d.IX[a + 9 * e] - 1;
      for (int64_t k = 0; k < d.ndf; ++k) {
        int64_t g = d.ID[k + d.ndf * node];
        if (g > 0) {
          lo = std::min(lo, g);
          hi = std::max(hi, g);
        }
      }
    }
    if (hi >= 0) b = std::max(b, hi - lo);
  }
  return b;
}

// Panel width: the FP64 panel and its trailing-update CTA keep (nb + kl) x nb
// values in shared memory.
static int choose_nb(int kl, int precision) {
  const size_t limit = 220 * 1024;
  const size_t esz = precision == MAFEM_PLAIN_FP64 ? 8 : 4;
  for (int nb : {32, 16, 8}) {
    size_t R = (size_t)nb + kl;
    size_t apply = R * nb * esz + 8 * R * esz + R * 4;
    if (apply <= limit) return nb;
  }
  return 0;
}

}  // namespace mafem

using namespace mafem;

struct mafem_handle {
  std::string err;
  int precision = 0;
  mafem_params p{};
  mafem_args a{};
  int ndf = 0, nq = 0, numel = 0, numnp = 0;
  int64_t nmdf = 0;
  DevPatch P{};
  PhysParams pp{};
  BandLayout L{};
  int rmax = 0;
  int64_t npan = 0;
  int apply_threads = 256, apply_blocks = 152;
  std::vector<void*> allocs;
  int64_t bytes = 0;
  double *d_rel = nullptr, *d_r = nullptr, *d_x = nullptr, *d_res = nullptr, *d_dx = nullptr;
  double *d_part = nullptr, *d_out = nullptr;
  void *d_Kel = nullptr, *d_band = nullptr, *d_band0 = nullptr;
  int *d_ipiv = nullptr, *d_perm = nullptr, *d_info = nullptr;
  double* h_out = nullptr;  // pinned: [0] eps [1] |r| [2] nan [3] refine |res| [4] info
  cudaStream_t st = nullptr;
  cudaStream_t st2 = nullptr;          // LU lookahead stream
  std::vector<cudaEvent_t> ev_pool;    // 2*npan + 2 ordering events for the lookahead
  cudaEvent_t ev[6] = {};
  bool factored = false;
  int max_refine = 30;
  double refine_tol = 1e-10;
  int64_t launches = 0;  // kernels enqueued by this handle
  // node-block pivoting (band_lu_blk.cu): the default; full partial pivoting
  // (band_lu.cu) is the fallback for a block without a usable pivot
  bool use_blk = false;
  bool last_blk = false;  // which factorisation the band currently holds
  BlkPlan blk;
  int* d_blk_end = nullptr;
  int* d_flags = nullptr;  // per-panel completion flags of the cooperative back substitution
  int epoch = 0;           // value the flags are set to by the next back substitution
  int bwd_grid = 0;        // CTAs of the cooperative back substitution (0: single-CTA kernel)
  BlkPersist pers;         // persistent cooperative factorisation (grid 0: per-panel launches)
  std::vector<int> h_ix;   // IX, 0-based [element][9] (pull-force neighbourhood)
  int bwd_max = 0;         // back-substitution CTAs before any cap
  // the time step in progress (step_begin / iter_enqueue / iter_finish)
  double ss_time = 0, ss_dt = 0, ss_eps = 0;
  int ss_iter = 0, ss_sweeps = 0;
  bool ss_async = false;
  mafem_step_stats ss_S{};
  int* d_pull_list = nullptr;
  double* d_pull_r = nullptr;
  int lu_path = MAFEM_LU_AUTO;
  int patch_nr = 0;  // CTAs per cluster of the batched FP32 factor (0: chosen per round)
  int round_nr = 0;  // the cluster size the autotuner chose for this round (0: by band width)
  int fepoch = 0;          // epoch of the last persistent factorisation
  void* d_rdiag = nullptr;
  int64_t fallbacks = 0;
  // batched FP32 form (band_lu_patch.cu): the handle's job, usable when its band fits
  float* d_inv = nullptr;
  double* d_zbuf = nullptr;  // npan x 32: z = U11^-1 y1 per panel (cooperative forward substitution)
  double* d_pinv = nullptr;  // npan x 2 x 32 x 32: L11^-1, U11^-1 per panel (cooperative substitutions)
  bool patch_ok = false;
  bool ss_patch = false;  // the iteration in progress ran through a batch's patch solve
  PatchJob job{};
  WaitTest wait_test;                   // mafem_set_wait_test (failure-detection tests)
  const double* host_band = nullptr;    // mafem_solve_band: the caller's band (padded layout), for the fallback
  int n_dir = 0;                        // inhomogeneous Dirichlet entries of the state (mafem_set_dirichlet_scale)
  int* d_dir_idx = nullptr;             // their index dof * numnp + node into cps
  double* d_dir_val = nullptr;          // their values
  int* d_rstate = nullptr;              // refinement state {done, sweeps, status} (FP32 form)
  int* h_rstate = nullptr;              // its pinned host copy
  bool no_async = false;                // the next iteration waits for its solve (a redo)
  std::unique_ptr<StateWriter> writer;  // state files, created by the first write
  double* d_snap = nullptr;             // device snapshots: nsnap x [xms | cps]
  int nsnap = 0;
};

#define CK(x)                                                               \
  do {                                                                      \
    cudaError_t e_ = (x);                                                   \
    if (e_ != cudaSuccess) {                                                \
      h->err = std::string(#x) + ": " + cudaGetErrorString(e_);             \
      return MAFEM_ERR_CUDA;                                                \
    }                                                                       \
  } while (0)

template <class X>
static int dalloc(mafem_handle* h, X** p, size_t count) {
  void* v = nullptr;
  size_t bytes = std::max<size_t>(count, 1) * sizeof(X);
  cudaError_t e = cudaMalloc(&v, bytes);
  if (e != cudaSuccess) {
    h->err = std::string("cudaMalloc of ") + std::to_string(bytes) + " bytes: " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? MAFEM_ERR_OOM : MAFEM_ERR_CUDA;
  }
  h->allocs.push_back(v);
  h->bytes += (int64_t)bytes;
  *p = reinterpret_cast<X*>(v);
  return MAFEM_OK;
}
template <class X>
static int dupload(mafem_handle* h, X** p, const std::vector<X>& v) {
  int rc = dalloc(h, p, v.size());
  if (rc) return rc;
  CK(cudaMemcpy(*p, v.data(), v.size() * sizeof(X), cudaMemcpyHostToDevice));
  return MAFEM_OK;
}

// Gᵀ H⁻¹ G of the Dohrmann-Bochev projection (FiniteElement.jl:279-323) for one
// unique element: G = Σ NDB Nᵀ w, H = Σ NDB NDBᵀ w, NDB = (ξ¹, ξ², 1).
static void db_matrix(const double* uf /* 9 x 55 */, double out[81]) {
  const double xi[3] = {-std::sqrt(3.0 / 5), 0.0, std::sqrt(3.0 / 5)};
  double G[3][9] = {}, H[3][3] = {};
  for (int gp = 0; gp < 9; ++gp) {
    const double* f = uf + gp * 55;
    const double w = f[0];
    const double nd[3] = {xi[gp % 3], xi[gp / 3], 1.0};
    for (int r = 0; r < 3; ++r) {
      for (int a = 0; a < 9; ++a) G[r][a] += nd[r] * f[1 + a] * w;
      for (int c = 0; c < 3; ++c) H[r][c] += nd[r] * nd[c] * w;
    }
  }
  // 3x3 inverse by cofactors
  double c00 = H[1][1] * H[2][2] - H[1][2] * H[2][1], c01 = H[1][2] * H[2][0] - H[1][0] * H[2][2],
         c02 = H[1][0] * H[2][1] - H[1][1] * H[2][0];
  double det = H[0][0] * c00 + H[0][1] * c01 + H[0][2] * c02;
  double Hi[3][3] = {{c00 / det, (H[0][2] * H[2][1] - H[0][1] * H[2][2]) / det, (H[0][1] * H[1][2] - H[0][2] * H[1][1]) / det},
                     {c01 / det, (H[0][0] * H[2][2] - H[0][2] * H[2][0]) / det, (H[0][2] * H[1][0] - H[0][0] * H[1][2]) / det},
                     {c02 / det, (H[0][1] * H[2][0] - H[0][0] * H[2][1]) / det, (H[0][0] * H[1][1] - H[0][1] * H[1][0]) / det}};
  double HG[3][9];
  for (int r = 0; r < 3; ++r)
    for (int a = 0; a < 9; ++a) HG[r][a] = Hi[r][0] * G[0][a] + Hi[r][1] * G[1][a] + Hi[r][2] * G[2][a];
  for (int a = 0; a < 9; ++a)
    for (int b = 0; b < 9; ++b) out[a * 9 + b] = G[0][a] * HG[0][b] + G[1][a] * HG[1][b] + G[2][a] * HG[2][b];
}

static int validate(const mafem_mesh_desc* d, const mafem_params* p, std::string& err) {
  if (!d || !p) { err = "null argument"; return MAFEM_ERR_ARG; }
  if (p->poly != 2 || p->nen != 9 || p->nders != 2 || p->gp1d != 3) {
    err = "only poly = 2, nen = 9, nders = 2, gp1d = 3 are supported (Params.jl:93-95)";
    return MAFEM_ERR_UNSUPPORTED;
  }
  if (d->ndf < 1 || d->ndf > 8 || d->numel != d->num1el * d->num2el || d->numnp != d->num1np * d->num2np ||
      d->num1np != d->num1el + 2 || d->num2np != d->num2el + 2 || d->nmdf < 1) {
    err = "inconsistent mesh sizes (flat patch expected: num?np = num?el + 2)";
    return MAFEM_ERR_ARG;
  }
  if (!d->IX || !d->ID || !d->uel_ids || !d->ufns) { err = "missing mesh arrays"; return MAFEM_ERR_ARG; }
  if (d->n_dir < 0 || (d->n_dir > 0 && (!d->dir_unknown || !d->dir_node || !d->dir_val))) {
    err = "missing Dirichlet arrays";
    return MAFEM_ERR_ARG;
  }
  // The gathers and the pull-force neighbourhood rely on the tensor-product
  // connectivity of construct_IX (Mesh.jl:574-593): node (a1, a2) of element
  // (e1, e2) is control point (e1 + a1) + num1np (e2 + a2) (0-based).  Any other
  // IX -- or an entry out of range -- is rejected rather than silently misread.
  for (int64_t e2 = 0; e2 < d->num2el; ++e2)
    for (int64_t e1 = 0; e1 < d->num1el; ++e1)
      for (int a = 0; a < 9; ++a) {
        const int64_t want = 1 + (e1 + a % 3) + d->num1np * (e2 + a / 3);
        if (d->IX[a + 9 * (e1 + d->num1el * e2)] != want) {
          err = "IX differs from the tensor-product connectivity (Mesh.jl:574-593) at element " +
                std::to_string(1 + e1 + d->num1el * e2) + ", node " + std::to_string(a + 1);
          return MAFEM_ERR_ARG;
        }
      }
  for (int64_t k = 0; k < d->ndf * d->numnp; ++k)
    if (d->ID[k] < 0 || d->ID[k] > d->nmdf) { err = "ID entry outside 0..nmdf"; return MAFEM_ERR_ARG; }
  if (d->n_uel < 1) { err = "n_uel must be >= 1"; return MAFEM_ERR_ARG; }
  for (int64_t e = 0; e < d->numel; ++e)
    if (d->uel_ids[e] < 1 || d->uel_ids[e] > d->n_uel) { err = "uel_ids entry outside 1..n_uel"; return MAFEM_ERR_ARG; }
  for (int b = 0; b < 4; ++b) {
    const int64_t nb = (b == 0 || b == 2) ? d->num1el : d->num2el;
    if (d->bdry_n_uel[b] > 0 && d->bdry_uel_ids[b] && d->bdry_ufns[b]) {
      for (int64_t k = 0; k < nb; ++k)
        if (d->bdry_uel_ids[b][k] < 1 || d->bdry_uel_ids[b][k] > d->bdry_n_uel[b]) {
          err = "bdry_uel_ids entry outside 1..bdry_n_uel";
          return MAFEM_ERR_ARG;
        }
    } else if (d->bdry_n_uel[b] != 0) {
      err = "missing boundary tables";
      return MAFEM_ERR_ARG;
    }
  }
  for (int u = 0; u < 8; ++u)
    if (d->dofs[u] < 0 || d->dofs[u] > d->ndf) { err = "dofs entry outside 0..ndf"; return MAFEM_ERR_ARG; }
  if (d->n_neu < 0 || d->n_neu > kMaxNeu) { err = "at most 8 Neumann entries are supported"; return MAFEM_ERR_ARG; }
  for (int64_t k = 0; k < d->n_neu; ++k) {
    if (d->neu_bdry[k] < 1 || d->neu_bdry[k] > 4) { err = "bad Neumann boundary"; return MAFEM_ERR_ARG; }
    int t = (int)d->neu_type[k];
    if (t != MAFEM_STRETCH && t != MAFEM_SHEAR && !(t == MAFEM_MOMENT && p->scenario == MAFEM_F_BEND)) {
      err = "Neumann boundary condition not implemented (FiniteElement.jl:382)";
      return MAFEM_ERR_UNSUPPORTED;
    }
  }
  if (p->motion < MAFEM_STATIC || p->motion > MAFEM_ALEVB) { err = "unknown motion"; return MAFEM_ERR_ARG; }
  return MAFEM_OK;
}

static int64_t footprint(const mafem_mesh_desc* d, int precision, int64_t kl) {
  const int nb = choose_nb((int)kl, precision);
  BandLayout L = make_band_layout(d->nmdf, (int)kl, (int)kl, nb ? nb : 8);
  const int64_t esz = precision == MAFEM_PLAIN_FP64 ? 8 : 4;
  const int64_t nq = 9 * d->ndf;
  int64_t b = L.ldb * d->nmdf * esz * (precision == MAFEM_PLAIN_FP64 ? 1 : 2);  // band (+ unfactored copy)
  b += d->numel * nq * nq * esz + d->numel * nq * 8;                             // element staging
  b += d->numnp * (3 + d->ndf) * 8 + d->nmdf * 8 * 6;                           // state + vectors
  b += ((d->nmdf + nb - 1) / std::max(nb, 1)) * ((int64_t)nb + kl) * 4;           // panel permutations
  b += d->nmdf * (esz + 4);                                                      // pivot reciprocals, blocks
  b += (d->nmdf / 24 + 1) * 2 * 32 * 32 * 8;                                     // panel triangle inverses
  return b;
}

extern "C" int64_t mafem_mesh_half_bandwidth(const mafem_mesh_desc* d) { return d ? half_bandwidth(*d) : -1; }

extern "C" int64_t mafem_footprint_bytes(const mafem_mesh_desc* d, int32_t precision) {
  if (!d || !d->IX || !d->ID) return -1;
  return footprint(d, precision, half_bandwidth(*d));
}

extern "C" int mafem_create(const mafem_mesh_desc* d, const mafem_params* p, const mafem_args* a,
                            int32_t precision, mafem_handle** out) {
  if (!out) return MAFEM_ERR_ARG;
  *out = nullptr;
  std::string err;
  int rc = validate(d, p, err);
  if (rc) {
    set_global_error(err);
    return rc;
  }
  if (precision != MAFEM_PLAIN_FP64 && precision != MAFEM_FP32_REFINE) {
    set_global_error("unknown precision mode");
    return MAFEM_ERR_ARG;
  }
  auto hp = std::make_unique<mafem_handle>();
  mafem_handle* h = hp.get();
  h->precision = precision;
  h->p = *p;
  if (a) h->a = *a;
  h->ndf = (int)d->ndf;
  h->nq = 9 * h->ndf;
  h->numel = (int)d->numel;
  h->numnp = (int)d->numnp;
  h->nmdf = d->nmdf;
  const int ndf = h->ndf, nq = h->nq, numel = h->numel, numnp = h->numnp;
  const int64_t n = h->nmdf;

  // physics parameters and dof maps
  PhysParams& pp = h->pp;
  std::memset(&pp, 0, sizeof pp);
  pp.motion = p->motion;
  pp.scenario = p->scenario;
  pp.ndf = ndf;
  pp.nq = nq;
  pp.kb = p->kb; pp.kg = p->kg; pp.zv = p->zeta_v; pp.pn = p->pn; pp.adb = p->alpha_db; pp.am = p->alpha_m;
  pp.bend_tm = h->a.bend_tm;
  for (int u = 0; u < 8; ++u) pp.dof_of[u] = (int)d->dofs[u] - 1;
  for (int k = 0; k < 8; ++k) pp.unk_of[k] = -1;
  for (int u = 0; u < 8; ++u)
    if (pp.dof_of[u] >= 0) pp.unk_of[pp.dof_of[u]] = u;
  for (int j = 0; j < 3; ++j) {  // get_m_motion_order (Mesh.jl:529-542)
    if (p->motion == MAFEM_STATIC) pp.mmo[j] = -1;
    else if (p->motion == MAFEM_LAG) pp.mmo[j] = pp.dof_of[j];
    else pp.mmo[j] = pp.dof_of[3 + j];
  }
  if (pp.dof_of[6] < 0) {
    set_global_error("λ must be an unknown (FiniteElement.jl:235)");
    return MAFEM_ERR_ARG;
  }
  pp.n_neu = (int)d->n_neu;
  for (int k = 0; k < pp.n_neu; ++k) {
    pp.neu_bdry[k] = (int)d->neu_bdry[k] - 1;
    pp.neu_type[k] = (int)d->neu_type[k];
    pp.neu_val[k] = d->neu_val[k];
  }

  // integer maps (0-based int32)
  std::vector<int> ix((size_t)numel * 9), lm((size_t)numel * nq), uel(numel), bref((size_t)numel * 4, -1);
  for (int e = 0; e < numel; ++e)
    for (int b = 0; b < 9; ++b) ix[e * 9 + b] = (int)(d->IX[b + 9 * (int64_t)e] - 1);
  for (int e = 0; e < numel; ++e)
    for (int b = 0; b < 9; ++b)
      for (int k = 0; k < ndf; ++k) lm[(size_t)e * nq + b * ndf + k] = (int)(d->ID[k + ndf * (int64_t)ix[e * 9 + b]] - 1);
  for (int e = 0; e < numel; ++e) uel[e] = (int)(d->uel_ids[e] - 1);
  std::vector<int> unk_node(n), unk_dof(n), node_unk((size_t)numnp * ndf, -1);
  for (int nd = 0; nd < numnp; ++nd)
    for (int k = 0; k < ndf; ++k) {
      int64_t g = d->ID[k + ndf * (int64_t)nd];
      if (g > 0) {
        if (g > n) {
          set_global_error("ID entry larger than nmdf");
          return MAFEM_ERR_ARG;
        }
        unk_node[g - 1] = nd;
        unk_dof[g - 1] = k;
        node_unk[(size_t)nd * ndf + k] = (int)(g - 1);
      }
    }
  // GP tables padded to kTab doubles per record
  std::vector<double> tab((size_t)d->n_uel * 9 * kTab, 0.0), db((size_t)d->n_uel * 81);
  for (int64_t u = 0; u < d->n_uel; ++u) {
    for (int g = 0; g < 9; ++g)
      std::memcpy(&tab[((size_t)u * 9 + g) * kTab], d->ufns + ((size_t)u * 9 + g) * 55, 55 * sizeof(double));
    db_matrix(d->ufns + (size_t)u * 9 * 55, &db[(size_t)u * 81]);
  }
  // boundary tables and the per-element boundary row map (Mesh.jl:126-131,
  // get_basis_fns(bdry, ...) Mesh.jl:390-403)
  std::vector<double> btab;
  int64_t boff[4];
  {
    int64_t rows = 0;
    for (int b = 0; b < 4; ++b) {
      boff[b] = rows;
      rows += d->bdry_n_uel[b];
    }
    btab.assign((size_t)std::max<int64_t>(rows, 1) * 3 * kTab, 0.0);
    for (int b = 0; b < 4; ++b)
      for (int64_t u = 0; u < d->bdry_n_uel[b]; ++u)
        for (int g = 0; g < 3; ++g)
          std::memcpy(&btab[((size_t)(boff[b] + u) * 3 + g) * kTab], d->bdry_ufns[b] + ((size_t)u * 3 + g) * 55,
                      55 * sizeof(double));
    const int n1 = (int)d->num1el, n2 = (int)d->num2el;
    for (int e2 = 0; e2 < n2; ++e2)
      for (int e1 = 0; e1 < n1; ++e1) {
        const int e = e1 + n1 * e2;
        auto set = [&](int b, int bel) {
          if (d->bdry_uel_ids[b] && d->bdry_n_uel[b] > 0) bref[e * 4 + b] = (int)(boff[b] + d->bdry_uel_ids[b][bel] - 1);
        };
        if (e2 == 0) set(0, e1);        // BOTTOM
        if (e1 == n1 - 1) set(1, e2);   // RIGHT
        if (e2 == n2 - 1) set(2, e1);   // TOP
        if (e1 == 0) set(3, e2);        // LEFT
      }
  }
  const int64_t kl = half_bandwidth(*d);
  const int nb = choose_nb((int)kl, precision);
  if (!nb) {
    set_global_error("half bandwidth too large for the banded LU's shared-memory panel");
    return MAFEM_ERR_UNSUPPORTED;
  }
  h->L = make_band_layout(n, (int)kl, (int)kl, nb);
  h->npan = (n + nb - 1) / nb;
  h->rmax = nb + (int)kl;

  cudaError_t ce = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
  if (ce != cudaSuccess) {
    set_global_error(std::string("cudaStreamCreate: ") + cudaGetErrorString(ce));
    return MAFEM_ERR_CUDA;
  }
  for (auto& e : h->ev) cudaEventCreate(&e);
  ce = cudaStreamCreateWithFlags(&h->st2, cudaStreamNonBlocking);
  if (ce != cudaSuccess) {
    set_global_error(std::string("cudaStreamCreate: ") + cudaGetErrorString(ce));
    mafem_destroy(hp.release());
    return MAFEM_ERR_CUDA;
  }
  h->ev_pool.resize((size_t)2 * h->npan + 2);
  for (auto& e : h->ev_pool) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  int* d_ix;
  int* d_lm;
  int* d_uel;
  int* d_bref;
  int *d_un, *d_ud, *d_nu;
  double *d_tab, *d_db, *d_btab;
#define UP(ptr, vec)                          \
  do {                                        \
    int r_ = dupload(h, &ptr, vec);           \
    if (r_) {                                 \
      set_global_error(h->err);               \
      mafem_destroy(hp.release());            \
      return r_;                              \
    }                                         \
  } while (0)
#define AL(ptr, cnt)                          \
  do {                                        \
    int r_ = dalloc(h, &ptr, cnt);            \
    if (r_) {                                 \
      set_global_error(h->err);               \
      mafem_destroy(hp.release());            \
      return r_;                              \
    }                                         \
  } while (0)
  UP(d_ix, ix);
  h->h_ix = ix;
  {  // inhomogeneous Dirichlet entries as prepare_input applies them (Input.jl:103-108)
    std::vector<int> didx;
    std::vector<double> dval;
    for (int64_t k = 0; k < d->n_dir; ++k) {
      const int64_t u = d->dir_unknown[k], nd = d->dir_node[k];
      if (u < 1 || u > 8 || nd < 1 || nd > numnp || pp.dof_of[u - 1] < 0) {
        set_global_error("Dirichlet entry with an unknown or node out of range");
        mafem_destroy(hp.release());
        return MAFEM_ERR_ARG;
      }
      didx.push_back(pp.dof_of[u - 1] * numnp + (int)(nd - 1));
      dval.push_back(d->dir_val[k]);
      if (p->scenario == MAFEM_F_PULL && p->motion == MAFEM_EUL && pp.dof_of[5] >= 0) {
        didx.push_back(pp.dof_of[5] * numnp + (int)(nd - 1));
        dval.push_back(d->dir_val[k]);
      }
    }
    h->n_dir = (int)didx.size();
    UP(h->d_dir_idx, didx);
    UP(h->d_dir_val, dval);
  }
  AL(h->d_pull_list, 25);
  AL(h->d_pull_r, (size_t)25 * nq);
  UP(d_lm, lm);
  UP(d_uel, uel);
  UP(d_bref, bref);
  UP(d_un, unk_node);
  UP(d_ud, unk_dof);
  UP(d_nu, node_unk);
  UP(d_tab, tab);
  UP(d_db, db);
  UP(d_btab, btab);
  // pivot blocks: the unknowns of one node (consecutive in the ID numbering)
  std::vector<int> blk_end(n);
  int maxblk = 1;
  for (int64_t q = 0; q < n;) {
    int64_t e = q;
    while (e < n && unk_node[e] == unk_node[q]) ++e;
    for (int64_t k = q; k < e; ++k) blk_end[k] = (int)e;
    maxblk = std::max(maxblk, (int)(e - q));
    q = e;
  }
  UP(h->d_blk_end, blk_end);
  {
    const int wmax = precision == MAFEM_PLAIN_FP64 ? blk_lu_setup<double>(h->L) : blk_lu_setup<float>(h->L);
    cudaGetLastError();
    if (wmax && maxblk <= wmax && blk_plan(blk_end, wmax, (int)h->L.ku, h->blk)) {
      UP(h->blk.d_ps, h->blk.ps);
      h->blk.d_blk_end = h->d_blk_end;
      h->use_blk = true;
      AL(h->d_flags, (size_t)h->blk.npan());
      AL(h->d_zbuf, (size_t)h->blk.npan() * kBlkW);
      AL(h->d_pinv, (size_t)h->blk.npan() * 2 * kBlkW * kBlkW);
      cudaMemset(h->d_flags, 0, (size_t)h->blk.npan() * sizeof(int));
      h->bwd_grid = precision == MAFEM_PLAIN_FP64 ? blk_backward_grid<double, double>() : blk_backward_grid<double, float>();
      h->bwd_max = h->bwd_grid;
      cudaGetLastError();
      const int pg = precision == MAFEM_PLAIN_FP64 ? blk_persist_setup<double>(h->L, h->blk, h->pers)
                                                   : blk_persist_setup<float>(h->L, h->blk, h->pers);
      cudaGetLastError();
      if (pg > 0) {
        const size_t np = (size_t)h->blk.npan();
        AL(h->pers.d_pdone, np);
        AL(h->pers.d_critcnt, np);
        AL(h->pers.d_a21cnt, np);
        cudaMemset(h->pers.d_pdone, 0, np * sizeof(int));
        cudaMemset(h->pers.d_critcnt, 0, np * sizeof(int));
        cudaMemset(h->pers.d_a21cnt, 0, np * sizeof(int));
      } else {
        h->pers.grid = 0;
      }
      const size_t nev = (size_t)2 * h->blk.npan() + 2;
      while (h->ev_pool.size() < nev) {
        cudaEvent_t e = nullptr;
        cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        h->ev_pool.push_back(e);
      }
    }
  }
  double *d_xms, *d_cps;
  AL(d_xms, (size_t)numnp * 3);
  AL(d_cps, (size_t)numnp * ndf);
  AL(h->d_rel, (size_t)numel * nq);
  AL(h->d_r, n);
  AL(h->d_x, n);
  AL(h->d_res, n);
  AL(h->d_dx, n);
  AL(h->d_part, 2048);
  AL(h->d_out, 16);
  AL(h->d_ipiv, n);
  AL(h->d_perm, std::max((size_t)h->npan * h->rmax, (size_t)h->blk.npan() * kBlkW));
  AL(h->d_rstate, 4);
  AL(h->d_info, 4);  // [0] zero-pivot column (1-based), [1] nonzero: a bounded device wait ran out
  cudaMemset(h->d_info, 0, 4 * sizeof(int));
  const size_t band_elems = (size_t)h->L.ldb * n;
  if (precision == MAFEM_PLAIN_FP64) {
    double *kel, *band, *rd;
    AL(kel, (size_t)numel * nq * nq);
    AL(band, band_elems);
    AL(rd, n);
    h->d_Kel = kel;
    h->d_band = band;
    h->d_rdiag = rd;
  } else {
    float *kel, *band, *band0, *rd;
    AL(kel, (size_t)numel * nq * nq);
    AL(band, band_elems);
    AL(band0, band_elems);
    AL(rd, n);
    h->d_Kel = kel;
    h->d_band = band;
    h->d_band0 = band0;
    h->d_rdiag = rd;
  }
  ce = cudaMallocHost(&h->h_out, 20 * sizeof(double));
  if (ce == cudaSuccess) h->h_rstate = reinterpret_cast<int*>(h->h_out + 16);
  if (ce != cudaSuccess) {
    set_global_error("cudaMallocHost failed");
    mafem_destroy(hp.release());
    return MAFEM_ERR_OOM;
  }
  // (the refinement residual reads every band window without bounds checks:
  // it needs nb >= 32 rows of padding)
  if (precision != MAFEM_PLAIN_FP64 && h->use_blk && h->L.nb >= 32) {
    const int dyn = patch_solve_setup();
    cudaGetLastError();
    if (dyn > 0 && patch_factor_smem(h->L.kl) <= (size_t)dyn && patch_refine_smem(n) <= (size_t)dyn) {
      AL(h->d_inv, (size_t)h->blk.npan() * 2 * kBlkW * kBlkW);
      PatchJob& J = h->job;
      J.a21_rows = patch_a21_rows(h->L.kl);
      AL(J.a21, (size_t)8 * 2 * J.a21_rows * 4);
      J.band = (float*)h->d_band;
      J.band0 = (const float*)h->d_band0;
      J.inv = h->d_inv;
      J.ps = h->blk.d_ps;
      J.blk_end = h->d_blk_end;
      J.perm = h->d_perm;
      J.rdiag = (float*)h->d_rdiag;
      J.info = h->d_info;
      J.stat = h->d_info + 2;
      J.rhs = h->d_r;
      J.x = h->d_x;
      J.res = h->d_res;
      J.xs = reinterpret_cast<float2*>(h->d_dx);  // d_dx: n doubles, unused by this form
      J.L = h->L;
      J.kuf = h->blk.kuf;
      J.npan = h->blk.npan();
      J.num1np = (int)d->num1np;
      J.num2np = (int)d->num2np;
      // first unknown of every control point, when the unknowns are numbered
      // control point by control point (the reference's ID numbering)
      std::vector<int> nf((size_t)numnp + 1, 0);
      bool mono = true;
      for (int64_t q = 0; q < n; ++q) {
        mono &= q == 0 || unk_node[q] >= unk_node[q - 1];
        ++nf[(size_t)unk_node[q] + 1];
      }
      for (int v = 0; v < numnp; ++v) nf[(size_t)v + 1] += nf[v];
      if (mono) {
        int* d_nf = nullptr;
        UP(d_nf, nf);
        J.node_first = d_nf;
        J.unk_node = d_un;
      }
      h->patch_ok = patch_a21_map(J);
    }
  }
  DevPatch& P = h->P;
  P.numel = numel; P.numnp = numnp; P.num1el = (int)d->num1el; P.num2el = (int)d->num2el;
  P.num1np = (int)d->num1np; P.num2np = (int)d->num2np; P.nmdf = n;
  P.kl = (int)kl; P.ku = (int)kl;
  P.ix = d_ix; P.lm = d_lm; P.uel = d_uel; P.tab = d_tab; P.db = d_db; P.bref = d_bref; P.btab = d_btab;
  P.unk_node = d_un; P.unk_dof = d_ud; P.node_unk = d_nu;
  P.xms = d_xms; P.cps = d_cps;
  cudaError_t e1, e2;
  if (precision == MAFEM_PLAIN_FP64) {
    e1 = band_lu_setup<double>(h->L, h->apply_threads);
    e2 = band_solve_setup<double, double>(h->L);
  } else {
    e1 = band_lu_setup<float>(h->L, h->apply_threads);
    e2 = band_solve_setup<float, double>(h->L);
  }
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    set_global_error(std::string("kernel attribute setup: ") + cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
    mafem_destroy(hp.release());
    return MAFEM_ERR_CUDA;
  }
  *out = hp.release();
  return MAFEM_OK;
}

extern "C" int mafem_destroy(mafem_handle* h) {
  if (!h) return MAFEM_OK;
  if (h->st) cudaStreamSynchronize(h->st);
  h->writer.reset();  // finishes the pending state files
  for (void* p : h->allocs) cudaFree(p);
  if (h->h_out) cudaFreeHost(h->h_out);
  if (h->st2) cudaStreamSynchronize(h->st2);
  for (auto& e : h->ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : h->ev_pool)
    if (e) cudaEventDestroy(e);
  if (h->st2) cudaStreamDestroy(h->st2);
  if (h->st) cudaStreamDestroy(h->st);
  delete h;
  return MAFEM_OK;
}

extern "C" const char* mafem_last_error(const mafem_handle* h) {
  if (h) return h->err.c_str();
  std::lock_guard<std::mutex> lk(g_err_mu);
  return g_err.c_str();
}

extern "C" int64_t mafem_device_bytes(const mafem_handle* h) { return h ? h->bytes : -1; }

extern "C" int mafem_upload_state(mafem_handle* h, const double* xms, const double* cps) {
  if (!h || !xms || !cps) return MAFEM_ERR_ARG;
  CK(cudaMemcpyAsync(h->P.xms, xms, sizeof(double) * 3 * h->numnp, cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(h->P.cps, cps, sizeof(double) * h->ndf * h->numnp, cudaMemcpyHostToDevice, h->st));
  CK(cudaStreamSynchronize(h->st));
  return MAFEM_OK;
}

extern "C" int mafem_download_state(mafem_handle* h, double* xms, double* cps) {
  if (!h) return MAFEM_ERR_ARG;
  if (xms) CK(cudaMemcpyAsync(xms, h->P.xms, sizeof(double) * 3 * h->numnp, cudaMemcpyDeviceToHost, h->st));
  if (cps) CK(cudaMemcpyAsync(cps, h->P.cps, sizeof(double) * h->ndf * h->numnp, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return MAFEM_OK;
}

// element kernel + gathers: r -> d_r, K -> d_band
static int assemble(mafem_handle* h, double time, double dt, bool both_bands = false) {
  cudaError_t e;
  if (h->precision == MAFEM_PLAIN_FP64) {
    e = launch_elem<double>(h->P, h->pp, time, dt, h->d_rel, (double*)h->d_Kel, h->st);
    if (e != cudaSuccess) {
      h->err = std::string("element kernel: ") + cudaGetErrorString(e);
      return MAFEM_ERR_CUDA;
    }
    launch_band_gather<double>(h->P, h->ndf, h->nq, h->L, (const double*)h->d_Kel, (double*)h->d_band, h->st);
    h->launches += 2;
  } else {
    e = launch_elem<float>(h->P, h->pp, time, dt, h->d_rel, (float*)h->d_Kel, h->st);
    if (e != cudaSuccess) {
      h->err = std::string("element kernel: ") + cudaGetErrorString(e);
      return MAFEM_ERR_CUDA;
    }
    launch_band_gather<float>(h->P, h->ndf, h->nq, h->L, (const float*)h->d_Kel, (float*)h->d_band, h->st,
                              both_bands ? (float*)h->d_band0 : nullptr);
    h->launches += 2;
  }
  launch_resid_gather(h->P, h->ndf, h->nq, h->d_rel, h->d_r, h->st);
  h->launches += 1;
  CK(cudaGetLastError());
  h->factored = false;
  return MAFEM_OK;
}

// Factorise the assembled band: node-block pivoting first; if a node block has
// no usable pivot, re-gather the band from the element blocks and factor it
// with full partial pivoting.  `x` (may be null) is the right-hand side that
// rides along the factorisation (forward substitution); `rhs0` restores it for
// the fallback.
// Launch the node-block factorisation (persistent kernel, or per-panel launches)
// without waiting for it; `info` tells later whether a block had no usable pivot.
// The panels' triangle inverses for the cooperative substitutions, stream-ordered
// after a node-block factorisation.
static void blk_after_factor(mafem_handle* h) {
  if (!h->d_pinv) return;
  if (h->precision == MAFEM_PLAIN_FP64)
    blk_inverses<double, double>((const double*)h->d_band, h->L, h->blk, (const double*)h->d_rdiag, h->d_pinv, h->st);
  else
    blk_inverses<double, float>((const float*)h->d_band, h->L, h->blk, (const float*)h->d_rdiag, h->d_pinv, h->st);
  h->launches += 1;
}

static int factor_enqueue(mafem_handle* h, double* x) {
  const bool fp64 = h->precision == MAFEM_PLAIN_FP64;
  CK(cudaMemsetAsync(h->d_info, 0, sizeof(int), h->st));
  bool launched = false;
  if (h->pers.grid > 0 && h->lu_path == MAFEM_LU_AUTO) {
    ++h->fepoch;
    const int nl = fp64 ? blk_lu_factor_persist<double>((double*)h->d_band, h->L, h->blk, h->pers, h->fepoch, h->d_perm,
                                                        (double*)h->d_rdiag, h->d_info, x, h->d_info + 1, h->st)
                        : blk_lu_factor_persist<float>((float*)h->d_band, h->L, h->blk, h->pers, h->fepoch, h->d_perm,
                                                       (float*)h->d_rdiag, h->d_info, nullptr, h->d_info + 1, h->st);
    if (nl < 0) {
      cudaGetLastError();
      h->pers.grid = 0;  // cooperative launch refused: per-panel launches from now on
    } else {
      h->launches += nl;
      launched = true;
    }
  }
  if (!launched) {
    const int nl = fp64 ? blk_lu_factor<double>((double*)h->d_band, h->L, h->blk, h->d_perm, (double*)h->d_rdiag,
                                                h->d_info, x, h->st, h->st2, h->ev_pool.data(), nullptr)
                        : blk_lu_factor<float>((float*)h->d_band, h->L, h->blk, h->d_perm, (float*)h->d_rdiag,
                                               h->d_info, nullptr, h->st, h->st2, h->ev_pool.data(), nullptr);
    h->launches += nl;
  }
  blk_after_factor(h);
  CK(cudaGetLastError());
  h->factored = true;
  h->last_blk = true;
  return MAFEM_OK;
}

// Factorise the assembled band: node-block pivoting first; if a node block has
// no usable pivot, re-gather the band from the element blocks and factor it
// with full partial pivoting.  `x` (may be null) is the right-hand side that
// rides along the factorisation (forward substitution); `rhs0` restores it for
// the fallback.
static int factor(mafem_handle* h, double* x, const double* rhs0) {
  const int64_t n = h->nmdf;
  const bool fp64 = h->precision == MAFEM_PLAIN_FP64;
  if (h->use_blk && h->lu_path != MAFEM_LU_FULL) {
    int rc = factor_enqueue(h, x);
    if (rc) return rc;
    int info2[2] = {0, 0};
    CK(cudaMemcpyAsync(info2, h->d_info, sizeof info2, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    const int info = info2[0];
    if (info2[1]) {
      h->err = "banded LU: a bounded wait for another CTA ran out";
      return MAFEM_ERR_CUDA;
    }
    if (info == 0) {
      h->factored = true;
      h->last_blk = true;
      return MAFEM_OK;
    }
    // fallback: rebuild the band from the element blocks (or the caller's band
    // of mafem_solve_band), then full pivoting
    ++h->fallbacks;
    if (fp64 && h->host_band)
      CK(cudaMemcpyAsync(h->d_band, h->host_band, (size_t)h->L.ldb * n * sizeof(double), cudaMemcpyHostToDevice,
                         h->st));
    else if (fp64)
      launch_band_gather<double>(h->P, h->ndf, h->nq, h->L, (const double*)h->d_Kel, (double*)h->d_band, h->st);
    else
      CK(cudaMemcpyAsync(h->d_band, h->d_band0, (size_t)h->L.ldb * n * sizeof(float), cudaMemcpyDeviceToDevice,
                         h->st));
    if (x && rhs0) CK(cudaMemcpyAsync(x, rhs0, n * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  }
  CK(cudaMemsetAsync(h->d_info, 0, sizeof(int), h->st));
  const int nl = fp64 ? band_lu_factor<double>((double*)h->d_band, h->L, h->d_ipiv, h->d_perm, h->rmax, h->d_info, x,
                                               h->apply_threads, h->apply_blocks, h->st, h->st2, h->ev_pool.data(),
                                               nullptr)
                      : band_lu_factor<float>((float*)h->d_band, h->L, h->d_ipiv, h->d_perm, h->rmax, h->d_info,
                                              nullptr, h->apply_threads, h->apply_blocks, h->st, h->st2,
                                              h->ev_pool.data(), nullptr);
  if (nl < 0) {
    h->err = "banded LU launch failed: " + std::string(cudaGetErrorString(cudaGetLastError()));
    return MAFEM_ERR_CUDA;
  }
  h->launches += nl;
  h->factored = true;
  h->last_blk = false;
  // full partial pivoting found no usable pivot either: the matrix is singular
  // (or not finite); report it before any solve uses the factors
  int zp = 0;
  CK(cudaMemcpyAsync(&zp, h->d_info, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  if (zp) {
    h->err = "zero pivot in column " + std::to_string(zp);
    return MAFEM_ZERO_PIVOT;
  }
  return MAFEM_OK;
}

// Back substitution with the node-block factors, in place on y (device).
template <class T>
static void blk_back_solve(mafem_handle* h, double* y, const int* gate = nullptr) {
  if (h->bwd_grid > 0) {
    ++h->epoch;
    if (blk_backward<double, T>((const T*)h->d_band, h->L, h->blk, h->d_pinv, y, h->d_flags, h->epoch,
                                h->d_info + 1, h->bwd_grid, h->st, h->wait_test, gate) == 0) {
      h->launches += 1;
      return;
    }
    cudaGetLastError();
    h->bwd_grid = 0;  // cooperative launch refused: use the single-CTA kernel from now on
  }
  blk_backward_1cta<double, T>((const T*)h->d_band, h->L, h->blk, (const T*)h->d_rdiag, y, h->st);
  h->launches += 1;
}

// Forward substitution with the node-block factors, in place on y (device):
// the cooperative multi-CTA kernel where the device allows it.
template <class T>
static void blk_fwd_solve(mafem_handle* h, double* y, const int* gate = nullptr) {
  if (h->bwd_grid > 0) {
    ++h->epoch;
    if (blk_forward_coop<double, T>((const T*)h->d_band, h->L, h->blk, h->d_perm, h->d_pinv, y, h->d_zbuf,
                                    h->d_flags, h->epoch, h->d_info + 1, h->bwd_grid, h->st, h->wait_test,
                                    gate) == 0) {
      h->launches += 1;
      return;
    }
    cudaGetLastError();
  }
  blk_forward<double, T>((const T*)h->d_band, h->L, h->blk, h->d_perm, (const T*)h->d_rdiag, y, h->st);
  h->launches += 1;
}

// info[0]: zero-pivot column, info[1]: a bounded device wait ran out (h_out + 5 holds both)
static int check_info(mafem_handle* h) {
  int info[2] = {0, 0};
  std::memcpy(info, h->h_out + 5, sizeof info);
  if (info[1]) {
    h->err = "back substitution: a bounded wait for another CTA ran out";
    return MAFEM_ERR_CUDA;
  }
  if (info[0]) {
    h->err = "zero pivot in column " + std::to_string(info[0]);
    return MAFEM_ZERO_PIVOT;
  }
  return MAFEM_OK;
}

// FP32 form: FP64 iterative refinement of K x = rhs with the FP32 factors, run
// on the device with a device-side stopping test.  refine_begin sets x = 0,
// res = rhs and the handle's refinement state {done, sweeps, status};
// refine_sweeps enqueues `count` sweeps (d = LU^-1 res, x += d, res = rhs - A0 x
// in FP64), each ending with a check kernel that updates the state; the kernels
// of a sweep read `done` first and return at once once it is set.  The stopping
// rule: |rhs - A0 x| <= tol |rhs| (this solver is also the fallback of the
// batched solve when that one stalls on an ill-conditioned tangent, where a
// small correction says nothing about the error of x); stall after the fourth
// sweep if |r| > |r_prev| / 2; max_refine sweeps at most.
static void refine_begin(mafem_handle* h, const double* rhs_dev) {
  const int64_t n = h->nmdf;
  cudaMemsetAsync(h->d_x, 0, n * sizeof(double), h->st);
  launch_band_residual<float>((const float*)h->d_band0, h->L, h->d_x, rhs_dev, h->d_res, h->d_part, h->d_out + 4,
                              h->st);  // res = rhs, |rhs|
  launch_refine_init(h->d_out + 4, h->d_rstate, h->d_out + 12, h->st);
  h->launches += 3;
}
static void refine_sweeps(mafem_handle* h, const double* rhs_dev, int count) {
  const int64_t n = h->nmdf;
  int* gate = h->d_rstate;
  for (int k = 0; k < count; ++k) {
    launch_copy_gated(n, h->d_res, h->d_dx, gate, h->st);
    if (h->last_blk) {
      blk_fwd_solve<float>(h, h->d_dx, gate);
      blk_back_solve<float>(h, h->d_dx, gate);
    } else {  // full partial pivoting: single-CTA substitutions (ungated: they only rewrite d_dx)
      band_forward<float, double>((const float*)h->d_band, h->L, h->d_perm, h->rmax, h->d_dx, h->st);
      band_backward<float, double>((const float*)h->d_band, h->L, h->d_dx, h->st);
      h->launches += 2;
    }
    launch_axpy_norms(n, h->d_dx, h->d_x, h->d_part, h->d_out + 8, h->st, gate);
    launch_band_residual<float>((const float*)h->d_band0, h->L, h->d_x, rhs_dev, h->d_res, h->d_part, h->d_out + 3,
                                h->st, gate);
    launch_refine_check(h->d_out + 3, h->d_out + 8, gate, h->d_out + 12, h->refine_tol, h->max_refine, h->st);
    h->launches += 6;
  }
}

// Solve K x = rhs (rhs in d_x on entry for the plain form; x in d_x on exit).
// Factors the band if needed.  Returns the number of refinement sweeps in *sweeps.
static int factor_and_solve(mafem_handle* h, const double* rhs_dev, int* sweeps) {
  const int64_t n = h->nmdf;
  *sweeps = 0;
  if (h->precision == MAFEM_PLAIN_FP64) {
    CK(cudaMemcpyAsync(h->d_x, rhs_dev, n * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    if (!h->factored) {
      int rc = factor(h, h->d_x, rhs_dev);
      if (rc) return rc;
    } else if (h->last_blk) {
      blk_fwd_solve<double>(h, h->d_x);
    } else {
      band_forward<double, double>((const double*)h->d_band, h->L, h->d_perm, h->rmax, h->d_x, h->st);
      h->launches += 1;
    }
    cudaEventRecord(h->ev[2], h->st);
    if (h->last_blk) {
      blk_back_solve<double>(h, h->d_x);
    } else {
      band_backward<double, double>((const double*)h->d_band, h->L, h->d_x, h->st);
      h->launches += 1;
    }
    CK(cudaGetLastError());
    return MAFEM_OK;
  }
  // FP32 factor of the FP32 tangent, FP64 iterative refinement
  if (!h->factored) {
    CK(cudaMemcpyAsync(h->d_band0, h->d_band, (size_t)h->L.ldb * n * sizeof(float), cudaMemcpyDeviceToDevice, h->st));
    int rc = factor(h, nullptr, nullptr);
    if (rc) return rc;
  }
  cudaEventRecord(h->ev[2], h->st);
  constexpr int kRefineChunk = 3;
  refine_begin(h, rhs_dev);
  int state[3] = {0, 0, MAFEM_OK};
  for (int chunk = 0; !state[0]; ++chunk) {
    refine_sweeps(h, rhs_dev, kRefineChunk);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h->h_rstate, h->d_rstate, 3 * sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    std::memcpy(state, h->h_rstate, sizeof state);
    if (!state[0] && state[1] >= h->max_refine) break;  // cannot happen: the check stops at max_sweeps
  }
  *sweeps = state[1];
  if (state[2] == MAFEM_NAN_DETECTED) {
    h->err = "non-finite refinement residual or correction";
    return MAFEM_NAN_DETECTED;
  }
  if (state[2] == MAFEM_REFINE_STALLED) {
    h->err = "iterative refinement stalled or did not reach its tolerance in " + std::to_string(state[1]) + " sweeps";
    return MAFEM_REFINE_STALLED;
  }
  return MAFEM_OK;
}

extern "C" int mafem_calc_r_K(mafem_handle* h, double time, double dt, double* r_out, double* band_out,
                              int64_t ldab_out) {
  if (!h) return MAFEM_ERR_ARG;
  const BandLayout& L = h->L;
  if (band_out && ldab_out < 2LL * L.kl + L.ku + 1) {
    h->err = "ldab_out must be >= 2*kl + ku + 1";
    return MAFEM_ERR_ARG;
  }
  int rc = assemble(h, time, dt);
  if (rc) return rc;
  if (r_out) CK(cudaMemcpyAsync(r_out, h->d_r, h->nmdf * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  if (band_out) {
    const size_t rows = 2 * (size_t)L.kl + L.ku + 1;
    if (h->precision == MAFEM_PLAIN_FP64) {
      CK(cudaMemcpy2DAsync(band_out, ldab_out * sizeof(double), (const double*)h->d_band + L.nb, L.ldb * sizeof(double),
                           rows * sizeof(double), L.n, cudaMemcpyDeviceToHost, h->st));
      CK(cudaStreamSynchronize(h->st));
    } else {
      std::vector<float> tmp((size_t)L.ldb * L.n);
      CK(cudaMemcpyAsync(tmp.data(), h->d_band, tmp.size() * sizeof(float), cudaMemcpyDeviceToHost, h->st));
      CK(cudaStreamSynchronize(h->st));
      for (int64_t j = 0; j < L.n; ++j)
        for (size_t r = 0; r < rows; ++r) band_out[j * ldab_out + r] = tmp[(size_t)j * L.ldb + L.nb + r];
    }
  }
  CK(cudaStreamSynchronize(h->st));
  return MAFEM_OK;
}

extern "C" int mafem_solve(mafem_handle* h, const double* r, double* du_out) {
  if (!h || !r || !du_out) return MAFEM_ERR_ARG;
  const int64_t n = h->nmdf;
  CK(cudaMemsetAsync(h->d_info, 0, 2 * sizeof(int), h->st));
  CK(cudaMemcpyAsync(h->d_res, r, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
  // keep the right-hand side in d_dx for the plain path (factor_and_solve reads rhs_dev)
  double* rhs = h->precision == MAFEM_PLAIN_FP64 ? h->d_dx : h->d_r;
  if (h->precision != MAFEM_PLAIN_FP64) {
    // d_r is the assembled residual; the refinement uses d_res as workspace, so
    // stage the caller's rhs in d_r only for this call
    CK(cudaMemcpyAsync(h->d_r, h->d_res, n * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  } else {
    CK(cudaMemcpyAsync(h->d_dx, h->d_res, n * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  }
  int sweeps = 0;
  int rc = factor_and_solve(h, rhs, &sweeps);
  if (rc) return rc;
  CK(cudaMemcpyAsync(du_out, h->d_x, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(h->h_out + 5, h->d_info, 2 * sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  for (int64_t i = 0; i < n; ++i) du_out[i] = -du_out[i];
  return check_info(h);
}

extern "C" int mafem_predict(mafem_handle* h, double dt) {
  if (!h) return MAFEM_ERR_ARG;
  launch_predictor(h->P, h->pp, dt, h->st);
  h->launches += 1;
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(h->st));
  return MAFEM_OK;
}

// Whether the assembled residual d_r is finite (one norm, waits for the stream).
static bool residual_finite(mafem_handle* h) {
  launch_axpy_norms(h->nmdf, h->d_r, h->d_res, h->d_part, h->d_out + 10, h->st);  // |r| (d_res is scratch here)
  double nr[2] = {0.0, 0.0};
  if (cudaMemcpyAsync(nr, h->d_out + 10, sizeof nr, cudaMemcpyDeviceToHost, h->st) != cudaSuccess ||
      cudaStreamSynchronize(h->st) != cudaSuccess)
    return true;
  return std::isfinite(nr[0]);
}

// Refinement sweeps enqueued per Newton iteration of the FP32 form when the
// iteration runs without a host wait (the refinement stops within 2-5 sweeps
// on the benchmark tangents at the default tolerance).
constexpr int kAsyncSweeps = 8;

// ---- a time step as step_begin / iter_enqueue / iter_finish: mafem_time_step
// runs them for one handle, mafem_batch_step interleaves many handles ----

static void step_begin(mafem_handle* h, double time, double dt) {
  h->ss_time = time;
  h->ss_dt = dt;
  h->ss_iter = 1;
  h->ss_eps = INFINITY;
  std::memset(&h->ss_S, 0, sizeof h->ss_S);
  cudaEventRecord(h->ev[5], h->st);
}

// Enqueue Newton iteration ss_iter (FiniteElement.jl:29-57).  The plain FP64
// node-block path does not wait for its factorisation: a block without a
// usable pivot shows in `info`, the update kernel then leaves the state
// unchanged, and iter_finish redoes the iteration with full pivoting.  The
// other forms run factor_and_solve, which waits where it must.
static int iter_enqueue(mafem_handle* h) {
  const int64_t n = h->nmdf;
  h->ss_patch = false;
  CK(cudaMemsetAsync(h->d_info, 0, 2 * sizeof(int), h->st));  // zero-pivot column, wait-ran-out word
  cudaEventRecord(h->ev[0], h->st);
  int rc = assemble(h, h->ss_time, h->ss_dt);
  if (rc) return rc;
  cudaEventRecord(h->ev[1], h->st);
  h->ss_sweeps = 0;
  h->ss_async = h->use_blk && h->lu_path != MAFEM_LU_FULL && !h->no_async;
  if (h->ss_async && h->precision == MAFEM_PLAIN_FP64) {
    CK(cudaMemcpyAsync(h->d_x, h->d_r, n * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    if ((rc = factor_enqueue(h, h->d_x)) != MAFEM_OK) return rc;
    cudaEventRecord(h->ev[2], h->st);
    blk_back_solve<double>(h, h->d_x);
  } else if (h->ss_async) {
    // FP32 form without a host wait: factor, then a fixed number of gated
    // refinement sweeps (those after convergence return at once); a node block
    // without a usable pivot, or a refinement that did not converge within
    // them, leaves the state unchanged and iter_finish redoes or reports it
    CK(cudaMemcpyAsync(h->d_band0, h->d_band, (size_t)h->L.ldb * n * sizeof(float), cudaMemcpyDeviceToDevice,
                       h->st));
    if ((rc = factor_enqueue(h, nullptr)) != MAFEM_OK) return rc;
    cudaEventRecord(h->ev[2], h->st);
    refine_begin(h, h->d_r);
    refine_sweeps(h, h->d_r, std::min(h->max_refine, kAsyncSweeps));
    launch_refine_seal(h->d_rstate, h->st);
    h->launches += 1;
  } else if ((rc = factor_and_solve(h, h->d_r, &h->ss_sweeps)) != MAFEM_OK) {
    // a singular or stalled solve of a non-finite system: report the NaN (the
    // residual itself is not finite), as the other paths do
    if (rc > 0 && !residual_finite(h)) {
      h->err = "non-finite residual";
      return MAFEM_NAN_DETECTED;
    }
    return rc;
  }
  cudaEventRecord(h->ev[3], h->st);
  const bool fp32_async = h->ss_async && h->precision != MAFEM_PLAIN_FP64;
  launch_newton_update(h->P, h->pp, h->ss_dt, h->d_x, h->d_r, h->d_part, h->d_out, h->st, h->d_info,
                       h->d_info + 1, fp32_async ? h->d_rstate + 3 : nullptr);
  h->launches += 2;
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(h->h_out, h->d_out, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(h->h_out + 5, h->d_info, 4 * sizeof(int), cudaMemcpyDeviceToHost, h->st));
  if (fp32_async) CK(cudaMemcpyAsync(h->h_rstate, h->d_rstate, 4 * sizeof(int), cudaMemcpyDeviceToHost, h->st));
  cudaEventRecord(h->ev[4], h->st);
  return MAFEM_OK;
}

// Batched FP32 form, first half of a Newton iteration: assembly into both
// bands (the factorisation overwrites one, the refinement multiplies by the
// other).  The batch then factors and solves every patch in one launch each
// (patch_solve) and iter_enqueue_patch_end applies the update.
static int iter_enqueue_patch_begin(mafem_handle* h) {
  h->ss_patch = true;
  h->ss_async = false;
  h->ss_sweeps = 0;
  cudaEventRecord(h->ev[0], h->st);
  int rc = assemble(h, h->ss_time, h->ss_dt, true);
  if (rc) return rc;
  CK(cudaMemsetAsync(h->d_info, 0, 4 * sizeof(int), h->st));
  cudaEventRecord(h->ev[1], h->st);
  return MAFEM_OK;
}

static int iter_enqueue_patch_end(mafem_handle* h, cudaEvent_t solved) {
  CK(cudaStreamWaitEvent(h->st, solved, 0));
  cudaEventRecord(h->ev[2], h->st);
  cudaEventRecord(h->ev[3], h->st);
  // the update is skipped when the patch solve failed (status word nonzero)
  launch_newton_update(h->P, h->pp, h->ss_dt, h->d_x, h->d_r, h->d_part, h->d_out, h->st, h->d_info + 2,
                       h->d_info + 1);
  h->launches += 2;
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(h->h_out, h->d_out, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(h->h_out + 5, h->d_info, 4 * sizeof(int), cudaMemcpyDeviceToHost, h->st));
  cudaEventRecord(h->ev[4], h->st);
  return MAFEM_OK;
}

static void accum_times(mafem_handle* h) {
  float ms_a = 0, ms_f = 0, ms_s = 0;
  cudaEventElapsedTime(&ms_a, h->ev[0], h->ev[1]);
  cudaEventElapsedTime(&ms_f, h->ev[1], h->ev[2]);
  cudaEventElapsedTime(&ms_s, h->ev[2], h->ev[4]);
  h->ss_S.ms_assemble += ms_a;
  h->ss_S.ms_factor += ms_f;
  h->ss_S.ms_solve += ms_s;
}

enum { kIterAgain = -100, kIterDone = -101 };

// Wait for the enqueued iteration and apply the Newton criterion: kIterAgain,
// kIterDone (converged), or a status.
static int iter_decide(mafem_handle* h);
static int iter_finish(mafem_handle* h) {
  CK(cudaEventSynchronize(h->ev[4]));
  accum_times(h);
  return iter_decide(h);
}
// The Newton criterion on the iteration's results in h_out (eps, |r|, the
// non-finite flag and the info words), redoing the iteration with the
// handle's own solver where the solve failed.
static int iter_decide(mafem_handle* h) {
  if (!std::isfinite(h->h_out[1])) {  // the FP64 residual itself is not finite: nothing to redo
    h->err = "non-finite residual";
    return MAFEM_NAN_DETECTED;
  }
  if (h->ss_patch) {
    int ps[4];
    std::memcpy(ps, h->h_out + 5, sizeof ps);
    h->ss_sweeps = ps[3];
    if (ps[1] != 0) {
      h->err = "batched FP32 factorisation: a bounded wait ran out";
      return MAFEM_ERR_CUDA;
    }
    if (ps[2] != MAFEM_OK) {
      // the patch solve found no usable pivot in a node block, or its
      // refinement failed: the update was skipped; redo this iteration with
      // the handle's own solve (full partial pivoting where needed)
      ++h->fallbacks;
      const int sw = h->ss_sweeps;
      const int rc = iter_enqueue(h);
      if (rc) return rc;
      CK(cudaEventSynchronize(h->ev[4]));
      accum_times(h);
      h->ss_sweeps += sw;
    }
  }
  int info[2] = {0, 0};
  std::memcpy(info, h->h_out + 5, sizeof info);
  if (info[1] == 0 && info[0] != 0 && h->ss_async) {
    // a node block without a usable pivot: the update was skipped; redo this
    // iteration with full partial pivoting
    ++h->fallbacks;
    const int saved = h->lu_path;
    h->lu_path = MAFEM_LU_FULL;
    const int rc = iter_enqueue(h);
    h->lu_path = saved;
    if (rc) return rc;
    CK(cudaEventSynchronize(h->ev[4]));
    accum_times(h);
  }
  if (h->ss_async && h->precision != MAFEM_PLAIN_FP64 && info[0] == 0 && info[1] == 0) {
    int rs[4];
    std::memcpy(rs, h->h_rstate, sizeof rs);
    h->ss_sweeps = rs[1];
    if (rs[3]) {  // the update was skipped: the refinement did not succeed within its sweeps
      if (rs[2] == MAFEM_NAN_DETECTED) {
        h->err = "non-finite refinement residual or correction";
        return MAFEM_NAN_DETECTED;
      }
      // still converging (or stalled): redo the iteration with the waiting
      // solver, which runs up to max_refine sweeps and reports a stall
      ++h->fallbacks;
      const int sw = h->ss_sweeps;
      h->no_async = true;
      const int rc = iter_enqueue(h);
      h->no_async = false;
      if (rc) return rc;
      CK(cudaEventSynchronize(h->ev[4]));
      accum_times(h);
      h->ss_sweeps += sw;
    }
  }
  mafem_step_stats& S = h->ss_S;
  const int iter = h->ss_iter;
  S.refine_iters += h->ss_sweeps;
  const double eps = h->h_out[0];
  h->ss_eps = eps;
  S.eps[iter - 1] = eps;
  S.res_norm[iter - 1] = h->h_out[1];
  S.newton_iters = iter;
  int rc = check_info(h);
  if (rc != MAFEM_OK) return rc;
  if (h->h_out[2] != 0.0 || !std::isfinite(eps)) {
    h->err = "non-finite residual or Newton update";
    return MAFEM_NAN_DETECTED;
  }
  h->ss_iter = iter + 1;
  if (eps < h->p.eps_nr) return kIterDone;
  if (h->ss_iter >= 15) {  // FiniteElement.jl:29,61
    h->err = "did not reach Newton--Raphson tolerance";
    return MAFEM_NEWTON_NOT_CONVERGED;
  }
  return kIterAgain;
}

static void step_stats(mafem_handle* h, mafem_step_stats* stats, cudaEvent_t end = nullptr) {
  float ms_t = 0;
  cudaEventElapsedTime(&ms_t, h->ev[5], end ? end : h->ev[4]);
  h->ss_S.ms_total = ms_t;
  if (stats) *stats = h->ss_S;
}

extern "C" int mafem_time_step(mafem_handle* h, double time, double dt, mafem_step_stats* stats) {
  if (!h) return MAFEM_ERR_ARG;
  step_begin(h, time, dt);
  int rc;
  do {
    rc = iter_enqueue(h);
    if (rc != MAFEM_OK) return rc;
    rc = iter_finish(h);
  } while (rc == kIterAgain);
  step_stats(h, stats);
  return rc == kIterDone ? MAFEM_OK : rc;
}

extern "C" int mafem_set_launch_ctas(mafem_handle* h, int32_t ctas) {
  if (!h || ctas < 0) return MAFEM_ERR_ARG;
  if (h->pers.max_grid > 0)
    h->pers.grid = ctas == 0 ? h->pers.max_grid : std::max(h->pers.min_grid, std::min(ctas, h->pers.max_grid));
  if (h->bwd_max > 0) h->bwd_grid = ctas == 0 ? h->bwd_max : std::max(1, std::min((int)ctas, h->bwd_max));
  return h->pers.max_grid > 0 ? h->pers.grid : h->bwd_grid;
}

// Order of a round's batched solves: the patches factored on four-CTA
// clusters first, then those on two-CTA clusters, then the single-CTA ones,
// each group largest first.  Returns the size of the first group in *n4 and of
// the second in *n2.
// CTAs that factor the handle's patch in the batched FP32 form: the caller's
// choice, else the autotuner's for this round, else by band width
static int patch_ctas(const mafem_handle* h) {
  return h->patch_nr ? h->patch_nr : h->round_nr ? h->round_nr : patch_cluster_ctas(h->blk.kuf);
}

// ---- autotuner of the batched FP32 factorisation's cluster sizes ----------------------
// The time of factoring one patch on 1, 2 and 4 CTAs is measured once per
// device and patch shape (synthetic band, CUDA events) and cached for the
// process.  Each round then picks a cluster size per shape: more CTAs shorten a
// patch's factorisation but cost more SM-time (on a 48 x 48 patch about 1.5x
// faster on 2 CTAs and 2.4x on 4), so a round with many patches wants small
// clusters and a round with few large ones big clusters.
namespace {
using PatchShape = std::tuple<int, int64_t, int, int, int>;  // device, n, kl, kuf, panels
std::mutex g_tune_mu;
std::map<PatchShape, std::array<float, 3>> g_tune;  // ms on 1, 2, 4 CTAs
int g_num_sms = 0;
PatchShape patch_shape(const mafem_handle* h) {
  int dev = 0;
  cudaGetDevice(&dev);
  return PatchShape{dev, h->L.n, h->L.kl, h->blk.kuf, h->blk.npan()};
}
}  // namespace

// Measure the cluster-size times of h's patch shape if not cached yet, with
// h's job (d_jobs[slot]) on stream st; d_tmp: one device int.  The job's band is
// overwritten (the next assembly rewrites it).
static int patch_tune(mafem_handle* h, const PatchJob* d_jobs, int slot, int* d_tmp, cudaStream_t st) {
  const PatchShape key = patch_shape(h);
  {
    std::lock_guard<std::mutex> g(g_tune_mu);
    if (g_tune.count(key)) return MAFEM_OK;
  }
  std::array<float, 3> ms{};
  CK(cudaMemcpyAsync(d_tmp, &slot, sizeof(int), cudaMemcpyHostToDevice, st));
  const int nrs[3] = {1, 2, 4};
  for (int k = 0; k < 3; ++k) {
    const cudaError_t e = patch_time_factor(d_jobs, d_tmp, nrs[k], patch_factor_smem(h->L.kl), st, &ms[k]);
    if (e != cudaSuccess) {
      h->err = std::string("factorisation autotuning: ") + cudaGetErrorString(e);
      return MAFEM_ERR_CUDA;
    }
  }
  CK(cudaMemsetAsync(h->d_info, 0, 4 * sizeof(int), st));
  CK(cudaStreamSynchronize(st));
  h->factored = false;
  std::lock_guard<std::mutex> g(g_tune_mu);
  g_tune[key] = ms;
  if (!g_num_sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
  }
  return MAFEM_OK;
}

// Cluster size per patch shape for the round's jobs hv[idx]: the choice in
// {1, 2, 4} per shape that minimises the estimated makespan
//   max(longest factorisation, sum of jobs x CTAs x time / SMs)
// (exhaustive over up to 8 shapes, the rest by band width).  Patches whose
// caller fixed the size, or whose shape has no times, keep theirs.
static void choose_patch_ctas(std::vector<mafem_handle*>& hv, const std::vector<int>& idx) {
  std::map<PatchShape, int> count;
  std::vector<std::pair<PatchShape, std::array<float, 3>>> shapes;
  {
    std::lock_guard<std::mutex> g(g_tune_mu);
    for (int k : idx) {
      mafem_handle* h = hv[k];
      h->round_nr = 0;
      if (h->patch_nr) continue;
      const PatchShape key = patch_shape(h);
      auto it = g_tune.find(key);
      if (it == g_tune.end()) continue;
      if (count[key]++ == 0 && shapes.size() < 8) shapes.push_back(*it);
    }
  }
  if (shapes.empty() || g_num_sms <= 0) return;
  const int ns = (int)shapes.size();
  const int nrs[3] = {1, 2, 4};
  std::vector<int> pick(ns, 0), best(ns, 0);
  double best_t = INFINITY;
  int combos = 1;
  for (int c = 0; c < ns; ++c) combos *= 3;
  for (int code = 0; code < combos; ++code) {
    int x = code;
    double lg[3] = {0.0, 0.0, 0.0}, work = 0.0;  // longest factorisation per group (1, 2, 4 CTAs)
    for (int c = 0; c < ns; ++c) {
      pick[c] = x % 3;
      x /= 3;
      const double t = shapes[c].second[pick[c]];
      lg[pick[c]] = std::max(lg[pick[c]], t);
      work += count[shapes[c].first] * nrs[pick[c]] * t;
    }
    // patch_solve runs the first non-empty group (4, 2, 1 CTAs) on one stream
    // and the others one after the other on a second
    const int first = lg[2] > 0.0 ? 2 : lg[1] > 0.0 ? 1 : 0;
    double rest = 0.0;
    for (int g = 0; g < 3; ++g)
      if (g != first) rest += lg[g];
    const double est = std::max(std::max(lg[first], rest), work / g_num_sms);
    if (est < best_t - 1e-9) {
      best_t = est;
      best = pick;
    }
  }
  std::map<PatchShape, int> nr;
  for (int c = 0; c < ns; ++c) nr[shapes[c].first] = nrs[best[c]];
  for (int k : idx) {
    mafem_handle* h = hv[k];
    if (h->patch_nr) continue;
    auto it = nr.find(patch_shape(h));
    if (it != nr.end()) h->round_nr = it->second;
  }
}

// ---- autotuner of the batched FP32 tangent kernel's elements per CTA -------------------
// Two or four elements per CTA: four share a CTA's launch overhead, two fit
// more CTAs on an SM (the kernel holds over 100 registers per thread).  The
// time of each is measured once per device, motion and element size on the
// first patch of that kind (CUDA events, the fastest of three launches after
// one untimed) and the faster is cached for the process.
namespace {
using TanShape = std::tuple<int, int, int>;  // device, motion, nq
std::map<TanShape, int> g_tan_epb;           // guarded by g_tune_mu
std::map<TanShape, std::array<float, 2>> g_tan_ms;  // ms with 2 and 4 elements per CTA
TanShape tan_shape(const mafem_handle* h) {
  int dev = 0;
  cudaGetDevice(&dev);
  return TanShape{dev, h->pp.motion, h->pp.nq};
}
}  // namespace

static int tan_epb(const mafem_handle* h) {
  std::lock_guard<std::mutex> g(g_tune_mu);
  auto it = g_tan_epb.find(tan_shape(h));
  return it == g_tan_epb.end() ? 4 : it->second;
}

// Tunes h's kind of patch if not cached yet, with h's job (slot of d_ajobs)
// alone in a one-item round written to h_buf (pinned) and d_buf (at least
// round_layout(1).bytes each) on stream st, which it synchronises.  The
// patch's element tangents are overwritten (the next assembly rewrites them).
static int tan_tune(mafem_handle* h, const AsmJob* d_ajobs, int slot, unsigned char* d_buf, unsigned char* h_buf,
                    cudaStream_t st);

static void order_patch_jobs(std::vector<mafem_handle*>& hv, std::vector<int>& idx, int* n4, int* n2) {
  auto nr = [&](int k) { return patch_ctas(hv[k]); };
  auto cost = [&](int k) { return (double)hv[k]->blk.npan() * hv[k]->L.kl * hv[k]->blk.kuf; };
  std::sort(idx.begin(), idx.end(), [&](int a, int b) {
    if (nr(a) != nr(b)) return nr(a) > nr(b);
    return cost(a) > cost(b);
  });
  *n4 = *n2 = 0;
  for (int k : idx) {
    *n4 += nr(k) == 4 ? 1 : 0;
    *n2 += nr(k) == 2 ? 1 : 0;
  }
}

// A batched round's host/device buffer: the items (patches of the round in
// motion groups), then per kernel kind the CTA offsets off[0 .. m] --
// 0 residual, 1 tangent, 2 band gather, 3 residual gather, 4 update, 5 predictor.
namespace {
constexpr int kOffKinds = 6;
struct RoundLayout {
  size_t off[kOffKinds];
  size_t bytes;
};
RoundLayout round_layout(int m) {
  RoundLayout R{};
  size_t p = ((size_t)m * sizeof(AsmItem) + 15) & ~(size_t)15;
  for (int t = 0; t < kOffKinds; ++t) {
    R.off[t] = p;
    p = (p + (size_t)(m + 1) * sizeof(int) + 15) & ~(size_t)15;
  }
  R.bytes = p;
  return R;
}
constexpr int kOffDir = kOffKinds;  // 6: Dirichlet scaling (a seventh offset array)

// One stream of batched Newton rounds (a batch has one, a server one per
// solve lane): its streams, round buffers, result rows, timing events and the
// CUDA graphs of the rounds it has run.
struct RoundRunner {
  cudaStream_t st = nullptr, st2 = nullptr;  // clusters / single CTAs of the factorisation
  cudaEvent_t efork = nullptr, ejoin = nullptr;
  cudaEvent_t rev[4] = {};  // start, assembled, solved, done
  unsigned char* d_round = nullptr;
  unsigned char* h_round = nullptr;  // pinned
  AsmOut* d_outs = nullptr;
  AsmOut* h_outs = nullptr;  // pinned
  int* d_order = nullptr;
  int* h_order = nullptr;  // pinned
  int cap = 0;              // patches per round at most
  bool graph_on = true;
  std::map<std::vector<int64_t>, cudaGraphExec_t> graphs;
  int64_t graph_launches = 0, graph_captures = 0;
  std::vector<int> items_of;  // the last round's result rows: index of each row's handle
  bool busy = false;

  RoundRunner() = default;
  RoundRunner(const RoundRunner&) = delete;  // owns its streams, events, buffers and graphs
  RoundRunner& operator=(const RoundRunner&) = delete;
  cudaError_t init(int max_patches) {
    cap = max_patches;
    const size_t rb = round_layout(cap).bytes + (size_t)(cap + 1) * sizeof(int) + 16;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&efork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ejoin, cudaEventDisableTiming);
    for (int k = 0; k < 4 && e == cudaSuccess; ++k) e = cudaEventCreate(&rev[k]);
    if (e == cudaSuccess) e = cudaMalloc(&d_round, rb);
    if (e == cudaSuccess) e = cudaMallocHost(&h_round, rb);
    if (e == cudaSuccess) e = cudaMalloc(&d_outs, (size_t)cap * sizeof(AsmOut));
    if (e == cudaSuccess) e = cudaMallocHost(&h_outs, (size_t)cap * sizeof(AsmOut));
    if (e == cudaSuccess) e = cudaMalloc(&d_order, (size_t)cap * sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost(&h_order, (size_t)cap * sizeof(int));
    return e;
  }
  ~RoundRunner() {
    if (st) cudaStreamSynchronize(st);
    if (st2) cudaStreamSynchronize(st2);
    for (auto& g : graphs) cudaGraphExecDestroy(g.second);
    for (cudaEvent_t e : {efork, ejoin, rev[0], rev[1], rev[2], rev[3]})
      if (e) cudaEventDestroy(e);
    if (d_round) cudaFree(d_round);
    if (h_round) cudaFreeHost(h_round);
    if (d_outs) cudaFree(d_outs);
    if (h_outs) cudaFreeHost(h_outs);
    if (d_order) cudaFree(d_order);
    if (h_order) cudaFreeHost(h_order);
    if (st2) cudaStreamDestroy(st2);
    if (st) cudaStreamDestroy(st);
  }
};

}  // namespace

// The batched-round view of a handle's FP32 patch (its job in a round).
static AsmJob asm_job(const mafem_handle* h) {
  AsmJob a{};
  a.P = h->P;
  a.pp = h->pp;
  a.L = h->L;
  a.r_el = h->d_rel;
  a.K_el = (float*)h->d_Kel;
  a.band = (float*)h->d_band;
  a.band0 = (float*)h->d_band0;
  a.r = h->d_r;
  a.x = h->d_x;
  a.part = h->d_part;
  a.out = h->d_out;
  a.info = h->d_info;
  a.dir_idx = h->d_dir_idx;
  a.dir_val = h->d_dir_val;
  a.n_dir = h->n_dir;
  return a;
}

static int tan_tune(mafem_handle* h, const AsmJob* d_ajobs, int slot, unsigned char* d_buf, unsigned char* h_buf,
                    cudaStream_t st) {
  const TanShape key = tan_shape(h);
  {
    std::lock_guard<std::mutex> g(g_tune_mu);
    if (g_tan_epb.count(key)) return MAFEM_OK;
  }
  const RoundLayout RL = round_layout(1);
  AsmItem* item = reinterpret_cast<AsmItem*>(h_buf);
  item->job = slot;
  item->start = 0;
  item->time = h->ss_time;
  item->dt = h->ss_dt > 0.0 ? h->ss_dt : 1e-3;
  item->dscale = 1.0;
  int* off = reinterpret_cast<int*>(h_buf + RL.off[1]);
  const AsmItem* d_item = reinterpret_cast<const AsmItem*>(d_buf);
  const int* d_off = reinterpret_cast<const int*>(d_buf + RL.off[1]);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CK(cudaEventCreate(&e0));
  cudaError_t e = cudaEventCreate(&e1);
  float best = INFINITY;
  int best_epb = 4;
  std::array<float, 2> times{INFINITY, INFINITY};
  for (int epb : {4, 2}) {
    if (e != cudaSuccess) break;
    off[0] = 0;
    off[1] = batch_tan_ctas(h->numel, epb);
    e = cudaMemcpyAsync(d_buf, h_buf, RL.bytes, cudaMemcpyHostToDevice, st);
    float t = INFINITY;
    for (int r = 0; r < 4 && e == cudaSuccess; ++r) {
      e = cudaEventRecord(e0, st);
      if (e == cudaSuccess) e = launch_batch_tan(h->pp.motion, epb, d_ajobs, d_item, d_off, 1, off[1], h->pp.nq, st);
      if (e == cudaSuccess) e = cudaEventRecord(e1, st);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float ms = 0.0f;
      if (e == cudaSuccess && r > 0 && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess) t = std::min(t, ms);
    }
    times[epb == 2 ? 0 : 1] = t;
    if (t < best) {
      best = t;
      best_epb = epb;
    }
  }
  cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (e != cudaSuccess) {
    h->err = std::string("tangent kernel autotuning: ") + cudaGetErrorString(e);
    return MAFEM_ERR_CUDA;
  }
  std::lock_guard<std::mutex> g(g_tune_mu);
  g_tan_epb[key] = best_epb;
  g_tan_ms[key] = times;
  return MAFEM_OK;
}

extern "C" int mafem_tangent_tile(const mafem_handle* h, int32_t* epb, double* ms_2, double* ms_4) {
  if (!h) return MAFEM_ERR_ARG;
  std::lock_guard<std::mutex> g(g_tune_mu);
  const TanShape key = tan_shape(h);
  auto it = g_tan_epb.find(key);
  if (it == g_tan_epb.end()) return MAFEM_ERR_UNSUPPORTED;
  const std::array<float, 2>& t = g_tan_ms[key];
  if (epb) *epb = it->second;
  if (ms_2) *ms_2 = t[0];
  if (ms_4) *ms_4 = t[1];
  return MAFEM_OK;
}

struct mafem_batch {
  std::vector<mafem_handle*> hs;
  // batched FP32 solve: the handles whose band fits one CTA (patch_ok)
  bool patch_on = false;
  std::vector<int> slot;  // per handle: its job index, or -1
  std::vector<double> cost;
  PatchJob* d_jobs = nullptr;
  int* d_order = nullptr;
  int* h_order = nullptr;  // pinned
  cudaStream_t bst = nullptr, bst2 = nullptr;  // clusters / single CTAs
  cudaEvent_t bev = nullptr, efork = nullptr, ejoin = nullptr;
  size_t smem_f = 0, smem_r = 0;
  int max_sweeps = 30;
  double tol = 1e-10;
  // batched rounds of the FP32 patch jobs: one launch per kernel (per motion
  // for the element kernels) per Newton round, indexed by slot like d_jobs
  bool asm_on = false;
  AsmJob* d_ajobs = nullptr;
  std::unique_ptr<RoundRunner> rr;
  ~mafem_batch() {
    if (bst) cudaStreamSynchronize(bst);
    if (bst2) cudaStreamSynchronize(bst2);
    rr.reset();
    if (d_ajobs) cudaFree(d_ajobs);
    if (efork) cudaEventDestroy(efork);
    if (ejoin) cudaEventDestroy(ejoin);
    if (bst2) cudaStreamDestroy(bst2);
    if (d_jobs) cudaFree(d_jobs);
    if (d_order) cudaFree(d_order);
    if (h_order) cudaFreeHost(h_order);
    if (bev) cudaEventDestroy(bev);
    if (bst) cudaStreamDestroy(bst);
  }
};


extern "C" int mafem_batch_create(mafem_handle* const* hs, int32_t n, int32_t ctas, mafem_batch** out) {
  if (!out || n < 0 || (n > 0 && !hs) || ctas < 0) {
    set_global_error("mafem_batch_create: bad arguments");
    return MAFEM_ERR_ARG;
  }
  auto b = std::make_unique<mafem_batch>();
  std::vector<PatchJob> jobs;
  for (int i = 0; i < n; ++i) {
    if (!hs[i]) {
      set_global_error("mafem_batch_create: null handle");
      return MAFEM_ERR_ARG;
    }
    for (mafem_handle* o : b->hs)
      if (o == hs[i]) {
        set_global_error("mafem_batch_create: a handle appears twice");
        return MAFEM_ERR_ARG;
      }
    mafem_handle* h = hs[i];
    b->hs.push_back(h);
    // ctas == 0: each patch's smallest persistent grid, so that many patches' factorisations fit at once
    const int c = ctas > 0 ? ctas : std::max(1, h->pers.min_grid);
    mafem_set_launch_ctas(h, c);
    if (h->patch_ok) {
      b->slot.push_back((int)jobs.size());
      jobs.push_back(h->job);
      b->cost.push_back((double)h->blk.npan() * h->L.kl * h->blk.kuf);
      b->smem_f = std::max(b->smem_f, patch_factor_smem(h->L.kl));
      b->smem_r = std::max(b->smem_r, patch_refine_smem(h->L.n));
    } else {
      b->slot.push_back(-1);
    }
  }
  if (!jobs.empty()) {
    const size_t nj = jobs.size();
    cudaError_t e = cudaMalloc(&b->d_jobs, nj * sizeof(PatchJob));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_order, nj * sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_order, nj * sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(b->d_jobs, jobs.data(), nj * sizeof(PatchJob), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->bst, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->bst2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->bev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->efork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ejoin, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      set_global_error(std::string("mafem_batch_create: ") + cudaGetErrorString(e));
      return MAFEM_ERR_CUDA;
    }
    for (int i = 0; i < n; ++i) {  // the autotuner's times of every patch shape not yet measured
      if (b->slot[i] < 0) continue;
      const int rc = patch_tune(b->hs[i], b->d_jobs, b->slot[i], b->d_order, b->bst);
      if (rc != MAFEM_OK) {
        set_global_error("mafem_batch_create: " + b->hs[i]->err);
        return rc;
      }
    }
    b->patch_on = true;
    // the batched rounds' job table and runner
    std::vector<AsmJob> aj;
    for (int i = 0; i < n; ++i)
      if (b->slot[i] >= 0) aj.push_back(asm_job(b->hs[i]));
    e = batch_asm_setup();
    if (e == cudaSuccess) e = cudaMalloc(&b->d_ajobs, nj * sizeof(AsmJob));
    if (e == cudaSuccess) e = cudaMemcpy(b->d_ajobs, aj.data(), nj * sizeof(AsmJob), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
      b->rr = std::make_unique<RoundRunner>();
      e = b->rr->init((int)nj);
    }
    for (int i = 0; i < n && e == cudaSuccess; ++i) {  // the tangent kernel's tile of every kind of patch
      if (b->slot[i] < 0) continue;
      const int rc = tan_tune(b->hs[i], b->d_ajobs, b->slot[i], b->rr->d_round, b->rr->h_round, b->rr->st);
      if (rc != MAFEM_OK) {
        set_global_error("mafem_batch_create: " + b->hs[i]->err);
        return rc;
      }
    }
    if (e != cudaSuccess) {
      set_global_error(std::string("mafem_batch_create: ") + cudaGetErrorString(e));
      return MAFEM_ERR_CUDA;
    }
    b->asm_on = true;
  }
  *out = b.release();
  return MAFEM_OK;
}

extern "C" int mafem_batch_set_patch_solve(mafem_batch* b, int32_t on) {
  if (!b) return MAFEM_ERR_ARG;
  b->patch_on = on != 0 && b->d_jobs != nullptr;
  return b->patch_on ? 1 : 0;
}

extern "C" int mafem_batch_destroy(mafem_batch* b) {
  delete b;
  return MAFEM_OK;
}

// One batched Newton round of the FP32 patches hv[pj] (ordered for the
// factorisation: the first n4 on four-CTA clusters, the next n2 on two; job
// index slot_of[i], step-start flags start[i] and Dirichlet scale dscale[i]
// per handle) on R's streams: the Dirichlet scaling and the predictor of the
// patches that start a time step, the FP64 residual and FP32 tangent kernels
// per motion, both band gathers and the residual gather, the batched factor /
// refine (patch_solve), the Newton update and norms of every patch, and the
// copy of the results to R.h_outs (row k: handle R.items_of[k]).  With
// R.graph_on a round is captured as a CUDA graph the first time its sequence
// of patches occurs and replayed from then on.  *launches: kernels per round.
static cudaError_t run_round(RoundRunner& R, const PatchJob* d_jobs, const AsmJob* d_ajobs, size_t smem_f,
                             size_t smem_r, const std::vector<mafem_handle*>& hv, const std::vector<int>& slot_of,
                             const std::vector<int>& pj, int n4, int n2, int max_sweeps, double tol,
                             const std::vector<int>& start, const std::vector<double>& dscale, int* launches) {
  const int m = (int)pj.size();
  if (m > R.cap) return cudaErrorInvalidValue;
  const RoundLayout RL = round_layout(m);
  const size_t dir_off = RL.bytes;  // the seventh offset array follows the layout
  std::vector<int>& it = R.items_of;
  it.assign(pj.begin(), pj.end());
  auto gkey = [&](int i) { return std::make_pair(hv[i]->pp.motion, hv[i]->pp.nq); };
  std::stable_sort(it.begin(), it.end(), [&](int a, int c) { return gkey(a) < gkey(c); });
  AsmItem* items = reinterpret_cast<AsmItem*>(R.h_round);
  int* off[kOffKinds + 1];
  for (int t = 0; t < kOffKinds; ++t) off[t] = reinterpret_cast<int*>(R.h_round + RL.off[t]);
  off[kOffDir] = reinterpret_cast<int*>(R.h_round + dir_off);
  for (int t = 0; t <= kOffDir; ++t) off[t][0] = 0;
  std::vector<int> groups{0};  // item ranges of one (motion, nq)
  std::vector<int> epb(m);     // the tangent kernel's elements per CTA (the same within a group)
  bool any_pred = false, any_dir = false;
  for (int k = 0; k < m; ++k) {
    const int i = it[k];
    const mafem_handle* h = hv[i];
    epb[k] = k > 0 && gkey(it[k - 1]) == gkey(i) ? epb[k - 1] : tan_epb(h);
    items[k].job = slot_of[i];
    items[k].start = start[i];
    items[k].time = h->ss_time;
    items[k].dt = h->ss_dt;
    items[k].dscale = dscale[i];
    off[0][k + 1] = off[0][k] + batch_resid_ctas(h->numel);
    off[1][k + 1] = off[1][k] + batch_tan_ctas(h->numel, epb[k]);
    off[2][k + 1] = off[2][k] + batch_gather_ctas(h->L.n);
    off[3][k + 1] = off[3][k] + batch_rgather_ctas(h->nmdf);
    off[4][k + 1] = off[4][k] + newton_update_blocks(h->nmdf);
    off[5][k + 1] = off[5][k] + ((start[i] & kStartPredict) ? batch_pred_ctas(h->numnp) : 0);
    off[kOffDir][k + 1] = off[kOffDir][k] + ((start[i] & kStartDirichlet) ? batch_dir_ctas(h->n_dir) : 0);
    any_pred |= (start[i] & kStartPredict) != 0;
    any_dir |= (start[i] & kStartDirichlet) != 0 && h->n_dir > 0;
    if (k + 1 < m && gkey(it[k + 1]) != gkey(it[k])) groups.push_back(k + 1);
  }
  groups.push_back(m);
  const size_t bytes = dir_off + (size_t)(m + 1) * sizeof(int);
  for (int k = 0; k < m; ++k) R.h_order[k] = slot_of[pj[k]];
  const unsigned char* dr = R.d_round;
  const AsmItem* d_items = reinterpret_cast<const AsmItem*>(dr);
  auto d_off = [&](int t, int g0) {
    return reinterpret_cast<const int*>(dr + (t == kOffDir ? dir_off : RL.off[t])) + g0;
  };
  const int ng = (int)groups.size() - 1;
  *launches = (any_dir ? 1 : 0) + (any_pred ? 1 : 0) + 2 * ng + 2 + patch_solve_launches(n4, n2, m) + 2;

  auto enqueue = [&](bool capturing) -> cudaError_t {
    const unsigned fl = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
    cudaStream_t st = R.st;
    cudaError_t e = cudaMemcpyAsync(R.d_round, R.h_round, bytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(R.d_order, R.h_order, m * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaEventRecordWithFlags(R.rev[0], st, fl);
    if (e == cudaSuccess && any_dir) {
      launch_batch_dirichlet(d_ajobs, d_items, d_off(kOffDir, 0), m, off[kOffDir][m], st);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess && any_pred) {
      launch_batch_predictor(d_ajobs, d_items, d_off(5, 0), m, off[5][m], st);
      e = cudaGetLastError();
    }
    for (int g = 0; g < ng && e == cudaSuccess; ++g) {
      const int g0 = groups[g], g1 = groups[g + 1];
      const mafem_handle* h = hv[it[g0]];
      e = launch_batch_resid(h->pp.motion, d_ajobs, d_items + g0, d_off(0, g0), g1 - g0, off[0][g1] - off[0][g0],
                             h->pp.nq, st);
      if (e == cudaSuccess)
        e = launch_batch_tan(h->pp.motion, epb[g0], d_ajobs, d_items + g0, d_off(1, g0), g1 - g0,
                             off[1][g1] - off[1][g0], h->pp.nq, st);
    }
    if (e == cudaSuccess) {
      launch_batch_gather(d_ajobs, d_items, d_off(2, 0), m, off[2][m], st);
      launch_batch_rgather(d_ajobs, d_items, d_off(3, 0), m, off[3][m], st);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecordWithFlags(R.rev[1], st, fl);
    if (e == cudaSuccess)
      e = patch_solve(d_jobs, R.d_order, n4, n2, m, smem_f, smem_r, max_sweeps, tol, st, R.st2, R.efork, R.ejoin);
    if (e == cudaSuccess) e = cudaEventRecordWithFlags(R.rev[2], st, fl);
    if (e == cudaSuccess) {
      launch_batch_update(d_ajobs, d_items, d_off(4, 0), m, off[4][m], R.d_outs, st);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(R.h_outs, R.d_outs, m * sizeof(AsmOut), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaEventRecordWithFlags(R.rev[3], st, fl);
    return e;
  };

  if (!R.graph_on) return enqueue(false);
  // the graph's key: everything its nodes bake in (grids, copy sizes, kernel arguments)
  // (a job's shape too: a slot of a server may hold another patch later)
  std::vector<int64_t> key{m, n4, n2, max_sweeps, (int64_t)smem_f, (int64_t)smem_r};
  int64_t tb;
  std::memcpy(&tb, &tol, sizeof tb);
  key.push_back(tb);
  for (int k = 0; k < m; ++k) {
    const mafem_handle* h = hv[it[k]];
    key.push_back((int64_t)items[k].job * 4 + items[k].start);
    key.push_back(((int64_t)h->numel << 32) | (uint32_t)h->numnp);
    key.push_back((h->nmdf << 24) | ((int64_t)h->n_dir << 8) | (h->pp.motion << 4) | (h->ndf & 15));
    key.push_back(epb[k]);
  }
  for (int k = 0; k < m; ++k) key.push_back(R.h_order[k]);
  auto found = R.graphs.find(key);
  if (found == R.graphs.end()) {
    if (R.graphs.size() >= 256) {
      for (auto& g : R.graphs) cudaGraphExecDestroy(g.second);
      R.graphs.clear();
    }
    cudaError_t e = cudaStreamBeginCapture(R.st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    const cudaError_t ee = enqueue(true);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(R.st, &graph);
    cudaGraphExec_t exec = nullptr;
    if (ee == cudaSuccess && e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (ee != cudaSuccess || e != cudaSuccess) {
      cudaGetLastError();
      R.graph_on = false;  // capture refused: plain stream launches from now on
      return enqueue(false);
    }
    found = R.graphs.emplace(key, exec).first;
    ++R.graph_captures;
  }
  ++R.graph_launches;
  return cudaGraphLaunch(found->second, R.st);
}

// After R's round completed: each patch's results into its handle's h_out
// (eps, |r|, the non-finite flag, the info words) and the round's phase times
// into its step stats.
static void round_results(RoundRunner& R, const std::vector<mafem_handle*>& hv) {
  float ms_a = 0, ms_f = 0, ms_s = 0;
  cudaEventElapsedTime(&ms_a, R.rev[0], R.rev[1]);
  cudaEventElapsedTime(&ms_f, R.rev[1], R.rev[2]);
  cudaEventElapsedTime(&ms_s, R.rev[2], R.rev[3]);
  for (size_t k = 0; k < R.items_of.size(); ++k) {
    mafem_handle* h = hv[R.items_of[k]];
    const AsmOut& o = R.h_outs[k];
    h->h_out[0] = o.out[0];
    h->h_out[1] = o.out[1];
    h->h_out[2] = o.out[2];
    std::memcpy(h->h_out + 5, o.info, sizeof o.info);
    h->ss_patch = true;
    h->ss_async = false;
    h->ss_sweeps = 0;
    h->factored = false;
    h->ss_S.ms_assemble += ms_a;
    h->ss_S.ms_factor += ms_f;
    h->ss_S.ms_solve += ms_s;
  }
}

// One time step of every patch: predictor + Newton, the patches' iterations
// interleaved -- every active patch's iteration k is enqueued before any is
// waited for, so their kernels overlap.  FP32 patches whose band fits the
// batched solve run as batched rounds (batch_round: one launch per kernel for
// all of them, replayed from a CUDA graph); the other patches run their own
// iterations on their own streams beside them.
extern "C" int mafem_batch_step(mafem_batch* b, const double* times, const double* dts, int32_t* status,
                                mafem_step_stats* stats) {
  if (!b || !times || !dts) return MAFEM_ERR_ARG;
  const int n = (int)b->hs.size();
  const bool basm = b->asm_on && b->patch_on && b->rr;
  std::vector<int> active, st(n, MAFEM_OK);
  std::vector<int> start(n, 0);
  const std::vector<double> dscale(n, 1.0);
  for (int i = 0; i < n; ++i) {
    mafem_handle* h = b->hs[i];
    const bool bp = basm && b->slot[i] >= 0;
    if (!bp) {
      launch_predictor(h->P, h->pp, dts[i], h->st);  // update_xms! (Analysis.jl:70)
      h->launches += 1;
    }
    step_begin(h, times[i], dts[i]);
    if (bp) {
      start[i] = kStartPredict;  // the predictor runs in the step's first round
      cudaStreamWaitEvent(b->rr->st, h->ev[5], 0);  // the caller's work on the handle's stream first
    }
    active.push_back(i);
  }
  std::vector<int> pj;
  std::vector<char> batched(n, 0);
  while (!active.empty()) {
    std::vector<int> next;
    pj.clear();
    for (int i : active) {
      mafem_handle* h = b->hs[i];
      const bool patch = b->patch_on && b->slot[i] >= 0;
      if (patch && basm) {
        pj.push_back(i);
        continue;
      }
      const int rc = patch ? iter_enqueue_patch_begin(h) : iter_enqueue(h);
      if (rc != MAFEM_OK)
        st[i] = rc;
      else if (patch)
        pj.push_back(i);
    }
    bool round_ok = false;
    if (!pj.empty()) {
      int n4 = 0, n2 = 0;
      choose_patch_ctas(b->hs, pj);
      order_patch_jobs(b->hs, pj, &n4, &n2);
      // one launch serves every patch: the strictest tolerance and the largest sweep cap among them
      b->max_sweeps = 1;
      b->tol = 1.0;
      for (int i : pj) {
        b->max_sweeps = std::max(b->max_sweeps, b->hs[i]->max_refine);
        b->tol = std::min(b->tol, b->hs[i]->refine_tol);
      }
      if (basm) {
        int nl = 0;
        cudaError_t e = run_round(*b->rr, b->d_jobs, b->d_ajobs, b->smem_f, b->smem_r, b->hs, b->slot, pj, n4, n2,
                                  b->max_sweeps, b->tol, start, dscale, &nl);
        if (e == cudaSuccess) e = cudaEventSynchronize(b->rr->rev[3]);
        for (int i : pj) start[i] = 0;
        if (e != cudaSuccess) {
          for (int i : pj) {
            b->hs[i]->err = std::string("batched round: ") + cudaGetErrorString(e);
            st[i] = MAFEM_ERR_CUDA;
          }
        } else {
          round_ok = true;
          b->hs[pj[0]]->launches += nl;
          round_results(*b->rr, b->hs);
          for (int i : b->rr->items_of) batched[i] = 1;
        }
      } else {
        for (size_t k = 0; k < pj.size(); ++k) {
          b->h_order[k] = b->slot[pj[k]];
          cudaStreamWaitEvent(b->bst, b->hs[pj[k]]->ev[1], 0);
        }
        cudaError_t e =
            cudaMemcpyAsync(b->d_order, b->h_order, pj.size() * sizeof(int), cudaMemcpyHostToDevice, b->bst);
        if (e == cudaSuccess)
          e = patch_solve(b->d_jobs, b->d_order, n4, n2, (int)pj.size(), b->smem_f, b->smem_r, b->max_sweeps,
                          b->tol, b->bst, b->bst2, b->efork, b->ejoin);
        if (e == cudaSuccess) e = cudaEventRecord(b->bev, b->bst);
        for (int i : pj) {
          mafem_handle* h = b->hs[i];
          if (e != cudaSuccess) {
            h->err = std::string("batched FP32 solve: ") + cudaGetErrorString(e);
            st[i] = MAFEM_ERR_CUDA;
            continue;
          }
          if (i == pj[0]) h->launches += patch_solve_launches(n4, n2, (int)pj.size());  // counted once
          const int rc = iter_enqueue_patch_end(h, b->bev);
          if (rc != MAFEM_OK) st[i] = rc;
        }
      }
    }
    for (int i : active) {
      if (st[i] != MAFEM_OK) continue;
      mafem_handle* h = b->hs[i];
      const bool in_round = basm && round_ok && batched[i];
      const int64_t fb = h->fallbacks;
      const int rc = in_round ? iter_decide(h) : iter_finish(h);
      if (rc == kIterAgain) {
        next.push_back(i);
      } else {
        st[i] = rc == kIterDone ? MAFEM_OK : rc;
        // a batched patch's step ends with its round (or with its own redo of the last iteration)
        step_stats(h, stats ? stats + i : nullptr, in_round && h->fallbacks == fb ? b->rr->rev[3] : nullptr);
      }
    }
    std::fill(batched.begin(), batched.end(), 0);
    active.swap(next);
  }
  int first = MAFEM_OK;
  for (int i = 0; i < n; ++i) {
    if (status) status[i] = st[i];
    if (first == MAFEM_OK && st[i] != MAFEM_OK) {
      first = st[i];
      set_global_error("patch " + std::to_string(i) + ": " + b->hs[i]->err);
    }
  }
  return first;
}

extern "C" int mafem_batch_set_rounds(mafem_batch* b, int32_t batched_assembly, int32_t graphs) {
  if (!b) return MAFEM_ERR_ARG;
  b->asm_on = batched_assembly != 0 && b->rr != nullptr;
  if (b->rr) b->rr->graph_on = graphs != 0;
  return MAFEM_OK;
}

extern "C" int mafem_batch_get_stats(const mafem_batch* b, mafem_batch_stats* out) {
  if (!b || !out) return MAFEM_ERR_ARG;
  out->graph_launches = b->rr ? b->rr->graph_launches : 0;
  out->graph_captures = b->rr ? b->rr->graph_captures : 0;
  out->graphs_cached = b->rr ? (int64_t)b->rr->graphs.size() : 0;
  int64_t l = 0;
  for (const mafem_handle* h : b->hs) l += h->launches;
  out->kernel_launches = l;
  return MAFEM_OK;
}

// ---- serving: continuous batching of many solves ------------------------------------
// Requests (a patch, its initial state, a number of time steps) are admitted
// while their device footprint fits the server's HBM budget and run as one
// continuous batch.  An FP32 request whose band fits the batched solve takes
// a slot of the server's job tables and advances through batched Newton rounds
// on one of kLanes solve lanes: a lane's round assembles, factors, refines and
// updates its requests with one launch per kernel (run_round), and each
// request that finishes an iteration goes into the next round of a free lane,
// so small patches iterate while a large one is still in its round.  The
// ready requests are grouped by the cost of their factorisation (groups within
// a factor of 8), the costliest group first, one group per free lane.  Other
// requests run their own iterations on their own streams beside the lanes.
// A finished request's state is copied out and its memory freed at once,
// which admits the next.  Each request computes exactly what mafem_time_step
// computes on its handle: results do not depend on the mix.

namespace {
struct ServerReq {
  enum State { IDLE, READY, LANE, FLIGHT };
  int64_t id = 0;
  mafem_request r{};
  std::vector<double> xms, cps;  // initial state, then the result
  int64_t est = 0, bytes = 0;
  mafem_handle* h = nullptr;
  int slot = -1;
  int step = 0;
  double t = 0.0;
  bool in_step = false;
  State state = IDLE;
  int start = 0;         // step-start flags of the next lane round (kStartPredict | kStartDirichlet)
  double dscale = 1.0;   // the ramp's Dirichlet scale of the step
  double t_start = 0.0;  // host seconds at the step's first iteration
  int status = MAFEM_OK;
  bool done = false;
  mafem_step_stats last{};
};
constexpr int kLanes = 4;
double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
// the factorisation cost of a patch, for the grouping of a lane's round
double patch_cost(const mafem_handle* h) { return (double)h->blk.npan() * h->L.kl * h->blk.kuf; }
}  // namespace

struct mafem_server {
  int64_t budget = 0, used = 0;
  int max_active = 0;
  int64_t next_id = 1;
  std::deque<ServerReq*> pending;
  std::vector<ServerReq*> active;
  std::map<int64_t, ServerReq*> finished;
  std::vector<int> free_slots;
  PatchJob* d_jobs = nullptr;
  PatchJob* h_jobs = nullptr;  // pinned staging of the job tables
  AsmJob* d_ajobs = nullptr;
  AsmJob* h_ajobs = nullptr;
  unsigned char* d_tune = nullptr;  // the tangent autotuner's one-item round
  unsigned char* h_tune = nullptr;  // pinned
  cudaStream_t admin = nullptr;  // job-table uploads
  RoundRunner lanes[kLanes];
  std::vector<ServerReq*> lane_reqs[kLanes];  // the requests of each lane's round in flight
  size_t smem_dyn = 0;
  std::vector<double> step_ms;  // wall latency of every completed step
  int64_t steps_done = 0, rounds = 0;
  ~mafem_server() {
    for (RoundRunner& l : lanes) {
      if (l.st) cudaStreamSynchronize(l.st);
      if (l.st2) cudaStreamSynchronize(l.st2);
    }
    for (ServerReq* q : pending) delete q;
    for (ServerReq* q : active) {
      if (q->h) mafem_destroy(q->h);
      delete q;
    }
    for (auto& kv : finished) delete kv.second;
    if (d_jobs) cudaFree(d_jobs);
    if (h_jobs) cudaFreeHost(h_jobs);
    if (d_ajobs) cudaFree(d_ajobs);
    if (h_ajobs) cudaFreeHost(h_ajobs);
    if (d_tune) cudaFree(d_tune);
    if (h_tune) cudaFreeHost(h_tune);
    if (admin) cudaStreamDestroy(admin);
  }
};

extern "C" int mafem_server_create(int64_t hbm_budget_bytes, int32_t max_active, mafem_server** out) {
  if (!out || hbm_budget_bytes < 0 || max_active < 0) return MAFEM_ERR_ARG;
  auto s = std::make_unique<mafem_server>();
  size_t fr = 0, tot = 0;
  cudaError_t e = cudaMemGetInfo(&fr, &tot);
  if (e != cudaSuccess) {
    set_global_error(std::string("mafem_server_create: ") + cudaGetErrorString(e));
    return MAFEM_ERR_CUDA;
  }
  s->budget = hbm_budget_bytes > 0 ? hbm_budget_bytes : (int64_t)(0.8 * (double)fr);
  s->max_active = max_active > 0 ? max_active : 1024;
  const size_t m = (size_t)s->max_active;
  e = cudaMalloc(&s->d_jobs, m * sizeof(PatchJob));
  if (e == cudaSuccess) e = cudaMallocHost(&s->h_jobs, m * sizeof(PatchJob));
  if (e == cudaSuccess) e = cudaMalloc(&s->d_ajobs, m * sizeof(AsmJob));
  if (e == cudaSuccess) e = cudaMallocHost(&s->h_ajobs, m * sizeof(AsmJob));
  if (e == cudaSuccess) e = cudaMalloc(&s->d_tune, round_layout(1).bytes);
  if (e == cudaSuccess) e = cudaMallocHost(&s->h_tune, round_layout(1).bytes);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->admin, cudaStreamNonBlocking);
  for (RoundRunner& l : s->lanes)
    if (e == cudaSuccess) e = l.init(s->max_active);
  if (e == cudaSuccess) e = batch_asm_setup();
  if (e != cudaSuccess) {
    set_global_error(std::string("mafem_server_create: ") + cudaGetErrorString(e));
    return MAFEM_ERR_CUDA;
  }
  const int dyn = patch_solve_setup();
  cudaGetLastError();
  s->smem_dyn = dyn > 0 ? (size_t)dyn : 0;
  for (int k = s->max_active - 1; k >= 0; --k) s->free_slots.push_back(k);
  *out = s.release();
  return MAFEM_OK;
}

extern "C" int mafem_server_destroy(mafem_server* s) {
  delete s;
  return MAFEM_OK;
}

extern "C" int mafem_server_submit(mafem_server* s, const mafem_request* r, int64_t* id) {
  if (!s || !r || !id || !r->mesh || !r->params || !r->args || !r->xms0 || !r->cps0 || r->nsteps < 1 ||
      !(r->dt > 0.0))
    return MAFEM_ERR_ARG;
  const int64_t fp = mafem_footprint_bytes(r->mesh, r->precision);
  if (fp < 0) return MAFEM_ERR_ARG;
  // the footprint estimate plus the FP32 form's per-panel inverses and slack
  const int64_t est = fp + fp / 8 + (16LL << 20);
  if (est > s->budget) {
    set_global_error("request needs about " + std::to_string(est) + " device bytes, more than the server's budget of " +
                     std::to_string(s->budget));
    return MAFEM_ERR_ADMISSION;
  }
  auto q = std::make_unique<ServerReq>();
  q->id = s->next_id++;
  q->r = *r;
  q->xms.assign(r->xms0, r->xms0 + 3 * r->mesh->numnp);
  q->cps.assign(r->cps0, r->cps0 + r->mesh->ndf * r->mesh->numnp);
  q->est = est;
  q->t = r->t0;
  *id = q->id;
  s->pending.push_back(q.release());
  return MAFEM_OK;
}

static void server_retire(mafem_server* s, ServerReq* q) {
  mafem_handle* h = q->h;
  if (q->status == MAFEM_OK || q->status == MAFEM_NEWTON_NOT_CONVERGED)
    mafem_download_state(h, q->xms.data(), q->cps.data());
  s->used -= q->bytes;
  mafem_destroy(h);
  q->h = nullptr;
  if (q->slot >= 0) s->free_slots.push_back(q->slot);
  q->slot = -1;
  q->done = true;
  s->finished[q->id] = q;
}

// The Newton criterion on a request's completed iteration: the next iteration,
// the next step, or the end of the request (pushed onto retire).
static void server_after_iter(mafem_server* s, ServerReq* q, int rc, std::vector<ServerReq*>& retire,
                              cudaEvent_t end) {
  q->state = ServerReq::IDLE;
  if (rc == kIterAgain) return;
  if (rc == kIterDone) {
    step_stats(q->h, &q->last, end);
    s->step_ms.push_back((now_s() - q->t_start) * 1e3);
    ++s->steps_done;
    q->t += q->r.dt;
    q->in_step = false;
    if (++q->step < q->r.nsteps) return;
    rc = MAFEM_OK;
  }
  q->status = rc;
  retire.push_back(q);
}

// One pass of the event-driven loop: admit what fits; collect the completed
// lane rounds and own iterations; start the next iteration of every request
// that is not on the GPU (starting a time step first if it is between steps);
// hand the ready FP32 requests to the free lanes as batched rounds.
extern "C" int mafem_server_round(mafem_server* s, int32_t* n_active, int32_t* n_pending) {
  if (!s) return MAFEM_ERR_ARG;
  // admission, first come first served, while the footprint fits
  while (!s->pending.empty() && (int)s->active.size() < s->max_active) {
    ServerReq* q = s->pending.front();
    if (s->used + q->est > s->budget) break;
    mafem_handle* h = nullptr;
    int rc = mafem_create(q->r.mesh, q->r.params, q->r.args, q->r.precision, &h);
    // Out of device memory: try again once an active request frees its memory;
    // with none active, nothing of this server's will free up, so fail it.
    if (rc == MAFEM_ERR_OOM && !s->active.empty()) break;
    s->pending.pop_front();
    if (rc == MAFEM_OK) rc = mafem_upload_state(h, q->xms.data(), q->cps.data());
    if (rc == MAFEM_OK && q->r.refine_tol > 0.0) rc = mafem_set_refinement(h, 30, q->r.refine_tol);
    if (rc != MAFEM_OK) {
      q->status = rc;
      q->done = true;
      if (h) mafem_destroy(h);
      s->finished[q->id] = q;
      continue;
    }
    q->h = h;
    q->bytes = h->bytes;
    s->used += h->bytes;
    if (h->patch_ok && s->smem_dyn >= patch_factor_smem(h->L.kl) && s->smem_dyn >= patch_refine_smem(h->L.n) &&
        !s->free_slots.empty()) {
      q->slot = s->free_slots.back();
      s->free_slots.pop_back();
      s->h_jobs[q->slot] = h->job;
      s->h_ajobs[q->slot] = asm_job(h);
      cudaMemcpyAsync(s->d_jobs + q->slot, s->h_jobs + q->slot, sizeof(PatchJob), cudaMemcpyHostToDevice, s->admin);
      cudaMemcpyAsync(s->d_ajobs + q->slot, s->h_ajobs + q->slot, sizeof(AsmJob), cudaMemcpyHostToDevice, s->admin);
      cudaStreamSynchronize(s->admin);
      // the tangent kernel's tile for a kind of patch not seen yet (optional: the default on failure)
      if (tan_tune(h, s->d_ajobs, q->slot, s->d_tune, s->h_tune, s->admin) != MAFEM_OK) cudaGetLastError();
    }
    s->active.push_back(q);
  }
  std::vector<ServerReq*> retire;
  bool progressed = false;
  // completed lane rounds
  for (int l = 0; l < kLanes; ++l) {
    RoundRunner& L = s->lanes[l];
    if (!L.busy) continue;
    const cudaError_t qe = cudaEventQuery(L.rev[3]);
    if (qe == cudaErrorNotReady) continue;
    L.busy = false;
    progressed = true;
    std::vector<mafem_handle*> hv;
    for (ServerReq* q : s->lane_reqs[l]) hv.push_back(q->h);
    if (qe == cudaSuccess) round_results(L, hv);
    for (ServerReq* q : s->lane_reqs[l]) {
      const int64_t fb = q->h->fallbacks;
      int rc = MAFEM_ERR_CUDA;
      if (qe == cudaSuccess)
        rc = iter_decide(q->h);
      else
        q->h->err = std::string("batched round: ") + cudaGetErrorString(qe);
      server_after_iter(s, q, rc, retire, q->h->fallbacks == fb ? L.rev[3] : nullptr);
    }
    s->lane_reqs[l].clear();
  }
  // completed own iterations
  for (ServerReq* q : s->active) {
    if (q->state != ServerReq::FLIGHT || q->status != MAFEM_OK) continue;
    const cudaError_t qe = cudaEventQuery(q->h->ev[4]);
    if (qe == cudaErrorNotReady) continue;
    progressed = true;
    int rc = qe == cudaSuccess ? iter_finish(q->h) : MAFEM_ERR_CUDA;
    if (qe != cudaSuccess) q->h->err = std::string("iteration: ") + cudaGetErrorString(qe);
    server_after_iter(s, q, rc, retire, nullptr);
  }
  // the next iteration of every request not on the GPU
  const double t_now = now_s();
  for (ServerReq* q : s->active) {
    if (q->state != ServerReq::IDLE || q->status != MAFEM_OK) continue;
    if (std::find(retire.begin(), retire.end(), q) != retire.end()) continue;
    mafem_handle* h = q->h;
    if (!q->in_step) {  // predictor (Analysis.jl:70) + step_begin
      const double sc = q->r.ramp_steps > 0 ? std::min(1.0, (double)(q->step + 1) / q->r.ramp_steps) : 1.0;
      if (q->slot >= 0) {  // in the step's first lane round
        q->start = kStartPredict | (q->r.ramp_steps > 0 ? kStartDirichlet : 0);
        q->dscale = sc;
      } else {
        // the Dirichlet values ramped over the request's first steps
        if (q->r.ramp_steps > 0) launch_dirichlet_scale(h->P.cps, h->d_dir_idx, h->d_dir_val, h->n_dir, sc, h->st);
        launch_predictor(h->P, h->pp, q->r.dt, h->st);
        h->launches += 1;
      }
      step_begin(h, q->t + q->r.dt, q->r.dt);
      q->in_step = true;
      q->t_start = t_now;
    }
    if (q->slot >= 0) {
      q->state = ServerReq::READY;
      continue;
    }
    const int rc = iter_enqueue(h);
    if (rc != MAFEM_OK) {
      q->status = rc;
      retire.push_back(q);
      continue;
    }
    q->state = ServerReq::FLIGHT;
  }
  // the ready FP32 requests as batched rounds on the free lanes: groups of
  // similar factorisation cost, the costliest first
  std::vector<ServerReq*> ready;
  for (ServerReq* q : s->active)
    if (q->state == ServerReq::READY && q->status == MAFEM_OK) ready.push_back(q);
  std::sort(ready.begin(), ready.end(), [](ServerReq* a, ServerReq* b) { return patch_cost(a->h) > patch_cost(b->h); });
  size_t next = 0;
  for (int l = 0; l < kLanes && next < ready.size(); ++l) {
    RoundRunner& L = s->lanes[l];
    if (L.busy) continue;
    const double top = patch_cost(ready[next]->h);
    size_t end = next + 1;
    while (end < ready.size() && patch_cost(ready[end]->h) * 8.0 >= top) ++end;
    std::vector<ServerReq*>& rq = s->lane_reqs[l];
    rq.assign(ready.begin() + next, ready.begin() + end);
    next = end;
    const int m = (int)rq.size();
    std::vector<mafem_handle*> hv(m);
    std::vector<int> slot_of(m), start(m), pj(m);
    std::vector<double> dscale(m);
    size_t smf = 0, smr = 0;
    int max_sw = 1;
    double tol = 1.0;
    for (int k = 0; k < m; ++k) {
      ServerReq* q = rq[k];
      mafem_handle* h = q->h;
      hv[k] = h;
      slot_of[k] = q->slot;
      start[k] = q->start;
      dscale[k] = q->dscale;
      pj[k] = k;
      smf = std::max(smf, patch_factor_smem(h->L.kl));
      smr = std::max(smr, patch_refine_smem(h->L.n));
      max_sw = std::max(max_sw, h->max_refine);
      tol = std::min(tol, h->refine_tol);
      if (q->start) cudaStreamWaitEvent(L.st, h->ev[5], 0);  // the handle's own work before the step
    }
    int n4 = 0, n2 = 0;
    choose_patch_ctas(hv, pj);
    order_patch_jobs(hv, pj, &n4, &n2);
    int nl = 0;
    cudaError_t e = run_round(L, s->d_jobs, s->d_ajobs, smf, smr, hv, slot_of, pj, n4, n2, max_sw, tol, start, dscale,
                              &nl);
    for (ServerReq* q : rq) q->start = 0;
    if (e != cudaSuccess) {
      for (ServerReq* q : rq) {
        q->h->err = std::string("batched round: ") + cudaGetErrorString(e);
        q->status = MAFEM_ERR_CUDA;
        retire.push_back(q);
      }
      rq.clear();
      continue;
    }
    hv[0]->launches += nl;
    L.busy = true;
    for (ServerReq* q : rq) q->state = ServerReq::LANE;
  }
  if (!retire.empty()) {
    std::vector<ServerReq*> keep;
    for (ServerReq* q : s->active)
      if (std::find(retire.begin(), retire.end(), q) == retire.end()) keep.push_back(q);
    // A request retired on an error path may still be read by a round in
    // flight on some lane: wait for the lanes before its memory is freed.
    bool drain = false;
    for (ServerReq* q : retire) drain |= q->status != MAFEM_OK && q->status != MAFEM_NEWTON_NOT_CONVERGED;
    if (drain)
      for (RoundRunner& L : s->lanes) {
        cudaStreamSynchronize(L.st);
        cudaStreamSynchronize(L.st2);
      }
    for (ServerReq* q : retire) {
      if (q->h) cudaStreamSynchronize(q->h->st);
      server_retire(s, q);
    }
    s->active.swap(keep);
  }
  if (!progressed && !s->active.empty()) std::this_thread::sleep_for(std::chrono::microseconds(20));
  ++s->rounds;
  if (n_active) *n_active = (int32_t)s->active.size();
  if (n_pending) *n_pending = (int32_t)s->pending.size();
  return MAFEM_OK;
}

extern "C" int mafem_server_result(mafem_server* s, int64_t id, double* xms, double* cps, int32_t* status,
                                   int32_t* steps_done) {
  if (!s) return MAFEM_ERR_ARG;
  auto it = s->finished.find(id);
  if (it == s->finished.end()) {
    for (ServerReq* q : s->pending)
      if (q->id == id) return 1;
    for (ServerReq* q : s->active)
      if (q->id == id) return 1;
    return MAFEM_ERR_ARG;  // unknown id, or its result was already taken
  }
  ServerReq* q = it->second;
  if (xms) std::memcpy(xms, q->xms.data(), q->xms.size() * sizeof(double));
  if (cps) std::memcpy(cps, q->cps.data(), q->cps.size() * sizeof(double));
  if (status) *status = q->status;
  if (steps_done) *steps_done = q->step;
  s->finished.erase(it);
  delete q;
  return MAFEM_OK;
}

extern "C" int mafem_server_get_stats(const mafem_server* s, mafem_server_stats* out) {
  if (!s || !out) return MAFEM_ERR_ARG;
  std::vector<double> v = s->step_ms;
  std::sort(v.begin(), v.end());
  auto pct = [&](double q) { return v.empty() ? 0.0 : v[std::min(v.size() - 1, (size_t)(q * (double)v.size()))]; };
  out->steps_done = s->steps_done;
  out->rounds = s->rounds;
  out->p50_step_ms = pct(0.50);
  out->p99_step_ms = pct(0.99);
  out->max_step_ms = v.empty() ? 0.0 : v.back();
  out->bytes_in_use = s->used;
  out->budget_bytes = s->budget;
  out->active = (int32_t)s->active.size();
  out->pending = (int32_t)s->pending.size();
  return MAFEM_OK;
}

extern "C" int mafem_time_step_host(mafem_handle* h, double* xms, double* cps, double time, double dt,
                                    mafem_step_stats* stats) {
  int rc = mafem_upload_state(h, xms, cps);
  if (rc) return rc;
  rc = mafem_time_step(h, time, dt, stats);
  int rc2 = mafem_download_state(h, xms, cps);
  return rc ? rc : rc2;
}

extern "C" int mafem_run(mafem_handle* h, const double* dts, int32_t nsteps, double t0, mafem_step_stats* last) {
  if (!h || (!dts && nsteps > 0)) return MAFEM_ERR_ARG;
  double t = t0;
  for (int k = 0; k < nsteps; ++k) {
    // the step's end time, accumulated left to right from t0; the reference
    // forms [sum(Δts[1:i]) for i] .+ t0 (Analysis.jl:30), whose summation
    // order Julia's sum chooses: the two agree to rounding
    t += dts[k];
    launch_predictor(h->P, h->pp, dts[k], h->st);
    h->launches += 1;
    CK(cudaGetLastError());
    int rc = mafem_time_step(h, t, dts[k], last);
    if (rc) return rc;
  }
  return MAFEM_OK;
}

extern "C" int64_t mafem_launch_count(const mafem_handle* h) { return h ? h->launches : -1; }

// Per-kernel device time of one assembly + factorisation of the resident
// state (CUDA events on the handle's stream around every launch).
// FLOPs of one factorisation as the kernels execute it (matrix columns only;
// the fused right-hand side is not counted).
static void lu_flops(const mafem_handle* h, double* fpanel, double* fapply) {
  const int64_t n = h->nmdf, kl = h->L.kl, ku = h->L.ku;
  double fp = 0, fa = 0;
  if (h->use_blk) {
    const BlkPlan& B = h->blk;
    for (int p = 0; p < B.npan(); ++p) {
      const int64_t j0 = B.ps[p], j1 = B.ps[p + 1], w = j1 - j0;
      const int64_t R = std::min(n - j0, w + kl);
      const int64_t ncol = std::min(n, j1 + B.kuf) - j1;
      // per column: unit-lower solve w(w-1), U11 solve w^2, A21 y 2(R-w)w
      fa += (double)ncol * (double)(w * (w - 1) + w * w + 2 * (R - w) * w);
      for (int64_t k = 0; k < w; ++k) fp += (double)(w - k - 1) * (1 + 2 * (w - k - 1));
    }
  } else {
    const int64_t nb = h->L.nb;
    for (int64_t j0 = 0; j0 < n; j0 += nb) {
      const int64_t w = std::min(nb, n - j0), R = std::min(n - j0, w + kl);
      const int64_t ncol = std::min(n, j0 + w + kl + ku) - (j0 + w);
      fa += (double)ncol * (double)(w * (w - 1) + 2 * (R - w) * w);
      for (int64_t k = 0; k < w; ++k) {
        const int64_t rows = std::min(R, k + kl + 1) - (k + 1);
        fp += (double)rows * (1 + 2 * (w - k - 1));
      }
    }
  }
  *fpanel = fp;
  *fapply = fa;
}

// Diagnostic: assemble at (time, dt), factor once with the persistent kernel
// and copy its per-panel clock stamps (12 int64 per panel, see
// blk_lu_factor_persist) to out[0 .. 12 * npan).  Returns npan, or a negative
// status.
extern "C" int mafem_trace_factor(mafem_handle* h, double time, double dt, int64_t* out, int64_t cap) {
  if (!h || !out || !h->use_blk || h->pers.grid <= 0) return MAFEM_ERR_UNSUPPORTED;
  const int npan = h->blk.npan();
  if (cap < 12LL * npan) return MAFEM_ERR_ARG;
  long long* d_tr = nullptr;
  CK(cudaMalloc(&d_tr, sizeof(long long) * 12 * npan));
  CK(cudaMemsetAsync(d_tr, 0, sizeof(long long) * 12 * npan, h->st));
  int rc = assemble(h, time, dt);
  if (rc) return rc;
  CK(cudaMemcpyAsync(h->d_x, h->d_r, h->nmdf * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  CK(cudaMemsetAsync(h->d_info, 0, sizeof(int), h->st));
  ++h->fepoch;
  const bool fp64 = h->precision == MAFEM_PLAIN_FP64;
  const int nl = fp64 ? blk_lu_factor_persist<double>((double*)h->d_band, h->L, h->blk, h->pers, h->fepoch, h->d_perm,
                                                      (double*)h->d_rdiag, h->d_info, h->d_x, h->d_info + 1, h->st,
                                                      d_tr)
                      : blk_lu_factor_persist<float>((float*)h->d_band, h->L, h->blk, h->pers, h->fepoch, h->d_perm,
                                                     (float*)h->d_rdiag, h->d_info, nullptr, h->d_info + 1, h->st,
                                                     d_tr);
  blk_after_factor(h);
  h->factored = true;
  h->last_blk = true;
  CK(cudaMemcpyAsync(out, d_tr, sizeof(long long) * 12 * npan, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  cudaFree(d_tr);
  return nl < 0 ? MAFEM_ERR_CUDA : npan;
}

// Assemble the resident state and run the batched FP32 solve on this handle
// alone with its factorisation traced: 6 stamps per panel into out (see
// patch_factor_kernel), plus the factor and refine kernels' device times in
// out[6 npan], out[6 npan + 1] (ns).  Returns npan.
extern "C" int mafem_trace_patch_solve(mafem_handle* h, double time, double dt, int64_t* out, int64_t cap) {
  if (!h || !out || !h->patch_ok) return MAFEM_ERR_UNSUPPORTED;
  const int npan = h->blk.npan();
  // factor stamps, 4 per refinement sweep (up to 32), 16 phase sums, 32 relative residuals
  const int64_t ntr = 6LL * npan + 4 * 32 + 16 + 32;
  if (cap < ntr + 4) return MAFEM_ERR_ARG;  // 6 npan + 182
  long long* d_tr = nullptr;
  PatchJob* d_job = nullptr;
  int* d_ord = nullptr;
  CK(cudaMalloc(&d_tr, sizeof(long long) * ntr));
  CK(cudaMalloc(&d_job, sizeof(PatchJob)));
  CK(cudaMalloc(&d_ord, sizeof(int)));
  PatchJob J = h->job;
  J.trace = d_tr;
  CK(cudaMemcpyAsync(d_job, &J, sizeof J, cudaMemcpyHostToDevice, h->st));
  CK(cudaMemsetAsync(d_ord, 0, sizeof(int), h->st));
  CK(cudaMemsetAsync(d_tr, 0, sizeof(long long) * ntr, h->st));
  int rc = assemble(h, time, dt, true);
  if (rc) return rc;
  CK(cudaMemsetAsync(h->d_info, 0, 4 * sizeof(int), h->st));
  cudaEvent_t e0, e1, e2;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventCreate(&e2);
  const int dyn = patch_solve_setup();
  cudaEventRecord(e0, h->st);
  const int nr = patch_ctas(h);  // as a batch would run it
  patch_solve_stage(d_job, d_ord, 1, nr, patch_factor_smem(h->L.kl), 0, 0, 0.0, h->st);
  cudaEventRecord(e1, h->st);
  patch_solve_stage(d_job, d_ord, 1, 1, 0, patch_refine_smem(h->L.n), h->max_refine, h->refine_tol, h->st);
  cudaEventRecord(e2, h->st);
  std::vector<long long> tr((size_t)ntr);
  CK(cudaMemcpyAsync(tr.data(), d_tr, tr.size() * sizeof(long long), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  float mf = 0, mr = 0;
  cudaEventElapsedTime(&mf, e0, e1);
  cudaEventElapsedTime(&mr, e1, e2);
  for (int64_t k = 0; k < 6LL * npan; ++k) out[k] = tr[(size_t)k];
  out[6 * npan] = (int64_t)(mf * 1e6);
  out[6 * npan + 1] = (int64_t)(mr * 1e6);
  for (int64_t k = 0; k < 4 * 32 + 16 + 32; ++k) out[6 * npan + 2 + k] = tr[(size_t)(6 * npan + k)];
  int st2[2] = {0, 0};  // the refinement's status and sweeps
  CK(cudaMemcpy(st2, h->d_info + 2, sizeof st2, cudaMemcpyDeviceToHost));
  out[ntr + 2] = st2[0];
  out[ntr + 3] = st2[1];
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  cudaFree(d_tr);
  cudaFree(d_job);
  cudaFree(d_ord);
  h->factored = false;
  return dyn > 0 ? npan : MAFEM_ERR_CUDA;
}

// calc_pull_force (PullForce.jl:61-80) with get_pull_el_id / get_adj_maps
// (PullForce.jl:8-53): the velocity residual rv of calc_elem_dof_residuals
// (area Gauss points only) of the (2·poly+1)² elements around the pulled
// element (ceil(numel/2), or the centre element with args.pull_centre),
// summed over that element's nodes.  The element rows come
// from the element kernel (area-only mode on the 25-element list); the sum is
// done here in a fixed order.
extern "C" int mafem_pull_force(mafem_handle* h, double* f_out) {
  if (!h || !f_out) return MAFEM_ERR_ARG;
  const int poly = h->p.poly, n1 = h->p.num1el, numel = h->numel, nq = h->nq, ndf = h->ndf;
  const int pull = pull_element(n1, h->p.num2el, h->a) - 1;  // get_pull_el_id (or the centre rule), 0-based
  std::vector<int> adj;
  for (int i = -poly; i <= poly; ++i)
    for (int j = -poly; j <= poly; ++j) adj.push_back(pull + i * n1 + j);
  for (int e : adj)
    if (e < 0 || e >= numel) {
      h->err = "the pull element's neighbourhood leaves the patch";
      return MAFEM_ERR_ARG;
    }
  if ((int)adj.size() > 25) {
    h->err = "pull-force neighbourhood larger than 5 x 5 elements";
    return MAFEM_ERR_UNSUPPORTED;
  }
  const int na = (int)adj.size();
  CK(cudaMemcpyAsync(h->d_pull_list, adj.data(), na * sizeof(int), cudaMemcpyHostToDevice, h->st));
  CK(launch_elem<double>(h->P, h->pp, 0.0, 0.0, h->d_pull_r, (double*)nullptr, h->st, h->d_pull_list, na, 1));
  h->launches += 1;
  std::vector<double> r((size_t)na * nq);
  CK(cudaMemcpyAsync(r.data(), h->d_pull_r, r.size() * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  const int* pn = h->h_ix.data() + (size_t)pull * 9;
  double f[3] = {0.0, 0.0, 0.0};
  for (int k = 0; k < na; ++k)
    for (int a = 0; a < 9; ++a) {
      const int node = h->h_ix[(size_t)adj[k] * 9 + a];
      if (std::find(pn, pn + 9, node) == pn + 9) continue;
      for (int c = 0; c < 3; ++c) {
        const int d = h->pp.dof_of[c];
        if (d >= 0) f[c] += r[(size_t)k * nq + a * ndf + d];
      }
    }
  for (int c = 0; c < 3; ++c) f_out[c] = f[c];
  return MAFEM_OK;
}

// x_pull of run_analysis! (src/Analysis.jl:83-84): the mean position of the
// pull element's nine nodes, summed in IX order and divided by 9.
extern "C" int mafem_pull_position(mafem_handle* h, double* x_out) {
  if (!h || !x_out) return MAFEM_ERR_ARG;
  const int pull = pull_element(h->p.num1el, h->p.num2el, h->a) - 1;
  std::vector<double> xms((size_t)h->numnp * 3);
  CK(cudaMemcpyAsync(xms.data(), h->P.xms, xms.size() * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  for (int c = 0; c < 3; ++c) {
    double s = 0.0;
    for (int a = 0; a < 9; ++a) s += xms[(size_t)c * h->numnp + h->h_ix[(size_t)pull * 9 + a]];
    x_out[c] = s / 9.0;
  }
  return MAFEM_OK;
}

// ---- state files and device snapshots ------------------------------------------
// The files run_analysis! writes after each step (src/Analysis.jl:75-78) and
// restart / prepare_input read (src/MembraneAleFem.jl:75-107,
// src/Input.jl:35-37); the formatting and the writer thread are in
// state_io.cpp.

static int snap_ptrs(mafem_handle* h, int32_t slot, double** xms, double** cps) {
  if (slot == -1) {
    *xms = h->P.xms;
    *cps = h->P.cps;
    return MAFEM_OK;
  }
  if (slot < 0 || slot >= h->nsnap) {
    h->err = "snapshot slot " + std::to_string(slot) + " out of range (" + std::to_string(h->nsnap) + " reserved)";
    return MAFEM_ERR_ARG;
  }
  const size_t per = (size_t)h->numnp * (3 + h->ndf);
  *xms = h->d_snap + per * slot;
  *cps = *xms + (size_t)h->numnp * 3;
  return MAFEM_OK;
}

extern "C" int mafem_write_state_async(mafem_handle* h, int32_t slot, const char* dir, int64_t t_id) {
  if (!h || !dir) return MAFEM_ERR_ARG;
  double *xms, *cps;
  int rc = snap_ptrs(h, slot, &xms, &cps);
  if (rc) return rc;
  if (!h->writer) {
    auto w = std::make_unique<StateWriter>();
    rc = w->init(h->numnp, h->ndf, 3, h->err);
    if (rc) return rc;
    h->writer = std::move(w);
  }
  return h->writer->submit(xms, cps, h->st, state_file(dir, t_id, "xms"), state_file(dir, t_id, "cps"), h->err);
}

extern "C" int mafem_flush_state_writes(mafem_handle* h) {
  if (!h) return MAFEM_ERR_ARG;
  return h->writer ? h->writer->flush(h->err) : MAFEM_OK;
}

extern "C" int mafem_write_state(mafem_handle* h, const char* dir, int64_t t_id) {
  const int rc = mafem_write_state_async(h, -1, dir, t_id);
  const int rf = h ? mafem_flush_state_writes(h) : MAFEM_ERR_ARG;
  return rc ? rc : rf;
}

extern "C" int mafem_read_state(mafem_handle* h, const char* xms_file, const char* cps_file) {
  if (!h || !xms_file || !cps_file) return MAFEM_ERR_ARG;
  std::vector<double> xms((size_t)h->numnp * 3), cps((size_t)h->numnp * h->ndf);
  int rc = readdlm(xms_file, xms.data(), h->numnp, 3, h->err);
  if (!rc) rc = readdlm(cps_file, cps.data(), h->numnp, h->ndf, h->err);
  if (rc) return rc;
  return mafem_upload_state(h, xms.data(), cps.data());
}

extern "C" int mafem_snapshot_reserve(mafem_handle* h, int32_t nslots) {
  if (!h || nslots < 1) return MAFEM_ERR_ARG;
  if (h->nsnap) {
    if (nslots == h->nsnap) return MAFEM_OK;
    h->err = "snapshots are already reserved with another slot count";
    return MAFEM_ERR_ARG;
  }
  const int rc = dalloc(h, &h->d_snap, (size_t)nslots * h->numnp * (3 + h->ndf));
  if (rc) return rc;
  h->nsnap = nslots;
  return MAFEM_OK;
}

extern "C" int mafem_snapshot(mafem_handle* h, int32_t slot) {
  if (!h || slot < 0) return MAFEM_ERR_ARG;
  double *xms, *cps;
  const int rc = snap_ptrs(h, slot, &xms, &cps);
  if (rc) return rc;
  CK(cudaMemcpyAsync(xms, h->P.xms, sizeof(double) * h->numnp * 3, cudaMemcpyDeviceToDevice, h->st));
  CK(cudaMemcpyAsync(cps, h->P.cps, sizeof(double) * h->numnp * h->ndf, cudaMemcpyDeviceToDevice, h->st));
  return MAFEM_OK;
}

extern "C" int mafem_restore(mafem_handle* h, int32_t slot) {
  if (!h || slot < 0) return MAFEM_ERR_ARG;
  double *xms, *cps;
  const int rc = snap_ptrs(h, slot, &xms, &cps);
  if (rc) return rc;
  CK(cudaMemcpyAsync(h->P.xms, xms, sizeof(double) * h->numnp * 3, cudaMemcpyDeviceToDevice, h->st));
  CK(cudaMemcpyAsync(h->P.cps, cps, sizeof(double) * h->numnp * h->ndf, cudaMemcpyDeviceToDevice, h->st));
  return MAFEM_OK;
}

extern "C" int mafem_set_dirichlet_scale(mafem_handle* h, double scale) {
  if (!h || !std::isfinite(scale)) return MAFEM_ERR_ARG;
  launch_dirichlet_scale(h->P.cps, h->d_dir_idx, h->d_dir_val, h->n_dir, scale, h->st);
  h->launches += h->n_dir > 0 ? 1 : 0;
  CK(cudaGetLastError());
  return MAFEM_OK;
}

extern "C" int mafem_set_wait_test(mafem_handle* h, int32_t limit_polls, int32_t withhold_panel) {
  if (!h || limit_polls < 0 || withhold_panel < -1) return MAFEM_ERR_ARG;
  h->wait_test.limit = limit_polls;
  h->wait_test.withhold = withhold_panel;
  return MAFEM_OK;
}

// Solve K x = rhs for a caller's K (host band in mafem_calc_r_K's layout)
// through the handle's own factorisation and solves: the band replaces the
// assembled tangent (and, in the FP32 form, the refinement's A0).
extern "C" int mafem_solve_band(mafem_handle* h, const double* band, int64_t ldab, const double* rhs, double* x_out) {
  if (!h || !band || !rhs || !x_out) return MAFEM_ERR_ARG;
  const BandLayout& L = h->L;
  if (ldab < 2LL * L.kl + L.ku + 1) {
    h->err = "ldab must be >= 2*kl + ku + 1";
    return MAFEM_ERR_ARG;
  }
  const int64_t n = h->nmdf;
  const size_t rows = 2 * (size_t)L.kl + L.ku + 1;
  // the handle's padded layout: column j at j*ldb, the caller's row r at row nb + r
  // (rows 0..nb-1 and nb+rows..ldb-1 of every column are padding, zero)
  std::vector<double> hb64;
  if (h->precision == MAFEM_PLAIN_FP64) {
    hb64.assign((size_t)L.ldb * n, 0.0);
    for (int64_t j = 0; j < n; ++j)
      for (size_t r = 0; r < rows; ++r) hb64[(size_t)j * L.ldb + L.nb + r] = band[j * ldab + r];
    CK(cudaMemcpyAsync(h->d_band, hb64.data(), hb64.size() * sizeof(double), cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
  } else {
    std::vector<float> tmp((size_t)L.ldb * n, 0.0f);
    for (int64_t j = 0; j < n; ++j)
      for (size_t r = 0; r < rows; ++r) tmp[(size_t)j * L.ldb + L.nb + r] = (float)band[j * ldab + r];
    CK(cudaMemcpyAsync(h->d_band, tmp.data(), tmp.size() * sizeof(float), cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
  }
  h->factored = false;
  CK(cudaMemsetAsync(h->d_info, 0, 2 * sizeof(int), h->st));
  CK(cudaMemcpyAsync(h->d_res, rhs, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
  double* rdev = h->precision == MAFEM_PLAIN_FP64 ? h->d_dx : h->d_r;
  CK(cudaMemcpyAsync(rdev, h->d_res, n * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  int sweeps = 0;
  const int64_t fb0 = h->fallbacks;
  h->host_band = h->precision == MAFEM_PLAIN_FP64 ? hb64.data() : nullptr;
  int rc = factor_and_solve(h, rdev, &sweeps);
  if (rc == MAFEM_OK) CK(cudaStreamSynchronize(h->st));  // hb64 must outlive the fallback's copy
  h->host_band = nullptr;
  h->factored = false;  // the band holds the caller's matrix, not the assembled tangent
  if (rc) return rc;
  CK(cudaMemcpyAsync(x_out, h->d_x, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(h->h_out + 5, h->d_info, 2 * sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  rc = check_info(h);
  if (rc == MAFEM_OK && h->fallbacks > fb0) h->err = "solved with full partial pivoting (a node block had no usable pivot)";
  return rc;
}

extern "C" int64_t mafem_fallback_count(const mafem_handle* h) { return h ? h->fallbacks : -1; }

extern "C" int mafem_set_refinement(mafem_handle* h, int32_t max_sweeps, double tol) {
  if (!h || max_sweeps < 1 || max_sweeps > 1000 || !(tol > 0.0) || !(tol < 1.0)) return MAFEM_ERR_ARG;
  h->max_refine = max_sweeps;
  h->refine_tol = tol;
  return MAFEM_OK;
}

extern "C" int mafem_set_lu_path(mafem_handle* h, int32_t path) {
  if (!h || path < MAFEM_LU_AUTO || path > MAFEM_LU_FULL) return MAFEM_ERR_ARG;
  if (path == MAFEM_LU_PANELS && !h->use_blk) {
    h->err = "the node-block LU is not available for this band";
    return MAFEM_ERR_UNSUPPORTED;
  }
  h->lu_path = path;
  h->factored = false;
  return MAFEM_OK;
}

extern "C" int mafem_autotune_patch(mafem_handle* h) {
  if (!h) return MAFEM_ERR_ARG;
  if (!h->patch_ok) {
    h->err = "the batched FP32 form does not serve this handle";
    return MAFEM_ERR_UNSUPPORTED;
  }
  PatchJob* d_job = nullptr;
  int* d_tmp = nullptr;
  cudaError_t e = cudaMalloc(&d_job, sizeof(PatchJob));
  if (e == cudaSuccess) e = cudaMalloc(&d_tmp, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_job, &h->job, sizeof(PatchJob), cudaMemcpyHostToDevice, h->st);
  int rc = e == cudaSuccess ? patch_tune(h, d_job, 0, d_tmp, h->st) : MAFEM_ERR_CUDA;
  if (e != cudaSuccess) h->err = std::string("mafem_autotune_patch: ") + cudaGetErrorString(e);
  cudaStreamSynchronize(h->st);
  if (d_job) cudaFree(d_job);
  if (d_tmp) cudaFree(d_tmp);
  return rc;
}

extern "C" int mafem_set_patch_ctas(mafem_handle* h, int32_t ctas) {
  if (!h || (ctas != 0 && ctas != 1 && ctas != 2 && ctas != 4)) return MAFEM_ERR_ARG;
  h->patch_nr = ctas;
  return MAFEM_OK;
}

extern "C" int mafem_profile_factor(mafem_handle* h, double time, double dt, mafem_kernel_times* out) {
  if (!h || !out) return MAFEM_ERR_ARG;
  std::memset(out, 0, sizeof *out);
  cudaEvent_t a0, a1;
  CK(cudaEventCreate(&a0));
  CK(cudaEventCreate(&a1));
  const int64_t npan = h->use_blk ? h->blk.npan() : h->npan;
  std::vector<cudaEvent_t> ev((size_t)3 * npan);
  for (auto& e : ev) CK(cudaEventCreate(&e));
  CK(cudaStreamSynchronize(h->st));
  CK(cudaEventRecord(a0, h->st));
  int rc = assemble(h, time, dt);
  if (rc) return rc;
  CK(cudaEventRecord(a1, h->st));
  CK(cudaMemcpyAsync(h->d_x, h->d_r, h->nmdf * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  CK(cudaMemsetAsync(h->d_info, 0, sizeof(int), h->st));
  const bool fp64 = h->precision == MAFEM_PLAIN_FP64;
  if (h->use_blk) {
    if (fp64)
      blk_lu_factor<double>((double*)h->d_band, h->L, h->blk, h->d_perm, (double*)h->d_rdiag, h->d_info, h->d_x, h->st,
                            nullptr, nullptr, ev.data());
    else
      blk_lu_factor<float>((float*)h->d_band, h->L, h->blk, h->d_perm, (float*)h->d_rdiag, h->d_info, nullptr, h->st,
                           nullptr, nullptr, ev.data());
    blk_after_factor(h);
  } else if (fp64) {
    band_lu_factor<double>((double*)h->d_band, h->L, h->d_ipiv, h->d_perm, h->rmax, h->d_info, h->d_x,
                           h->apply_threads, h->apply_blocks, h->st, nullptr, nullptr, ev.data());
  } else {
    band_lu_factor<float>((float*)h->d_band, h->L, h->d_ipiv, h->d_perm, h->rmax, h->d_info, nullptr,
                          h->apply_threads, h->apply_blocks, h->st, nullptr, nullptr, ev.data());
  }
  h->factored = true;
  h->last_blk = h->use_blk;
  CK(cudaStreamSynchronize(h->st));
  float ms = 0;
  cudaEventElapsedTime(&ms, a0, a1);
  out->ms_assemble = ms;
  for (int64_t p = 0; p < npan; ++p) {
    float m1 = 0, m2 = 0;
    cudaEventElapsedTime(&m1, ev[3 * p], ev[3 * p + 1]);
    cudaEventElapsedTime(&m2, ev[3 * p + 1], ev[3 * p + 2]);
    out->ms_panel += m1;
    out->ms_apply += m2;
  }
  out->n_panel = npan;
  out->n_apply = npan;
  out->n = h->nmdf;
  out->kl = h->L.kl;
  out->ku = h->L.ku;
  out->nb = h->L.nb;
  out->ndfp = h->use_blk ? h->blk.ndfp : -1;
  lu_flops(h, &out->flop_panel, &out->flop_apply);
  for (auto& e : ev) cudaEventDestroy(e);
  cudaEventDestroy(a0);
  cudaEventDestroy(a1);
  return MAFEM_OK;
}

// FP64 FMA throughput of the current device (independent FMA chains, all SMs):
// the compute roof of the FP64 kernels, measured rather than assumed.
__global__ void fp64_fma_probe_kernel(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

extern "C" int mafem_probe_fp64_tflops(double* tflops) {
  if (!tflops) return MAFEM_ERR_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    set_global_error("no CUDA device");
    return MAFEM_ERR_CUDA;
  }
  const int nb = sms * 8, nt = 256, iters = 2000;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * nb * nt) != cudaSuccess) return MAFEM_ERR_OOM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  for (int w = 0; w < 2; ++w) fp64_fma_probe_kernel<<<nb, nt>>>(out, iters, 0.999999, 1e-7);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    fp64_fma_probe_kernel<<<nb, nt>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    best = std::min(best, ms);
  }
  cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) {
    set_global_error(cudaGetErrorString(e));
    return MAFEM_ERR_CUDA;
  }
  *tflops = 2.0 * 8 * (double)iters * nb * nt / (best * 1e-3) / 1e12;
  return MAFEM_OK;
}
