// mafem_internal.h -- internal types shared by the library's translation units.
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <vector>

#include "mafem.h"

namespace mafem {

// Host copy of the reference's Mesh fields, in the C ABI's layout
// (mafem_mesh_desc): 1-based, column-major, int64.
struct HostMesh {
  int num1el = 0, num2el = 0, numel = 0, num1np = 0, num2np = 0, numnp = 0, ndf = 0;
  int64_t nmdf = 0;
  int64_t dofs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  std::vector<double> kv1, kv2;
  std::vector<int64_t> IX, ID;
  int64_t n_uel = 0;
  std::vector<int64_t> uel_ids;
  std::vector<double> ufns;
  int64_t bdry_n_uel[4] = {0, 0, 0, 0};
  std::vector<int64_t> bdry_uel_ids[4];
  std::vector<double> bdry_ufns[4];
  std::vector<int64_t> neu_bdry, neu_type;
  std::vector<double> neu_val;
  std::vector<int64_t> dir_unknown, dir_node;
  std::vector<double> dir_val;
  double lambda0 = 0.0;  // F_PULL edge tension and initial λ (kb / 4 unless mafem_args.lambda0 > 0)
};

// 1-based id of the pulled element: ceil(numel / 2) (get_pull_el_id,
// PullForce.jl:8-13), or with a.pull_centre the element
// (floor(n1/2) + 1, floor(n2/2) + 1) numbered e1 + n1 (e2 - 1) (Mesh.jl:582-589).
inline int pull_element(int n1, int n2, const mafem_args& a) {
  if (a.pull_centre) return (n1 / 2 + 1) + n1 * (n2 / 2);
  return (n1 * n2 + 1) / 2;
}
// F_PULL's tension value: kb / 4 (Bc.jl:259, Input.jl:85) unless a.lambda0 > 0.
inline double pull_tension(const mafem_params& p, const mafem_args& a) { return a.lambda0 > 0 ? a.lambda0 : p.kb / 4; }

// ---- state files (state_io.cpp) -------------------------------------------------
// Julia's print(::Float64), appended to out.
void format_double(double x, std::string& out);
// writedlm / readdlm of a column-major rows x cols matrix (a[i + rows*j]).
int writedlm(const char* path, const double* a, int64_t rows, int64_t cols, std::string& err);
int readdlm(const char* path, double* a, int64_t rows, int64_t cols, std::string& err);
// "<dir>/t<t_id>-<which>.txt", the names run_analysis! writes.
std::string state_file(const char* dir, int64_t t_id, const char* which);

int build_mesh(const mafem_params& p, const mafem_args& a, HostMesh& m, std::string& err);
void mesh_desc(const HostMesh& m, mafem_mesh_desc& d);
int prepare_input(const HostMesh& m, const mafem_params& p, double* xms, double* cps, std::string& err);
void set_global_error(const std::string& s);

// ---------------------------------------------------------------------------
// Device-side description of one patch.  All pointers are device pointers.
// Control-point state is stored exactly like the host arrays: xms as 3
// columns of numnp doubles, cps as ndf columns of numnp doubles (SoA).
constexpr int kMaxNeu = 8;
constexpr int kTab = 56;  // doubles per GP record: w, N[9], dN[18], ddN[27], pad

struct PhysParams {
  int motion, scenario, ndf, nq;      // nq = 9*ndf element dofs (tangent directions)
  double kb, kg, zv, pn, adb, am;
  int dof_of[8];                      // 0-based dof of Unknown u (vx..pm), -1 if absent
  int unk_of[8];                      // Unknown (0..7) of dof d (0-based), for d < ndf
  int mmo[3];                         // 0-based dof of m_motion_order[j], -1 if none
  int n_neu;
  int neu_bdry[kMaxNeu];              // 0..3 = BOTTOM, RIGHT, TOP, LEFT
  int neu_type[kMaxNeu];              // SHEAR/STRETCH/MOMENT
  double neu_val[kMaxNeu];
  double bend_tm;
};

struct DevPatch {
  int numel, numnp, num1el, num2el, num1np, num2np;
  int64_t nmdf;
  int kl, ku;                         // half bandwidths of K
  // mesh tables
  const int* ix;                      // [numel][9] 0-based node numbers
  const int* lm;                      // [numel][nq] 0-based unknown, -1 = Dirichlet
  const int* uel;                     // [numel] unique area element (0-based)
  const double* tab;                  // [n_uel][9][kTab]
  const double* db;                   // [n_uel][81] Dohrmann-Bochev Gᵀ H⁻¹ G
  const int* bref;                    // [numel][4] boundary GP table row per boundary, -1 if not on it
  const double* btab;                 // [rows][3][kTab] boundary GP tables
  const int* unk_node;                // [nmdf] node of unknown q (0-based)
  const int* unk_dof;                 // [nmdf] dof of unknown q (0-based)
  const int* node_unk;                // [numnp][ndf] unknown of (node, dof), -1 if Dirichlet
  // state
  double* xms;                        // [3][numnp]
  double* cps;                        // [ndf][numnp]
};

// Band storage of an n x n matrix with lower/upper half bandwidths kl, ku and
// panel width nb: column-major, ldb rows per column; A(i, j) lives at
// ab[(size_t)j * ldb + off + i - j] with off = kl + ku + nb.  Rows
// [0, nb) hold U entries beyond the pivoting fill (kept zero), rows
// [off + kl + 1, off + kl + nb] hold panel-local L fill (lower-left triangle).
struct BandLayout {
  int64_t n;
  int kl, ku, nb;
  int64_t ldb, off;
};
BandLayout make_band_layout(int64_t n, int kl, int ku, int nb);

}  // namespace mafem

// ---- kernel launchers (elem.cu, assemble.cu, band_lu.cu) ----------------------
#include <cuda.h>  // CUtensorMap
#include <cuda_runtime.h>
namespace mafem {
template <class T>
size_t elem_smem_bytes(int nq, int epb);
template <class T>
cudaError_t launch_elem(const DevPatch& P, const PhysParams& pp, double time, double dt, double* r_el, T* K_el,
                        cudaStream_t st, const int* elist = nullptr, int nlist = 0, int area_only = 0);
template <class T>
void launch_band_gather(const DevPatch& P, int ndf, int nq, const BandLayout& L, const T* K_el, T* ab,
                        cudaStream_t st, T* ab2 = nullptr);
void launch_resid_gather(const DevPatch& P, int ndf, int nq, const double* r_el, double* r, cudaStream_t st);
void launch_predictor(const DevPatch& P, const PhysParams& pp, double dt, cudaStream_t st);
// cps[idx[k]] = s * val[k] for k < n (the scaled inhomogeneous Dirichlet values)
void launch_dirichlet_scale(double* cps, const int* idx, const double* val, int n, double s, cudaStream_t st);
int newton_update_blocks(int64_t nmdf);
void launch_newton_update(const DevPatch& P, const PhysParams& pp, double dt, const double* x, const double* r,
                          double* part, double* out, cudaStream_t st, const int* skip = nullptr,
                          const int* skip2 = nullptr, const int* skip3 = nullptr);
int band_residual_blocks(int64_t n);
template <class T>
void launch_band_residual(const T* a0, const BandLayout& L, const double* x, const double* r, double* res,
                          double* part, double* out, cudaStream_t st, const int* gate = nullptr);
void launch_axpy(int64_t n, const double* dx, double* x, cudaStream_t st);
// x += dx; out[0] = |dx|, out[1] = |x| (part: 2048 doubles of scratch)
void launch_axpy_norms(int64_t n, const double* dx, double* x, double* part, double* out, cudaStream_t st,
                       const int* gate = nullptr);
// Device-side stopping test of a handle's iterative refinement (assemble.cu):
// st = {done, sweeps, status}, nrm = {|r0|, previous |r|}; kernels given
// gate = st do nothing once done is set.
void launch_refine_init(const double* r0, int* st, double* nrm, cudaStream_t s);
void launch_refine_check(const double* rn, const double* dxn, int* st, double* nrm, double tol, int max_sweeps,
                         cudaStream_t s);
void launch_copy_gated(int64_t n, const double* src, double* dst, const int* gate, cudaStream_t s);
// st[3] = 1 unless the refinement has stopped with MAFEM_OK.
void launch_refine_seal(int* st, cudaStream_t s);

template <class T>
size_t apply_smem_bytes(const BandLayout& L, int threads);
template <class T>
cudaError_t band_lu_setup(const BandLayout& L, int apply_threads);
// Enqueues the blocked factorisation; returns the number of kernels launched.
// st2 + ev_pool (2*npan+2 events) enable the two-stream lookahead; with
// prof != nullptr it runs serially on st and records prof[3p], prof[3p+1],
// prof[3p+2] around panel p's two kernels.
template <class T>
int band_lu_factor(T* ab, const BandLayout& L, int* ipiv, int* perm_all, int rmax, int* info, T* rhs,
                   int apply_threads, int apply_blocks, cudaStream_t st, cudaStream_t st2, cudaEvent_t* ev_pool,
                   cudaEvent_t* prof);
template <class T, class V>
cudaError_t band_solve_setup(const BandLayout& L);
template <class T, class V>
void band_forward(const T* ab, const BandLayout& L, const int* perm_all, int rmax, V* b, cudaStream_t st);
template <class T, class V>
void band_backward(const T* ab, const BandLayout& L, V* y, cudaStream_t st);

// node-block pivoted banded LU (band_lu_blk.cu).  Panels are runs of whole
// pivot blocks (the unknowns of one control point), at most wmax <= 32 wide.
constexpr int kBlkW = 32;  // widest panel; also the stride of the per-panel permutations
struct BlkPlan {
  int ndfp = 0;          // largest block size - 1
  int wmax = 0;          // widest panel
  int kuf = 0;           // bandwidth of U after the interchanges: ku + ndfp
  std::vector<int> ps;   // panel starts; ps.back() == n
  int* d_ps = nullptr;   // device copy of ps
  const int* d_blk_end = nullptr;  // per unknown: one past the last unknown of its block
  int npan() const { return (int)ps.size() - 1; }
};
// Host: panel starts for blocks `blk_end` (false if a block is wider than wmax).
bool blk_plan(const std::vector<int>& blk_end, int wmax, int ku, BlkPlan& out);
// Widest panel (<= kBlkW, <= L.nb) whose kernels fit the device's shared memory; 0 if none.
template <class T>
int blk_lu_setup(const BandLayout& L);
template <class T>
int blk_lu_factor(T* ab, const BandLayout& L, const BlkPlan& B, int* perm_all, T* rdiag, int* info, T* rhs,
                  cudaStream_t st, cudaStream_t st2, cudaEvent_t* ev_pool, cudaEvent_t* prof);
template <class V, class T>
void blk_forward(const T* ab, const BandLayout& L, const BlkPlan& B, const int* perm_all, const T* rdiag, V* b,
                 cudaStream_t st);
// Back substitution U x = y in place on many SMs (one cooperative launch of
// `grid` CTAs, grid <= blk_backward_grid()).  flags: npan ints, epoch: a value
// they do not hold yet (incremented per call); err: nonzero after a bounded
// wait ran out.  Returns -1 if the launch failed.
// Failure-detection test hook of the cooperative substitutions: limit = polls
// before a wait gives up (<= 0: the default), withhold = k: the back
// substitution never publishes the flag of panel npan - 1 - k (-1: none).
struct WaitTest {
  int limit = 0;
  int withhold = -1;
};
// Explicit inverses of the stored panels' L11 and U11 (inv: npan x 2 x 32 x
// 32 in V) for the cooperative substitutions; run after each factorisation.
template <class V, class T>
void blk_inverses(const T* ab, const BandLayout& L, const BlkPlan& B, const T* rdiag, V* inv, cudaStream_t st);
template <class V, class T>
int blk_backward(const T* ab, const BandLayout& L, const BlkPlan& B, const V* inv, V* y, int* flags, int epoch,
                 int* err, int grid, cudaStream_t st, WaitTest wt = WaitTest(), const int* gate = nullptr);
template <class V, class T>
int blk_backward_grid();
// Forward substitution (P, L11, A21 of the stored panels) on `grid` CTAs of one
// cooperative launch, in place on b; zbuf: npan x 32 scratch; flags/epoch as
// for blk_backward.  Returns 0, or -1 if the cooperative launch was refused.
template <class V, class T>
int blk_forward_coop(const T* ab, const BandLayout& L, const BlkPlan& B, const int* perm_all, const V* inv, V* b,
                     V* zbuf, int* flags, int epoch, int* err, int grid, cudaStream_t st, WaitTest wt = WaitTest(),
                     const int* gate = nullptr);
// Persistent cooperative factorisation (band_lu_persist.cu): launch shape and
// per-panel flags.  Flags are zeroed once; epochs make them reusable.
struct BlkPersist {
  int grid = 0;            // CTAs of the launch: min_grid <= grid <= max_grid
  int min_grid = 0;        // fewest CTAs that give every worker <= kMaxCols columns per panel
  int max_grid = 0;        // the device's SM count
  size_t smem = 0;
  int* d_pdone = nullptr;
  int* d_critcnt = nullptr;
  int* d_a21cnt = nullptr;
};
// Fills S (host part); returns the grid (0: not available on this device / size).
template <class T>
int blk_persist_setup(const BandLayout& L, const BlkPlan& B, BlkPersist& S);
// One launch; returns 1, or -1 if the cooperative launch was refused.
template <class T>
// trace (optional, device): 12 globaltimer stamps per panel t -- [0] the
// factorising CTA starts waiting for t's columns, [1] they are ready, [2] t is
// published; for the owner of t's first column: [3] it starts step t - 1,
// [4] its waits are over, [5] panel t - 1 is staged, [6] its columns are
// solved, [7] the rows t reads are written, [8] the rest of the rows,
// [9] its column copies are issued, [10] the A21 copies are issued, [11] the
// diagonal block is in shared memory.
int blk_lu_factor_persist(T* ab, const BandLayout& L, const BlkPlan& B, const BlkPersist& S, int epoch, int* perm_all,
                          T* rdiag, int* info, T* rhs, int* err, cudaStream_t st, long long* trace = nullptr);
template <class V, class T>
void blk_backward_1cta(const T* ab, const BandLayout& L, const BlkPlan& B, const T* rdiag, V* y, cudaStream_t st);
}  // namespace mafem

namespace mafem {
// ---- batched assembly of the FP32 form (elem.cu, assemble.cu) -----------------------
// A batch's Newton round assembles, updates and measures every patch of the
// round with one launch per kernel (per motion for the element kernels): a
// CTA finds its patch by the round's block offsets (off[k] <= CTA < off[k+1]
// for item k) and reads the patch's tables from the job table.  Each patch is
// cut into exactly the CTAs its single-patch launch would use: the same
// arithmetic as the per-patch kernels (the element kernels are compiled
// separately, so a multiply-add may round differently).
struct AsmJob {
  DevPatch P;
  PhysParams pp;
  BandLayout L;
  double* r_el;  // [numel][nq] element residuals
  float* K_el;   // [numel][nq][nq] element tangents
  float* band;   // the band the factorisation overwrites
  float* band0;  // its unfactored copy (refinement residual)
  double* r;     // [nmdf] residual
  double* x;     // [nmdf] the round's solution
  double* part;  // per-CTA partial sums of the Newton update
  double* out;   // [3] eps, |r|, non-finite flag
  int* info;     // [4] zero-pivot column, wait ran out, solve status, sweeps
  const int* dir_idx;     // [n_dir] inhomogeneous Dirichlet entries of cps (dof * numnp + node)
  const double* dir_val;  // [n_dir] their values
  int n_dir;
  int pad;
};
enum { kStartPredict = 1, kStartDirichlet = 2 };  // AsmItem::start
struct AsmItem {  // one patch of a round
  int job;        // index into the job table
  int start;      // first round of a time step: kStartPredict | kStartDirichlet (scale the Dirichlet values first)
  double time, dt;
  double dscale;  // the Dirichlet values' scale (kStartDirichlet)
};
struct AsmOut {  // one patch's results of a round, read by the host
  double out[3];
  int info[4];
};
constexpr int kGatherCols = 4;  // band columns per CTA of the batched gather
// CTAs per patch of each batched kernel
int batch_resid_ctas(int numel);
int batch_tan_ctas(int numel, int epb);  // epb: elements per CTA of the tangent kernel, 2 or 4
inline int batch_gather_ctas(int64_t n) { return (int)((n + kGatherCols - 1) / kGatherCols); }
inline int batch_rgather_ctas(int64_t nmdf) { return (int)((nmdf + 255) / 256); }
inline int batch_pred_ctas(int numnp) { return (3 * numnp + 255) / 256; }
inline int batch_dir_ctas(int n_dir) { return (n_dir + 255) / 256; }
// Sets the batched element kernels' shared-memory limits (once per process and device).
cudaError_t batch_asm_setup();
// The launches of one round.  items / off point at the round's slice (m items,
// off[0 .. m]); each launch covers CTAs off[0] .. off[m] - 1.
cudaError_t launch_batch_resid(int motion, const AsmJob* jobs, const AsmItem* items, const int* off, int m, int ctas,
                               int nq, cudaStream_t st);
cudaError_t launch_batch_tan(int motion, int epb, const AsmJob* jobs, const AsmItem* items, const int* off, int m,
                             int ctas, int nq, cudaStream_t st);
// Both bands and the residual; the residual gather also zeroes each patch's info words.
void launch_batch_gather(const AsmJob* jobs, const AsmItem* items, const int* off, int m, int ctas, cudaStream_t st);
void launch_batch_rgather(const AsmJob* jobs, const AsmItem* items, const int* off, int m, int ctas, cudaStream_t st);
// Newton update of every patch (skipped for a patch whose solve failed) and the
// fixed-order norms, written to the job's out and to outs[k].
void launch_batch_update(const AsmJob* jobs, const AsmItem* items, const int* off, int m, int ctas, AsmOut* outs,
                         cudaStream_t st);
void launch_batch_predictor(const AsmJob* jobs, const AsmItem* items, const int* off, int m, int ctas,
                            cudaStream_t st);
// cps[dir_idx[k]] = dscale * dir_val[k] for the items that start a step with kStartDirichlet
void launch_batch_dirichlet(const AsmJob* jobs, const AsmItem* items, const int* off, int m, int ctas,
                            cudaStream_t st);

// One patch's FP32 solve in the batched form (band_lu_patch.cu): device
// pointers of the handle that owns them.
struct PatchJob {
  CUtensorMap a21_map;  // TMA view of a21: 3-D (k % 4, row, k / 4), box 4 x 128 x 8
  float* band;          // factored in place
  const float* band0;   // the unfactored band (refinement residual)
  float* inv;           // [npan][2][32][32]: L11^-1, U11^-1 per panel, column-major
  const int* ps;        // panel starts [npan + 1]
  const int* blk_end;   // [n]
  int* perm;            // [npan][32]
  float* rdiag;         // [n]
  int* info;            // [0] zero-pivot column, [2] status, [3] sweeps
  int* stat;            // = info + 2
  const double* rhs;    // [n]
  double* x;            // [n] solution
  double* res;          // [n] FP64 residual (workspace)
  float2* xs;           // [n] x as two floats (workspace)
  BandLayout L;
  int kuf, npan;
  long long* trace;     // optional: 6 globaltimer stamps per panel (patch_factor_kernel)
  float* a21;           // split A21 of the current panel: [8][2 a21_rows][4] floats (TF32 hi rows, then lo rows)
  int a21_rows;         // rows per part, a multiple of 128 (patch_a21_rows)
  // the tangent's sparsity for the refinement residual: unknowns couple only
  // within 5 x 5 control points (biquadratic elements); null: walk the whole band
  const int* unk_node;    // [n] control point of each unknown (non-decreasing)
  const int* node_first;  // [numnp + 1] first unknown of each control point
  int num1np, num2np;     // the control-point grid
};
// Rows per part of a patch's split-A21 buffer for half bandwidth kl.
int patch_a21_rows(int kl);
// Encodes J.a21_map over J.a21 (J.a21, J.a21_rows set); returns false if the
// driver refuses the tensor map.
bool patch_a21_map(PatchJob& J);
size_t patch_factor_smem(int kl);
size_t patch_refine_smem(int64_t n);
// Sets the kernels' shared-memory limits; returns the dynamic bytes available (0: unusable).
int patch_solve_setup();
// Trailing columns per chunk of the factorisation (at most).
int patch_chunk_cols();
// CTAs that factor a patch with kuf trailing columns: 4 (a cluster, one chunk
// per CTA) above two chunks, 2 above one chunk, else 1.
int patch_cluster_ctas(int kuf);
// The factor kernel alone (smem_refine == 0; nr = CTAs per patch, 1, 2 or 4) or
// the refine kernel alone (smem_factor == 0).
cudaError_t patch_solve_stage(const PatchJob* d_jobs, const int* d_order, int njobs, int nr, size_t smem_factor,
                              size_t smem_refine, int max_sweeps, double tol, cudaStream_t st);
// Time (ms, CUDA events) of factoring job d_order1[0] on a cluster of nr CTAs,
// on a synthetic band of its shape written over the job's band (which the
// next assembly rewrites); synchronises st.
cudaError_t patch_time_factor(const PatchJob* d_jobs, const int* d_order1, int nr, size_t smem, cudaStream_t st,
                              float* ms);
// kernel launches patch_solve makes for these group sizes
int patch_solve_launches(int n4, int n2, int njobs);
// Factor and solve the jobs d_order[0 .. njobs): the first n4 on four-CTA
// clusters, the next n2 on two-CTA clusters, the rest one CTA each -- the first
// non-empty group on st, the others after one another on st2 (forked from and
// joined to st with ev_fork / ev_join); each stream refines its own jobs after
// their factorisations.
cudaError_t patch_solve(const PatchJob* d_jobs, const int* d_order, int n4, int n2, int njobs, size_t smem_factor,
                        size_t smem_refine, int max_sweeps, double tol, cudaStream_t st, cudaStream_t st2,
                        cudaEvent_t ev_fork, cudaEvent_t ev_join);
}  // namespace mafem

#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
namespace mafem {
// Writes state files off the time loop's critical path: submit() copies
// device xms / cps into a free pinned slot on stream st and returns; a thread
// waits for that copy and writes the two files.  submit() blocks only while
// every slot is still being written.  flush() waits for all pending files and
// returns the first failure since the previous flush.
class StateWriter {
 public:
  ~StateWriter();
  int init(int numnp, int ndf, int depth, std::string& err);
  int submit(const double* d_xms, const double* d_cps, cudaStream_t st, std::string xms_path,
             std::string cps_path, std::string& err);
  int flush(std::string& err);

 private:
  struct Slot {
    double* host = nullptr;  // pinned: xms (numnp x 3) then cps (numnp x ndf)
    cudaEvent_t ev = nullptr;
    bool busy = false;
    std::string xms_path, cps_path;
  };
  void run();
  int numnp_ = 0, ndf_ = 0, device_ = 0;
  std::vector<Slot> slots_;
  std::deque<int> queue_;
  std::mutex mu_;
  std::condition_variable cv_job_, cv_free_;
  bool stop_ = false;
  int first_rc_ = 0;
  std::string first_err_;
  std::thread th_;
};
}  // namespace mafem
