/*
 * mafem.h -- C ABI of libmafem.so, the GB300 (sm_103a) assemble-and-solve
 * library for MembraneAleFem.jl's Newton step.
 *
 * The library replaces the two lines of the reference's `time_step!`
 *     r_gl, K_gl = calc_r_K(mesh, xms, cps, time, Δt, p; args...)   # src/analysis/FiniteElement.jl:35
 *     Δu = -K_gl \ r_gl                                              # src/analysis/FiniteElement.jl:38
 * and, optionally, the whole Newton loop around them (FiniteElement.jl:11-63).
 * Mesh construction, input preparation and the time loop stay with the caller
 * (src/Input.jl, src/Analysis.jl), exactly as in the reference.
 *
 * Conventions
 *  - Every array that crosses this boundary uses the reference's layout:
 *    Julia column-major, 1-based node / unknown numbers, 0 = Dirichlet in ID.
 *    xms is numnp x 3 and cps is numnp x ndf (column-major, Float64).
 *  - Return codes: 0 = OK; > 0 = numerical outcome (the cases where the
 *    reference @asserts); < 0 = usage, CUDA or memory error.  The message of
 *    the last failure is available from mafem_last_error().
 *  - A handle is used by one host thread at a time.  Handles are independent.
 *  - No function allocates device memory after mafem_create() (the
 *    diagnostic mafem_trace_patch_solve excepted: it allocates and frees its
 *    trace buffer); every device buffer of a handle is allocated there and
 *    freed by mafem_destroy().
 */
#ifndef MAFEM_H
#define MAFEM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------- */
#define MAFEM_OK 0
#define MAFEM_NEWTON_NOT_CONVERGED 1 /* FiniteElement.jl:61 @assert */
#define MAFEM_ZERO_PIVOT 2           /* exactly singular tangent */
#define MAFEM_NAN_DETECTED 3         /* non-finite residual or update */
#define MAFEM_REFINE_STALLED 4       /* FP32 factor + FP64 refinement did not converge */
#define MAFEM_ERR_ARG (-1)
#define MAFEM_ERR_CUDA (-2)
#define MAFEM_ERR_OOM (-3)
#define MAFEM_ERR_UNSUPPORTED (-4)
#define MAFEM_ERR_ADMISSION (-5)

/* ---- enums: same numeric values as the reference (src/input/Enums.jl) --------- */
enum mafem_motion { MAFEM_STATIC = 1, MAFEM_EUL = 2, MAFEM_LAG = 3, MAFEM_ALEV = 4, MAFEM_ALEVB = 5 };
enum mafem_scenario { MAFEM_F_CAVI = 1, MAFEM_F_COUE = 2, MAFEM_F_POIS = 3, MAFEM_F_PULL = 4, MAFEM_F_BEND = 5 };
enum mafem_boundary { MAFEM_BOTTOM = 1, MAFEM_RIGHT = 2, MAFEM_TOP = 3, MAFEM_LEFT = 4 };
enum mafem_neumann { MAFEM_SHEAR = 1, MAFEM_STRETCH = 2, MAFEM_MOMENT = 3 };

/* Linear-algebra form of a handle. */
enum mafem_precision {
  MAFEM_PLAIN_FP64 = 0, /* FP64 tangent, FP64 banded LU (node-block partial pivoting) */
  MAFEM_FP32_REFINE = 1 /* FP64 residual; FP32 tangent and FP32 banded LU (same
                           algorithm); FP64 iterative refinement of every solve */
};

/* Which banded LU a handle uses (mafem_set_lu_path; no reference counterpart:
 * the reference calls Julia's sparse `\`).  Testing and diagnostics. */
enum mafem_lu_path {
  MAFEM_LU_AUTO = 0,   /* node-block pivoting as one persistent cooperative launch when the
                          device allows it, else per-panel launches; full partial pivoting
                          when a node block has no usable pivot (the default) */
  MAFEM_LU_PANELS = 1, /* node-block pivoting, per-panel launches */
  MAFEM_LU_FULL = 2    /* full partial pivoting (LAPACK gbtrf's pivot rule) */
};

/* Params (src/input/Params.jl:36-55), field for field. */
typedef struct mafem_params {
  int32_t motion, scenario, num1el, num2el;
  double length, kb, kg, zeta_v, pn;
  int32_t poly, gp1d, nders, nen;
  double alpha_db, alpha_m, eps_k, eps_nr;
} mafem_params;

/* The keyword arguments (`args...`) the hot path reads:
 * pull_speed (src/input/Bc.jl:234,240), bend_tm and bend_mf
 * (src/analysis/FiniteElement.jl:379, src/input/Bc.jl:389-390).
 * Two F_PULL extensions follow; the reference has no such keywords, and their
 * zero values give the reference's behaviour:
 *  - lambda0: the edge tension of the four STRETCH conditions and the initial
 *    λ of every node.  The reference fixes both at kb / 4 (Bc.jl:259,
 *    Input.jl:85); 0 keeps kb / 4.
 *  - pull_centre: which element is pulled.  0 = element ceil(numel / 2)
 *    (get_pull_el_id, PullForce.jl:8-13), which for an even num1el lies on the
 *    right edge; 1 = element (floor(num1el/2) + 1, floor(num2el/2) + 1), the
 *    centre element for any size (the same element as the reference's rule
 *    when num1el == num2el is odd).  The pull force and x_pull use the same
 *    element. */
typedef struct mafem_args {
  double pull_speed, bend_tm, bend_mf;
  double lambda0;
  int32_t pull_centre;
  int32_t reserved; /* 0 */
} mafem_args;

/* A view of the reference's `Mesh` struct (src/input/Mesh.jl:48-80): the fields
 * the hot path reads, in the reference's own layout.  A Julia caller fills it
 * from its `mesh`; mafem_mesh_view() fills it from a mesh
 * built by mafem_mesh_build().  GP tables pack one GpBasisFnsζα
 * (src/input/GpBasisFn.jl:96-112) as 55 doubles: w, N[9], ∂Nα (9x2
 * column-major), ∂∂Nαβ (9x3 column-major, Voigt order 11, 22, 12). */
/* mafem_create checks IX against the tensor-product connectivity of
 * construct_IX (src/input/Mesh.jl:574-593) and every ID, uel_ids and dofs entry
 * against its range, and rejects (MAFEM_ERR_ARG) a mesh that differs. */
typedef struct mafem_mesh_desc {
  int64_t num1el, num2el, numel, num1np, num2np, numnp, ndf, nmdf;
  int64_t dofs[8];        /* mesh.dofs[Dof.vx .. Dof.pm]: 1-based dof index, 0 if absent */
  const int64_t* IX;      /* mesh.IX: 9 x numel, 1-based node numbers */
  const int64_t* ID;      /* mesh.ID: ndf x numnp, 1-based unknown numbers, 0 = Dirichlet */
  int64_t n_uel;          /* size(mesh.area_gp_fns.ufns, 1) */
  const int64_t* uel_ids; /* mesh.area_gp_fns.uel_ids (numel, 1-based) */
  const double* ufns;     /* mesh.area_gp_fns.ufns: [uel][gp 1..9] x 55 */
  int64_t bdry_n_uel[4];            /* per Boundary (BOTTOM, RIGHT, TOP, LEFT) */
  const int64_t* bdry_uel_ids[4];   /* mesh.bdry_gp_fns[b].uel_ids (num1el or num2el) */
  const double* bdry_ufns[4];       /* mesh.bdry_gp_fns[b].ufns: [uel][gp 1..3] x 55 */
  int64_t n_neu;                    /* length(mesh.inh_neu_bcs) (<= 8) */
  const int64_t* neu_bdry;          /* Boundary of each entry */
  const int64_t* neu_type;          /* Neumann type of each entry */
  const double* neu_val;            /* value of each entry */
  int64_t n_dir;                    /* length(mesh.inh_dir_bcs) */
  const int64_t* dir_unknown;       /* Dof.Unknown of each entry (1..8) */
  const int64_t* dir_node;          /* node (1-based) */
  const double* dir_val;            /* value */
} mafem_mesh_desc;

typedef struct mafem_mesh mafem_mesh;     /* host mesh owned by the library */
typedef struct mafem_handle mafem_handle; /* device-resident solver state */

typedef struct mafem_step_stats {
  int32_t newton_iters;       /* Newton iterations taken */
  int32_t refine_iters;       /* total refinement sweeps (FP32 form) */
  double eps[14];             /* ‖Δu‖₂ / nmdf per iteration (FiniteElement.jl:48) */
  double res_norm[14];        /* ‖r‖₂ at the start of each iteration */
  double ms_assemble, ms_factor, ms_solve, ms_total; /* device time */
} mafem_step_stats;

/* ---- host mesh (restates Mesh(p; args...) and prepare_input) ----------------- */

/* Mesh(p; args...) -- src/input/Mesh.jl:79,94-302, src/input/Bc.jl.  Rejects
 * (MAFEM_ERR_ARG / MAFEM_ERR_UNSUPPORTED) what check_params does
 * (src/input/Params.jl:89-119): other element orders, F_BEND with a static or
 * ALEVB mesh, bend_mf != kb / 2 / length or a normal pressure, the flat flows
 * with a moving mesh, F_PULL with a normal pressure (Bc.jl:266). */
int mafem_mesh_build(const mafem_params* p, const mafem_args* a, mafem_mesh** out);
/* Fill `out` with pointers into `m` (valid until mafem_mesh_free). */
int mafem_mesh_view(const mafem_mesh* m, mafem_mesh_desc* out);
void mafem_mesh_free(mafem_mesh* m);
/* prepare_input's default initial state (src/Input.jl:40-108, non-F_BEND
 * scenarios): xms numnp x 3 and cps numnp x ndf, column-major. */
int mafem_prepare_input(const mafem_mesh* m, const mafem_params* p, double* xms, double* cps);
/* Half bandwidth of K in the reference's ID ordering. */
int64_t mafem_mesh_half_bandwidth(const mafem_mesh_desc* d);

/* ---- device handle ------------------------------------------------------------ */

/* Allocate every device buffer for one patch and upload the mesh tables. */
int mafem_create(const mafem_mesh_desc* d, const mafem_params* p, const mafem_args* a,
                 int32_t precision, mafem_handle** out);
int mafem_destroy(mafem_handle* h);
const char* mafem_last_error(const mafem_handle* h); /* h may be NULL */
/* Bytes of device memory the handle holds (state + band factor + staging). */
int64_t mafem_device_bytes(const mafem_handle* h);
/* Same figure for a mesh before creating a handle (admission control). */
int64_t mafem_footprint_bytes(const mafem_mesh_desc* d, int32_t precision);

/* Copy state host -> device / device -> host (xms numnp x 3, cps numnp x ndf). */
int mafem_upload_state(mafem_handle* h, const double* xms, const double* cps);
int mafem_download_state(mafem_handle* h, double* xms, double* cps);

/* calc_r_K (FiniteElement.jl:75-200) on the resident state.  r_out (nmdf) may be
 * NULL.  If band_out is not NULL it receives K in LAPACK band layout: column j
 * (0-based) at band_out + j*ldab_out, A(i,j) at row kl+ku+i-j with
 * kl = ku = mafem_mesh_half_bandwidth(); the top kl rows are zero. */
int mafem_calc_r_K(mafem_handle* h, double time, double dt, double* r_out, double* band_out,
                   int64_t ldab_out);
/* Δu = -K \ r for the K of the last mafem_calc_r_K and a host r (nmdf). */
int mafem_solve(mafem_handle* h, const double* r, double* du_out);
/* update_xms! (FiniteElement.jl:408-423) on the resident state: the predictor
 * xms[:, j] += Δt * cps[:, m_motion_order[j]] (Analysis.jl:70). */
int mafem_predict(mafem_handle* h, double dt);
/* time_step! (FiniteElement.jl:11-63) on the resident state. */
int mafem_time_step(mafem_handle* h, double time, double dt, mafem_step_stats* stats);
/* time_step! with host state: upload xms/cps, Newton on the device, download
 * the updated xms/cps into the same arrays -- the drop-in for the reference. */
int mafem_time_step_host(mafem_handle* h, double* xms, double* cps, double time, double dt,
                         mafem_step_stats* stats);
/* run_analysis!'s time loop (src/Analysis.jl:60-93) on the resident state:
 * predictor + time_step! for each Δt; step k ends at t0 + dts[0] + ... + dts[k],
 * summed left to right. */
int mafem_run(mafem_handle* h, const double* dts, int32_t nsteps, double t0, mafem_step_stats* last);

/* calc_pull_force (src/analysis/PullForce.jl:61-80) on the resident state:
 * the velocity residual of calc_elem_dof_residuals over the 5x5 elements around
 * the pulled element (ceil(numel/2), or the centre element with
 * args.pull_centre; get_adj_maps, PullForce.jl:25-53), summed over that
 * element's nodes -> f_out[3].  The reference writes it to f-pull.txt after
 * each step of an F_PULL run (src/Analysis.jl:81-91). */
int mafem_pull_force(mafem_handle* h, double* f_out);
/* x_pull of the same f-pull.txt line (src/Analysis.jl:83-84): the mean of the
 * pull element's nine node positions -> x_out[3]. */
int mafem_pull_position(mafem_handle* h, double* x_out);

/* ---- state files and checkpoints ---------------------------------------------------
 * The files run_analysis! writes after every step with writedlm
 * (src/Analysis.jl:75-78; the initial state at src/Input.jl:113-114) and
 * prepare_input / restart read back with readdlm (src/Input.jl:35-37,
 * src/MembraneAleFem.jl:75-107): "<dir>/t<t_id>-xms.txt" (numnp rows of 3) and
 * "<dir>/t<t_id>-cps.txt" (numnp rows of ndf), one matrix row per line, entries
 * separated by a tab, each Float64 printed as Julia's print does (shortest
 * round-trip digits: "1.0", "0.0001", "100000.0", "1.0e-5", "1.0e6"), so a
 * restart from these files continues bit for bit. */

/* Julia's print(::Float64) into buf (NUL-terminated); returns its length, or
 * MAFEM_ERR_ARG if cap is too small (32 bytes always suffice). */
int mafem_format_double(double x, char* buf, int32_t cap);
/* writedlm / readdlm of a column-major rows x cols matrix (a[i + rows*j]).
 * readdlm accepts tabs or spaces between entries and fails (MAFEM_ERR_ARG, the
 * message in mafem_last_error(NULL)) unless the file holds exactly that shape. */
int mafem_writedlm(const char* path, const double* a, int64_t rows, int64_t cols);
int mafem_readdlm(const char* path, double* a, int64_t rows, int64_t cols);
/* Write the resident state as <dir>/t<t_id>-{xms,cps}.txt and wait for the files. */
int mafem_write_state(mafem_handle* h, const char* dir, int64_t t_id);
/* The same without waiting: the state (slot -1) or device snapshot `slot` is
 * copied to pinned host memory on the handle's stream, after every step already
 * enqueued, and a library thread writes the files while later steps run.
 * Blocks only while three earlier writes are still pending. */
int mafem_write_state_async(mafem_handle* h, int32_t slot, const char* dir, int64_t t_id);
/* Wait for every pending write; returns the first write failure since the last flush. */
int mafem_flush_state_writes(mafem_handle* h);
/* readdlm both files into the resident state (restart, or prepare_input's
 * in_path / in_xms / in_cps initial state). */
int mafem_read_state(mafem_handle* h, const char* xms_file, const char* cps_file);
/* Device-resident checkpoints (no reference counterpart): nslots copies of the
 * state kept in HBM beside it.  mafem_snapshot copies the state into a slot and
 * mafem_restore copies a slot back, both stream-ordered device-to-device copies
 * that do not wait -- e.g. to retry a step with a smaller Δt after
 * MAFEM_NEWTON_NOT_CONVERGED without a host round trip.  Reserve once per handle. */
int mafem_snapshot_reserve(mafem_handle* h, int32_t nslots);
int mafem_snapshot(mafem_handle* h, int32_t slot);
int mafem_restore(mafem_handle* h, int32_t slot);

/* ---- batching (no reference counterpart: the reference steps one patch) -----------
 * Many independent patches (handles of any sizes, motions and precisions) advance
 * together: mafem_batch_step runs predictor + time_step! for every patch, each
 * patch's Newton iterations enqueued on its own stream and interleaved with the
 * others', so their kernels overlap on the GPU.  Results are those of
 * mafem_time_step on each handle alone.  A handle belongs to at most one batch
 * at a time; the batch does not own the handles. */
typedef struct mafem_batch mafem_batch;
/* ctas: CTAs of each patch's persistent factorisation (0: each patch's smallest
 * grid, which lets the most factorisations run at once). */
int mafem_batch_create(mafem_handle* const* handles, int32_t n, int32_t ctas, mafem_batch** out);
/* times[i], dts[i] per patch; status[i] (optional) = the patch's mafem_time_step
 * status; stats (optional, n entries).  Returns the first nonzero status. */
int mafem_batch_step(mafem_batch* b, const double* times, const double* dts, int32_t* status,
                     mafem_step_stats* stats);
int mafem_batch_destroy(mafem_batch* b);
/* FP32 + refinement patches whose band fits one CTA's shared memory are, by
 * default, factored and solved together: one launch factors every such patch
 * (one CTA each, largest first) and one more runs their FP32 triangular
 * solves and FP64 iterative refinement.  on = 0 steps them like the other
 * patches instead (each with its own multi-CTA factorisation).  Returns 1 if
 * the batched solve is in use. */
int mafem_batch_set_patch_solve(mafem_batch* b, int32_t on);
/* Newton rounds of the batched solve's patches (no counterpart in the
 * reference, whose time_step! advances one patch).  batched_assembly != 0 (the
 * default): every round assembles all of those patches with one launch per
 * kernel (the element kernels once per motion), factors and refines them
 * (mafem_batch_set_patch_solve), then updates them and forms their Newton
 * norms with one launch each, and reads all their results with one copy --
 * a fixed number of launches per round, whatever the patch count.  They
 * run the per-patch kernels' arithmetic on the same element-to-CTA map (the
 * element kernels compiled separately, so a multiply-add may round
 * differently).  graphs != 0 (the
 * default): such a round is captured as a CUDA graph the first time its
 * sequence of patches occurs and replayed from then on.  Returns MAFEM_OK. */
int mafem_batch_set_rounds(mafem_batch* b, int32_t batched_assembly, int32_t graphs);
typedef struct mafem_batch_stats {
  int64_t graph_launches;   /* rounds replayed from a CUDA graph */
  int64_t graph_captures;   /* rounds captured */
  int64_t graphs_cached;    /* graphs held now */
  int64_t kernel_launches;  /* kernels enqueued by the batch's handles and rounds */
} mafem_batch_stats;
int mafem_batch_get_stats(const mafem_batch* b, mafem_batch_stats* out);
/* CTAs of this handle's persistent factorisation and back substitution (0: all
 * SMs); clamped to what the band needs.  Returns the CTAs the factorisation uses. */
int mafem_set_launch_ctas(mafem_handle* h, int32_t ctas);

/* ---- serving: continuous batching (no reference counterpart) -------------------------
 * A request is one solve: a patch (the mesh view, Params and args of
 * mafem_create), its initial state and a number of time steps.  The server
 * admits requests first come first served while their device footprint fits
 * its HBM budget and runs the admitted ones as one continuous batch.  Each
 * mafem_server_round collects the Newton iterations that have completed,
 * starts the next iteration of every admitted request that is not on the GPU
 * (a time step -- predictor + time_step! -- for one between steps), and hands
 * the ready FP32-form requests to free solve lanes: a lane runs one batched
 * Newton round of its requests (mafem_batch_set_rounds), the requests grouped
 * by the cost of their factorisation so that small patches iterate while a
 * large one is still in its round.  Other requests run their own iterations.
 * A finished request's state is kept on the host and its device memory freed
 * at once.  Each request's results are those of mafem_time_step on its own
 * handle, whatever else runs beside it. */
typedef struct mafem_server mafem_server;
typedef struct mafem_request {
  const mafem_mesh_desc* mesh;  /* must stay valid until the request is admitted */
  const mafem_params* params;   /* likewise */
  const mafem_args* args;       /* likewise */
  int32_t precision;            /* enum mafem_precision */
  int32_t nsteps;               /* time steps to run */
  double t0, dt;                /* step k ends at t0 + (k + 1) dt */
  const double* xms0;           /* initial state, copied at submit */
  const double* cps0;
  double refine_tol;            /* FP32 form: mafem_set_refinement's tol; 0 = default */
  int32_t ramp_steps;           /* > 0: before step k the inhomogeneous Dirichlet values are scaled by
                                   min(1, (k + 1) / ramp_steps), as mafem_set_dirichlet_scale does */
  int32_t reserved;             /* 0 */
} mafem_request;
typedef struct mafem_server_stats {
  int64_t steps_done, rounds;
  double p50_step_ms, p99_step_ms, max_step_ms; /* wall time of each completed step */
  int64_t bytes_in_use, budget_bytes;
  int32_t active, pending;
} mafem_server_stats;
/* hbm_budget_bytes 0: 80 % of the device memory free now; max_active 0: 1024. */
int mafem_server_create(int64_t hbm_budget_bytes, int32_t max_active, mafem_server** out);
int mafem_server_destroy(mafem_server* s);
/* Queue a request; MAFEM_ERR_ADMISSION if it can never fit the budget. */
int mafem_server_submit(mafem_server* s, const mafem_request* r, int64_t* id);
/* Admit what fits, collect completed iterations, start the next ones (see above). */
int mafem_server_round(mafem_server* s, int32_t* n_active, int32_t* n_pending);
/* A finished request's final state (xms, cps as in mafem_download_state; either
 * may be NULL) and status; the server then forgets it.  Returns 1 while it is
 * still queued or running. */
int mafem_server_result(mafem_server* s, int64_t id, double* xms, double* cps, int32_t* status,
                        int32_t* steps_done);
int mafem_server_get_stats(const mafem_server* s, mafem_server_stats* out);

/* ---- diagnostics --------------------------------------------------------------- */

/* Assemble the resident state at (time, dt), factor once with the persistent
 * node-block LU and copy its per-panel clock stamps (12 int64 per panel) to
 * out[0 .. 12 npan).  cap >= 12 npan.  Returns npan, or MAFEM_ERR_UNSUPPORTED if
 * the handle does not use that factorisation. */
int mafem_trace_factor(mafem_handle* h, double time, double dt, int64_t* out, int64_t cap);

/* FP32 form: assemble the resident state and run the batched one-CTA solve on
 * this handle alone, its factorisation traced -- 6 globaltimer stamps (ns) per
 * panel in out[6p .. 6p+5] (start, diagonal block factored, panel staged and
 * inverses formed, first chunk's U12/Y, its trailing update, panel done), then
 * the factor and refine kernels' event times in ns, then 4 stamps per
 * refinement sweep for up to 32 sweeps (start, substitutions done, x updated,
 * residual done; 0 where not reached), then 16 phase sums (ns) of the first
 * sweep's substitutions (see patch_lu_solve), then the relative residual
 * |r - A0 x| / |r| after each sweep (up to 32, as double bit patterns), then
 * the refinement's status and sweep count.  cap >= 6 npan + 182.
 * Returns npan, or MAFEM_ERR_UNSUPPORTED if the handle cannot use that solve. */
int mafem_trace_patch_solve(mafem_handle* h, double time, double dt, int64_t* out, int64_t cap);

/* Number of kernels this handle has enqueued since mafem_create. */
int64_t mafem_launch_count(const mafem_handle* h);

/* Solve K x = rhs (host arrays, nmdf entries) for a caller's K -- a host band in
 * the layout mafem_calc_r_K writes (column j at band + j*ldab, A(i,j) at row
 * kl+ku+i-j, kl = ku = mafem_mesh_half_bandwidth()) -- through the handle's own
 * factorisation: node-block pivoting, full partial pivoting when a node block
 * has no usable pivot, FP64 refinement in the FP32 form.  The reference solves
 * with `K \ r` (src/analysis/FiniteElement.jl:38); this entry point exposes the
 * same solver to systems the assembly would not produce (tests, diagnostics).
 * MAFEM_ZERO_PIVOT when K is singular.  The next mafem_solve needs a new
 * mafem_calc_r_K. */
int mafem_solve_band(mafem_handle* h, const double* band, int64_t ldab, const double* rhs, double* x_out);
/* Factorisations this handle redid with full partial pivoting because a node
 * block had no usable pivot (or the batched FP32 solve handed the iteration
 * back). */
int64_t mafem_fallback_count(const mafem_handle* h);
/* Set the inhomogeneous Dirichlet entries of the resident state (the mesh's
 * dir_unknown / dir_node / dir_val, as prepare_input applies them,
 * src/Input.jl:103-108) to scale * value, stream-ordered before the next step:
 * a pull whose speed is ramped up over the first steps.  The reference sets
 * these entries once; a run that changes them goes through restart with an
 * edited cps file (src/MembraneAleFem.jl:75-107), which this replaces without
 * a host round trip. */
int mafem_set_dirichlet_scale(mafem_handle* h, double scale);
/* Failure-detection test hook (no reference counterpart; the reference has no
 * inter-CTA waits).  The cooperative forward and back substitutions' waits for
 * another CTA give up after limit_polls polls (0: the default, 2^22), and the
 * back substitution never publishes the completion flag of the panel
 * withhold_panel places before the last (0: the last panel, which every panel
 * whose columns reach it waits for; -1: none).  A Newton iteration
 * whose wait ran out leaves the state unchanged and returns MAFEM_ERR_CUDA
 * ("a bounded wait ... ran out"); every CTA returns, the device stays usable,
 * and the next call (after mafem_set_wait_test(h, 0, -1)) runs normally. */
int mafem_set_wait_test(mafem_handle* h, int32_t limit_polls, int32_t withhold_panel);

/* FP32 form: FP64 iterative refinement of each linear solve stops at tol
 * (default 1e-10) or fails after max_sweeps sweeps (default 30) or when it stops
 * converging (MAFEM_REFINE_STALLED).  A handle stepped on its own stops when
 * |r - A x| <= tol |r|; the batched solve of mafem_batch_step stops when its
 * last correction is at most tol |x| (a bound on the forward error of x that
 * holds on ill-conditioned tangents too) and hands a stalled solve to the
 * handle's own solver.  A looser tol trades refinement sweeps for Newton
 * iterations: the Newton criterion (FiniteElement.jl:48) on the FP64 residual
 * still decides convergence, so the converged state does not depend on tol. */
int mafem_set_refinement(mafem_handle* h, int32_t max_sweeps, double tol);

/* Select the banded LU (enum mafem_lu_path) for the following factorisations.
 * MAFEM_ERR_UNSUPPORTED if the handle cannot run that path (e.g. the node-block
 * forms when the band is too wide for their shared-memory panels). */
int mafem_set_lu_path(mafem_handle* h, int32_t path);

/* Batched FP32 form: the CTAs (one thread-block cluster) that factor this
 * handle's patch -- 1, 2 or 4; 0 (the default) chooses by band width: one CTA
 * up to 256 trailing columns, two up to 512, four beyond.  Any choice gives the
 * same factors; it trades the factorisation's latency against the SMs it holds. */
int mafem_set_patch_ctas(mafem_handle* h, int32_t ctas);

/* Autotuner of the batched FP32 factorisation: measure (CUDA events, on a
 * synthetic band of this handle's shape written over its band, so call it
 * between steps and with the GPU otherwise idle) the time of factoring this
 * patch on 1, 2 and 4 CTAs, once per device and patch shape, cached for the
 * process.  mafem_batch_create measures every shape of its patches; each
 * batched round (mafem_batch_step, mafem_server_round) then picks per shape
 * the cluster size that minimises the round's estimated makespan, max(longest
 * factorisation, summed CTA-time / SMs).  Shapes without times keep the
 * width rule of mafem_set_patch_ctas.  MAFEM_ERR_UNSUPPORTED for a handle the
 * batched FP32 form does not serve. */
int mafem_autotune_patch(mafem_handle* h);
/* The batched rounds' FP32 tangent kernel evaluates 2 or 4 elements per CTA
 * (no reference counterpart).  mafem_batch_create (and a server, when it
 * admits the first FP32 request of a kind) times both on the first patch of
 * each motion and element size, once per device, and every round uses the
 * faster.  This returns that choice for h's kind of patch and the two
 * measured times (ms); MAFEM_ERR_UNSUPPORTED before it was measured. */
int mafem_tangent_tile(const mafem_handle* h, int32_t* epb, double* ms_2, double* ms_4);

typedef struct mafem_kernel_times {
  double ms_assemble;         /* element kernel + gathers */
  double ms_panel, ms_apply;  /* summed device time of the LU's two kernels */
  int64_t n_panel, n_apply;   /* launches of each */
  int64_t n, kl, ku, nb;      /* factorised system */
  int64_t ndfp;               /* node-block pivoting: max block size - 1; -1 = full partial pivoting */
  double flop_panel, flop_apply;  /* FLOPs of the factorisation's panel and trailing-update kernels */
} mafem_kernel_times;
/* Assemble and factor the resident state once, timing every LU launch with
 * CUDA events on the handle's stream (for roofline reporting). */
int mafem_profile_factor(mafem_handle* h, double time, double dt, mafem_kernel_times* out);
/* Measured FP64 FMA throughput of the current device in TFLOP/s (the roof of
 * the FP64 kernels; a short FMA-chain kernel on every SM). */
int mafem_probe_fp64_tflops(double* tflops);

/* ---- allocation-free solve --------------------------------------------------------- */

/* Factor and solve A x = rhs for a banded A (LAPACK band layout, A(i,j) at
 * band_dev[j*ldab + kl+ku+i-j], kl == ku, ldab >= 2kl+ku+1; all three arrays are
 * device pointers owned by the caller) without allocating device memory.  No
 * counterpart in the reference: it exists for callers that must not call
 * cudaMalloc -- e.g. a Julia host whose CUDA.jl memory pool accounts for every
 * device byte, or a loop that cannot afford cudaMalloc's device-wide
 * synchronisation.  Its scratch is one static 32 MiB device array inside the
 * library (held by every GPU that loads it until exit): systems needing more --
 * about 8*n*(3kl+65) + 4*n*(kl+33)/32 bytes, e.g. a 16x16 ALEVB tangent fits and
 * a 24x24 one does not -- return MAFEM_ERR_ARG.  All calls share that array, so
 * calls that overlap on the GPU race; order them on one stream.  Each call looks
 * the array up on the current device (cudaGetSymbolAddress).  Full partial
 * pivoting (LAPACK gbtrf's pivot rule); a zero, infinite or NaN pivot gives
 * MAFEM_ZERO_PIVOT, a NaN or infinity in x MAFEM_NAN_DETECTED.  Runs on
 * `stream` (NULL = default stream) and returns after synchronising it. */
int mafem_band_solve_noalloc(const double* band_dev, int64_t n, int64_t kl, int64_t ku, int64_t ldab,
                             const double* rhs_dev, double* x_dev, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MAFEM_H */
