// sfd_internal.cuh -- the engine object shared by the orchestration files
// (sfd_api.cu: forward path and C ABI; sfd_adjoint.cu: reverse mode).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <map>
#include <vector>

#include "sfd_kernels.cuh"

#include "../../include/sfd.h"
#include "sfd_engine.cuh"
#include "sfd_kernels.cuh"

// kernel classes of the per-launch profile
enum {
  SFD_K_OTHER = 0,
  SFD_K_SPECTRAL,
  SFD_K_NODE,
  SFD_K_SUMS64,
  SFD_K_SUMSDF,
  SFD_K_SUMS32,
  SFD_K_EPILOGUE,  // no launches: the sum epilogue runs inside the boundary-sum kernels
  SFD_K_ASSEMBLE,
  SFD_K_DIAG,
  SFD_K_PANEL,
  SFD_K_UPDATE,
  SFD_K_TRSV,
  SFD_K_GEMV,
  SFD_K_VELOCITY,
  SFD_K_RK4,
  SFD_K_UPDATE_TC,
  SFD_K_F4_COLS,   // four-step transforms: forward column FFTs
  SFD_K_F4_ROWS,   // row FFTs, multipliers, inverse row FFTs
  SFD_K_F4_ICOLS,  // inverse column FFTs and outputs
  SFD_K_EXTRA,     // extra corrections (gated: they return at once where the residual is converged)
  SFD_K_AP_REDO,   // a' transformed again after extra corrections (gated likewise)
  SFD_K_AP,        // the a' transform (forked beside the last pass while stepping on graphs)
  SFD_K_GEMV0,     // the starting product a0 = X phi' (returns at once on warm starts)
  SFD_NCLASS
};

struct AdjWork;

struct sfd_engine {
  int device = 0;
  int nsm = 0;  // SMs of the device
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  // auxiliary stream of the a' transform, forked from `stream` once a is final
  // and joined before the velocity epilogue (also inside captured graphs)
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  bool ap_forked = false;
  sfd_options opt{};
  int nsurf = 0, ntot = 0, max_n = 0, max_np = 0;
  int nblk = 3;  // state blocks: [x | y | phi] or, with an augmented drive, [x | y | phi | D]
  int sum_groups[3] = {4, 4, 4};  // boundary-sum source groups per CTA, by pass precision
  bool tune_pending = false;
  long long mat_elems = 0, panel_elems = 0;
  bool any_rho = false;
  std::vector<SurfaceDesc> hs;
  SurfaceDesc* d_surf = nullptr;
  int* d_node_surf = nullptr;
  std::map<int, cd*> d_tw;
  std::map<int, cd*> d_ctw;  // cluster-transform twiddle tables by n
  // work lists
  int2* d_jobs_first = nullptr; int njobs_first = 0;
  int2* d_jobs_ap = nullptr; int njobs_ap = 0;
  int2* d_cjobs_first = nullptr; int ncjobs_first = 0;  // cluster-distributed transforms
  int2* d_cjobs_ap = nullptr; int ncjobs_ap = 0;
  int max_n_single = 0, max_n_cluster = 0;
  // four-step transforms of the power-of-two surfaces: z', z'', phi' and a'
  // plans, and their L2 scratch (4 ntot complex: z' rows, z'' rows, phi' rows,
  // a' rows; a' runs on the auxiliary stream beside the main stream's work)
  F4Plan f4_first, f4_ap;
  cd* f4_scr = nullptr;
  int2* d_sum_items = nullptr; int nsum = 0;
  // FP32 pass: (tile, source slice) work entries, per-entry partials, per-tile counters
  F32Work* d_f32_work = nullptr; int nf32 = 0;
  int f32_max_per = 0;  // sources of the widest slice
  float4* f32_part = nullptr;
  float2* f32_wsum = nullptr;
  unsigned int* f32_count = nullptr;
  float4* df_part = nullptr;  // double-float pass on the same work entries: 128 float4 per entry
  int4* d_asm_tiles = nullptr; int nasm = 0;
  int2* d_gemv_rows = nullptr; int ngemv = 0;
  long long* d_poff = nullptr;
  int max_blocks64 = 0, max_blocks128 = 0;
  // state (each 3 * ntot): [x | y | phi]
  double *y0 = nullptr, *ys = nullptr, *kacc = nullptr, *kcur = nullptr;
  // stage data
  cd *zp = nullptr, *zpp = nullptr, *ap = nullptr;
  double *phip = nullptr, *a = nullptr, *r = nullptr, *delta = nullptr, *phi_im = nullptr;
  float2 *adf = nullptr, *ddf = nullptr;  // double-float copies of a and delta
  float *rf = nullptr, *phipf = nullptr;   // FP32 copies of r and phi' (inputs of the preconditioner product)
  NodeData nd{};
  cd *cacc = nullptr, *dacc = nullptr, *vel_low1 = nullptr;
  unsigned int* status = nullptr;
  double *lmax = nullptr, *rnorm = nullptr, *inv_out = nullptr;
  // refinement bookkeeping: per-evaluation residual slots (SFD_RSLOTS per
  // surface) and max |phi'|, cleared by k_node_prep; per-surface max final
  // relative residual and count of extra corrections since the last clear
  double *rslot = nullptr, *bnorm = nullptr, *rrel = nullptr;
  unsigned long long* extra_count = nullptr;
  // host-mapped word the velocity kernel sets on a refinement stall (mixed
  // mode): the next step the host enqueues after seeing it rebuilds the
  // preconditioner in-step
  unsigned int* stall_host = nullptr;
  unsigned int* stall_dev = nullptr;
  // mixed mode: per surface 0 when the last solve converged, 1e300 otherwise
  // (written by the velocity kernel).  During fixed-step RK4 stepping
  // (allow_warm) a converged solve's a is the starting point of the next one
  // (the product a0 = X phi' is gated off for that surface); every other
  // evaluation, and every evaluation that rebuilds the preconditioner, starts
  // cold.  SFD_WARM=0 in the environment turns warm starts off.
  double* warm = nullptr;
  bool allow_warm = false;
  long long stall_rebuilds = 0;
  // matrices
  double* m64 = nullptr;
  float* m32 = nullptr;
  __half* m16 = nullptr;     // FP16 copy of the preconditioner (rows scaled by powers of two)
  float* rscale = nullptr;   // per-row inverse scales of m16
  int gemv_spw = 0;          // streamed product (one surface): row slots per warp, 0 = register-pipelined
  int gemv_smem = 0;         // its dynamic shared memory
  bool m16_written = false;  // the last kernel enqueued wrote m16: the next product may not prefetch it
  bool node_written = false; // node data written since the last product: FP32 passes may not prefetch them
  float *pbuf = nullptr, *rbuf = nullptr, *cbuf = nullptr;
  __nv_bfloat16 *cparts = nullptr, *rparts = nullptr;  // tensor-core operands: 3 bf16 parts, panel_elems apart
  // TMA tensor maps of cparts / rparts (opaque 128-byte descriptors) and the
  // row groups per tile column of the tensor-core update
  struct alignas(64) TensorMap {
    unsigned char bytes[128];
  } tmap_c{}, tmap_r{};
  TensorMap* d_tmap_out = nullptr;  // per surface: its FP32 matrix, the target of the update's reduce-adds
  int tc_groups = 1;
  // graphs
  cudaGraphExec_t g_step[2] = {nullptr, nullptr};
  double g_dt = 0.0;
  int g_kernels[2] = {0, 0};
  long long step_count = 0;
  long long launches = 0;
  bool have_precond = false;
  // per-kernel-class timing (eager launches only)
  bool profile = false;
  struct Pending {
    int cls;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> event_pool;
  double class_ms[SFD_NCLASS] = {};
  long long class_count[SFD_NCLASS] = {};
  // reverse-mode workspace (checkpoints and per-stage records), allocated on first use
  AdjWork* adj = nullptr;
  // adaptive RKF45 workspace, allocated on first use
  struct RkfWork* rkf = nullptr;
  // complex-layout staging of the C++ facade (sfd_facade.cu), allocated on first use
  double* fc_in = nullptr;
  double* fc_out = nullptr;
  // background preconditioner rebuild (opt.refactor_lag > 0): a low-priority
  // side stream assembles and inverts M from a snapshot of the state into
  // m16_next / rscale_next; the main stream switches at step bg_swap_at
  struct Background {
    cudaStream_t side = nullptr;
    cudaEvent_t ev_snap = nullptr, ev_done = nullptr;
    double* snap = nullptr;     // state copy [x | y | phi]
    cd *zp = nullptr, *zpp = nullptr;
    double* phip = nullptr;
    NodeData nd{};
    __half* m16_next = nullptr;
    float* rscale_next = nullptr;
    cd* f4_scr = nullptr;       // four-step scratch of the side stream's transforms (3 ntot)
    long long swap_at = -1;     // step index of the switch; -1: none pending
    long long rebuilds = 0;
  } bg;
  // the problem of each surface as given to sfd_create (helper engines copy it)
  std::vector<sfd_problem> hp;
  // implicit Gauss-Legendre workspace (sfd_gl2.cu), allocated on first use
  struct Gl2Work* gl2 = nullptr;
};

// Batched dense FP64 solver (sfd_facade.cu): `batch` systems of order n held
// as padded row-major matrices (np = pad_n(n), identity padding) in `mat`.
struct sfd_dense_solver {
  int n = 0, np = 0, batch = 0;
  SurfaceDesc* d_surf = nullptr;
  double* mat = nullptr;
  double* lmax = nullptr;
  int* piv = nullptr;  // row exchanges of the pivoted factorisation, batch x np
  unsigned int* status = nullptr;
  cudaStream_t stream = nullptr;
};
// Factor d->mat in place and solve for each system's right-hand side b
// (batch x n) into x: with `pivoted`, blocked LU with partial pivoting (getrf /
// getrs semantics); otherwise blocked LU without row exchanges, recording
// max |l_ij|.  status (host, nullable, batch words) as sfd_dense_solve.
// Asynchronous unless status is given.
int sfd_internal_dense_factor_solve(sfd_dense_solver* d, const double* b, double* x, unsigned int* status,
                                    bool pivoted);

// Entry points of sfd_api.cu used by the reverse mode.
int sfd_internal_error(int code, const char* msg);
int sfd_internal_cuda(cudaError_t err, const char* what);
// One FP64 RHS evaluation (state [x|y|phi] -> [dx|dy|dphi]) on the engine
// stream; leaves z', z'', a, a', C, D, w, p and the LU factors of M in the
// engine's buffers.
int sfd_internal_rhs(sfd_engine* e, const double* st, double* out);
// As sfd_internal_rhs, for either precision; refactor = rebuild the mixed
// preconditioner at this evaluation (it is built anyway if there is none).
int sfd_internal_rhs_ex(sfd_engine* e, const double* st, double* out, bool refactor);
// Whether warm starts are enabled (SFD_WARM=0 in the environment: off; read once).
bool sfd_warm_enabled();
// Row slots per warp of the streamed single-surface product at most
// (SFD_GEMV_SPW in the environment, default kGemvSDefaultSpw; 0: the
// register-pipelined product; read once).
int sfd_gemv_stream_cap();
// Whether the streamed product requests its first rows before waiting on its
// predecessor (SFD_GEMV_PREFETCH=0: never; read once).
bool sfd_gemv_prefetch_enabled();
// Whether the FP32 boundary-sum passes stage the node data before waiting on
// their predecessor (SFD_SUMS_PREFETCH=0: never; read once).
bool sfd_sums_prefetch_enabled();
// Switch in a pending background preconditioner rebuild now (not allowed
// while the engine stream is being captured).
int sfd_internal_bg_flush(sfd_engine* e);
// reverse-mode workspace release (sfd_adjoint.cu)
void sfd_adjoint_free(sfd_engine* e);
// adaptive-integrator workspace release (sfd_rkf45.cu)
void sfd_rkf45_free(sfd_engine* e);
// First half of an RHS evaluation (z', z'', phi', the solve of M a = phi',
// C and D) on state [x|y|phi]; leaves a, z', z'' in the engine's buffers.
int sfd_internal_solve(sfd_engine* e, const double* st);
// Dynamic shared-memory limits of the solver kernels on the current device.
cudaError_t sfd_solve_configure();
// Why reverse mode does not cover the engine, or null when it does (sfd_adjoint.cu).
const char* sfd_adjoint_unsupported(const sfd_engine* e);
// implicit Gauss-Legendre workspace release (sfd_gl2.cu)
void sfd_gl2_free(sfd_engine* e);
// GL2 from t0 to t1 on the engine state (sfd_gl2.cu); times / states (host,
// nullable) are appended the time and the 3n state after each accepted step.
int sfd_internal_gl2(sfd_engine* e, double t0, double t1, const sfd_gl2_options& o, sfd_gl2_result& r,
                     std::vector<double>* times, std::vector<double>* states, sfd_gl2_step_fn fn = nullptr,
                     void* user = nullptr);
