// sfd_api.cu -- engine orchestration and the C ABI (include/sfd.h).
//
// One engine = one batch of surfaces resident in HBM.  An RHS evaluation is
//   spectral derivatives -> node prep -> solve (FP64 LU, or mixed: FP32
//   Gauss-Jordan preconditioner + double-float refinement) -> a' -> velocity
//   and Bernoulli,
// all enqueued on the engine stream with no host synchronisation; one RK4
// step (4 evaluations + stage combines) is captured once into a CUDA graph and
// replayed.  Host code never touches the per-stage data.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/sfd.h"
#include "../../include/sfd_h5.hpp"
#include "sfd_engine.cuh"
#include "sfd_kernels.cuh"
#include "sfd_solve.cuh"
#include "sfd_internal.cuh"


namespace {

thread_local std::string g_last_error;
int g_default_precision = SFD_PRECISION_FP64;

int set_error(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  // A CUDA failure is reported here once: consume the runtime's record of it,
  // so that a later, unrelated launch check does not report it again (errors
  // that leave the context unusable persist regardless).
  if (code == SFD_ERR_CUDA || code == SFD_ERR_NO_DEVICE) (void)cudaGetLastError();
  return code;
}

int sfd_fail(cudaError_t e) { return set_error(SFD_ERR_CUDA, "CUDA error: %s", cudaGetErrorString(e)); }

#define CK(expr)                                                                                        \
  do {                                                                                                  \
    cudaError_t _e = (expr);                                                                            \
    if (_e != cudaSuccess)                                                                              \
      return set_error(SFD_ERR_CUDA, "%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), __FILE__, \
                       __LINE__);                                                                       \
  } while (0)

template <typename T>
cudaError_t dalloc(T** p, size_t count) {
  *p = nullptr;
  if (count == 0) return cudaSuccess;
  return cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
}

// exp(-2 pi i e / n), computed in long double (80- or 128-bit) and rounded.
std::vector<cd> twiddles(int n) {
  std::vector<cd> t(n);
  const long double two_pi = 6.283185307179586476925286766559005768L;
  for (int e = 0; e < n; ++e) {
    long double ang = two_pi * (long double)e / (long double)n;
    t[e] = cd{(double)cosl(ang), (double)(-sinl(ang))};
  }
  // exact values at the quarter points
  if (n % 4 == 0) {
    t[0] = {1.0, 0.0};
    t[n / 4] = {0.0, -1.0};
    t[n / 2] = {-1.0, 0.0};
    t[3 * n / 4] = {0.0, 1.0};
  } else if (n % 2 == 0) {
    t[0] = {1.0, 0.0};
    t[n / 2] = {-1.0, 0.0};
  } else {
    t[0] = {1.0, 0.0};
  }
  return t;
}

// Twiddles of the cluster transform of length n = C M (C CTAs, R = M / C),
// laid out so that each CTA reads its own slice contiguously:
// [W_n^{C e}, e < M | for c < C: W_n^{c e}, e < M; W_n^{q (c R + t)}, q < C, t < R].
std::vector<cd> cluster_twiddles(int n, const std::vector<cd>& tw) {
  const int C = SFD_FFT_CLUSTER, M = n / C, R = M / C;
  std::vector<cd> t((size_t)(1 + 2 * C) * M);
  for (int e = 0; e < M; ++e) t[e] = tw[(size_t)C * e];
  for (int c = 0; c < C; ++c) {
    cd* twc = t.data() + M + (size_t)c * 2 * M;
    cd* twq = twc + M;
    for (int e = 0; e < M; ++e) twc[e] = tw[(size_t)c * e];
    for (int q = 0; q < C; ++q)
      for (int r = 0; r < R; ++r) twq[q * R + r] = tw[(size_t)q * (c * R + r)];
  }
  return t;
}

// radices: 4s, then a 2, then odd primes ascending
bool factorize(int n, std::vector<int>& rad) {
  rad.clear();
  while (n % 4 == 0) { rad.push_back(4); n /= 4; }
  while (n % 2 == 0) { rad.push_back(2); n /= 2; }
  for (int p = 3; n > 1; p += 2) {
    while (n % p == 0) { rad.push_back(p); n /= p; }
    if (p > 8192) return false;
  }
  return (int)rad.size() <= SFD_MAX_RADICES;
}

}  // namespace


namespace {

// ------------------------------------------------------------------ enqueue helpers
int launch_check(sfd_engine* e) {
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return set_error(SFD_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString(err));
  e->launches++;
  return 0;
}

cudaEvent_t get_event(sfd_engine* e) {
  if (!e->event_pool.empty()) {
    cudaEvent_t ev = e->event_pool.back();
    e->event_pool.pop_back();
    return ev;
  }
  cudaEvent_t ev = nullptr;
  cudaEventCreate(&ev);
  return ev;
}

// Collect finished profile intervals (called after a stream synchronisation).
void drain_profile(sfd_engine* e) {
  for (auto& p : e->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      e->class_ms[p.cls] += ms;
      e->class_count[p.cls] += 1;
    }
    e->event_pool.push_back(p.a);
    e->event_pool.push_back(p.b);
  }
  e->pending.clear();
}

// LAUNCHC(e, class, launch-expression): launch, check, count, and when
// profiling bracket the launch with events on the engine stream.
#define LAUNCHC(e, cls, ...)                                     \
  do {                                                           \
    cudaEvent_t _ea = nullptr, _eb = nullptr;                    \
    if ((e)->profile) {                                          \
      _ea = get_event(e);                                        \
      _eb = get_event(e);                                        \
      cudaEventRecord(_ea, (e)->stream);                         \
    }                                                            \
    __VA_ARGS__;                                                 \
    int _rc = launch_check(e);                                   \
    if (_rc) return _rc;                                         \
    if ((e)->profile) {                                          \
      cudaEventRecord(_eb, (e)->stream);                         \
      (e)->pending.push_back({(cls), _ea, _eb});                 \
    }                                                            \
  } while (0)
#define LAUNCH(e, ...) LAUNCHC(e, SFD_K_OTHER, __VA_ARGS__)

inline int blocks_for(long long n, int t) { return (int)((n + t - 1) / t); }

// Extra corrections of the solve this engine runs (0 when the residual check
// is off).
int extra_iters(const sfd_engine* e) {
  if (!e->rslot || !(e->opt.refine_tol > 0.0)) return 0;
  return std::max(0, std::min(SFD_MAX_EXTRA, e->opt.extra_iters));
}

// Gate on the residual slot `slot` of the current evaluation (-1: ungated).
Gate make_gate(const sfd_engine* e, int slot) {
  if (slot < 0 || !e->rslot) return Gate{nullptr, nullptr, 0, 0.0};
  return Gate{e->rslot + slot, e->bnorm, SFD_RSLOTS, e->opt.refine_tol};
}

// One boundary-sum pass over every surface with weights `weights`
// (`weights_df` its double-float copy for the DF / FP32 passes); the fused
// epilogue writes C, D and the residual (mode 0: r = phi' - M a, C/D
// overwritten; mode 1: r -= M a, C/D accumulated).  track >= 0: the pass
// records max |r| in that residual slot; gate >= 0: it runs only for the
// surfaces whose residual in that slot is above the tolerance.
int enqueue_sums(sfd_engine* e, int prec, const double* weights, const float2* weights_df, int mode, bool track,
                 int gate = -1) = delete;  // the slot is an index: a bool would silently mean slot 0 or 1
int enqueue_sums(sfd_engine* e, int prec, const double* weights, const float2* weights_df, int mode, int track,
                 int gate = -1) {
  SumArgs A{e->d_surf, e->d_sum_items, e->nsurf, e->ntot, e->nd.w, e->nd.p, weights, e->nd.wdf,
            e->nd.pdf, weights_df, e->nd.mdiag, e->zp, e->phip,
            e->cacc, e->dacc, e->r, (track >= 0 && e->rslot) ? e->rslot + track : nullptr, mode, e->rf,
            (mode == 0 && e->rslot) ? e->bnorm : nullptr, make_gate(e, gate),
            e->d_f32_work, e->f32_part, e->f32_wsum, e->f32_count};
  if (prec == SFD_PREC_F32 && e->d_f32_work) {
    // node data staged before the wait unless the preceding kernel wrote them
    A.prefetch = (gate < 0 && !e->node_written && sfd_sums_prefetch_enabled()) ? 1 : 0;
    LAUNCHC(e, gate >= 0 ? SFD_K_EXTRA : SFD_K_SUMS32, sfd_launch_sums_f32(A, e->nf32, e->f32_max_per, e->stream));
    return 0;
  }
  if (prec == SFD_PREC_DF && e->d_f32_work && e->df_part) {
    LAUNCHC(e, gate >= 0 ? SFD_K_EXTRA : SFD_K_SUMSDF,
            sfd_launch_sums_dfs(A, e->df_part, e->nf32, e->f32_max_per, e->sum_groups[prec], e->stream));
    return 0;
  }
  int cls = prec == SFD_PREC_F64 ? SFD_K_SUMS64 : prec == SFD_PREC_DF ? SFD_K_SUMSDF : SFD_K_SUMS32;
  if (gate >= 0) cls = SFD_K_EXTRA;
  LAUNCHC(e, cls, sfd_launch_sums(prec, A, e->nsum, e->max_n, e->sum_groups[prec], e->stream));
  return 0;
}

// y = X v with the current preconditioner (FP16 copy or FP32); ydf: optional
// double-float copy of y; gate >= 0: only where that residual slot is above
// the tolerance.
int enqueue_gemv_gated(sfd_engine* e, const float* vf, double* y, float2* ydf, double* acc, float2* accdf,
                       const Gate& G, int cls) {
  // the first rows may be requested before the wait on the preceding kernel
  // unless the launch is gated or that kernel wrote the matrix
  const bool prefetch = !G.slot && !e->m16_written && sfd_gemv_prefetch_enabled();
  if (e->m16 && e->gemv_spw > 0) {
    // one surface: rows streamed into shared memory, one CTA per SM
    LAUNCHC(e, cls, sfd_launch_gemv_stream(e->d_surf, e->nsm, e->gemv_spw, e->gemv_smem, prefetch, e->m16, e->rscale,
                                           vf, y, ydf, acc, accdf, G, e->status, e->stream));
    e->m16_written = false;
  } else if (e->m16 && e->nsurf == 1 && e->nsm > 0) {
    // one surface: a whole number of waves of two CTAs per SM, rows interleaved
    const int wave = 2 * e->nsm, need = (e->max_n + kGemvRows - 1) / kGemvRows;
    const int grid = (need + wave - 1) / wave * wave;
    LAUNCHC(e, cls, sfd_launch(k_gemv_h, dim3(grid), dim3(512), e->max_np * sizeof(float), e->stream, true,
                                      e->d_surf, (const int2*)nullptr, 0, e->m16, e->rscale, vf, y, ydf, acc, accdf,
                                      G, prefetch ? 1 : 0));
    e->m16_written = false;
  } else if (e->m16) {
    // a batch: persistent CTAs (two per SM) over the (surface, row block) entries
    const int grid = e->nsm > 0 ? std::min(e->ngemv, 2 * e->nsm) : e->ngemv;
    LAUNCHC(e, cls, sfd_launch(k_gemv_h, dim3(grid), dim3(512), e->max_np * sizeof(float), e->stream, true,
                                      e->d_surf, e->d_gemv_rows, e->ngemv, e->m16, e->rscale, vf, y, ydf, acc, accdf,
                                      G, 0));
  } else
    LAUNCHC(e, cls, sfd_launch(k_gemv, dim3(e->ngemv), dim3(256), e->max_np * sizeof(float), e->stream, true,
                                      e->d_surf, e->d_gemv_rows, e->m32, vf, y, ydf, acc, accdf, G));
  e->node_written = false;  // node data are at least two kernels back from the next pass
  return 0;
}
int enqueue_gemv(sfd_engine* e, const float* vf, double* y, float2* ydf, double* acc, float2* accdf,
                 int gate = -1) {
  return enqueue_gemv_gated(e, vf, y, ydf, acc, accdf, make_gate(e, gate), gate >= 0 ? SFD_K_EXTRA : SFD_K_GEMV);
}

int bg_flush(sfd_engine* e);

int enqueue_precond(sfd_engine* e) {
  int rc = bg_flush(e);  // a rebuild in flight on the side stream owns the work buffers
  if (rc) return rc;
  const int nb = e->max_np / 128;
  LAUNCHC(e, SFD_K_ASSEMBLE, sfd_launch_assemble32(e->d_surf, e->d_asm_tiles, e->nasm, e->nd.wdf, e->nd.pdf, e->nd.p,
                                                   e->zp, e->nd.mdiag, e->m32, e->stream));
  const int tiles = e->max_np / 64;
  for (int kb = 0; kb < nb; ++kb) {
    LAUNCHC(e, SFD_K_DIAG, k_gj_diag<<<e->nsurf, 512, kGjDiagSmem, e->stream>>>(e->d_surf, e->nsurf, kb, e->m32,
                                                                                  e->pbuf, e->status));
    const bool tc = e->opt.tensor_cores != 0;
    LAUNCHC(e, SFD_K_PANEL,
            k_gj_panel<<<dim3(tiles, 1, e->nsurf), 256, 0, e->stream>>>(
                e->d_surf, e->nsurf, kb, e->m32, e->pbuf, e->rbuf, e->cbuf, e->d_poff, tc ? e->cparts : nullptr,
                tc ? e->rparts : nullptr, e->panel_elems));
    if (tc) {
      LAUNCHC(e, SFD_K_UPDATE,
              k_gj_update<<<dim3(4 * tiles - 4, 1, e->nsurf), 256, 0, e->stream>>>(
                  e->d_surf, e->nsurf, kb, e->m32, e->pbuf, e->rbuf, e->cbuf, e->d_poff, 1));
      LAUNCHC(e, SFD_K_UPDATE_TC,
              sfd_launch_gj_update_tc(&e->tmap_c, &e->tmap_r, e->d_tmap_out, e->d_surf, e->nsurf, kb, e->max_np,
                                      e->tc_groups, e->d_poff, e->status, e->stream));
    } else {
      LAUNCHC(e, SFD_K_UPDATE,
              k_gj_update<<<dim3(tiles, tiles, e->nsurf), 256, 0, e->stream>>>(
                  e->d_surf, e->nsurf, kb, e->m32, e->pbuf, e->rbuf, e->cbuf, e->d_poff, 0));
    }
  }
  if (e->m16) {
    LAUNCHC(e, SFD_K_GEMV, k_precond_to_half<<<e->ngemv, 256, 0, e->stream>>>(e->d_surf, e->d_gemv_rows, e->m32,
                                                                              e->m16, e->rscale));
    e->m16_written = true;  // the next product reads it only after its wait
  }
  return 0;
}

// The spectral transforms of one evaluation step on stream `st`: the first
// jobs (z', z'', phi') or the a' jobs, as single-CTA transforms, cluster
// transforms and four-step transforms (power-of-two surfaces; `scr` is
// their scratch).  *nlaunch counts the kernels launched.
cudaError_t launch_transforms(const sfd_engine* e, const DerivArgs& D, bool first, cudaStream_t st, cd* scr,
                              int* nlaunch) {
  const int nj = first ? e->njobs_first : e->njobs_ap, ncj = first ? e->ncjobs_first : e->ncjobs_ap;
  cudaError_t err = cudaSuccess;
  if (nj) {
    err = sfd_launch_spectral(D, first ? e->d_jobs_first : e->d_jobs_ap, nj, e->max_n_single, st);
    ++*nlaunch;
  }
  if (err == cudaSuccess && ncj) {
    err = sfd_launch_spectral_cluster(D, first ? e->d_cjobs_first : e->d_cjobs_ap, ncj, e->max_n_cluster, st);
    ++*nlaunch;
  }
  const F4Plan& p = first ? e->f4_first : e->f4_ap;
  for (int ph = 1; ph <= 3 && err == cudaSuccess && p.njobs; ++ph) {
    err = sfd_launch_f4(D, p, scr, st, ph);
    ++*nlaunch;
  }
  return err;
}

// The same on the engine stream as one profiled launch group.
// The same on the engine stream, each kernel a profiled launch of its own
// class (the four-step phases separately, so that per-kernel times compare
// with single-kernel classes).
int enqueue_transforms(sfd_engine* e, const DerivArgs& D, bool first) {
  const int nj = first ? e->njobs_first : e->njobs_ap, ncj = first ? e->ncjobs_first : e->ncjobs_ap;
  const bool redo = D.gate.slot != nullptr;  // gated a' after extra corrections: a class of its own
  // the a' transform has a class of its own too (off the step's critical path on graphs)
  const int c_single = redo ? SFD_K_AP_REDO : first ? SFD_K_SPECTRAL : SFD_K_AP;
  if (nj)
    LAUNCHC(e, c_single,
            sfd_launch_spectral(D, first ? e->d_jobs_first : e->d_jobs_ap, nj, e->max_n_single, e->stream));
  if (ncj)
    LAUNCHC(e, c_single,
            sfd_launch_spectral_cluster(D, first ? e->d_cjobs_first : e->d_cjobs_ap, ncj, e->max_n_cluster,
                                        e->stream));
  const F4Plan& p = first ? e->f4_first : e->f4_ap;
  if (p.njobs) {
    LAUNCHC(e, first ? SFD_K_F4_COLS : c_single, sfd_launch_f4(D, p, e->f4_scr, e->stream, 1));
    LAUNCHC(e, first ? SFD_K_F4_ROWS : c_single, sfd_launch_f4(D, p, e->f4_scr, e->stream, 2));
    LAUNCHC(e, first ? SFD_K_F4_ICOLS : c_single, sfd_launch_f4(D, p, e->f4_scr, e->stream, 3));
  }
  return 0;
}

// a' = d a / d xi (FftDerivative on a, BaseBoundaryIntegrator.cuh:201-203):
// on the engine stream, or forked onto the auxiliary stream so that it runs
// beside the last boundary-sum pass (that pass reads the weights delta and
// writes C, D and r; the transform reads a and writes a').  Where the fork
// is not possible (no auxiliary stream, or per-kernel profiling, whose events
// live on the engine stream) nothing is launched here: enqueue_rhs transforms
// a once the solve, extra corrections included, is done.
int enqueue_ap(sfd_engine* e, bool fork) {
  DerivArgs D{e->d_surf, e->nsurf, nullptr, nullptr, nullptr, nullptr, e->a, e->zp, e->zpp, e->phip, e->ap, nullptr};
  if (fork) {
    if (!e->aux || e->profile) return 0;
    CK(cudaEventRecord(e->ev_fork, e->stream));
    CK(cudaStreamWaitEvent(e->aux, e->ev_fork, 0));
    int nl = 0;
    CK(launch_transforms(e, D, false, e->aux, e->f4_scr, &nl));
    CK(cudaEventRecord(e->ev_join, e->aux));
    e->launches += nl;
    e->ap_forked = true;
    return 0;
  }
  return enqueue_transforms(e, D, false);
}

// First half of an RHS evaluation (calculateVorticities,
// BaseBoundaryIntegrator.cuh:275-306): z', z'', phi', M a = phi' and the
// boundary sums C, D of the solution.
int enqueue_solve(sfd_engine* e, const double* st, const double* phi_im, bool refactor, bool fork_ap = false) {
  const int nt = e->ntot;
  const double *x = st, *y = st + nt, *phi = st + 2 * nt;
  DerivArgs D{e->d_surf, e->nsurf, x, y, phi, phi_im, e->a, e->zp, e->zpp, e->phip, e->ap, e->phipf};
  {
    int rc = enqueue_transforms(e, D, true);
    if (rc) return rc;
  }
  LAUNCHC(e, SFD_K_NODE, sfd_launch(k_node_prep, dim3(blocks_for(nt, 32)), dim3(64), 0, e->stream, true, e->d_surf,
                                    e->d_node_surf, nt, x, y, e->zp, e->zpp, e->nd, e->rslot, e->bnorm));
  e->node_written = true;  // the next boundary-sum pass stages them only after its wait
  const int extra = extra_iters(e);
  if (e->opt.precision == SFD_PRECISION_FP64) {
    LAUNCHC(e, SFD_K_ASSEMBLE, sfd_launch_assemble64(e->d_surf, e->d_asm_tiles, e->nasm, e->nd.w, e->nd.p, e->zp, e->nd.mdiag,
                                    e->m64, e->stream));
    const int nb = e->max_np / 64;
    for (int kb = 0; kb < nb; ++kb) {
      LAUNCHC(e, SFD_K_DIAG, k_lu64_diag<<<e->nsurf, 256, 0, e->stream>>>(e->d_surf, e->nsurf, kb, e->m64, e->status, e->lmax));
      int rem = nb - kb - 1;
      if (rem > 0) {
        LAUNCHC(e, SFD_K_PANEL, k_lu64_trsm<<<dim3(rem, 2, e->nsurf), 64, kTrsmSmem, e->stream>>>(e->d_surf, e->nsurf, kb, e->m64, e->lmax));
        LAUNCHC(e, SFD_K_UPDATE, k_lu64_gemm<<<dim3(2 * rem, 2 * rem, e->nsurf), 256, 0, e->stream>>>(e->d_surf, e->nsurf, kb, e->m64));
      }
    }
    LAUNCHC(e, SFD_K_TRSV, k_lu64_solve<<<e->nsurf, 256, e->max_np * sizeof(double), e->stream>>>(
                               e->d_surf, e->m64, e->phip, e->a, nullptr, nullptr, Gate{}, e->lmax, e->status));
    if (fork_ap) {
      int rc = enqueue_ap(e, true);
      if (rc) return rc;
    }
    int rc = enqueue_sums(e, SFD_PREC_F64, e->a, nullptr, 0, 0);
    if (rc) return rc;
    // FP64 refinement where the residual is above the tolerance (an LU
    // without exchanges that lost accuracy where partial pivoting would have
    // exchanged rows): delta = (LU)^-1 r, a += delta, r -= M delta
    for (int i = 1; i <= extra; ++i) {
      LAUNCHC(e, SFD_K_EXTRA, k_lu64_solve<<<e->nsurf, 256, e->max_np * sizeof(double), e->stream>>>(
                                  e->d_surf, e->m64, e->r, e->delta, e->a, nullptr, make_gate(e, i - 1), nullptr, nullptr));
      rc = enqueue_sums(e, SFD_PREC_F64, e->delta, nullptr, 1, i, i - 1);
      if (rc) return rc;
    }
  } else {
    if (refactor || !e->have_precond) {
      int rc = enqueue_precond(e);
      if (rc) return rc;
      e->have_precond = true;
      // cold starts after a rebuild: every byte 0x7F is a large positive double, an open gate
      if (e->warm) CK(cudaMemsetAsync(e->warm, 0x7F, (size_t)e->nsurf * sizeof(double), e->stream));
    }
    // a0 = X phi'; FP32 pre-iterations (full residual in FP32) bring a within
    // ~1e-7 of the solution; one double-float pass then gives the accurate
    // residual and C(a); FP32 post-iterations correct the small remainder.
    // The products read FP32 copies of phi' and r written by their producers;
    // the updates a += delta run in the product's epilogue.
    // a is final after the last product: a' forks from there
    // a0 = X phi' where the surface's previous solve did not converge (or
    // there is none); elsewhere the previous solution a is the start
    const Gate cold = (e->warm && e->allow_warm && sfd_warm_enabled()) ? Gate{e->warm, e->warm, 1, 0.0} : Gate{};
    int rc = enqueue_gemv_gated(e, e->phipf, e->a, e->adf, nullptr, nullptr, cold, SFD_K_GEMV0);
    if (rc) return rc;
    for (int it = 0; it < e->opt.pre_iters; ++it) {
      rc = enqueue_sums(e, SFD_PREC_F32, e->a, e->adf, 0, -1);
      if (rc) return rc;
      rc = enqueue_gemv(e, e->rf, nullptr, nullptr, e->a, e->adf);
      if (rc) return rc;
    }
    if (fork_ap && e->opt.refine_iters == 0) {
      rc = enqueue_ap(e, true);
      if (rc) return rc;
    }
    rc = enqueue_sums(e, SFD_PREC_DF, e->a, e->adf, 0, e->opt.refine_iters == 0 ? 0 : -1);
    if (rc) return rc;
    for (int it = 0; it < e->opt.refine_iters; ++it) {
      rc = enqueue_gemv(e, e->rf, e->delta, e->ddf, e->a, e->adf);
      if (rc) return rc;
      if (fork_ap && it == e->opt.refine_iters - 1) {
        rc = enqueue_ap(e, true);
        if (rc) return rc;
      }
      rc = enqueue_sums(e, SFD_PREC_F32, e->delta, e->ddf, 1, it == e->opt.refine_iters - 1 ? 0 : -1);
      if (rc) return rc;
    }
    // extra corrections where the residual of the regular passes is above the
    // tolerance (a stale or inaccurate preconditioner)
    for (int i = 1; i <= extra; ++i) {
      rc = enqueue_gemv(e, e->rf, e->delta, e->ddf, e->a, e->adf, i - 1);
      if (rc) return rc;
      rc = enqueue_sums(e, SFD_PREC_F32, e->delta, e->ddf, 1, i, i - 1);
      if (rc) return rc;
    }
  }
  return 0;
}

// One RHS evaluation: state [x|y|phi] -> out [dx|dy|dphi].
int enqueue_rhs(sfd_engine* e, const double* st, double* out, bool refactor) {
  e->ap_forked = false;
  int rc = enqueue_solve(e, st, nullptr, refactor, true);
  if (rc) return rc;
  const int nt = e->ntot;
  const double* y = st + nt;
  // a' (forked during the solve, or here) and the velocity / Bernoulli epilogue
  const int extra = extra_iters(e);
  if (e->ap_forked) {
    CK(cudaStreamWaitEvent(e->stream, e->ev_join, 0));
    e->ap_forked = false;
    if (extra > 0) {
      // the forked transform read a before any extra correction: where one ran
      // (the residual of the regular passes is above the tolerance), a' is
      // transformed again from the final a
      DerivArgs D{e->d_surf, e->nsurf, nullptr, nullptr, nullptr, nullptr, e->a, e->zp, e->zpp, e->phip, e->ap,
                  nullptr, make_gate(e, 0)};
      rc = enqueue_transforms(e, D, false);
      if (rc) return rc;
    }
  } else {
    rc = enqueue_ap(e, false);
    if (rc) return rc;
  }
  VelArgs V{e->d_surf, e->d_node_surf, e->nsurf, nt, e->cacc, e->dacc, e->a, e->ap, e->nd.v1low, e->nd.v1up,
            e->nd.v2, y, st, e->nblk == 4 ? st + 3 * nt : nullptr, e->nblk == 4 ? out + 3 * nt : nullptr,
            e->zp, e->zpp, e->vel_low1, out, out + nt, out + 2 * nt, e->status,
            e->rslot, 1 + extra, e->bnorm, e->opt.refine_tol, e->rnorm, e->rrel, e->extra_count,
            e->opt.precision == SFD_PRECISION_MIXED ? e->stall_dev : nullptr, e->warm};
  if (e->any_rho) LAUNCHC(e, SFD_K_VELOCITY, sfd_launch(k_velocity_node1, dim3(1), dim3(32), 0, e->stream, true, V));
  LAUNCHC(e, SFD_K_VELOCITY,
          sfd_launch(k_velocity_bernoulli, dim3(blocks_for(nt, 32)), dim3(32), 0, e->stream, true, V));
  return 0;
}

int enqueue_step(sfd_engine* e, double dt, bool refactor) {
  const int n3 = e->nblk * e->ntot;  // [x | y | phi (| D)]
  const int nb = blocks_for(n3, 256);
  const double wk[4] = {1.0, 2.0, 2.0, 1.0};
  const double cy[4] = {dt * 0.5, dt * 0.5, dt, 0.0};
  for (int s = 0; s < 4; ++s) {
    const double* in = s == 0 ? e->y0 : e->ys;
    int rc = enqueue_rhs(e, in, e->kcur, refactor && s == 0);
    if (rc) return rc;
    LAUNCHC(e, SFD_K_RK4, sfd_launch(k_rk4_stage, dim3(nb), dim3(256), 0, e->stream, true, n3, e->y0, e->kcur, e->kacc,
                                     s < 3 ? e->ys : nullptr, wk[s], cy[s], s == 0 ? 1 : 0));
  }
  LAUNCHC(e, SFD_K_RK4, sfd_launch(k_rk4_final, dim3(nb), dim3(256), 0, e->stream, true, n3, e->y0, e->kacc, dt / 6.0));
  return 0;
}

void destroy_graphs(sfd_engine* e) {
  for (int i = 0; i < 2; ++i)
    if (e->g_step[i]) {
      cudaGraphExecDestroy(e->g_step[i]);
      e->g_step[i] = nullptr;
    }
}

int build_graph(sfd_engine* e, double dt, int variant) {
  cudaGraph_t g = nullptr;
  long long before = e->launches;
  bool had = e->have_precond;
  if (variant == 0) e->have_precond = true;  // capture the no-refactor variant as such
  CK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_step(e, dt, variant == 1);
  cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
  e->have_precond = had;
  e->launches = before;
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (ce != cudaSuccess) return sfd_fail(ce);
  size_t nn = 0;
  cudaGraphGetNodes(g, nullptr, &nn);
  e->g_kernels[variant] = (int)nn;
  ce = cudaGraphInstantiate(&e->g_step[variant], g, 0);
  cudaGraphDestroy(g);
  if (ce != cudaSuccess) return sfd_fail(ce);
  return 0;
}

// Autotuner of the boundary-sum CTA shape: one eager RHS evaluation on the
// resident state (it leaves valid weights and node data behind), then each
// candidate group count is timed over three launches of every pass precision
// the engine uses; the fastest is kept if it beats the default 4 groups by 3 %.
// The group count sets the per-thread summation order, so runs are bitwise
// repeatable only with autotune off (or the same choice).  The timed launches overwrite C, D
// and r, which the next evaluation recomputes before reading.  Skipped while
// the stream is being captured.
int autotune_sums(sfd_engine* e) {
  e->tune_pending = false;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(e->stream, &cs));
  if (cs != cudaStreamCaptureStatusNone) return 0;
  const bool prof = e->profile;
  e->profile = false;
  int rc = enqueue_rhs(e, e->y0, e->kcur, true);
  if (rc) return rc;
  const bool mixed = e->opt.precision == SFD_PRECISION_MIXED;
  // the FP32 pass (slice-parallel kernel) has no CTA shape to choose
  const int prec_tuned = mixed ? SFD_PREC_DF : SFD_PREC_F64;
  cudaEvent_t a = nullptr, b = nullptr;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  for (int pi = 0; pi < 1 && !rc; ++pi) {
    const int prec = prec_tuned;
    const float2* wdf = prec == SFD_PREC_F64 ? nullptr : e->adf;
    float best = 0.f, t4 = 0.f;
    int best_g = 4;
    for (int g : kSumGroupChoices) {
      e->sum_groups[prec] = g;
      rc = enqueue_sums(e, prec, e->a, wdf, 0, -1);  // warm-up
      if (rc) break;
      cudaEventRecord(a, e->stream);
      for (int r = 0; r < 3 && !rc; ++r) rc = enqueue_sums(e, prec, e->a, wdf, 0, -1);
      cudaEventRecord(b, e->stream);
      if (rc) break;
      cudaError_t err = cudaEventSynchronize(b);
      float ms = 0.f;
      if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, a, b);
      if (err != cudaSuccess) {
        rc = sfd_fail(err);
        break;
      }
      if (g == 4) t4 = ms;
      if (g == kSumGroupChoices[0] || ms < best) {
        best = ms;
        best_g = g;
      }
    }
    // keep the default unless another shape is clearly faster (timing noise
    // would otherwise flip the choice, and with it the summation order)
    e->sum_groups[prec] = best < 0.97f * t4 ? best_g : 4;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  e->profile = prof;
  return rc;
}

// ------------------------------------------------------- background rebuild
// With refactor_lag = k > 0 the preconditioner due at step s is built on a
// low-priority side stream: the main stream copies the state and records
// ev_snap; the side stream waits for it, recomputes z', z'' and the node data
// of the copy into its own buffers, assembles M, runs the Gauss-Jordan
// inverse and writes the FP16 copy into m16_next / rscale_next, then records
// ev_done.  Before the graph of step s + k the main stream waits for ev_done
// and copies m16_next / rscale_next over the live preconditioner.  The switch
// step does not depend on timing, so runs are deterministic.  The work
// buffers of the inverse (m32, panels, parts) belong to the side stream while
// a rebuild is in flight; any synchronous rebuild first flushes it.
namespace {
int bg_alloc(sfd_engine* e) {
  auto& B = e->bg;
  if (B.side) return 0;
  int least = 0, greatest = 0;
  CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  CK(cudaStreamCreateWithPriority(&B.side, cudaStreamNonBlocking, least));
  CK(cudaEventCreateWithFlags(&B.ev_snap, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&B.ev_done, cudaEventDisableTiming));
  const int nt = e->ntot;
  CK(dalloc(&B.snap, 3LL * nt));
  CK(dalloc(&B.zp, nt));
  CK(dalloc(&B.zpp, nt));
  CK(dalloc(&B.phip, nt));
  CK(dalloc(&B.nd.w, nt));
  CK(dalloc(&B.nd.p, nt));
  CK(dalloc(&B.nd.wdf, nt));
  CK(dalloc(&B.nd.pdf, nt));
  CK(dalloc(&B.nd.mdiag, nt));
  CK(dalloc(&B.nd.v1low, nt));
  CK(dalloc(&B.nd.v1up, nt));
  CK(dalloc(&B.nd.v2, nt));
  CK(dalloc(&B.m16_next, e->mat_elems));
  CK(dalloc(&B.rscale_next, nt));
  if (e->f4_first.njobs) CK(dalloc(&B.f4_scr, 3LL * nt));
  return 0;
}

// Enqueue the rebuild of the preconditioner from the current state.
int bg_start(sfd_engine* e) {
  int rc = bg_alloc(e);
  if (rc) return rc;
  auto& B = e->bg;
  const int nt = e->ntot;
  cudaStream_t side = B.side;
  CK(cudaMemcpyAsync(B.snap, e->y0, 3LL * nt * sizeof(double), cudaMemcpyDeviceToDevice, e->stream));
  CK(cudaEventRecord(B.ev_snap, e->stream));
  CK(cudaStreamWaitEvent(side, B.ev_snap, 0));
  const double *x = B.snap, *y = B.snap + nt, *phi = B.snap + 2 * nt;
  DerivArgs D{e->d_surf, e->nsurf, x, y, phi, nullptr, nullptr, B.zp, B.zpp, B.phip, nullptr, nullptr};
  int nl = 0;
  CK(launch_transforms(e, D, true, side, B.f4_scr, &nl));
  e->launches += nl;
  k_node_prep<<<blocks_for(nt, 32), 64, 0, side>>>(e->d_surf, e->d_node_surf, nt, x, y, B.zp, B.zpp, B.nd, nullptr,
                                                    nullptr);
  CK(cudaGetLastError());
  CK(sfd_launch_assemble32(e->d_surf, e->d_asm_tiles, e->nasm, B.nd.wdf, B.nd.pdf, B.nd.p, B.zp, B.nd.mdiag,
                           e->m32, side));
  const int nb = e->max_np / 128, tiles = e->max_np / 64;
  for (int kb = 0; kb < nb; ++kb) {
    k_gj_diag<<<e->nsurf, 512, kGjDiagSmem, side>>>(e->d_surf, e->nsurf, kb, e->m32, e->pbuf, e->status);
    k_gj_panel<<<dim3(tiles, 1, e->nsurf), 256, 0, side>>>(e->d_surf, e->nsurf, kb, e->m32, e->pbuf, e->rbuf, e->cbuf,
                                                            e->d_poff, e->cparts, e->rparts, e->panel_elems);
    k_gj_update<<<dim3(4 * tiles - 4, 1, e->nsurf), 256, 0, side>>>(e->d_surf, e->nsurf, kb, e->m32, e->pbuf, e->rbuf,
                                                                     e->cbuf, e->d_poff, 1);
    CK(sfd_launch_gj_update_tc(&e->tmap_c, &e->tmap_r, e->d_tmap_out, e->d_surf, e->nsurf, kb, e->max_np,
                               e->tc_groups, e->d_poff, e->status, side));
  }
  k_precond_to_half<<<e->ngemv, 256, 0, side>>>(e->d_surf, e->d_gemv_rows, e->m32, B.m16_next, B.rscale_next);
  CK(cudaGetLastError());
  CK(cudaEventRecord(B.ev_done, side));
  e->launches += 4 + 4LL * nb;
  B.rebuilds++;
  return 0;
}

// Switch to the rebuilt preconditioner (main stream waits for it).
int bg_swap(sfd_engine* e) {
  auto& B = e->bg;
  CK(cudaStreamWaitEvent(e->stream, B.ev_done, 0));
  CK(cudaMemcpyAsync(e->m16, B.m16_next, (size_t)e->mat_elems * sizeof(__half), cudaMemcpyDeviceToDevice, e->stream));
  e->m16_written = true;
  CK(cudaMemcpyAsync(e->rscale, B.rscale_next, (size_t)e->ntot * sizeof(float), cudaMemcpyDeviceToDevice, e->stream));
  B.swap_at = -1;
  return 0;
}

bool bg_usable(const sfd_engine* e) {
  return e->opt.precision == SFD_PRECISION_MIXED && e->opt.refactor_lag > 0 && e->m16 && e->opt.tensor_cores &&
         e->opt.refactor_lag < std::max(1, e->opt.refactor_every);
}
}  // namespace

// Apply a pending background rebuild now (before anything else uses the
// inverse's work buffers or replaces the preconditioner).
int bg_flush(sfd_engine* e) {
  if (e->bg.swap_at < 0) return 0;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(e->stream, &cs));
  if (cs != cudaStreamCaptureStatusNone) return set_error(SFD_ERR_INVALID, "background rebuild pending during capture");
  return bg_swap(e);
}

int run_steps_body(sfd_engine* e, double dt, int steps);
// Fixed-step RK4 on the resident state; its evaluations may start warm.
int run_steps(sfd_engine* e, double dt, int steps) {
  e->allow_warm = true;
  const int rc = run_steps_body(e, dt, steps);
  e->allow_warm = false;
  return rc;
}
int run_steps_body(sfd_engine* e, double dt, int steps) {
  if (steps < 0) return set_error(SFD_ERR_INVALID, "negative step count");
  if (!std::isfinite(dt)) return set_error(SFD_ERR_INVALID, "time step must be finite");
  CK(cudaSetDevice(e->device));
  if (e->tune_pending && steps > 0) {
    int rc = autotune_sums(e);
    if (rc) return rc;
    destroy_graphs(e);  // captured with the previous shapes
  }
  const bool mixed = e->opt.precision == SFD_PRECISION_MIXED;
  const int every = std::max(1, e->opt.refactor_every);
  const bool graphs = e->opt.use_graphs && !e->profile;
  if (graphs && e->g_dt != dt) {
    destroy_graphs(e);
    e->g_dt = dt;
  }
  for (int s = 0; s < steps; ++s) {
    const bool due = (e->step_count % every) == 0;
    bool refactor = !mixed || !e->have_precond || due;
    if (mixed && e->have_precond && bg_usable(e)) {
      if (e->bg.swap_at == e->step_count) {
        int rc = bg_swap(e);
        if (rc) return rc;
      }
      if (due && e->bg.swap_at < 0) {
        int rc = bg_start(e);
        if (rc) return rc;
        e->bg.swap_at = e->step_count + e->opt.refactor_lag;
      }
      refactor = false;
    }
    // A refinement stall seen by a step that already ran (the kernels set the
    // host-mapped word; the GPU may be several steps behind the host, so this
    // is the first step enqueued after the host sees it) rebuilds the
    // preconditioner inside this step.  A background rebuild in flight owns
    // the inverse's work buffers, so it is switched in first.
    if (mixed && e->have_precond && e->stall_host && *reinterpret_cast<volatile unsigned int*>(e->stall_host)) {
      *reinterpret_cast<volatile unsigned int*>(e->stall_host) = 0u;
      if (!refactor) {
        refactor = true;
        e->stall_rebuilds++;
        if (e->bg.swap_at >= 0) {
          int rc = bg_swap(e);
          if (rc) return rc;
        }
      }
    }
    if (graphs) {
      const int variant = refactor ? 1 : 0;
      if (!e->g_step[variant]) {
        int rc = build_graph(e, dt, variant);
        if (rc) return rc;
      }
      CK(cudaGraphLaunch(e->g_step[variant], e->stream));
      e->launches += e->g_kernels[variant];
    } else {
      int rc = enqueue_step(e, dt, refactor);
      if (rc) return rc;
    }
    if (refactor && mixed) e->have_precond = true;
    e->step_count++;
  }
  return 0;
}

void free_engine(sfd_engine* e) {
  if (!e) return;
  cudaSetDevice(e->device);
  if (e->stream) cudaStreamSynchronize(e->stream);
  if (e->bg.side) cudaStreamSynchronize(e->bg.side);  // a background rebuild uses the inverse's buffers
  destroy_graphs(e);
  void* ptrs[] = {e->d_surf, e->d_node_surf, e->d_jobs_first, e->d_jobs_ap, e->d_cjobs_first, e->d_cjobs_ap, e->d_sum_items,
                  e->d_f32_work, e->f32_part, e->f32_wsum, e->f32_count, e->df_part, e->d_asm_tiles,
                  e->d_gemv_rows, e->d_poff, e->y0, e->ys, e->kacc, e->kcur, e->zp, e->zpp, e->ap, e->phip, e->a,
                  e->r, e->delta, e->phi_im, e->nd.w, e->nd.p, e->nd.wdf, e->nd.pdf, e->adf, e->ddf, e->nd.mdiag, e->nd.v1low, e->nd.v1up, e->nd.v2,
                  e->cacc, e->dacc, e->vel_low1, e->status, e->lmax, e->rnorm, e->rslot, e->bnorm, e->rrel,
                  e->extra_count,
                  e->inv_out, e->m64, e->m32, e->m16, e->rscale, e->fc_in, e->fc_out, e->rf, e->phipf, e->pbuf, e->rbuf, e->cbuf, e->cparts, e->rparts,
                  e->d_tmap_out, e->warm};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  {
    auto& B = e->bg;
    void* bp[] = {B.snap, B.zp, B.zpp, B.phip, B.nd.w, B.nd.p, B.nd.wdf, B.nd.pdf, B.nd.mdiag, B.nd.v1low, B.nd.v1up,
                  B.nd.v2, B.m16_next, B.rscale_next, B.f4_scr};
    for (void* p : bp)
      if (p) cudaFree(p);
    if (B.ev_snap) cudaEventDestroy(B.ev_snap);
    if (B.ev_done) cudaEventDestroy(B.ev_done);
    if (B.side) cudaStreamDestroy(B.side);
  }
  sfd_adjoint_free(e);
  sfd_rkf45_free(e);
  sfd_gl2_free(e);
  drain_profile(e);
  for (cudaEvent_t ev : e->event_pool) cudaEventDestroy(ev);
  for (F4Plan* p : {&e->f4_first, &e->f4_ap}) {
    if (p->jobs) cudaFree(p->jobs);
    for (int ph = 0; ph < 3; ++ph)
      if (p->units[ph]) cudaFree(p->units[ph]);
  }
  if (e->f4_scr) cudaFree(e->f4_scr);
  for (auto& kv : e->d_tw) cudaFree(kv.second);
  for (auto& kv : e->d_ctw) cudaFree(kv.second);
  if (e->aux) cudaStreamSynchronize(e->aux);
  if (e->ev_fork) cudaEventDestroy(e->ev_fork);
  if (e->ev_join) cudaEventDestroy(e->ev_join);
  if (e->aux) cudaStreamDestroy(e->aux);
  if (e->own_stream) cudaStreamDestroy(e->own_stream);
  if (e->stall_host) cudaFreeHost(e->stall_host);
  delete e;
}

int fill_surface(SurfaceDesc& S, const sfd_problem& p) {
  S.physics = p.physics;
  S.infinite_depth = p.infinite_depth ? 1 : 0;
  S.rho = p.rho;
  S.depth = p.depth;
  S.gravity = p.gravity > 0 ? p.gravity : 1.0;
  S.U = p.U;
  S.kappa = p.kappa;
  S.expansion_order = p.expansion_order;
  S.bern_variant = 0;
  if (p.physics != SFD_WATER && p.physics != SFD_HELIUM) return set_error(SFD_ERR_INVALID, "unknown physics %d", p.physics);
  if (p.physics == SFD_HELIUM) {
    if (!(p.depth > 0)) return set_error(SFD_ERR_INVALID, "helium needs depth > 0 (got %g)", p.depth);
    S.vdw = p.A3 > 0 ? p.A3 / (p.depth * p.depth * p.depth) : p.depth / 3.0;  // createM.cuh:113
    if (p.use_expansions) S.bern_variant = 1;      // HeliumBoundaryProblem.cuh:140-148
    else if (p.kappa != 0.0) S.bern_variant = 2;
  } else {
    S.vdw = 0.0;
  }
  return 0;
}

// Optomechanical drive of one surface (HeliumDrivenAutonomousProblem.cuh:10-28).
int fill_drive(SurfaceDesc& S, const sfd_drive& d) {
  S.drive = 1;
  S.drive_aug = d.augmented ? 1 : 0;
  if (S.physics != SFD_HELIUM) return set_error(SFD_ERR_INVALID, "a drive needs a helium surface");
  if (!(d.sigma != 0.0) || (d.augmented && !(d.tau != 0.0)))
    return set_error(SFD_ERR_INVALID, "drive: sigma and (augmented) tau must be nonzero");
  S.dr_detuning = d.detuning;
  S.dr_gamma = d.gamma;
  S.dr_G = d.G;
  S.dr_tau = d.tau;
  S.dr_imax = d.max_intensity;
  S.dr_x0 = d.x0;
  S.dr_sigma = d.sigma;
  S.dr_beta = d.beta;
  S.dr_damping = d.damping;
  S.dr_strength = d.strength;
  return 0;
}

}  // namespace

// Dynamic shared-memory limits of the solver kernels (per device context).
cudaError_t sfd_solve_configure() {
  cudaError_t e = cudaFuncSetAttribute(k_gj_diag, cudaFuncAttributeMaxDynamicSharedMemorySize, kGjDiagSmem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_lu64_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, 8320 * (int)sizeof(double));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_lu64_trsm, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrsmSmem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_lu64_trsm_u, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrsmSmem);
  return e;
}

int sfd_internal_error(int code, const char* msg) { return set_error(code, "%s", msg); }
int sfd_internal_cuda(cudaError_t err, const char* what) {
  return set_error(SFD_ERR_CUDA, "%s: %s", what, cudaGetErrorString(err));
}
int sfd_internal_rhs(sfd_engine* e, const double* st, double* out) { return enqueue_rhs(e, st, out, true); }
int sfd_internal_solve(sfd_engine* e, const double* st) { return enqueue_solve(e, st, nullptr, true); }
int sfd_internal_rhs_ex(sfd_engine* e, const double* st, double* out, bool refactor) {
  return enqueue_rhs(e, st, out, refactor);
}
int sfd_internal_bg_flush(sfd_engine* e) { return bg_flush(e); }
bool sfd_sums_prefetch_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("SFD_SUMS_PREFETCH");
    return !(v && v[0] == '0');
  }();
  return on;
}
bool sfd_gemv_prefetch_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("SFD_GEMV_PREFETCH");
    return !(v && v[0] == '0');
  }();
  return on;
}
int sfd_gemv_stream_cap() {
  static const int cap = [] {
    const char* v = std::getenv("SFD_GEMV_SPW");
    return v ? std::max(0, std::atoi(v)) : kGemvSDefaultSpw;
  }();
  return cap;
}
bool sfd_warm_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("SFD_WARM");
    return !(v && v[0] == '0');
  }();
  return on;
}

// ====================================================================== C ABI
extern "C" {

void sfd_default_options(sfd_options* o) {
  if (!o) return;
  o->precision = SFD_PRECISION_MIXED;
  o->refine_iters = 2;
  o->refactor_every = 1;
  o->use_graphs = 1;
  o->device = 0;
  o->tensor_cores = 1;
  o->pre_iters = 1;
  o->precond_half = 1;
  o->autotune = 1;
  o->refactor_lag = 0;
  o->extra_iters = 2;
  o->refine_tol = 1e-10;
}

void sfd_default_problem(sfd_problem* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->physics = SFD_WATER;
  p->depth = 1.0;
  p->gravity = 1.0;
}

const char* sfd_last_error(void) { return g_last_error.c_str(); }
const char* sfd_version(void) { return "sfd-gb300 0.1 (sm_103a)"; }

int sfd_set_default_precision(int precision) {
  if (precision != SFD_PRECISION_FP64 && precision != SFD_PRECISION_MIXED)
    return set_error(SFD_ERR_INVALID, "unknown precision %d", precision);
  g_default_precision = precision;
  return 0;
}

int sfd_create(const int* n, int nsurf, const sfd_problem* problems, int shared_problem, const sfd_options* opts,
               sfd_engine** out) {
  return sfd_create_driven(n, nsurf, problems, nullptr, shared_problem, opts, out);
}

// Source slices per surface for the FP32 pass, so that one launch fills the
// GPU evenly: the total work (tiles x sources) is spread over `slots`
// resident CTAs (in as many waves as keep a slice within kF32MaxPer
// sources), each surface's slice count proportional to its node count (the
// floor, so the entries never exceed the slots of the waves), with at least
// kF32MinPer sources per slice and at most kF32MaxSlices slices.
static void plan_f32_slices(const std::vector<SurfaceDesc>& hs, int nsurf, int slots, std::vector<int>& out) {
  int cap = kF32MaxSlices;
  if (const char* v = std::getenv("SFD_F32_SLICES")) cap = std::min(kF32MaxSlices, std::max(1, std::atoi(v)));
  long long total = 0;
  for (int s = 0; s < nsurf; ++s) total += (long long)((hs[s].n + kSumTile - 1) / kSumTile) * hs[s].n;
  const long long waves = std::max(1LL, (total + (long long)slots * kF32MaxPer - 1) / ((long long)slots * kF32MaxPer));
  out.assign(nsurf, 1);
  for (int s = 0; s < nsurf; ++s) {
    const long long n = hs[s].n;
    long long ns = total > 0 ? n * waves * slots / total : 1;
    ns = std::min(ns, (n + kF32MinPer - 1) / kF32MinPer);
    ns = std::max(ns, (n + kF32MaxPer - 1) / kF32MaxPer);  // slices within kF32MaxPer sources
    out[s] = (int)std::max(1LL, std::min<long long>(ns, cap));
  }
}

int sfd_create_driven(const int* n, int nsurf, const sfd_problem* problems, const sfd_drive* drives,
                      int shared_problem, const sfd_options* opts, sfd_engine** out) {
  if (!out || !n || !problems || nsurf <= 0) return set_error(SFD_ERR_INVALID, "sfd_create: bad arguments");
  *out = nullptr;
  sfd_options opt;
  if (opts) opt = *opts;
  else sfd_default_options(&opt);
  if (opt.precision != SFD_PRECISION_FP64 && opt.precision != SFD_PRECISION_MIXED)
    return set_error(SFD_ERR_INVALID, "unknown precision %d", opt.precision);
  if (opt.extra_iters < 0 || opt.extra_iters > SFD_MAX_EXTRA || !(opt.refine_tol == opt.refine_tol))
    return set_error(SFD_ERR_INVALID, "extra_iters must be 0..%d and refine_tol a number", SFD_MAX_EXTRA);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return set_error(SFD_ERR_NO_DEVICE, "no CUDA device available");
  sfd_engine* e = new sfd_engine();
  e->opt = opt;
  if (e->opt.refine_iters < 0) e->opt.refine_iters = 0;
  e->tune_pending = e->opt.autotune != 0;
  if (e->opt.pre_iters < 0) e->opt.pre_iters = 0;
  e->device = e->opt.device;
  if (e->device < 0 || e->device >= ndev) {
    const int device = e->device;
    delete e;
    return set_error(SFD_ERR_INVALID, "device %d out of range", device);
  }
  int rc = 0;
#define CKE(expr)                   \
  do {                              \
    cudaError_t _e = (expr);        \
    if (_e != cudaSuccess) {        \
      rc = sfd_fail(_e);            \
      free_engine(e);               \
      return rc;                    \
    }                               \
  } while (0)
  CKE(cudaSetDevice(e->device));
  CKE(cudaDeviceGetAttribute(&e->nsm, cudaDevAttrMultiProcessorCount, e->device));
  CKE(cudaStreamCreateWithFlags(&e->own_stream, cudaStreamNonBlocking));
  e->stream = e->own_stream;
  CKE(cudaStreamCreateWithFlags(&e->aux, cudaStreamNonBlocking));
  CKE(cudaEventCreateWithFlags(&e->ev_fork, cudaEventDisableTiming));
  CKE(cudaEventCreateWithFlags(&e->ev_join, cudaEventDisableTiming));
  e->nsurf = nsurf;
  e->hs.resize(nsurf);
  for (int s = 0; s < nsurf; ++s) e->hp.push_back(problems[shared_problem ? 0 : s]);
  long long off = 0, moff = 0, poff = 0;
  std::vector<long long> h_poff(nsurf);
  for (int s = 0; s < nsurf; ++s) {
    int ns = n[s];
    if (ns < 1 || ns > 8192) {
      free_engine(e);
      return set_error(SFD_ERR_INVALID, "surface %d: n = %d outside 1..8192", s, ns);
    }
    SurfaceDesc& S = e->hs[s];
    std::memset(&S, 0, sizeof(S));
    S.n = ns;
    S.off = (int)off;
    S.moff = moff;
    rc = fill_surface(S, problems[shared_problem ? 0 : s]);
    if (!rc && drives) rc = fill_drive(S, drives[shared_problem ? 0 : s]);
    if (rc) {
      free_engine(e);
      return rc;
    }
    if (S.drive_aug) e->nblk = 4;
    std::vector<int> rad;
    if (!factorize(ns, rad)) {
      free_engine(e);
      return set_error(SFD_ERR_INVALID, "surface %d: n = %d has too many factors", s, ns);
    }
    S.nrad = (int)rad.size();
    for (size_t i = 0; i < rad.size(); ++i) S.rad[i] = rad[i];
    S.nrad_m = 0;
    if (ns % (SFD_FFT_CLUSTER * SFD_FFT_CLUSTER) == 0 && ns >= SFD_FFT_CLUSTER_MIN_N) {
      std::vector<int> radm;
      if (factorize(ns / SFD_FFT_CLUSTER, radm)) {
        S.nrad_m = (int)radm.size();
        for (size_t i = 0; i < radm.size(); ++i) S.rad_m[i] = radm[i];
      }
    }
    if (!e->d_tw.count(ns)) {
      std::vector<cd> t = twiddles(ns);
      cd* d = nullptr;
      CKE(dalloc(&d, ns));
      e->d_tw[ns] = d;
      CKE(cudaMemcpy(d, t.data(), ns * sizeof(cd), cudaMemcpyHostToDevice));
    }
    S.tw = e->d_tw[ns];
    if (S.nrad_m > 0) {
      if (!e->d_ctw.count(ns)) {
        std::vector<cd> t = twiddles(ns), ct = cluster_twiddles(ns, t);
        cd* d = nullptr;
        CKE(dalloc(&d, (long long)ct.size()));
        e->d_ctw[ns] = d;
        CKE(cudaMemcpy(d, ct.data(), ct.size() * sizeof(cd), cudaMemcpyHostToDevice));
      }
      S.ctw = e->d_ctw[ns];
    }
    if (S.physics == 0 && S.rho != 0.0) e->any_rho = true;
    int np = pad_n(ns);
    h_poff[s] = poff;
    poff += 128LL * np;
    off += ns;
    moff += (long long)np * np;
    e->max_n = std::max(e->max_n, ns);
    e->max_np = std::max(e->max_np, np);
  }
  if (off > (1LL << 30)) {
    free_engine(e);
    return set_error(SFD_ERR_INVALID, "too many nodes");
  }
  e->ntot = (int)off;
  e->mat_elems = moff;
  e->panel_elems = poff;
  const int nt = e->ntot;
  // work lists
  std::vector<int> node_surf(nt);
  std::vector<int2> jf, ja, cjf, cja;
  std::vector<F4Job> f4f, f4a;
  std::vector<int2> items;
  std::vector<F32Work> f32work;
  std::vector<int4> tiles;
  std::vector<int2> rows;
  std::vector<int> f32_slices;
  if (e->opt.precision == SFD_PRECISION_MIXED) {
    int ctas = 0;
    CKE(sfd_f32_ctas_per_sm(kF32MaxPer, &ctas));
    plan_f32_slices(e->hs, nsurf, std::max(1, ctas) * std::max(1, e->nsm), f32_slices);
  }
  for (int s = 0; s < nsurf; ++s) {
    const SurfaceDesc& S = e->hs[s];
    for (int k = 0; k < S.n; ++k) node_surf[S.off + k] = s;
    if (sfd_f4_eligible(S.n)) {
      // four-step transforms over the whole GPU; scratch regions by node offset
      f4f.push_back({s, SFD_F4_Z, 0LL * nt + S.off, 1LL * nt + S.off});
      f4f.push_back({s, SFD_F4_PHI, 2LL * nt + S.off, 0});
      f4a.push_back({s, SFD_F4_AP, 3LL * nt + S.off, 0});
    } else if (S.nrad_m > 0) {
      cjf.push_back({s, SFD_JOB_ZP});  // z', z'' and phi' on three clusters side by side
      cjf.push_back({s, SFD_JOB_ZPP});
      cjf.push_back({s, SFD_JOB_PHIP});
      cja.push_back({s, SFD_JOB_AP});
      e->max_n_cluster = std::max(e->max_n_cluster, S.n);
    } else {
      jf.push_back({s, SFD_JOB_ZP});
      jf.push_back({s, SFD_JOB_ZPP});
      jf.push_back({s, SFD_JOB_PHIP});
      ja.push_back({s, SFD_JOB_AP});
      e->max_n_single = std::max(e->max_n_single, S.n);
    }
    for (int t0 = 0; t0 < S.n; t0 += kSumTile) {
      const int it = (int)items.size(), ns = f32_slices.empty() ? 0 : f32_slices[s];
      const int base = (int)f32work.size();
      if (ns) e->f32_max_per = std::max(e->f32_max_per, (S.n + ns - 1) / ns);
      for (int sl = 0; sl < ns; ++sl) {
        F32Work w{};
        w.item = it;
        w.slice = sl;
        w.base = base;
        w.nsl = ns;
        w.sidx = s;
        w.t0 = t0;
        w.n = S.n;
        w.off = S.off;
        w.image = (S.physics == 1 && !S.infinite_depth) ? 1 : 0;
        w.c1 = S.physics == 0 ? (float)(0.25 * (1 - S.rho) / SFD_PI) : (float)(0.25 / SFD_PI);
        f32work.push_back(w);
      }
      items.push_back({s, t0});
    }
    int np = pad_n(S.n);
    for (int r0 = 0; r0 < np; r0 += 64)
      for (int c0 = 0; c0 < np; c0 += 64) tiles.push_back({s, r0, c0, 0});
    for (int r0 = 0; r0 < S.n; r0 += kGemvRows) rows.push_back({s, r0});
  }
  e->njobs_first = (int)jf.size();
  e->njobs_ap = (int)ja.size();
  e->ncjobs_first = (int)cjf.size();
  e->ncjobs_ap = (int)cja.size();
  e->nsum = (int)items.size();
  e->nasm = (int)tiles.size();
  e->ngemv = (int)rows.size();
  CKE(dalloc(&e->d_surf, nsurf));
  CKE(cudaMemcpy(e->d_surf, e->hs.data(), nsurf * sizeof(SurfaceDesc), cudaMemcpyHostToDevice));
  CKE(dalloc(&e->d_node_surf, nt));
  CKE(cudaMemcpy(e->d_node_surf, node_surf.data(), nt * sizeof(int), cudaMemcpyHostToDevice));
  CKE(dalloc(&e->d_jobs_first, jf.size()));
  CKE(cudaMemcpy(e->d_jobs_first, jf.data(), jf.size() * sizeof(int2), cudaMemcpyHostToDevice));
  CKE(dalloc(&e->d_jobs_ap, ja.size()));
  CKE(cudaMemcpy(e->d_jobs_ap, ja.data(), ja.size() * sizeof(int2), cudaMemcpyHostToDevice));
  CKE(dalloc(&e->d_cjobs_first, cjf.size()));
  CKE(cudaMemcpy(e->d_cjobs_first, cjf.data(), cjf.size() * sizeof(int2), cudaMemcpyHostToDevice));
  CKE(dalloc(&e->d_cjobs_ap, cja.size()));
  CKE(cudaMemcpy(e->d_cjobs_ap, cja.data(), cja.size() * sizeof(int2), cudaMemcpyHostToDevice));
  // four-step plans: per phase the (job, unit) list; units of a job are
  // contiguous and their counts multiples of 4 (64 columns, n / 64 rows)
  for (int pi = 0; pi < 2; ++pi) {
    const std::vector<F4Job>& jl = pi == 0 ? f4f : f4a;
    F4Plan& p = pi == 0 ? e->f4_first : e->f4_ap;
    if (jl.empty()) continue;
    std::vector<int2> ul[3];
    for (int j = 0; j < (int)jl.size(); ++j) {
      const int n = e->hs[jl[j].surf].n;
      for (int u = 0; u < 64; ++u) ul[0].push_back({j, u});
      for (int u = 0; u < n / 64; ++u) ul[1].push_back({j, u});
      for (int u = 0; u < (jl[j].kind == SFD_F4_Z ? 128 : 64); ++u) ul[2].push_back({j, u});
    }
    p.njobs = (int)jl.size();
    CKE(dalloc(&p.jobs, jl.size()));
    CKE(cudaMemcpy(p.jobs, jl.data(), jl.size() * sizeof(F4Job), cudaMemcpyHostToDevice));
    for (int ph = 0; ph < 3; ++ph) {
      p.nunits[ph] = (int)ul[ph].size();
      CKE(dalloc(&p.units[ph], ul[ph].size()));
      CKE(cudaMemcpy(p.units[ph], ul[ph].data(), ul[ph].size() * sizeof(int2), cudaMemcpyHostToDevice));
    }
  }
  if (!f4f.empty()) CKE(dalloc(&e->f4_scr, 4LL * nt));
  CKE(dalloc(&e->d_sum_items, items.size()));
  CKE(cudaMemcpy(e->d_sum_items, items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice));
  if (e->opt.precision == SFD_PRECISION_MIXED) {
    e->nf32 = (int)f32work.size();
    int ctas = 0;  // shared-memory opt-in for the widest slice
    CKE(sfd_f32_ctas_per_sm(std::max(e->f32_max_per, kF32MaxPer), &ctas));
    CKE(dalloc(&e->d_f32_work, f32work.size()));
    CKE(cudaMemcpy(e->d_f32_work, f32work.data(), f32work.size() * sizeof(F32Work), cudaMemcpyHostToDevice));
    CKE(dalloc(&e->f32_part, 64LL * f32work.size()));
    CKE(dalloc(&e->df_part, 128LL * f32work.size()));
    CKE(dalloc(&e->f32_wsum, f32work.size()));
    CKE(dalloc(&e->f32_count, items.size()));
    CKE(cudaMemset(e->f32_count, 0, items.size() * sizeof(unsigned int)));
  }
  CKE(dalloc(&e->d_asm_tiles, tiles.size()));
  CKE(cudaMemcpy(e->d_asm_tiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice));
  CKE(dalloc(&e->d_gemv_rows, rows.size()));
  CKE(cudaMemcpy(e->d_gemv_rows, rows.data(), rows.size() * sizeof(int2), cudaMemcpyHostToDevice));
  CKE(dalloc(&e->d_poff, nsurf));
  CKE(cudaMemcpy(e->d_poff, h_poff.data(), nsurf * sizeof(long long), cudaMemcpyHostToDevice));
  // buffers
  CKE(dalloc(&e->y0, (long long)e->nblk * nt));
  CKE(dalloc(&e->ys, (long long)e->nblk * nt));
  CKE(dalloc(&e->kacc, (long long)e->nblk * nt));
  CKE(dalloc(&e->kcur, (long long)e->nblk * nt));
  CKE(dalloc(&e->zp, nt));
  CKE(dalloc(&e->zpp, nt));
  CKE(dalloc(&e->ap, nt));
  CKE(dalloc(&e->phip, nt));
  CKE(dalloc(&e->a, nt));
  CKE(dalloc(&e->r, nt));
  CKE(dalloc(&e->delta, nt));
  CKE(dalloc(&e->nd.w, nt));
  CKE(dalloc(&e->nd.p, nt));
  CKE(dalloc(&e->nd.wdf, nt));
  CKE(dalloc(&e->nd.pdf, nt));
  CKE(dalloc(&e->adf, nt));
  CKE(dalloc(&e->ddf, nt));
  if (e->opt.precision == SFD_PRECISION_MIXED) {
    CKE(dalloc(&e->rf, nt));
    CKE(dalloc(&e->phipf, nt));
  }
  CKE(dalloc(&e->nd.mdiag, nt));
  CKE(dalloc(&e->nd.v1low, nt));
  CKE(dalloc(&e->nd.v1up, nt));
  CKE(dalloc(&e->nd.v2, nt));
  CKE(dalloc(&e->cacc, nt));
  CKE(dalloc(&e->dacc, nt));
  CKE(dalloc(&e->vel_low1, 1));
  CKE(dalloc(&e->status, nsurf));
  CKE(dalloc(&e->lmax, nsurf));
  CKE(dalloc(&e->rnorm, nsurf));
  CKE(dalloc(&e->rslot, (long long)SFD_RSLOTS * nsurf));
  CKE(dalloc(&e->bnorm, nsurf));
  CKE(dalloc(&e->rrel, nsurf));
  CKE(dalloc(&e->extra_count, nsurf));
  CKE(dalloc(&e->inv_out, 5LL * nsurf));
  CKE(cudaMemset(e->status, 0, nsurf * sizeof(unsigned int)));
  CKE(cudaMemset(e->lmax, 0, nsurf * sizeof(double)));
  CKE(cudaMemset(e->rnorm, 0, nsurf * sizeof(double)));
  CKE(cudaMemset(e->rslot, 0, (size_t)SFD_RSLOTS * nsurf * sizeof(double)));
  CKE(cudaMemset(e->bnorm, 0, nsurf * sizeof(double)));
  CKE(cudaMemset(e->rrel, 0, nsurf * sizeof(double)));
  CKE(cudaMemset(e->extra_count, 0, nsurf * sizeof(unsigned long long)));
  if (e->opt.precision == SFD_PRECISION_MIXED) {
    CKE(dalloc(&e->warm, nsurf));
    CKE(cudaMemset(e->warm, 0x7F, nsurf * sizeof(double)));  // cold: no previous solve
    CKE(cudaHostAlloc(reinterpret_cast<void**>(&e->stall_host), sizeof(unsigned int), cudaHostAllocMapped));
    *e->stall_host = 0u;
    CKE(cudaHostGetDevicePointer(reinterpret_cast<void**>(&e->stall_dev), e->stall_host, 0));
  }
  CKE(cudaMemset(e->y0, 0, (long long)e->nblk * nt * sizeof(double)));
  CKE(cudaMemset(e->nd.p, 0, nt * sizeof(cd)));
  CKE(cudaMemset(e->nd.pdf, 0, nt * sizeof(float4)));
  CKE(cudaMemset(e->dacc, 0, nt * sizeof(cd)));
  if (e->opt.precision == SFD_PRECISION_FP64) {
    CKE(dalloc(&e->m64, e->mat_elems));
  } else {
    CKE(dalloc(&e->m32, e->mat_elems));
    if (e->opt.precond_half) {
      CKE(dalloc(&e->m16, e->mat_elems));
      CKE(dalloc(&e->rscale, nt));
      if (nsurf == 1 && e->nsm > 0 && e->hs[0].moff % 8 == 0 && sfd_gemv_stream_cap() > 0) {
        int smem_max = 0;
        CKE(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, e->device));
        sfd_gemv_stream_plan(e->hs[0].n, e->nsm, smem_max, sfd_gemv_stream_cap(), &e->gemv_spw, &e->gemv_smem);
        if (e->gemv_spw > 0) CKE(sfd_gemv_stream_configure(e->gemv_smem));
      }
    }
    CKE(dalloc(&e->pbuf, (long long)nsurf * 128 * 128));
    CKE(dalloc(&e->rbuf, e->panel_elems));
    CKE(dalloc(&e->cbuf, e->panel_elems));
    if (e->opt.tensor_cores) {
      CKE(dalloc(&e->cparts, 3 * e->panel_elems));
      CKE(dalloc(&e->rparts, 3 * e->panel_elems));
      CKE(sfd_tc_configure());
      CKE(sfd_tc_make_map(&e->tmap_c, e->cparts, e->panel_elems / 128, e->panel_elems));
      CKE(sfd_tc_make_map(&e->tmap_r, e->rparts, e->panel_elems / 128, e->panel_elems));
      {
        std::vector<sfd_engine::TensorMap> maps(nsurf);
        for (int s = 0; s < nsurf; ++s) CKE(sfd_tc_make_out_map(&maps[s], e->m32 + e->hs[s].moff, pad_n(e->hs[s].n)));
        CKE(dalloc(&e->d_tmap_out, nsurf));
        CKE(cudaMemcpy(e->d_tmap_out, maps.data(), nsurf * sizeof(sfd_engine::TensorMap), cudaMemcpyHostToDevice));
      }
      // row groups per tile column: a single surface spreads its columns'
      // rows over the SMs; a batch has columns enough
      long long cols = 0;
      int max_nt = 1;
      for (int s = 0; s < nsurf; ++s) {
        const int ntile = pad_n(e->hs[s].n) / 128;
        cols += std::max(1, ntile - 1);
        max_nt = std::max(max_nt, ntile);
      }
      e->tc_groups = cols >= e->nsm ? 1 : (int)std::max(1LL, std::min<long long>(max_nt, e->nsm / std::max(1LL, cols)));
    }
  }
  CKE(sfd_fft_configure());
  CKE(sfd_sums_configure());
  CKE(sfd_solve_configure());
#undef CKE
  *out = e;
  return 0;
}

int sfd_destroy(sfd_engine* e) {
  free_engine(e);
  return 0;
}

int sfd_set_problem(sfd_engine* e, int surface, const sfd_problem* problem) {
  if (!e || !problem || surface < 0 || surface >= e->nsurf) return set_error(SFD_ERR_INVALID, "invalid argument");
  SurfaceDesc S = e->hs[surface];
  int rc = fill_surface(S, *problem);
  if (rc) return rc;
  const SurfaceDesc& O = e->hs[surface];
  if (S.physics != O.physics || S.infinite_depth != O.infinite_depth || (S.physics == 0 && (S.rho != 0.0) != (O.rho != 0.0)))
    return set_error(SFD_ERR_INVALID, "sfd_set_problem: physics, depth mode and rho != 0 must not change");
  CK(cudaSetDevice(e->device));
  CK(cudaStreamSynchronize(e->stream));
  e->hs[surface] = S;
  CK(cudaMemcpy(e->d_surf + surface, &S, sizeof(SurfaceDesc), cudaMemcpyHostToDevice));
  return 0;
}

int sfd_get_tuning(const sfd_engine* e, int* g) {
  if (!e || !g) return set_error(SFD_ERR_INVALID, "null argument");
  for (int i = 0; i < 3; ++i) g[i] = e->sum_groups[i];
  return 0;
}

int sfd_set_stream(sfd_engine* e, void* st) {
  if (!e) return set_error(SFD_ERR_INVALID, "null engine");
  destroy_graphs(e);
  e->stream = st ? (cudaStream_t)st : e->own_stream;
  return 0;
}

int sfd_total_nodes(const sfd_engine* e) { return e ? e->ntot : 0; }

int sfd_set_state_host(sfd_engine* e, const double* x, const double* y, const double* phi) {
  if (!e || !x || !y || !phi) return set_error(SFD_ERR_INVALID, "null argument");
  CK(cudaSetDevice(e->device));
  size_t b = e->ntot * sizeof(double);
  CK(cudaMemcpyAsync(e->y0, x, b, cudaMemcpyHostToDevice, e->stream));
  CK(cudaMemcpyAsync(e->y0 + e->ntot, y, b, cudaMemcpyHostToDevice, e->stream));
  CK(cudaMemcpyAsync(e->y0 + 2 * e->ntot, phi, b, cudaMemcpyHostToDevice, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  return 0;
}

int sfd_get_state_host(sfd_engine* e, double* x, double* y, double* phi) {
  if (!e || !x || !y || !phi) return set_error(SFD_ERR_INVALID, "null argument");
  CK(cudaSetDevice(e->device));
  size_t b = e->ntot * sizeof(double);
  CK(cudaMemcpyAsync(x, e->y0, b, cudaMemcpyDeviceToHost, e->stream));
  CK(cudaMemcpyAsync(y, e->y0 + e->ntot, b, cudaMemcpyDeviceToHost, e->stream));
  CK(cudaMemcpyAsync(phi, e->y0 + 2 * e->ntot, b, cudaMemcpyDeviceToHost, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  return 0;
}

int sfd_set_aux_host(sfd_engine* e, const double* D) {
  if (!e || !D) return set_error(SFD_ERR_INVALID, "null argument");
  if (e->nblk != 4) return set_error(SFD_ERR_INVALID, "the engine has no delayed-intensity block (no augmented drive)");
  CK(cudaSetDevice(e->device));
  CK(cudaMemcpyAsync(e->y0 + 3LL * e->ntot, D, e->ntot * sizeof(double), cudaMemcpyHostToDevice, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  return 0;
}

int sfd_get_aux_host(sfd_engine* e, double* D) {
  if (!e || !D) return set_error(SFD_ERR_INVALID, "null argument");
  if (e->nblk != 4) return set_error(SFD_ERR_INVALID, "the engine has no delayed-intensity block (no augmented drive)");
  CK(cudaSetDevice(e->device));
  CK(cudaMemcpyAsync(D, e->y0 + 3LL * e->ntot, e->ntot * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  return 0;
}

int sfd_set_state_device(sfd_engine* e, const void* x, const void* y, const void* phi) {
  if (!e || !x || !y || !phi) return set_error(SFD_ERR_INVALID, "null argument");
  CK(cudaSetDevice(e->device));
  size_t b = e->ntot * sizeof(double);
  CK(cudaMemcpyAsync(e->y0, x, b, cudaMemcpyDeviceToDevice, e->stream));
  CK(cudaMemcpyAsync(e->y0 + e->ntot, y, b, cudaMemcpyDeviceToDevice, e->stream));
  CK(cudaMemcpyAsync(e->y0 + 2 * e->ntot, phi, b, cudaMemcpyDeviceToDevice, e->stream));
  return 0;
}

int sfd_get_state_device(sfd_engine* e, void* x, void* y, void* phi) {
  if (!e || !x || !y || !phi) return set_error(SFD_ERR_INVALID, "null argument");
  CK(cudaSetDevice(e->device));
  size_t b = e->ntot * sizeof(double);
  CK(cudaMemcpyAsync(x, e->y0, b, cudaMemcpyDeviceToDevice, e->stream));
  CK(cudaMemcpyAsync(y, e->y0 + e->ntot, b, cudaMemcpyDeviceToDevice, e->stream));
  CK(cudaMemcpyAsync(phi, e->y0 + 2 * e->ntot, b, cudaMemcpyDeviceToDevice, e->stream));
  return 0;
}

int sfd_state_device_ptr(sfd_engine* e, void** state) {
  if (!e || !state) return set_error(SFD_ERR_INVALID, "null argument");
  *state = e->y0;
  return 0;
}

int sfd_rhs_device(sfd_engine* e, const void* state_in, void* rhs_out) {
  if (!e || !state_in || !rhs_out) return set_error(SFD_ERR_INVALID, "null argument");
  CK(cudaSetDevice(e->device));
  return enqueue_rhs(e, (const double*)state_in, (double*)rhs_out, true);
}

int sfd_rhs_host(sfd_engine* e, double* dx, double* dy, double* dphi, double* a, double* zp, double* zpp) {
  if (!e || !dx || !dy || !dphi) return set_error(SFD_ERR_INVALID, "null argument");
  CK(cudaSetDevice(e->device));
  int rc = enqueue_rhs(e, e->y0, e->kcur, true);
  if (rc) return rc;
  size_t b = e->ntot * sizeof(double);
  CK(cudaMemcpyAsync(dx, e->kcur, b, cudaMemcpyDeviceToHost, e->stream));
  CK(cudaMemcpyAsync(dy, e->kcur + e->ntot, b, cudaMemcpyDeviceToHost, e->stream));
  CK(cudaMemcpyAsync(dphi, e->kcur + 2 * e->ntot, b, cudaMemcpyDeviceToHost, e->stream));
  if (a) CK(cudaMemcpyAsync(a, e->a, b, cudaMemcpyDeviceToHost, e->stream));
  if (zp) CK(cudaMemcpyAsync(zp, e->zp, 2 * b, cudaMemcpyDeviceToHost, e->stream));
  if (zpp) CK(cudaMemcpyAsync(zpp, e->zpp, 2 * b, cudaMemcpyDeviceToHost, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  return 0;
}

int sfd_rk4_steps_async(sfd_engine* e, double dt, int steps) {
  if (!e) return set_error(SFD_ERR_INVALID, "null engine");
  return run_steps(e, dt, steps);
}

int sfd_synchronize(sfd_engine* e) {
  if (!e) return set_error(SFD_ERR_INVALID, "null engine");
  CK(cudaSetDevice(e->device));
  CK(cudaStreamSynchronize(e->stream));
  if (e->profile) drain_profile(e);
  return 0;
}

int sfd_join_background(sfd_engine* e) {
  if (!e) return set_error(SFD_ERR_INVALID, "null engine");
  if (!e->bg.side) return 0;
  CK(cudaSetDevice(e->device));
  cudaEvent_t ev = nullptr;
  CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  cudaError_t err = cudaEventRecord(ev, e->bg.side);
  if (err == cudaSuccess) err = cudaStreamWaitEvent(e->stream, ev, 0);
  cudaEventDestroy(ev);
  CK(err);
  return 0;
}

int sfd_profile(sfd_engine* e, int enable) {
  if (!e) return set_error(SFD_ERR_INVALID, "null engine");
  CK(cudaSetDevice(e->device));
  CK(cudaStreamSynchronize(e->stream));
  drain_profile(e);
  e->profile = enable != 0;
  for (int i = 0; i < SFD_NCLASS; ++i) {
    e->class_ms[i] = 0.0;
    e->class_count[i] = 0;
  }
  return 0;
}

int sfd_profile_read(sfd_engine* e, double* ms, long long* counts, int nclass) {
  if (!e || !ms || !counts) return set_error(SFD_ERR_INVALID, "null argument");
  CK(cudaSetDevice(e->device));
  CK(cudaStreamSynchronize(e->stream));
  drain_profile(e);
  for (int i = 0; i < nclass && i < SFD_NCLASS; ++i) {
    ms[i] = e->class_ms[i];
    counts[i] = e->class_count[i];
  }
  return 0;
}

const char* sfd_profile_class_name(int cls) {
  static const char* names[SFD_NCLASS] = {"other", "spectral_deriv", "node_prep", "boundary_sums_fp64",
                                          "boundary_sums_df", "boundary_sums_fp32", "sum_epilogue", "assemble",
                                          "factor_diag", "factor_panel", "factor_update", "lu_trsv", "gemv",
                                          "velocity_bernoulli", "rk4_combine", "factor_update_tcgen05",
                                          "fft4_columns", "fft4_rows", "fft4_inverse_columns", "extra_corrections",
                                          "ap_redo", "ap_transform", "start_product"};
  return (cls >= 0 && cls < SFD_NCLASS) ? names[cls] : "";
}

int sfd_rk4_steps(sfd_engine* e, double dt, int steps) {
  int rc = sfd_rk4_steps_async(e, dt, steps);
  if (rc) return rc;
  return sfd_synchronize(e);
}

// The three state blocks between host arrays and the resident state, on the
// engine stream.
static cudaError_t copy_state_host(sfd_engine* e, double* x, double* y, double* phi, bool to_device) {
  const size_t b = (size_t)e->ntot * sizeof(double);
  if (y == x + e->ntot && phi == y + e->ntot)  // one [x | y | phi] buffer: one copy
    return to_device ? cudaMemcpyAsync(e->y0, x, 3 * b, cudaMemcpyHostToDevice, e->stream)
                     : cudaMemcpyAsync(x, e->y0, 3 * b, cudaMemcpyDeviceToHost, e->stream);
  double* h[3] = {x, y, phi};
  for (int k = 0; k < 3; ++k) {
    double* d = e->y0 + (size_t)k * e->ntot;
    const cudaError_t err = to_device ? cudaMemcpyAsync(d, h[k], b, cudaMemcpyHostToDevice, e->stream)
                                      : cudaMemcpyAsync(h[k], d, b, cudaMemcpyDeviceToHost, e->stream);
    if (err != cudaSuccess) return err;
  }
  return cudaSuccess;
}

int sfd_rk4_steps_host(sfd_engine* e, double* x, double* y, double* phi, double dt, int steps) {
  if (!e || !x || !y || !phi) return set_error(SFD_ERR_INVALID, "null argument");
  if (e->nblk != 3) return set_error(SFD_ERR_INVALID, "the engine carries a fourth state block: use the aux calls");
  if (steps < 0) return set_error(SFD_ERR_INVALID, "negative step count");
  if (!std::isfinite(dt)) return set_error(SFD_ERR_INVALID, "time step must be finite");
  CK(cudaSetDevice(e->device));
  // Once a copy is queued every exit waits for the stream, so that no copy
  // still reads or writes the caller's arrays when the call returns.
  cudaError_t err = copy_state_host(e, x, y, phi, true);
  int rc = err == cudaSuccess ? run_steps(e, dt, steps) : 0;
  if (err == cudaSuccess && rc == 0) err = copy_state_host(e, x, y, phi, false);
  const cudaError_t sync = cudaStreamSynchronize(e->stream);
  if (err != cudaSuccess) return set_error(SFD_ERR_CUDA, "sfd_rk4_steps_host: %s", cudaGetErrorString(err));
  if (rc) return rc;
  if (sync != cudaSuccess) return set_error(SFD_ERR_CUDA, "sfd_rk4_steps_host: %s", cudaGetErrorString(sync));
  return 0;
}

int sfd_invariants(sfd_engine* e, double kappa, double* out) {
  if (!e || !out) return set_error(SFD_ERR_INVALID, "null argument");
  CK(cudaSetDevice(e->device));
  int rc = enqueue_rhs(e, e->y0, e->kcur, true);
  if (rc) return rc;
  const int nt = e->ntot;
  LAUNCH(e, k_invariants<<<e->nsurf, 256, 0, e->stream>>>(e->d_surf, e->y0, e->y0 + nt, e->y0 + 2 * nt, e->zp, e->kcur,
                                                            e->kcur + nt, kappa, e->inv_out));
  CK(cudaMemcpyAsync(out, e->inv_out, 5 * e->nsurf * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  return 0;
}

int sfd_get_status(sfd_engine* e, unsigned int* status, double* lmax, double* rnorm) {
  if (!e) return set_error(SFD_ERR_INVALID, "null engine");
  CK(cudaSetDevice(e->device));
  CK(cudaStreamSynchronize(e->stream));
  if (status) CK(cudaMemcpy(status, e->status, e->nsurf * sizeof(unsigned int), cudaMemcpyDeviceToHost));
  if (lmax) CK(cudaMemcpy(lmax, e->lmax, e->nsurf * sizeof(double), cudaMemcpyDeviceToHost));
  if (rnorm) CK(cudaMemcpy(rnorm, e->rnorm, e->nsurf * sizeof(double), cudaMemcpyDeviceToHost));
  return 0;
}

int sfd_clear_status(sfd_engine* e) {
  if (!e) return set_error(SFD_ERR_INVALID, "null engine");
  CK(cudaSetDevice(e->device));
  CK(cudaMemsetAsync(e->status, 0, e->nsurf * sizeof(unsigned int), e->stream));
  CK(cudaMemsetAsync(e->lmax, 0, e->nsurf * sizeof(double), e->stream));
  CK(cudaMemsetAsync(e->rnorm, 0, e->nsurf * sizeof(double), e->stream));
  CK(cudaMemsetAsync(e->rrel, 0, e->nsurf * sizeof(double), e->stream));
  CK(cudaMemsetAsync(e->extra_count, 0, e->nsurf * sizeof(unsigned long long), e->stream));
  return 0;
}

int sfd_get_refinement(sfd_engine* e, double* rel_residual, long long* extra, long long* stall_rebuilds) {
  if (!e) return set_error(SFD_ERR_INVALID, "null engine");
  CK(cudaSetDevice(e->device));
  CK(cudaStreamSynchronize(e->stream));
  if (rel_residual) CK(cudaMemcpy(rel_residual, e->rrel, e->nsurf * sizeof(double), cudaMemcpyDeviceToHost));
  if (extra) CK(cudaMemcpy(extra, e->extra_count, e->nsurf * sizeof(long long), cudaMemcpyDeviceToHost));
  if (stall_rebuilds) *stall_rebuilds = e->stall_rebuilds;
  return 0;
}

long long sfd_kernel_launches(const sfd_engine* e) { return e ? e->launches : 0; }

}  // extern "C"

// ====================================================================== reference-compatible exports
namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kAlphaHamaker = 3.5e-24;  // constants.cuh:15
constexpr double kRhoHelium = 150.0;       // Export.cuh:82 default

struct NondimProps {
  double depth, rho, kappa, base_time, base_length, base_energy;
};

// adimensionalizeProperties (Export.cu:1222-1246) without the console output.
NondimProps adimensionalize(double L, double rho, double kappa, double depth) {
  NondimProps p;
  double base_length = L / (2.0 * kPi);
  double base_acc = 3 * kAlphaHamaker / std::pow(depth, 4);
  p.base_time = std::sqrt(base_length / base_acc);
  p.base_length = base_length;
  p.base_energy = 3.0 * kRhoHelium * kAlphaHamaker * std::pow(base_length, 4) / std::pow(depth, 4);
  double stf = kRhoHelium * base_length * base_length * base_length / (p.base_time * p.base_time);
  p.kappa = kappa / stf;
  p.depth = depth / base_length;
  p.rho = rho / kRhoHelium;
  return p;
}

sfd_problem helium_problem(const NondimProps& np, bool use_exp = false, int order = 1, bool inf = false) {
  sfd_problem p;
  sfd_default_problem(&p);
  p.physics = SFD_HELIUM;
  p.depth = np.depth;
  p.rho = np.rho;
  p.kappa = np.kappa;
  p.A3 = 0.0;  // the reference's fixed h^4 / 3
  p.use_expansions = use_exp ? 1 : 0;
  p.expansion_order = order;
  p.infinite_depth = inf ? 1 : 0;
  return p;
}

// Engines of the compatibility exports: eager launches, and no autotuning of
// the sum shape, so that repeated calls give bitwise the same results (the
// tuner keeps the fastest shape by timing, which sets the summation order).
int make_engine(int n, int batch, const sfd_problem& p, sfd_engine** e, const sfd_drive* drive = nullptr) {
  sfd_options o;
  sfd_default_options(&o);
  o.precision = g_default_precision;
  o.use_graphs = 0;
  o.autotune = 0;
  std::vector<int> ns(batch, n);
  return sfd_create_driven(ns.data(), batch, &p, drive, 1, &o, e);
}

constexpr double kHbar = 1.054571817e-34;  // constants.cuh:10

// adimensionalizeOptomechanicalVariables (Export.cu:1248-1270) and the
// instantaneous-intensity prefactor get_current_intensity_drive_strength
// (LightIntensity.cuh:34-37), for the augmented driven problem.
sfd_drive optomech_drive(const COptomechanicalVariables& v, const NondimProps& np) {
  sfd_drive d;
  std::memset(&d, 0, sizeof(d));
  d.gamma = v.gamma * np.base_time;
  d.detuning = v.detuning * np.base_time;
  d.G = v.G * np.base_time * np.base_length;
  d.tau = v.tau / np.base_time;
  d.x0 = v.location_x0_mode / np.base_length;
  d.sigma = v.sigma_optical_mode / np.base_length;
  const double hbar_adim = kHbar / np.base_energy / np.base_time;
  d.beta = v.beta * hbar_adim * d.G / d.tau / (d.sigma * d.sigma * np.rho);
  d.max_intensity = v.max_intensity;  // not rescaled by the reference either
  d.damping = v.damping_strength;
  d.strength = kHbar / (np.base_energy * np.base_time * np.rho) * d.G / (d.sigma * d.sigma);
  d.augmented = 1;
  return d;
}

int rhs_from_vectors(const double* x, const double* y, const double* phi, double* vx, double* vy, double* rhsPhi,
                     double L, double rho, double kappa, double depth, int n, int batch) {
  if (!x || !y || !phi || !vx || !vy || !rhsPhi) return set_error(SFD_ERR_INVALID, "null argument");
  sfd_engine* e = nullptr;
  int rc = make_engine(n, batch, helium_problem(adimensionalize(L, rho, kappa, depth)), &e);
  if (rc) return rc;
  rc = sfd_set_state_host(e, x, y, phi);
  if (!rc) rc = sfd_rhs_host(e, vx, vy, rhsPhi, nullptr, nullptr, nullptr);
  sfd_destroy(e);
  return rc;
}

}  // namespace

extern "C" {

int calculateRHSFromVectors(const double* x, const double* y, const double* phi, double* vx, double* vy,
                            double* rhsPhi, double L, double rho, double kappa, double depth, size_t N) {
  if (N < 1 || N > 8192) return set_error(SFD_ERR_INVALID, "unsupported particle number %zu (1..8192)", N);
  return rhs_from_vectors(x, y, phi, vx, vy, rhsPhi, L, rho, kappa, depth, (int)N, 1);
}

int calculateRHS256FromVectors(const double* x, const double* y, const double* phi, double* vx, double* vy,
                               double* rhsPhi, double L, double rho, double kappa, double depth) {
  return rhs_from_vectors(x, y, phi, vx, vy, rhsPhi, L, rho, kappa, depth, 256, 1);
}

int calculateRHS2048FromVectors(const double* x, const double* y, const double* phi, double* vx, double* vy,
                                double* rhsPhi, double L, double rho, double kappa, double depth) {
  return rhs_from_vectors(x, y, phi, vx, vy, rhsPhi, L, rho, kappa, depth, 2048, 1);
}

int calculateRHS256FromVectorsBatched(const double* x, const double* y, const double* phi, double* vx, double* vy,
                                      double* rhsPhi, double L, double rho, double kappa, double depth,
                                      int batchSize) {
  if (batchSize < 1) return set_error(SFD_ERR_INVALID, "unsupported batch size %d", batchSize);
  return rhs_from_vectors(x, y, phi, vx, vy, rhsPhi, L, rho, kappa, depth, 256, batchSize);
}

int calculateRHS256FromFile(const char* inputFile, const char* outputFile, double L, double rho, double kappa,
                            double depth) {
  // Export.cu:42-113: read a state file (y scaled by 2 pi / L), evaluate the
  // helium RHS at N = 256 and write it as a state file flagged rhs, with the
  // nondimensional properties and the amplitude (max y - min y) / 2.
  if (!inputFile || !outputFile) return set_error(SFD_ERR_INVALID, "null argument");
  const int n = 256;
  std::vector<std::complex<double>> Z;
  std::vector<double> phi;
  try {
    sfd::loadStateFile(inputFile, Z, phi, n, 2.0 * kPi / L);
  } catch (const std::exception& ex) {
    return set_error(SFD_ERR_INVALID, "calculateRHS256FromFile: %s: %s", inputFile, ex.what());
  }
  if (phi.size() != (size_t)n)
    return set_error(SFD_ERR_INVALID, "calculateRHS256FromFile: %s: potential holds %zu values, not %d", inputFile,
                     phi.size(), n);
  std::vector<double> x(n), y(n), vx(n), vy(n), dphi(n);
  for (int i = 0; i < n; ++i) {
    x[i] = Z[i].real();
    y[i] = Z[i].imag();
  }
  const auto mm = std::minmax_element(y.begin(), y.end());
  const double amplitude = (*mm.second - *mm.first) / 2.0;
  int rc = rhs_from_vectors(x.data(), y.data(), phi.data(), vx.data(), vy.data(), dphi.data(), L, rho, kappa, depth,
                            n, 1);
  if (rc) return rc;
  const NondimProps np = adimensionalize(L, rho, kappa, depth);
  std::vector<std::complex<double>> dz(n);
  for (int i = 0; i < n; ++i) dz[i] = {vx[i], vy[i]};
  try {
    sfd::saveStateFile(outputFile, dz, dphi, n, np.rho, np.kappa, 0.0, np.depth, amplitude, true);
  } catch (const std::exception& ex) {
    return set_error(SFD_ERR_INVALID, "calculateRHS256FromFile: %s: %s", outputFile, ex.what());
  }
  return 0;
}

int calculatePerturbedStates256(const double* x, const double* y, const double* phi, double* Zperturbed, double L,
                                double rho, double kappa, double depth, double epsilon) {
  // Export.cu:601-662 with JacobianCalculator.cuh:11-75 and :154-161: the 3N
  // states of the finite-difference Jacobian, each the complex state
  // [Z | Phi] = [x + i y | phi + 0 i] with one coordinate raised by epsilon.
  // Positions of perturbation b fill entries [b N, (b+1) N), potentials
  // [3N^2 + b N, 3N^2 + (b+1) N); b / N picks x, y or phi and b % N the node.
  // The output is a host array and the layout is a copy with one shifted
  // entry per block, so it is written on the host: a device pass would only
  // add the 6.3 MB copy back.  L, rho, kappa and depth are unused, as in the
  // reference.
  (void)L;
  (void)rho;
  (void)kappa;
  (void)depth;
  if (!x || !y || !phi || !Zperturbed) return set_error(SFD_ERR_INVALID, "null argument");
  constexpr size_t n = 256, m = 3 * n;
  double* pos = Zperturbed;
  double* pot = Zperturbed + 2 * m * n;
  for (size_t b = 0; b < m; ++b) {
    double* zp = pos + 2 * b * n;
    double* pp = pot + 2 * b * n;
    for (size_t t = 0; t < n; ++t) {
      zp[2 * t] = x[t];
      zp[2 * t + 1] = y[t];
      pp[2 * t] = phi[t];
      pp[2 * t + 1] = 0.0;
    }
    // the perturbed entry is the complex sum state + (eps, 0) or + (0, eps),
    // both parts added as the reference adds them (0.0 turns -0.0 into +0.0)
    const size_t j = b % n, c = b / n;
    double* e = c == 2 ? pp + 2 * j : zp + 2 * j;
    e[0] = e[0] + (c == 1 ? 0.0 : epsilon);
    e[1] = e[1] + (c == 1 ? epsilon : 0.0);
  }
  return 0;
}

int calculateVorticities256FromVectors(const double* Z, const double* phi, double* a, double* Zp, double* Zpp,
                                       double L, double rho, double kappa, double depth) {
  if (!Z || !phi || !a) return set_error(SFD_ERR_INVALID, "null argument");
  const int n = 256;
  sfd_engine* e = nullptr;
  int rc = make_engine(n, 1, helium_problem(adimensionalize(L, rho, kappa, depth)), &e);
  if (rc) return rc;
  std::vector<double> x(n), y(n), ph(n), phi_im(n), dx(n), dy(n), dp(n);
  for (int i = 0; i < n; ++i) {
    x[i] = Z[2 * i];
    y[i] = Z[2 * i + 1];
    ph[i] = phi[2 * i];
    phi_im[i] = phi[2 * i + 1];
  }
  bool imag = false;
  for (int i = 0; i < n; ++i) imag |= phi_im[i] != 0.0;
  rc = sfd_set_state_host(e, x.data(), y.data(), ph.data());
  if (!rc && imag) {
    // the reference transforms the complex phi as given (SimulationRunner.cuh:245-251)
    if (cudaMalloc(&e->phi_im, n * sizeof(double)) != cudaSuccess ||
        cudaMemcpy(e->phi_im, phi_im.data(), n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
      rc = set_error(SFD_ERR_CUDA, "phi_im upload failed");
  }
  if (!rc) rc = enqueue_solve(e, e->y0, e->phi_im, true);
  if (!rc) {
    cudaStreamSynchronize(e->stream);
    if (cudaMemcpy(a, e->a, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) rc = SFD_ERR_CUDA;
    if (!rc && Zp) cudaMemcpy(Zp, e->zp, n * sizeof(cd), cudaMemcpyDeviceToHost);
    if (!rc && Zpp) cudaMemcpy(Zpp, e->zpp, n * sizeof(cd), cudaMemcpyDeviceToHost);
  }
  sfd_destroy(e);
  return rc;
}

int calculateDerivativeFFT256(const double* input, double* output) {
  if (!input || !output) return set_error(SFD_ERR_INVALID, "null argument");
  const int n = 256;
  sfd_problem p;
  sfd_default_problem(&p);
  sfd_engine* e = nullptr;
  int rc = make_engine(n, 1, p, &e);
  if (rc) return rc;
  std::vector<double> re(n), im(n);
  for (int i = 0; i < n; ++i) {
    re[i] = input[2 * i];
    im[i] = input[2 * i + 1];
  }
  rc = sfd_set_state_host(e, re.data(), im.data(), re.data());
  if (!rc) {
    int2 job{0, SFD_JOB_RAW};
    int2* dj = nullptr;
    if (cudaMalloc(&dj, sizeof(int2)) != cudaSuccess) rc = SFD_ERR_CUDA;
    if (!rc) cudaMemcpy(dj, &job, sizeof(int2), cudaMemcpyHostToDevice);
    const int nt = e->ntot;
    DerivArgs D{e->d_surf, e->nsurf, e->y0, e->y0 + nt, e->y0 + 2 * nt, nullptr, e->a, e->zp, e->zpp, e->phip, e->ap, nullptr};
    if (!rc && sfd_launch_spectral(D, dj, 1, n, e->stream) != cudaSuccess) rc = SFD_ERR_CUDA;  // single-CTA job
    if (!rc) {
      cudaStreamSynchronize(e->stream);
      if (cudaMemcpy(output, e->ap, n * sizeof(cd), cudaMemcpyDeviceToHost) != cudaSuccess) rc = SFD_ERR_CUDA;
    }
    if (dj) cudaFree(dj);
    if (rc == SFD_ERR_CUDA) set_error(rc, "calculateDerivativeFFT256: CUDA failure");
  }
  sfd_destroy(e);
  return rc;
}

int integrateSimulationRK4(double* initialState, double** statesOut, size_t* statesCount, double** timesOut,
                           size_t* timesCount, SimProperties* sp, RK4SolverOptions* ro, size_t N) {
  if (!initialState || !statesOut || !statesCount || !timesOut || !timesCount || !sp || !ro)
    return set_error(SFD_ERR_INVALID, "null argument");
  if (N < 1 || N > 8192) return set_error(SFD_ERR_INVALID, "unsupported N %zu", N);
  NondimProps np = adimensionalize(sp->L, sp->rho, sp->kappa, sp->depth);
  // adimensionalizeRK4SolverOptions (Export.cu:1212-1219)
  double dt = ro->timeStep / np.base_time, t0 = ro->t0 / np.base_time, t1 = ro->t1 / np.base_time;
  if (!(dt > 0)) return set_error(SFD_ERR_INVALID, "timeStep must be > 0");
  size_t steps = (size_t)((t1 - t0) / dt);  // runEvolution (AutonomousRungeKuttaStepper.cuh:421)
  sfd_engine* e = nullptr;
  int rc = make_engine((int)N, 1, helium_problem(np, sp->use_expansions, sp->expansion_order, sp->infinite_depth), &e);
  if (rc) return rc;
  e->opt.use_graphs = 1;
  const size_t n3 = 3 * N;
  size_t nstates = ro->returnTrajectory ? steps + 1 : 1;
  double* states = (double*)std::malloc(nstates * n3 * sizeof(double));
  double* times = ro->returnTrajectory ? (double*)std::malloc(nstates * sizeof(double)) : nullptr;
  if (!states || (ro->returnTrajectory && !times)) {
    std::free(states);
    std::free(times);
    sfd_destroy(e);
    return set_error(SFD_ERR_INVALID, "host allocation failed");
  }
  rc = sfd_set_state_host(e, initialState, initialState + N, initialState + 2 * N);
  double t = t0;
  if (!rc && ro->returnTrajectory) {
    std::memcpy(states, initialState, n3 * sizeof(double));
    times[0] = t;
  }
  for (size_t s = 0; s < steps && !rc; ++s) {
    rc = sfd_rk4_steps_async(e, dt, 1);
    t += dt;
    if (!rc && ro->returnTrajectory) {
      double* dst = states + (s + 1) * n3;
      rc = sfd_get_state_host(e, dst, dst + N, dst + 2 * N);
      times[s + 1] = t;
    }
  }
  if (!rc && !ro->returnTrajectory) rc = sfd_get_state_host(e, states, states + N, states + 2 * N);
  sfd_destroy(e);
  if (rc) {
    std::free(states);
    std::free(times);
    return rc;
  }
  *statesOut = states;
  *statesCount = nstates;
  *timesOut = times;
  *timesCount = ro->returnTrajectory ? nstates : 0;
  return 0;
}

int integrateSimulationRK4_freeMemory(double* statesOut, double* timesOut) {
  std::free(statesOut);
  std::free(timesOut);
  return 0;
}

// integrateSimulationGL2 (Export.cu:665-738): helium (SI properties made
// nondimensional as the other exports), state and times nondimensional as the
// reference takes them, FP64 engine, GL2 options mapped one to one.
int integrateSimulationGL2(double* initialState, double** statesOut, size_t* statesCount, double** timesOut,
                           size_t* timesCount, SimProperties* sp, GaussLegendreOptions* gl, size_t N) {
  if (!initialState || !statesOut || !statesCount || !timesOut || !timesCount || !sp || !gl)
    return set_error(SFD_ERR_INVALID, "null argument");
  if (N < 1 || 6 * N > 8192) return set_error(SFD_ERR_INVALID, "unsupported N %zu (GL2 needs 6N <= 8192)", N);
  if (!(gl->stepSize > 0)) return set_error(SFD_ERR_INVALID, "Step size must be positive.");
  NondimProps np = adimensionalize(sp->L, sp->rho, sp->kappa, sp->depth);
  sfd_problem p = helium_problem(np, sp->use_expansions, sp->expansion_order, sp->infinite_depth);
  sfd_options o;
  sfd_default_options(&o);
  o.precision = SFD_PRECISION_FP64;
  o.use_graphs = 0;
  o.autotune = 0;
  int n = (int)N;
  sfd_engine* e = nullptr;
  int rc = sfd_create(&n, 1, &p, 1, &o, &e);
  if (rc) return rc;
  sfd_gl2_options go;
  sfd_default_gl2_options(&go);
  go.step = gl->stepSize;
  go.newton_tol = gl->newtonTolerance;
  go.max_newton = (long long)gl->maxNewtonIterations;
  go.allow_simplified = gl->allowSimplifiedFallback ? 1 : 0;
  go.armijo_c = gl->armijo_c;
  go.backtrack = gl->backtrack;
  go.min_alpha = gl->minAlpha;
  go.max_halvings = (long long)gl->maxStepsHalves;
  const size_t n3 = 3 * N;
  std::vector<double> T, Y;
  const bool traj = gl->returnTrajectory;
  if (traj) {
    T.push_back(gl->t0);
    Y.assign(initialState, initialState + n3);
  }
  rc = sfd_set_state_host(e, initialState, initialState + N, initialState + 2 * N);
  sfd_gl2_result r;
  if (!rc) rc = sfd_internal_gl2(e, gl->t0, gl->t1, go, r, traj ? &T : nullptr, traj ? &Y : nullptr);
  if (!rc && r.status != 0)
    rc = set_error(SFD_ERR_NUMERICS, "Gauss-Legendre 2nd Order method failed to converge at t=%g; residual=%.3e; last htry=%.3e",
                   r.t, r.residual, r.h);
  if (!rc && !traj) {
    Y.resize(n3);
    rc = sfd_get_state_host(e, Y.data(), Y.data() + N, Y.data() + 2 * N);
  }
  sfd_destroy(e);
  if (rc) return -1;
  double* states = (double*)std::malloc(Y.size() * sizeof(double) + 1);
  double* times = traj ? (double*)std::malloc(T.size() * sizeof(double) + 1) : nullptr;
  if (!states || (traj && !times)) {
    std::free(states);
    std::free(times);
    return set_error(SFD_ERR_INVALID, "host allocation failed");
  }
  std::memcpy(states, Y.data(), Y.size() * sizeof(double));
  if (traj) std::memcpy(times, T.data(), T.size() * sizeof(double));
  *statesOut = states;
  *statesCount = Y.size() / n3;
  *timesOut = times;
  *timesCount = traj ? T.size() : 0;
  return 0;
}

int integrateSimulationGL2_freeMemory(double* statesOut, double* timesOut) {
  std::free(statesOut);
  std::free(timesOut);
  return 0;
}

// calculateJacobian (Export.cu:393-519, JacobianCalculator.cuh:11-150):
// central differences of the helium RHS, J[col * 3N + row] = d rhs_row /
// d state_col (column-major, rows and columns ordered [x | y | phi]).  All
// perturbed copies of the state are surfaces of one batched FP64 engine
// (the reference batches them too); the batch is cut into chunks of at most
// kJacBatchBytes of matrix storage.
int calculateJacobian(const double* state, double* jac, double L, double rho, double kappa, double depth,
                      double epsilon, size_t N) {
  if (!state || !jac) return set_error(SFD_ERR_INVALID, "null argument");
  if (N < 1 || N > 8192) return set_error(SFD_ERR_INVALID, "unsupported N %zu", N);
  if (!(epsilon != 0.0)) return set_error(SFD_ERR_INVALID, "epsilon must be nonzero");
  constexpr double kJacBatchBytes = 8e9;
  const size_t n3 = 3 * N, np = (size_t)pad_n((int)N);
  const size_t per_var = 2 * 8 * np * np;  // +eps and -eps copies, FP64 matrices
  const size_t chunk = std::max<size_t>(1, std::min<size_t>(n3, (size_t)(kJacBatchBytes / (double)per_var)));
  NondimProps np_ = adimensionalize(L, rho, kappa, depth);
  sfd_problem p = helium_problem(np_);
  sfd_options o;
  sfd_default_options(&o);
  o.precision = SFD_PRECISION_FP64;
  o.use_graphs = 0;
  o.autotune = 0;
  std::vector<double> hx, hy, hp, dx, dy, dp;
  for (size_t c0 = 0; c0 < n3; c0 += chunk) {
    const size_t nc = std::min(chunk, n3 - c0), ns = 2 * nc;
    std::vector<int> sizes(ns, (int)N);
    sfd_engine* e = nullptr;
    int rc = sfd_create(sizes.data(), (int)ns, &p, 1, &o, &e);
    if (rc) return rc;
    hx.resize(ns * N);
    hy.resize(ns * N);
    hp.resize(ns * N);
    for (size_t b = 0; b < ns; ++b) {  // surface b: variable c0 + b % nc, sign + for b < nc
      std::memcpy(&hx[b * N], state, N * sizeof(double));
      std::memcpy(&hy[b * N], state + N, N * sizeof(double));
      std::memcpy(&hp[b * N], state + 2 * N, N * sizeof(double));
      const size_t var = c0 + b % nc, blk = var / N, j = var % N;
      const double d = b < nc ? epsilon : -epsilon;
      (blk == 0 ? hx : blk == 1 ? hy : hp)[b * N + j] += d;
    }
    dx.resize(ns * N);
    dy.resize(ns * N);
    dp.resize(ns * N);
    rc = sfd_set_state_host(e, hx.data(), hy.data(), hp.data());
    if (!rc) rc = sfd_rhs_host(e, dx.data(), dy.data(), dp.data(), nullptr, nullptr, nullptr);
    sfd_destroy(e);
    if (rc) return rc;
    for (size_t k = 0; k < nc; ++k) {
      double* col = jac + (c0 + k) * n3;
      const size_t bp = k * N, bm = (nc + k) * N;
      for (size_t r = 0; r < N; ++r) {
        col[r] = (dx[bp + r] - dx[bm + r]) / (2.0 * epsilon);
        col[N + r] = (dy[bp + r] - dy[bm + r]) / (2.0 * epsilon);
        col[2 * N + r] = (dp[bp + r] - dp[bm + r]) / (2.0 * epsilon);
      }
    }
  }
  return 0;
}

int calculateRhsAugmentedOptomechanical(double* state, double* rhs, SimProperties* sp, COptomechanicalVariables* ov,
                                        size_t N) {
  if (!state || !rhs || !sp || !ov) return set_error(SFD_ERR_INVALID, "null argument");
  if (N < 1 || N > 8192) return set_error(SFD_ERR_INVALID, "unsupported N %zu", N);
  NondimProps np = adimensionalize(sp->L, sp->rho, sp->kappa, sp->depth);
  sfd_drive d = optomech_drive(*ov, np);
  sfd_engine* e = nullptr;
  int rc = make_engine((int)N, 1, helium_problem(np, sp->use_expansions, sp->expansion_order, sp->infinite_depth),
                       &e, &d);
  if (rc) return rc;
  const size_t n4 = 4 * N;
  rc = sfd_set_state_host(e, state, state + N, state + 2 * N);
  if (!rc) rc = sfd_set_aux_host(e, state + 3 * N);
  if (!rc) rc = sfd_rhs_device(e, e->y0, e->kcur);
  if (!rc) {
    cudaError_t err = cudaMemcpyAsync(rhs, e->kcur, n4 * sizeof(double), cudaMemcpyDeviceToHost, e->stream);
    if (err == cudaSuccess) err = cudaStreamSynchronize(e->stream);
    if (err != cudaSuccess) rc = sfd_fail(err);
  }
  sfd_destroy(e);
  return rc;
}

int integrateAugmentedOptomechanicalSimulationRK4(double* initialState, double** statesOut, size_t* statesCount,
                                                  double** timesOut, size_t* timesCount, SimProperties* sp,
                                                  RK4SolverOptions* ro, COptomechanicalVariables* ov, size_t N) {
  if (!initialState || !statesOut || !statesCount || !timesOut || !timesCount || !sp || !ro || !ov)
    return set_error(SFD_ERR_INVALID, "null argument");
  if (N < 1 || N > 8192) return set_error(SFD_ERR_INVALID, "unsupported N %zu", N);
  NondimProps np = adimensionalize(sp->L, sp->rho, sp->kappa, sp->depth);
  sfd_drive d = optomech_drive(*ov, np);
  double dt = ro->timeStep / np.base_time, t0 = ro->t0 / np.base_time, t1 = ro->t1 / np.base_time;
  if (!(dt > 0)) return set_error(SFD_ERR_INVALID, "timeStep must be > 0");
  size_t steps = (size_t)((t1 - t0) / dt);  // runEvolution (AutonomousRungeKuttaStepper.cuh:421)
  sfd_engine* e = nullptr;
  int rc = make_engine((int)N, 1, helium_problem(np, sp->use_expansions, sp->expansion_order, sp->infinite_depth),
                       &e, &d);
  if (rc) return rc;
  e->opt.use_graphs = 1;
  const size_t n4 = 4 * N;
  size_t nstates = ro->returnTrajectory ? steps + 1 : 1;
  double* states = (double*)std::malloc(nstates * n4 * sizeof(double));
  double* times = ro->returnTrajectory ? (double*)std::malloc(nstates * sizeof(double)) : nullptr;
  if (!states || (ro->returnTrajectory && !times)) {
    std::free(states);
    std::free(times);
    sfd_destroy(e);
    return set_error(SFD_ERR_INVALID, "host allocation failed");
  }
  rc = sfd_set_state_host(e, initialState, initialState + N, initialState + 2 * N);
  if (!rc) rc = sfd_set_aux_host(e, initialState + 3 * N);
  double t = t0;
  if (!rc && ro->returnTrajectory) {
    std::memcpy(states, initialState, n4 * sizeof(double));
    times[0] = t;
  }
  auto fetch = [&](double* dst) {
    int r = sfd_get_state_host(e, dst, dst + N, dst + 2 * N);
    return r ? r : sfd_get_aux_host(e, dst + 3 * N);
  };
  for (size_t s = 0; s < steps && !rc; ++s) {
    rc = sfd_rk4_steps_async(e, dt, 1);
    t += dt;
    if (!rc && ro->returnTrajectory) {
      rc = fetch(states + (s + 1) * n4);
      times[s + 1] = t;
    }
  }
  if (!rc && !ro->returnTrajectory) rc = fetch(states);
  sfd_destroy(e);
  if (rc) {
    std::free(states);
    std::free(times);
    return rc;
  }
  *statesOut = states;
  *statesCount = nstates;
  *timesOut = times;
  *timesCount = ro->returnTrajectory ? nstates : 0;
  return 0;
}

int integrateAugmentedOptomechanicalSimulationRK4_freeMemory(double* statesOut, double* timesOut) {
  std::free(statesOut);
  std::free(timesOut);
  return 0;
}

}  // extern "C"

// ====================================================================== no-allocation RHS
// sfd_rhs_device_noalloc: one FP64 RHS evaluation of a single surface for
// callers that cannot call cudaMalloc (code running where the device memory
// is owned by someone else: inside another framework's allocator, a real-time
// loop that must not allocate after start-up, or a host that forbids runtime
// allocation).  All scratch lives in the file-scope array below; the caller
// passes only the state and the output.
namespace noalloc {
constexpr int kMaxN = 1024;  // stated maximum surface size
constexpr size_t align256(size_t b) { return (b + 255) & ~size_t(255); }
constexpr int kMaxItems = (kMaxN + kSumTile - 1) / kSumTile;
constexpr int kMaxTiles = (kMaxN / 64) * (kMaxN / 64);
constexpr size_t kBytes = align256(8ull * kMaxN * kMaxN)            // FP64 matrix (kMaxN is a multiple of 128)
                          + 13 * align256(16ull * kMaxN)            // complex node arrays, twiddles, df copies
                          + 5 * align256(8ull * kMaxN)              // real node arrays
                          + align256(4ull * kMaxN)                  // node -> surface map
                          + align256(sizeof(SurfaceDesc)) + 2 * align256(4 * sizeof(int2)) +
                          align256(kMaxItems * sizeof(int2)) + align256(kMaxTiles * sizeof(int4)) + align256(16) +
                          align256(4) + 2 * align256(8);
constexpr int kMaxDevices = 64;
}  // namespace noalloc

// About 8.7 MB; every GPU that loads the library keeps it until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[noalloc::kBytes];

namespace {

struct Bump {
  unsigned char* p;
  template <typename T>
  T* take(size_t count) {
    T* r = reinterpret_cast<T*>(p);
    p += noalloc::align256(count * sizeof(T));
    return r;
  }
};

// Device address of g_noalloc_scratch for the current device (resolved once
// per device, with that device current).
int noalloc_base(unsigned char** out) {
  static void* addr[noalloc::kMaxDevices] = {};
  static std::mutex mu;
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return sfd_fail(err);
  if (dev < 0 || dev >= noalloc::kMaxDevices) return set_error(SFD_ERR_INVALID, "device %d out of range", dev);
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* a = nullptr;
    err = cudaGetSymbolAddress(&a, g_noalloc_scratch);
    if (err != cudaSuccess) return set_error(SFD_ERR_CUDA, "cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(err));
    err = sfd_solve_configure();  // dynamic shared-memory limits of the FP64 LU kernels
    if (err != cudaSuccess) return sfd_fail(err);
    addr[dev] = a;
  }
  *out = static_cast<unsigned char*>(addr[dev]);
  return 0;
}

}  // namespace

// Descriptors of the allocation-free call, written on the device by one
// kernel from values passed by value (the twiddles travel in the kernel
// parameters, 16 KB at the 1024-node maximum), so the call issues no host to
// device copy.
struct NoallocSetup {
  SurfaceDesc S;  // S.tw already points into the scratch
  int n, np, nitems, ntiles;
  cd tw[noalloc::kMaxN];
};
static_assert(sizeof(NoallocSetup) < 32000, "kernel parameters are limited to 32 KB");

__global__ void k_noalloc_setup(const __grid_constant__ NoallocSetup P, SurfaceDesc* d_surf, cd* tw, int2* jobs_first,
                                int2* jobs_ap, int2* items, int4* tiles, int* node_surf, unsigned int* status,
                                double* lmax, double* rnorm) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0) {
    *d_surf = P.S;
    jobs_first[0] = make_int2(0, SFD_JOB_ZP);
    jobs_first[1] = make_int2(0, SFD_JOB_ZPP);
    jobs_first[2] = make_int2(0, SFD_JOB_PHIP);
    jobs_ap[0] = make_int2(0, SFD_JOB_AP);
    *status = 0u;
    *lmax = 0.0;
    *rnorm = 0.0;
  }
  if (t < P.n) {
    tw[t] = P.tw[t];
    node_surf[t] = 0;
  }
  if (t < P.nitems) items[t] = make_int2(0, t * kSumTile);
  if (t < P.ntiles) {
    const int per_row = P.np / 64;
    tiles[t] = make_int4(0, (t / per_row) * 64, (t % per_row) * 64, 0);
  }
}

extern "C" int sfd_rhs_device_noalloc(const sfd_problem* problem, int n, const void* state_in, void* rhs_out,
                                      void* stream) {
  if (!problem || !state_in || !rhs_out) return set_error(SFD_ERR_INVALID, "sfd_rhs_device_noalloc: null argument");
  if (n < 1 || n > noalloc::kMaxN)
    return set_error(SFD_ERR_INVALID,
                     "sfd_rhs_device_noalloc: n = %d is outside 1..%d, the size of its static scratch; use an engine "
                     "(sfd_create) for larger surfaces",
                     n, noalloc::kMaxN);
  unsigned char* base = nullptr;
  int rc = noalloc_base(&base);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int np = pad_n(n);

  // host-side descriptors (host memory only; the same radices and twiddles as
  // an engine's, from the same functions)
  static_assert(std::is_trivially_copyable<NoallocSetup>::value, "passed by value to a kernel");
  NoallocSetup P;
  std::memset(&P, 0, sizeof(P));
  SurfaceDesc& S = P.S;
  rc = fill_surface(S, *problem);
  if (rc) return rc;
  S.n = n;
  S.off = 0;
  S.moff = 0;
  std::vector<int> rad;
  if (!factorize(n, rad))
    return set_error(SFD_ERR_INVALID, "sfd_rhs_device_noalloc: n = %d has too many factors", n);
  S.nrad = (int)rad.size();
  for (size_t i = 0; i < rad.size(); ++i) S.rad[i] = rad[i];
  const std::vector<cd> tw = twiddles(n);
  std::memcpy(P.tw, tw.data(), n * sizeof(cd));
  P.n = n;
  P.np = np;
  P.nitems = (n + kSumTile - 1) / kSumTile;
  P.ntiles = (np / 64) * (np / 64);

  // carve the static scratch (same order as its size computation)
  Bump b{base};
  sfd_engine e;  // on the stack; owns nothing (its containers stay empty)
  e.m64 = b.take<double>((size_t)noalloc::kMaxN * noalloc::kMaxN);
  e.zp = b.take<cd>(noalloc::kMaxN);
  e.zpp = b.take<cd>(noalloc::kMaxN);
  e.ap = b.take<cd>(noalloc::kMaxN);
  e.nd.w = b.take<cd>(noalloc::kMaxN);
  e.nd.p = b.take<cd>(noalloc::kMaxN);
  e.nd.wdf = b.take<float4>(noalloc::kMaxN);
  e.nd.pdf = b.take<float4>(noalloc::kMaxN);
  e.nd.v1low = b.take<cd>(noalloc::kMaxN);
  e.nd.v1up = b.take<cd>(noalloc::kMaxN);
  e.nd.v2 = b.take<cd>(noalloc::kMaxN);
  e.cacc = b.take<cd>(noalloc::kMaxN);
  e.dacc = b.take<cd>(noalloc::kMaxN);
  cd* d_tw = b.take<cd>(noalloc::kMaxN);
  e.phip = b.take<double>(noalloc::kMaxN);
  e.a = b.take<double>(noalloc::kMaxN);
  e.r = b.take<double>(noalloc::kMaxN);
  e.delta = b.take<double>(noalloc::kMaxN);
  e.nd.mdiag = b.take<double>(noalloc::kMaxN);
  e.d_node_surf = b.take<int>(noalloc::kMaxN);
  e.d_surf = b.take<SurfaceDesc>(1);
  e.d_jobs_first = b.take<int2>(4);
  e.d_jobs_ap = b.take<int2>(4);
  e.d_sum_items = b.take<int2>(noalloc::kMaxItems);
  e.d_asm_tiles = b.take<int4>(noalloc::kMaxTiles);
  e.vel_low1 = b.take<cd>(1);
  e.status = b.take<unsigned int>(1);
  e.lmax = b.take<double>(1);
  e.rnorm = b.take<double>(1);
  if ((size_t)(b.p - base) > noalloc::kBytes) return set_error(SFD_ERR_INVALID, "scratch layout overflow");
  S.tw = d_tw;

  // descriptors on the device, then the evaluation, all on `stream`
  const int setup_threads = std::max(n, P.ntiles);
  k_noalloc_setup<<<(setup_threads + 255) / 256, 256, 0, st>>>(P, e.d_surf, d_tw, e.d_jobs_first, e.d_jobs_ap,
                                                               e.d_sum_items, e.d_asm_tiles, e.d_node_surf, e.status,
                                                               e.lmax, e.rnorm);
  CK(cudaGetLastError());
  CK(cudaGetDevice(&e.device));
  e.stream = st;
  sfd_default_options(&e.opt);
  e.opt.precision = SFD_PRECISION_FP64;
  e.opt.use_graphs = 0;
  e.opt.refine_iters = 0;
  e.opt.pre_iters = 0;
  e.opt.extra_iters = 0;
  e.nsurf = 1;
  e.ntot = n;
  e.max_n = n;
  e.max_n_single = n;
  e.max_np = np;
  e.njobs_first = 3;
  e.njobs_ap = 1;
  e.nsum = P.nitems;
  e.nasm = P.ntiles;
  e.any_rho = (S.physics == 0 && S.rho != 0.0);
  return enqueue_rhs(&e, static_cast<const double*>(state_in), static_cast<double*>(rhs_out), true);
}
