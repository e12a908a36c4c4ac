// sfd_rkf45.cu -- adaptive Runge-Kutta-Fehlberg 4(5) on the engine state
// (RK45Base / RK45_std_complex, RK45.cuh:195-406, RK45_Kernels.cuh:15-106).
//
// Fehlberg's 1969 tableau; the fifth-order solution is kept and the error is
// h sum (b - b*) k.  The error norm runs over the complex state entries the
// reference integrates (z = x + i y per node, then phi, then the delayed
// intensity D of an augmented drive):
//   err = sqrt(mean_entries(|e|^2 / (atol + rtol max(|y|, |y5|))^2)),
// reduced in a fixed order (per-block partials, then one block), so runs are
// bitwise repeatable.  Step control on the host after each trial step (one
// 8-byte read): factor 0.9 err^(-1/5) clamped to [0.2, 5] on acceptance and
// [0.2, 1] on rejection, then to [h_min, h_max]; k1 is reused after a
// rejection; the step is cut to the remaining interval.
#include <algorithm>
#include <cmath>

#include "sfd_internal.cuh"

namespace {

constexpr double kA[6][5] = {{0, 0, 0, 0, 0},
                             {1.0 / 4.0, 0, 0, 0, 0},
                             {3.0 / 32.0, 9.0 / 32.0, 0, 0, 0},
                             {1932.0 / 2197.0, -7200.0 / 2197.0, 7296.0 / 2197.0, 0, 0},
                             {439.0 / 216.0, -8.0, 3680.0 / 513.0, -845.0 / 4104.0, 0},
                             {-8.0 / 27.0, 2.0, -3544.0 / 2565.0, 1859.0 / 4104.0, -11.0 / 40.0}};
constexpr double kB[6] = {16.0 / 135.0, 0.0, 6656.0 / 12825.0, 28561.0 / 56430.0, -9.0 / 50.0, 2.0 / 55.0};
constexpr double kBs[6] = {25.0 / 216.0, 0.0, 1408.0 / 2565.0, 2197.0 / 4104.0, -1.0 / 5.0, 0.0};
constexpr int kRkfThreads = 256;
constexpr int kRkfErrBlocks = 304;  // 2 per SM on GB300; partial sums reduced in order afterwards

struct Ks {
  const double* k[6];
  double c[6];
};

// out = y + sum_{j < count} c_j k_j (left to right, as the reference's lincomb)
__global__ void k_rkf_stage(long long n, const double* __restrict__ y, Ks K, int count, double* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v = y[i];
  for (int j = 0; j < count; ++j) v += K.c[j] * K.k[j][i];
  out[i] = v;
}

// y5 = y + sum (h b_j) k_j; e = sum (h d_j) k_j; partial[block] = sum over
// this block's entries of (|e| / sc)^2.  Entry q < nt: z_q = (x_q, y_q);
// entry q >= nt: the real block q / nt + 1 (phi, then D).
__global__ void __launch_bounds__(kRkfThreads) k_rkf_error(int nt, int nblk, const double* __restrict__ y,
                                                            Ks Kb, Ks Kd, double atol, double rtol,
                                                            double* __restrict__ y5, double* __restrict__ partial) {
  __shared__ double red[kRkfThreads];
  const long long nent = (long long)(nblk - 1) * nt;
  double acc = 0.0;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nent; q += (long long)gridDim.x * blockDim.x) {
    const int ncomp = q < nt ? 2 : 1;
    double e2 = 0.0, y2 = 0.0, y52 = 0.0;
    for (int c = 0; c < ncomp; ++c) {
      const long long idx = q < nt ? q + (long long)c * nt : q + nt;  // (x, y) or block q / nt + 1
      double v5 = y[idx], ev = 0.0;
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        const double kj = Kb.k[j][idx];
        v5 += Kb.c[j] * kj;
        ev += Kd.c[j] * kj;
      }
      y5[idx] = v5;
      e2 += ev * ev;
      y2 += y[idx] * y[idx];
      y52 += v5 * v5;
    }
    double sc = atol + rtol * fmax(sqrt(y2), sqrt(y52));
    sc = fmax(sc, 1e-300);
    acc += e2 / (sc * sc);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kRkfThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void k_rkf_error_sum(int nparts, const double* partial, double* out) {
  __shared__ double red[kRkfThreads];
  double v = 0.0;
  for (int i = threadIdx.x; i < nparts; i += kRkfThreads) v += partial[i];
  red[threadIdx.x] = v;
  __syncthreads();
  for (int s = kRkfThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

}  // namespace

struct RkfWork {
  long long n = 0;
  double* k[6] = {};
  double *tmp = nullptr, *y5 = nullptr, *partial = nullptr, *err = nullptr;
  double* h_err = nullptr;  // pinned host copy of the error sum
};

void sfd_rkf45_free(sfd_engine* e) {
  if (!e || !e->rkf) return;
  RkfWork* W = e->rkf;
  for (double* p : W->k) cudaFree(p);
  cudaFree(W->tmp);
  cudaFree(W->y5);
  cudaFree(W->partial);
  cudaFree(W->err);
  if (W->h_err) cudaFreeHost(W->h_err);
  delete W;
  e->rkf = nullptr;
}

#define RCK(expr)                                                  \
  do {                                                             \
    cudaError_t _e = (expr);                                       \
    if (_e != cudaSuccess) return sfd_internal_cuda(_e, #expr);    \
  } while (0)

extern "C" void sfd_default_rkf45_options(sfd_rkf45_options* o) {
  if (!o) return;
  o->atol = 1e-6;  // RK45_Options (RK45.cuh:21-27)
  o->rtol = 1e-3;
  o->h_min = 1e-16;
  o->h_max = 1e10;
  o->h0 = 1e-2;
  o->max_rejected = 500;  // RK45Base::maxRejectedSteps
}

extern "C" int sfd_rkf45_evolve(sfd_engine* e, double t0, double t1, const sfd_rkf45_options* opt,
                                sfd_rkf45_result* res, double* times, long long cap) {
  if (!e || !opt || !res) return sfd_internal_error(SFD_ERR_INVALID, "null argument");
  if (!std::isfinite(t0) || !std::isfinite(t1)) return sfd_internal_error(SFD_ERR_INVALID, "t0 and t1 must be finite");
  if (!(opt->h0 > 0) || !std::isfinite(opt->h0)) return sfd_internal_error(SFD_ERR_INVALID, "h0 must be finite and > 0");
  RCK(cudaSetDevice(e->device));
  const long long n = (long long)e->nblk * e->ntot;
  if (!e->rkf) {
    RkfWork* W = e->rkf = new RkfWork();
    W->n = n;
    for (auto& p : W->k) RCK(cudaMalloc(&p, sizeof(double) * n));
    RCK(cudaMalloc(&W->tmp, sizeof(double) * n));
    RCK(cudaMalloc(&W->y5, sizeof(double) * n));
    RCK(cudaMalloc(&W->partial, sizeof(double) * kRkfErrBlocks));
    RCK(cudaMalloc(&W->err, sizeof(double)));
    RCK(cudaMallocHost(&W->h_err, sizeof(double)));
  }
  RkfWork* W = e->rkf;
  cudaStream_t s = e->stream;
  const int nb = (int)((n + kRkfThreads - 1) / kRkfThreads);
  const bool mixed = e->opt.precision == SFD_PRECISION_MIXED;
  const long long every = std::max(1, e->opt.refactor_every);
  const double nent = (double)(e->nblk - 1) * e->ntot;
  double t = t0, h = opt->h0;
  bool have_k1 = false;
  long long acc = 0, rej = 0;
  int status = 0;
  while (t < t1) {
    if (t1 - t < h) h = t1 - t;
    long long rej_here = 0;
    for (;;) {
      if (!have_k1) {  // the first stage of an accepted state may rebuild the preconditioner
        const bool refactor = !mixed || (e->step_count % every) == 0;
        int rc = sfd_internal_rhs_ex(e, e->y0, W->k[0], refactor);
        if (rc) return rc;
        have_k1 = true;
      }
      for (int st = 1; st < 6; ++st) {
        Ks K{};
        for (int j = 0; j < st; ++j) {
          K.k[j] = W->k[j];
          K.c[j] = kA[st][j] * h;
        }
        k_rkf_stage<<<nb, kRkfThreads, 0, s>>>(n, e->y0, K, st, W->tmp);
        RCK(cudaGetLastError());
        int rc = sfd_internal_rhs_ex(e, W->tmp, W->k[st], false);
        if (rc) return rc;
      }
      Ks Kb{}, Kd{};
      for (int j = 0; j < 6; ++j) {
        Kb.k[j] = Kd.k[j] = W->k[j];
        Kb.c[j] = h * kB[j];
        Kd.c[j] = h * (kB[j] - kBs[j]);
      }
      k_rkf_error<<<kRkfErrBlocks, kRkfThreads, 0, s>>>(e->ntot, e->nblk, e->y0, Kb, Kd, opt->atol, opt->rtol,
                                                        W->y5, W->partial);
      k_rkf_error_sum<<<1, kRkfThreads, 0, s>>>(kRkfErrBlocks, W->partial, W->err);
      RCK(cudaGetLastError());
      RCK(cudaMemcpyAsync(W->h_err, W->err, sizeof(double), cudaMemcpyDeviceToHost, s));
      RCK(cudaStreamSynchronize(s));
      const double err = std::sqrt(*W->h_err / nent);
      const bool ok = err <= 1.0;
      double fac, hn;
      if (err == 0.0) {
        fac = ok ? 5.0 : 1.0;
        hn = h * fac;
      } else if (!(err == err)) {  // NaN: treat as a rejection with the largest cut
        fac = 0.2;
        hn = std::min(std::max(h * fac, opt->h_min), opt->h_max);
      } else {
        fac = 0.9 * std::pow(err, -0.2);
        fac = std::min(std::max(fac, 0.2), ok ? 5.0 : 1.0);
        hn = std::min(std::max(h * fac, opt->h_min), opt->h_max);
      }
      if (ok) {
        RCK(cudaMemcpyAsync(e->y0, W->y5, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        have_k1 = false;
        t += h;
        if (times && acc < cap) times[acc] = t;
        ++acc;
        e->step_count++;
        h = hn;
        break;
      }
      h = hn;
      ++rej;
      if (++rej_here > opt->max_rejected) {
        status = 1;  // OdeSolverResult::StiffnessDetected
        break;
      }
    }
    if (status) break;
  }
  RCK(cudaStreamSynchronize(s));
  res->status = status;
  res->accepted = acc;
  res->rejected = rej;
  res->t = t;
  res->h = h;
  return 0;
}
