// sfd_gl2.cu -- implicit two-stage Gauss-Legendre (order 4) on the engine
// state (GaussLegendre2, GaussLegendre.cuh:216-605; GLCoefficients.hpp:5-17).
//
// Per step of size h the stage slopes k = (k1, k2) solve
//   R_i(k) = k_i - f(y + h sum_j A_ij k_j) = 0,   i = 1, 2,
// by damped Newton from k1 = k2 = f(y):
//   [delta_ij I - h A_ij J(y_i)] d = -R,  then an Armijo backtracking line
//   search on phi = |R|^2 / 2 (target phi(k) - c alpha |R(k)|^2),
// converged when |R| <= tol (1 + |k|) (2-norms over both stages).  A step
// whose Newton iteration fails is halved up to max_halvings times, down to
// hmin = |t1 - t0| / 2^20; the last accepted step size carries over.
//
// GB300 layout: the two stage states are the two surfaces of one batched
// FP64 engine ("stage" engine, state [x(2n) | y(2n) | phi(2n)], stage s at
// offset s n of each block), so both stage RHS evaluations are one pass; k,
// R and the Newton unknowns use that same interleaved layout, so R = k - f
// is elementwise.  The stage Jacobians are central differences over a
// batched FP64 engine of perturbed stage states (2 x 6n surfaces, chunked to
// a bounded matrix footprint; JacobianCalculator.cuh:223-284), or the exact
// reverse-mode Jacobian.  The 6n x 6n Newton matrix is assembled by a tiled
// transpose kernel straight into the dense solver's padded row-major storage
// and factored by the FP64 blocked LU.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "sfd_internal.cuh"
#include "sfd_solve.cuh"

namespace {

constexpr double kSq3 = 1.7320508075688772935;
constexpr double kA11 = 0.25, kA12 = 0.25 - kSq3 / 6.0, kA21 = 0.25 + kSq3 / 6.0, kA22 = 0.25;
constexpr double kB1 = 0.5, kB2 = 0.5;
constexpr int kT = 256;
constexpr double kFdChunkBytes = 8e9;  // FP64 matrix storage of one FD engine
constexpr int kExactMinN = 384;        // SFD_GL2_JACOBIAN_AUTO: exact Jacobian from this n up

inline int nbl(long long n, int t) { return (int)((n + t - 1) / t); }

// y (one surface, 3n) -> both surfaces of the stage layout
__global__ void k_gl2_broadcast(int n, const double* __restrict__ y, double* __restrict__ st) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= 3 * n) return;
  const int blk = v / n, p = v - blk * n;
  const double val = y[v];
  st[blk * 2 * n + p] = val;
  st[blk * 2 * n + n + p] = val;
}

// kt = k + alpha d (when d is given, else kt = k), then the stage states
// y_s = y + h (A_s1 kt_1 + A_s2 kt_2), one thread per state variable.
__global__ void k_gl2_stage(int n, double h, const double* __restrict__ y, const double* __restrict__ k,
                            const double* __restrict__ d, double alpha, double* __restrict__ kt,
                            double* __restrict__ st) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= 3 * n) return;
  const int blk = v / n, p = v - blk * n;
  const int i0 = blk * 2 * n + p, i1 = i0 + n;
  double k0 = k[i0], k1 = k[i1];
  if (d) {
    k0 = k0 + alpha * d[i0];
    k1 = k1 + alpha * d[i1];
    kt[i0] = k0;
    kt[i1] = k1;
  }
  const double yv = y[v];
  st[i0] = yv + h * (kA11 * k0 + kA12 * k1);
  st[i1] = yv + h * (kA21 * k0 + kA22 * k1);
}

// R = k - f over the 6n stage entries; red = [|R|^2, |k|^2] (one block,
// fixed-order tree, so the norms are bitwise repeatable).
constexpr int kRedT = 1024;
__global__ void __launch_bounds__(kRedT) k_gl2_residual(int m, const double* __restrict__ k,
                                                        const double* __restrict__ f, double* __restrict__ R,
                                                        double* __restrict__ red) {
  __shared__ double s1[kRedT], s2[kRedT];
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < m; i += kRedT) {
    const double kv = k[i], r = kv - f[i];
    R[i] = r;
    a += r * r;
    b += kv * kv;
  }
  s1[threadIdx.x] = a;
  s2[threadIdx.x] = b;
  __syncthreads();
  for (int s = kRedT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      s1[threadIdx.x] += s1[threadIdx.x + s];
      s2[threadIdx.x] += s2[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    red[0] = s1[0];
    red[1] = s2[0];
  }
}

// Newton matrix in the stage layout, padded row-major (np x np, identity
// padding): M[i][j] = delta_ij - h A[s_i][s_j] J_{s_i}[v_i][v_j], with the
// column-major Jacobians J_s[v_i + v_j 3n].  32 x 32 tiles through shared
// memory: reads run along v_i (contiguous in J), writes along j.
__global__ void __launch_bounds__(256) k_gl2_newton_matrix(int n, int np, double h, const double* __restrict__ J0,
                                                           const double* __restrict__ J1, double* __restrict__ M) {
  __shared__ double tile[32][33];
  const int m = 6 * n, n3 = 3 * n;
  const int i0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
  const int ti = threadIdx.x;
  const int i = i0 + ti;
  int si = 0, vi = 0;
  if (i < m) {
    const int blk = i / (2 * n), rem = i - blk * 2 * n;
    si = rem / n;
    vi = blk * n + (rem - si * n);
  }
  for (int tj = threadIdx.y; tj < 32; tj += 8) {
    const int j = j0 + tj;
    double val;
    if (i < m && j < m) {
      const int blk = j / (2 * n), rem = j - blk * 2 * n;
      const int sj = rem / n, vj = blk * n + (rem - sj * n);
      const double a = si == 0 ? (sj == 0 ? kA11 : kA12) : (sj == 0 ? kA21 : kA22);
      const double jv = (si == 0 ? J0 : J1)[(long long)vj * n3 + vi];
      val = (i == j ? 1.0 : 0.0) - h * a * jv;
    } else {
      val = i == j ? 1.0 : 0.0;
    }
    tile[tj][ti] = val;
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += 8) M[(long long)(i0 + r) * np + j0 + ti] = tile[ti][r];
}

// Surface b of the FD engine (ns = 2 nc surfaces; +eps for b < nc, -eps
// after) holds the source state of column c = c0 + b % nc, perturbed at
// variable v: column c is (stage s = c / 3n, variable v = c % 3n); the source
// of stage s, variable blk n + p sits at src[blk sstride + s soff + p].
// Slots b % nc >= cnt are unused (left unperturbed).
__global__ void k_gl2_fd_perturb(int n, int nc, int cnt, int c0, double eps, const double* __restrict__ src,
                                 int sstride, int soff, double* __restrict__ fy) {
  const long long ns = 2LL * nc;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * ns * n) return;
  const int blk = (int)(t / (ns * n));
  const long long rem = t - (long long)blk * ns * n;
  const int b = (int)(rem / n), p = (int)(rem - (long long)b * n);
  const int q = b % nc;
  int s = 0, v = -1;
  if (q < cnt) {
    const int c = c0 + q;
    s = c / (3 * n);
    v = c - s * 3 * n;
  }
  double val = src[(long long)blk * sstride + (long long)s * soff + p];
  if (blk * n + p == v) val += b < nc ? eps : -eps;
  fy[t] = val;
}

// J_s[v 3n + r] = (f+ - f-)[r] / (2 eps) for the cnt columns of the chunk.
__global__ void k_gl2_fd_columns(int n, int nc, int cnt, int c0, double eps, const double* __restrict__ fo,
                                 double* __restrict__ J0, double* __restrict__ J1) {
  const int n3 = 3 * n;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)cnt * n3) return;
  const int q = (int)(t / n3), r = (int)(t - (long long)q * n3);
  const int c = c0 + q, s = c / n3, v = c - s * n3;
  const long long ns = 2LL * nc;
  const int blk = r / n, p = r - blk * n;
  const double fp = fo[(long long)blk * ns * n + (long long)q * n + p];
  const double fm = fo[(long long)blk * ns * n + (long long)(nc + q) * n + p];
  (s == 0 ? J0 : J1)[(long long)v * n3 + r] = (fp - fm) / (2.0 * eps);
}

// stage s of the stage layout -> one contiguous 3n state
__global__ void k_gl2_gather(int n, int s, const double* __restrict__ st, double* __restrict__ y) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= 3 * n) return;
  const int blk = v / n, p = v - blk * n;
  y[v] = st[blk * 2 * n + s * n + p];
}

// y += h (b1 k1 + b2 k2)
__global__ void k_gl2_advance(int n, double h, double* __restrict__ y, const double* __restrict__ k) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= 3 * n) return;
  const int blk = v / n, p = v - blk * n;
  const int i0 = blk * 2 * n + p;
  y[v] = y[v] + h * (kB1 * k[i0] + kB2 * k[i0 + n]);
}

}  // namespace

struct Gl2Work {
  int n = 0;
  sfd_engine* stage = nullptr;  // two surfaces: the stage states
  sfd_engine* fd = nullptr;     // 2 fd_nc surfaces: perturbed states
  sfd_engine* jeng = nullptr;   // one surface: exact Jacobians
  int fd_nc = 0;
  sfd_dense_solver* lu = nullptr;
  double *k = nullptr, *kt = nullptr, *d = nullptr, *R = nullptr, *Rt = nullptr, *f = nullptr, *st = nullptr;
  double *J0 = nullptr, *J1 = nullptr, *yc = nullptr, *red = nullptr;
  double* h_red = nullptr;  // pinned
};

void sfd_gl2_free(sfd_engine* e) {
  if (!e || !e->gl2) return;
  Gl2Work* W = e->gl2;
  if (W->stage) sfd_destroy(W->stage);
  if (W->fd) sfd_destroy(W->fd);
  if (W->jeng) sfd_destroy(W->jeng);
  if (W->lu) sfd_dense_solver_destroy(W->lu);
  for (double* p : {W->k, W->kt, W->d, W->R, W->Rt, W->f, W->st, W->J0, W->J1, W->yc, W->red}) cudaFree(p);
  if (W->h_red) cudaFreeHost(W->h_red);
  delete W;
  e->gl2 = nullptr;
}

#define GCK(expr)                                                  \
  do {                                                             \
    cudaError_t _e = (expr);                                       \
    if (_e != cudaSuccess) return sfd_internal_cuda(_e, #expr);    \
  } while (0)

namespace {

// FP64 helper engine with the engine's problem, on the engine's stream.
int helper_engine(sfd_engine* e, int nsurf, sfd_engine** out) {
  sfd_options o;
  sfd_default_options(&o);
  o.precision = SFD_PRECISION_FP64;
  o.use_graphs = 0;
  o.autotune = 0;
  o.device = e->device;
  std::vector<int> ns(nsurf, e->hs[0].n);
  int rc = sfd_create(ns.data(), nsurf, &e->hp[0], 1, &o, out);
  if (rc) return rc;
  return sfd_set_stream(*out, e->stream);
}

int ensure_work(sfd_engine* e) {
  const int n = e->hs[0].n;
  if (e->gl2) {  // follow the engine's current stream
    Gl2Work* W = e->gl2;
    for (sfd_engine* h : {W->stage, W->fd, W->jeng})
      if (h && h->stream != e->stream) sfd_set_stream(h, e->stream);
    W->lu->stream = e->stream;
    return 0;
  }
  Gl2Work* W = e->gl2 = new Gl2Work();
  W->n = n;
  int rc = helper_engine(e, 2, &W->stage);
  if (rc) return rc;
  rc = sfd_dense_solver_create(6 * n, 1, &W->lu);
  if (rc) return rc;
  W->lu->stream = e->stream;
  const size_t m = 6 * (size_t)n, n3 = 3 * (size_t)n;
  for (double** p : {&W->k, &W->kt, &W->d, &W->R, &W->Rt, &W->f, &W->st}) GCK(cudaMalloc(p, m * sizeof(double)));
  GCK(cudaMalloc(&W->J0, n3 * n3 * sizeof(double)));
  GCK(cudaMalloc(&W->J1, n3 * n3 * sizeof(double)));
  GCK(cudaMalloc(&W->yc, n3 * sizeof(double)));
  GCK(cudaMalloc(&W->red, 2 * sizeof(double)));
  GCK(cudaMallocHost(&W->h_red, 2 * sizeof(double)));
  return 0;
}

struct Gl2Stats {
  long long newton = 0, rhs = 0, jac = 0;
};

// Reads [|R|^2, |k|^2] after k_gl2_residual.
int read_norms(sfd_engine* e, Gl2Work* W, double& r2, double& k2) {
  GCK(cudaMemcpyAsync(W->h_red, W->red, 2 * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
  GCK(cudaStreamSynchronize(e->stream));
  r2 = W->h_red[0];
  k2 = W->h_red[1];
  return 0;
}

// Jacobians of f at the stage states held in src (stage layout: sstride 2n,
// soff n, ncols 6n -> J0, J1) or at one state (sstride n, soff 0, ncols 3n -> J0).
int jacobians(sfd_engine* e, Gl2Work* W, const sfd_gl2_options& o, bool exact, const double* src, int sstride,
              int soff, int ncols, Gl2Stats& S) {
  const int n = W->n, n3 = 3 * n;
  cudaStream_t s = e->stream;
  if (exact) {
    for (int st = 0; st < ncols / n3; ++st) {
      const double* y = src;
      if (soff) {
        k_gl2_gather<<<nbl(n3, kT), kT, 0, s>>>(n, st, src, W->yc);
        GCK(cudaGetLastError());
        y = W->yc;
      }
      int rc = sfd_jacobian_device(W->jeng, y, st == 0 ? W->J0 : W->J1);
      if (rc) return rc;
      ++S.jac;
    }
    return 0;
  }
  if (!W->fd) {
    const double np = (double)pad_n(n);
    W->fd_nc = (int)std::max(1.0, std::min((double)(6 * n), std::floor(kFdChunkBytes / (2.0 * 8.0 * np * np))));
    int rc = helper_engine(e, 2 * W->fd_nc, &W->fd);
    if (rc) return rc;
  }
  const int nc = W->fd_nc;
  const long long nfd = 3LL * 2 * nc * n;
  for (int c0 = 0; c0 < ncols; c0 += nc) {
    const int cnt = std::min(nc, ncols - c0);
    k_gl2_fd_perturb<<<nbl(nfd, kT), kT, 0, s>>>(n, nc, cnt, c0, o.fd_eps, src, sstride, soff, W->fd->y0);
    GCK(cudaGetLastError());
    int rc = sfd_internal_rhs(W->fd, W->fd->y0, W->fd->kcur);
    if (rc) return rc;
    S.rhs += 2LL * cnt;
    k_gl2_fd_columns<<<nbl((long long)cnt * n3, kT), kT, 0, s>>>(n, nc, cnt, c0, o.fd_eps, W->fd->kcur, W->J0, W->J1);
    GCK(cudaGetLastError());
  }
  S.jac += ncols / n3;
  return 0;
}

// One Newton solve for a step of size h from the engine state.  On
// convergence the engine state is advanced.
int attempt(sfd_engine* e, Gl2Work* W, const sfd_gl2_options& o, bool exact, double h, Gl2Stats& S, bool& converged,
            double& resid) {
  const int n = W->n, n3 = 3 * n, m = 6 * n;
  cudaStream_t s = e->stream;
  converged = false;
  // k1 = k2 = f(y): y on both stage surfaces, one batched evaluation
  k_gl2_broadcast<<<nbl(n3, kT), kT, 0, s>>>(n, e->y0, W->st);
  GCK(cudaGetLastError());
  int rc = sfd_internal_rhs(W->stage, W->st, W->k);
  if (rc) return rc;
  S.rhs += 2;
  // residual at k
  k_gl2_stage<<<nbl(n3, kT), kT, 0, s>>>(n, h, e->y0, W->k, nullptr, 0.0, nullptr, W->st);
  GCK(cudaGetLastError());
  rc = sfd_internal_rhs(W->stage, W->st, W->f);
  if (rc) return rc;
  S.rhs += 2;
  k_gl2_residual<<<1, kRedT, 0, s>>>(m, W->k, W->f, W->R, W->red);
  GCK(cudaGetLastError());
  double r2, k2;
  rc = read_norms(e, W, r2, k2);
  if (rc) return rc;
  bool frozen = false;
  const int np = W->lu->np;
  for (long long it = 0; it < o.max_newton; ++it) {
    resid = std::sqrt(r2);
    if (resid <= o.newton_tol * (1.0 + std::sqrt(k2))) {
      converged = true;
      break;
    }
    ++S.newton;
    if (!frozen) {  // W->st holds the stage states of the current k
      rc = jacobians(e, W, o, exact, W->st, 2 * n, n, m, S);
      if (rc) return rc;
    }
    k_gl2_newton_matrix<<<dim3(np / 32, np / 32), dim3(32, 8), 0, s>>>(n, np, h, W->J0, frozen ? W->J0 : W->J1,
                                                                      W->lu->mat);
    GCK(cudaGetLastError());
    unsigned int lst = 0;
    rc = sfd_internal_dense_factor_solve(W->lu, W->R, W->d, &lst, false);  // M d = R; the update is k - alpha d
    if (rc) return rc;
    if (lst & SFD_STATUS_PIVOT_SWAP) {
      // partial pivoting would have exchanged rows: assemble the Newton matrix
      // again and factor it with the exchanges (the reference's getrf)
      k_gl2_newton_matrix<<<dim3(np / 32, np / 32), dim3(32, 8), 0, s>>>(n, np, h, W->J0, frozen ? W->J0 : W->J1,
                                                                        W->lu->mat);
      GCK(cudaGetLastError());
      rc = sfd_internal_dense_factor_solve(W->lu, W->R, W->d, &lst, true);
      if (rc) return rc;
    }
    if (lst & (SFD_STATUS_ZERO_PIVOT | SFD_STATUS_NONFINITE)) return 0;  // not converged
    const double phi = 0.5 * r2;
    double alpha = 1.0;
    for (;;) {
      k_gl2_stage<<<nbl(n3, kT), kT, 0, s>>>(n, h, e->y0, W->k, W->d, -alpha, W->kt, W->st);
      GCK(cudaGetLastError());
      rc = sfd_internal_rhs(W->stage, W->st, W->f);
      if (rc) return rc;
      S.rhs += 2;
      k_gl2_residual<<<1, kRedT, 0, s>>>(m, W->kt, W->f, W->Rt, W->red);
      GCK(cudaGetLastError());
      double rt2, kt2;
      rc = read_norms(e, W, rt2, kt2);
      if (rc) return rc;
      if (0.5 * rt2 <= phi - o.armijo_c * alpha * r2) {  // sufficient decrease: accept the trial
        std::swap(W->k, W->kt);
        std::swap(W->R, W->Rt);
        r2 = rt2;
        k2 = kt2;
        break;
      }
      alpha *= o.backtrack;
      if (alpha < o.min_alpha) {
        if (!frozen && o.allow_simplified) {  // simplified Newton with J(y) for the rest of the attempt
          frozen = true;
          rc = jacobians(e, W, o, exact, e->y0, n, 0, n3, S);
          if (rc) return rc;
          break;
        }
        resid = std::sqrt(rt2);
        return 0;  // not converged
      }
    }
  }
  if (!converged) resid = std::sqrt(r2);
  if (converged) {
    k_gl2_advance<<<nbl(n3, kT), kT, 0, s>>>(n, h, e->y0, W->k);
    GCK(cudaGetLastError());
  }
  return 0;
}

}  // namespace

int sfd_internal_gl2(sfd_engine* e, double t0, double t1, const sfd_gl2_options& o, sfd_gl2_result& r,
                     std::vector<double>* times, std::vector<double>* states, sfd_gl2_step_fn fn, void* user) {
  std::memset(&r, 0, sizeof(r));
  if (!e) return sfd_internal_error(SFD_ERR_INVALID, "null engine");
  if (e->nsurf != 1 || e->nblk != 3)
    return sfd_internal_error(SFD_ERR_INVALID, "GL2 integrates engines with one surface and no augmented drive");
  if (e->hs[0].drive) return sfd_internal_error(SFD_ERR_INVALID, "GL2 does not cover the optomechanical drive");
  const int n = e->hs[0].n;
  if (6 * n > 8192) return sfd_internal_error(SFD_ERR_INVALID, "GL2 supports n <= 1365 (Newton systems of order 6n)");
  if (!std::isfinite(t0) || !std::isfinite(t1)) return sfd_internal_error(SFD_ERR_INVALID, "t0 and t1 must be finite");
  if (!(o.step > 0) || !std::isfinite(o.step)) return sfd_internal_error(SFD_ERR_INVALID, "step must be finite and > 0");
  // The line search ends when alpha falls below min_alpha: with min_alpha <= 0
  // (or NaN) and a non-finite trial residual it would never end.
  if (o.max_newton < 0 || o.max_halvings < 0 || !(o.backtrack > 0 && o.backtrack < 1) ||
      !(o.min_alpha > 0 && o.min_alpha <= 1) || !(o.armijo_c >= 0 && o.armijo_c < 1) || !(o.newton_tol >= 0) ||
      !(std::isfinite(o.fd_eps) && o.fd_eps != 0))
    return sfd_internal_error(SFD_ERR_INVALID,
                              "invalid GL2 options: need max_newton, max_halvings >= 0, 0 < backtrack < 1, "
                              "0 < min_alpha <= 1, 0 <= armijo_c < 1, newton_tol >= 0 and a finite nonzero fd_eps");
  GCK(cudaSetDevice(e->device));
  int rc = ensure_work(e);
  if (rc) return rc;
  Gl2Work* W = e->gl2;
  bool exact = false;
  if (o.jacobian == SFD_GL2_JACOBIAN_EXACT || o.jacobian == SFD_GL2_JACOBIAN_AUTO) {
    if (!W->jeng) {
      rc = helper_engine(e, 1, &W->jeng);
      if (rc) return rc;
    }
    const char* why = sfd_adjoint_unsupported(W->jeng);
    if (o.jacobian == SFD_GL2_JACOBIAN_EXACT && why) return sfd_internal_error(SFD_ERR_INVALID, why);
    exact = !why && (o.jacobian == SFD_GL2_JACOBIAN_EXACT || n >= kExactMinN);
  } else if (o.jacobian != SFD_GL2_JACOBIAN_FD) {
    return sfd_internal_error(SFD_ERR_INVALID, "unknown Jacobian mode");
  }
  const size_t n3 = 3 * (size_t)n;
  const double fwd = t1 >= t0 ? 1.0 : -1.0;
  const double hmin = std::fabs(t1 - t0) / std::pow(2.0, 20);
  double step = o.step, t = t0;
  Gl2Stats S;
  long long steps = 0, halvings = 0;
  double resid = 0.0, last_h = 0.0;
  std::vector<double> step_host;
  int status = 0;
  while ((t - t1) * fwd < 0.0) {
    double htry = std::min(step, std::fabs(t1 - t)) * fwd;
    bool ok = false;
    for (long long i = 0;; ++i) {
      rc = attempt(e, W, o, exact, htry, S, ok, resid);
      if (rc) return rc;
      if (ok || std::fabs(htry) <= hmin || i == o.max_halvings) break;
      htry *= 0.5;
      ++halvings;
    }
    if (!ok) {
      status = 1;
      last_h = htry;
      break;
    }
    t += htry;
    step = std::fabs(htry);
    last_h = htry;
    ++steps;
    if (times) times->push_back(t);
    if (states) {
      const size_t off = states->size();
      states->resize(off + n3);
      GCK(cudaMemcpyAsync(states->data() + off, e->y0, n3 * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    }
    if (fn) {
      step_host.resize(n3);
      GCK(cudaMemcpyAsync(step_host.data(), e->y0, n3 * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
      GCK(cudaStreamSynchronize(e->stream));
      fn(user, t, step_host.data());
    }
  }
  GCK(cudaStreamSynchronize(e->stream));
  r.status = status;
  r.steps = steps;
  r.newton_iters = S.newton;
  r.rhs_evals = S.rhs;
  r.jacobians = S.jac;
  r.halvings = halvings;
  r.t = t;
  r.h = last_h;
  r.residual = resid;
  return 0;
}

extern "C" void sfd_default_gl2_options(sfd_gl2_options* o) {
  if (!o) return;
  o->step = 0.01;  // GaussLegendre2Options (GaussLegendre.cuh:83-104)
  o->newton_tol = 1e-10;
  o->max_newton = 20;
  o->allow_simplified = 0;
  o->armijo_c = 1e-4;
  o->backtrack = 0.5;
  o->min_alpha = 1e-6;
  o->max_halvings = 6;
  o->fd_eps = 1e-6;  // JacobianCalculator::eps
  o->jacobian = SFD_GL2_JACOBIAN_AUTO;
}

extern "C" int sfd_gl2_evolve_cb(sfd_engine* e, double t0, double t1, const sfd_gl2_options* opts,
                                 sfd_gl2_result* res, sfd_gl2_step_fn fn, void* user) {
  if (!opts || !res) return sfd_internal_error(SFD_ERR_INVALID, "null argument");
  return sfd_internal_gl2(e, t0, t1, *opts, *res, nullptr, nullptr, fn, user);
}

extern "C" int sfd_gl2_evolve(sfd_engine* e, double t0, double t1, const sfd_gl2_options* opts, sfd_gl2_result* res,
                              double* times, double* states, long long cap) {
  if (!opts || !res) return sfd_internal_error(SFD_ERR_INVALID, "null argument");
  std::vector<double> T, Y;
  int rc = sfd_internal_gl2(e, t0, t1, *opts, *res, times ? &T : nullptr, states ? &Y : nullptr);
  if (rc) return rc;
  const long long k = std::min<long long>(cap, res->steps);
  if (times && k > 0) std::memcpy(times, T.data(), (size_t)k * sizeof(double));
  if (states && k > 0) std::memcpy(states, Y.data(), (size_t)k * 3 * e->hs[0].n * sizeof(double));
  return 0;
}
