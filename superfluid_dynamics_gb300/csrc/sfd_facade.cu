// sfd_facade.cu -- C ABI pieces behind the C++ facade include/sfd.hpp, which
// mirrors the reference's in-process classes:
//   BaseBoundaryIntegralCalculator::run on interleaved complex state
//     [Z (n) | Phi (n, imaginary part 0)] -> [dZ/dt | dPhi/dt]
//     (BaseBoundaryIntegrator.cuh:137-262),
//   calculateVorticities + getDevA / getDevZp / getDevZpp (:275-314),
//   the RK4 stage combines of AutonomousRungeKuttaStepper (utilities.cuh:78-83)
//   for user-defined problems, and MatrixSolver::solve (MatrixSolver.cuh:113-172)
//   on column-major matrices.
#include <algorithm>
#include <cstring>
#include <vector>

#include "sfd_internal.cuh"
#include "sfd_solve.cuh"

namespace {

// [Z | Phi] complex (interleaved) -> [x | y | phi] (SoA)
__global__ void k_complex_to_soa(int n, const cd* __restrict__ zc, double* __restrict__ soa) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const cd z = zc[i];
  soa[i] = z.re;
  soa[n + i] = z.im;
  soa[2 * n + i] = zc[n + i].re;
}
// [dx | dy | dphi] -> [dx + i dy | dphi + 0 i]
__global__ void k_soa_to_complex(int n, const double* __restrict__ soa, cd* __restrict__ zc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  zc[i] = {soa[i], soa[n + i]};
  zc[n + i] = {soa[2 * n + i], 0.0};
}
// column-major n x n (batch b at b n^2) -> padded row-major with identity padding
__global__ void k_colmajor_to_padded(int n, int np, const double* __restrict__ src, double* __restrict__ dst) {
  const int b = blockIdx.z;
  const int r = blockIdx.y * 16 + threadIdx.y, c = blockIdx.x * 16 + threadIdx.x;
  if (r >= np || c >= np) return;
  double v;
  if (r < n && c < n) v = src[(long long)b * n * n + (long long)c * n + r];
  else v = (r == c) ? 1.0 : 0.0;
  dst[(long long)b * np * np + (long long)r * np + c] = v;
}

inline int nb(long long n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

#define FCK(expr)                                                     \
  do {                                                                \
    cudaError_t _e = (expr);                                          \
    if (_e != cudaSuccess) return sfd_internal_cuda(_e, #expr);       \
  } while (0)

namespace {
// complex <-> SoA staging buffers of the engine (allocated on first use, freed with it)
int ensure_scratch(sfd_engine* e) {
  if (e->fc_in && e->fc_out) return 0;
  const long long n3 = 3LL * e->ntot;
  if (!e->fc_in) FCK(cudaMalloc(&e->fc_in, n3 * sizeof(double)));
  FCK(cudaMalloc(&e->fc_out, n3 * sizeof(double)));
  return 0;
}
}  // namespace

extern "C" int sfd_rhs_device_complex(sfd_engine* e, const void* state_c, void* rhs_c) {
  if (!e || !state_c || !rhs_c) return sfd_internal_error(SFD_ERR_INVALID, "null argument");
  if (e->nblk != 3) return sfd_internal_error(SFD_ERR_INVALID, "complex layout: engines with an augmented drive are not supported");
  FCK(cudaSetDevice(e->device));
  int rc = ensure_scratch(e);
  if (rc) return rc;
  k_complex_to_soa<<<nb(e->ntot, 256), 256, 0, e->stream>>>(e->ntot, static_cast<const cd*>(state_c), e->fc_in);
  FCK(cudaGetLastError());
  rc = sfd_internal_rhs(e, e->fc_in, e->fc_out);
  if (rc) return rc;
  k_soa_to_complex<<<nb(e->ntot, 256), 256, 0, e->stream>>>(e->ntot, e->fc_out, static_cast<cd*>(rhs_c));
  FCK(cudaGetLastError());
  return 0;
}

extern "C" int sfd_vorticities_device(sfd_engine* e, const void* state_c, double** a, void** zp, void** zpp) {
  if (!e || !state_c) return sfd_internal_error(SFD_ERR_INVALID, "null argument");
  if (e->nblk != 3) return sfd_internal_error(SFD_ERR_INVALID, "complex layout: engines with an augmented drive are not supported");
  FCK(cudaSetDevice(e->device));
  int rc = ensure_scratch(e);
  if (rc) return rc;
  k_complex_to_soa<<<nb(e->ntot, 256), 256, 0, e->stream>>>(e->ntot, static_cast<const cd*>(state_c), e->fc_in);
  FCK(cudaGetLastError());
  rc = sfd_internal_solve(e, e->fc_in);
  if (rc) return rc;
  if (a) *a = e->a;
  if (zp) *zp = e->zp;
  if (zpp) *zpp = e->zpp;
  return 0;
}

// Generic RK4 stage combines (AutonomousRungeKuttaStepper.cuh:338-375), n doubles.
extern "C" int sfd_rk4_stage_device(long long n, const void* y0, const void* k, void* kacc, void* ystage, double wk,
                                    double cy, int first, void* stream) {
  if (!y0 || !k || !kacc || n < 0 || n > (1LL << 31) - 1) return sfd_internal_error(SFD_ERR_INVALID, "invalid argument");
  k_rk4_stage<<<nb(n, 256), 256, 0, (cudaStream_t)stream>>>((int)n, (const double*)y0, (const double*)k,
                                                             (double*)kacc, (double*)ystage, wk, cy, first);
  FCK(cudaGetLastError());
  return 0;
}
extern "C" int sfd_rk4_final_device(long long n, void* y0, const void* kacc, double c, void* stream) {
  if (!y0 || !kacc || n < 0 || n > (1LL << 31) - 1) return sfd_internal_error(SFD_ERR_INVALID, "invalid argument");
  k_rk4_final<<<nb(n, 256), 256, 0, (cudaStream_t)stream>>>((int)n, (double*)y0, (const double*)kacc, c);
  FCK(cudaGetLastError());
  return 0;
}

// ---------------------------------------------------------------- dense solver
// MatrixSolver::solve (MatrixSolver.cuh:113-172): batch column-major n x n
// systems M a = b.  The matrices are copied into padded row-major storage and
// factored by the engine's FP64 blocked LU without row exchanges (with the
// pivot-growth certificate: max |l_ij| <= 1 means partial pivoting would have
// chosen the same rows; otherwise the status word gets SFD_STATUS_PIVOT_SWAP).

extern "C" int sfd_dense_solver_create(int n, int batch, sfd_dense_solver** out) {
  if (!out || n < 1 || n > 8192 || batch < 1) return sfd_internal_error(SFD_ERR_INVALID, "invalid argument");
  *out = nullptr;
  sfd_dense_solver* d = new sfd_dense_solver();
  d->n = n;
  d->np = pad_n(n);
  d->batch = batch;
  std::vector<SurfaceDesc> hs(batch);
  for (int b = 0; b < batch; ++b) {
    std::memset(&hs[b], 0, sizeof(SurfaceDesc));
    hs[b].n = n;
    hs[b].off = b * n;
    hs[b].moff = (long long)b * d->np * d->np;
  }
  cudaError_t err = cudaMalloc(&d->d_surf, batch * sizeof(SurfaceDesc));
  if (err == cudaSuccess) err = cudaMemcpy(d->d_surf, hs.data(), batch * sizeof(SurfaceDesc), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMalloc(&d->mat, (size_t)batch * d->np * d->np * sizeof(double));
  if (err == cudaSuccess) err = cudaMalloc(&d->lmax, batch * sizeof(double));
  if (err == cudaSuccess) err = cudaMalloc(&d->piv, (size_t)batch * d->np * sizeof(int));
  if (err == cudaSuccess) err = cudaMalloc(&d->status, batch * sizeof(unsigned int));
  if (err == cudaSuccess) err = sfd_solve_configure();
  if (err != cudaSuccess) {
    cudaFree(d->d_surf);
    cudaFree(d->mat);
    cudaFree(d->lmax);
    cudaFree(d->piv);
    cudaFree(d->status);
    delete d;
    return sfd_internal_cuda(err, "sfd_dense_solver_create");
  }
  *out = d;
  return 0;
}

extern "C" int sfd_dense_solver_set_stream(sfd_dense_solver* d, void* stream) {
  if (!d) return sfd_internal_error(SFD_ERR_INVALID, "null solver");
  d->stream = (cudaStream_t)stream;
  return 0;
}

extern "C" int sfd_dense_solve(sfd_dense_solver* d, const double* M, const double* b, double* x, unsigned int* status) {
  if (!d || !M || !b || !x) return sfd_internal_error(SFD_ERR_INVALID, "null argument");
  dim3 blk(16, 16), grid(nb(d->np, 16), nb(d->np, 16), d->batch);
  k_colmajor_to_padded<<<grid, blk, 0, d->stream>>>(d->n, d->np, M, d->mat);
  FCK(cudaGetLastError());
  // MatrixSolver::solve factors with cusolverDnDgetrf / getrs (partial pivoting)
  return sfd_internal_dense_factor_solve(d, b, x, status, true);
}

int sfd_internal_dense_factor_solve(sfd_dense_solver* d, const double* b, double* x, unsigned int* status,
                                    bool pivoted) {
  cudaStream_t s = d->stream;
  FCK(cudaMemsetAsync(d->status, 0, d->batch * sizeof(unsigned int), s));
  FCK(cudaMemsetAsync(d->lmax, 0, d->batch * sizeof(double), s));
  const int nbk = d->np / 64;
  for (int kb = 0; kb < nbk; ++kb) {
    const int rem = nbk - kb - 1;
    if (pivoted) {
      k_lu64_panel_piv<<<d->batch, 1024, 0, s>>>(d->d_surf, d->batch, kb, d->mat, d->piv, d->status);
      if (nbk > 1) k_lu64_swap<<<dim3(nb(d->np - 64, 256), d->batch), 256, 0, s>>>(d->d_surf, d->batch, kb, d->mat, d->piv);
      if (rem > 0) k_lu64_trsm_u<<<dim3(rem, 1, d->batch), 64, kTrsmSmem, s>>>(d->d_surf, d->batch, kb, d->mat);
    } else {
      k_lu64_diag<<<d->batch, 256, 0, s>>>(d->d_surf, d->batch, kb, d->mat, d->status, d->lmax);
      if (rem > 0) k_lu64_trsm<<<dim3(rem, 2, d->batch), 64, kTrsmSmem, s>>>(d->d_surf, d->batch, kb, d->mat, d->lmax);
    }
    if (rem > 0) k_lu64_gemm<<<dim3(2 * rem, 2 * rem, d->batch), 256, 0, s>>>(d->d_surf, d->batch, kb, d->mat);
  }
  k_lu64_solve<<<d->batch, 256, d->np * sizeof(double), s>>>(d->d_surf, d->mat, b, x, nullptr,
                                                               pivoted ? d->piv : nullptr, Gate{}, nullptr, nullptr);
  FCK(cudaGetLastError());
  if (status) {
    std::vector<double> lm(d->batch);
    FCK(cudaMemcpyAsync(status, d->status, d->batch * sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
    FCK(cudaMemcpyAsync(lm.data(), d->lmax, d->batch * sizeof(double), cudaMemcpyDeviceToHost, s));
    FCK(cudaStreamSynchronize(s));
    if (!pivoted)
      for (int i = 0; i < d->batch; ++i)
        if (lm[i] > 1.0) status[i] |= SFD_STATUS_PIVOT_SWAP;
  }
  return 0;
}

extern "C" int sfd_dense_solver_destroy(sfd_dense_solver* d) {
  if (!d) return 0;
  if (d->stream) cudaStreamSynchronize(d->stream);
  cudaFree(d->d_surf);
  cudaFree(d->mat);
  cudaFree(d->lmax);
  cudaFree(d->piv);
  cudaFree(d->status);
  delete d;
  return 0;
}
