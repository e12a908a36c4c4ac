// sfd_solve.cuh -- dense-solver kernels (padded per-surface matrices).
#pragma once
#include "sfd_engine.cuh"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

// per-surface matrices are padded to a multiple of 128 rows/columns
__host__ __device__ __forceinline__ int pad_n(int n) { return (n + 127) / 128 * 128; }
constexpr int kGemvRows = 16;  // rows per CTA of k_gemv
constexpr int kTrsmSmem = 2 * 64 * 65 * 8;  // k_lu64_trsm dynamic shared memory
constexpr int kGjDiagSmem = (128 * 129 + 128 * 33 + 32 * 128 + 32 * 33) * 4;  // k_gj_diag dynamic shared memory

cudaError_t sfd_launch_assemble64(const SurfaceDesc* surf, const int4* tiles, int ntiles, const cd* w, const cd* p,
                                  const cd* zp, const double* mdiag, double* mat, cudaStream_t st);
cudaError_t sfd_launch_assemble32(const SurfaceDesc* surf, const int4* tiles, int ntiles, const float4* wdf,
                                  const float4* pdf, const cd* p, const cd* zp, const double* mdiag, float* mat,
                                  cudaStream_t st);
__global__ void k_lu64_diag(const SurfaceDesc* surf, int nsurf, int kb, double* mat, unsigned int* status,
                            double* lmax);
__global__ void k_lu64_trsm(const SurfaceDesc* surf, int nsurf, int kb, double* mat, double* lmax);
__global__ void k_lu64_gemm(const SurfaceDesc* surf, int nsurf, int kb, double* mat);
// x = (LU)^-1 b per surface (b, x at the surface's node offset; x may be
// null); acc (nullable) += the solution; piv (nullable) = row exchanges of a
// pivoted factorisation, applied to b first; where lmax[s] > 1 the surface's
// status gets SFD_ST_PIVOT_SWAP (lmax, status nullable); gated surfaces skip.
__global__ void k_lu64_solve(const SurfaceDesc* surf, const double* mat, const double* b, double* x, double* acc,
                             const int* piv, Gate gate, const double* lmax, unsigned int* status);
// Blocked LU with partial pivoting (getrf semantics: the first row of largest
// magnitude in the column is the pivot).  Step kb: k_lu64_panel_piv factors
// the 64-column panel [k0, np) x [k0, k0 + 64) in place and records the
// pivot rows piv[s * np + k] (absolute row indices); k_lu64_swap applies the
// panel's exchanges to the columns outside it; then the U12 part of
// k_lu64_trsm (blockIdx.y == 1) and k_lu64_gemm complete the step.
__global__ void k_lu64_panel_piv(const SurfaceDesc* surf, int nsurf, int kb, double* mat, int* piv,
                                 unsigned int* status);
__global__ void k_lu64_swap(const SurfaceDesc* surf, int nsurf, int kb, double* mat, const int* piv);
__global__ void k_lu64_trsm_u(const SurfaceDesc* surf, int nsurf, int kb, double* mat);
__global__ void k_gj_diag(const SurfaceDesc* surf, int nsurf, int kb, float* mat, float* pbuf, unsigned int* status);
__global__ void k_gj_panel(const SurfaceDesc* surf, int nsurf, int kb, const float* mat, const float* pbuf,
                           float* rbuf, float* cbuf, const long long* poff, __nv_bfloat16* cparts,
                           __nv_bfloat16* rparts, long long pstride);
__global__ void k_gj_update(const SurfaceDesc* surf, int nsurf, int kb, float* mat, const float* pbuf,
                            const float* rbuf, const float* cbuf, const long long* poff, int k_lines_only);
__global__ void k_precond_to_half(const SurfaceDesc* surf, const int2* rowblk, const float* mat, __half* mat16,
                                  float* rscale);
// y = X v (v FP32); optional double-float copy of y and in-place acc += y;
// prefetch: one surface (rowblk null), ungated, predecessor not writing mat16
__global__ void k_gemv_h(const SurfaceDesc* surf, const int2* rowblk, int nblk, const __half* mat16, const float* rscale,
                         const float* v, double* y, float2* ydf, double* acc, float2* accdf, Gate gate, int prefetch);
// y = X v for one surface with the FP16 rows streamed into shared memory
// (k_gemv_hs): kGemvSWarps warps per CTA, one CTA per SM, spw row slots per
// warp; the plan gives spw and the dynamic shared memory (spw = 0: the rows do
// not fit, use k_gemv_h); configure sets the kernel's shared-memory limit.
constexpr int kGemvSWarps = 8;
constexpr int kGemvSMaxSpw = 8;
// Default cap on the slots per warp.  At N = 4096 (27 rows per CTA) two slots
// (16 rows, 148 KB in flight per SM) stepped faster than three (214 KB) or
// one: the smaller footprint leaves room on the SM for the next kernel's CTAs,
// which programmatic dependent launch places there early.
constexpr int kGemvSDefaultSpw = 2;
constexpr int kGemvSHead = 1024;  // mbarriers (kGemvSWarps x kGemvSMaxSpw x 8 B), padded
void sfd_gemv_stream_plan(int n, int nsm, int smem_max, int cap, int* spw, int* smem);
cudaError_t sfd_gemv_stream_configure(int smem);
// prefetch: request the first rows before waiting on the preceding kernel
// (ungated launches whose predecessor does not write mat16 only).
cudaError_t sfd_launch_gemv_stream(const SurfaceDesc* surf, int nsm, int spw, int smem, bool prefetch,
                                   const __half* mat16, const float* rscale, const float* v, double* y, float2* ydf,
                                   double* acc, float2* accdf, const Gate& gate, unsigned int* status,
                                   cudaStream_t st);
cudaError_t sfd_tc_configure();
// TMA tensor map (128 bytes, written to map_out) of three bf16 part arrays of
// `rows` rows x 128 K-major values, parts `part_stride` elements apart.
cudaError_t sfd_tc_make_map(void* map_out, const __nv_bfloat16* parts, long long rows, long long part_stride);
// TMA tensor map (128 bytes) of one surface's np x np FP32 matrix at `mat`.
cudaError_t sfd_tc_make_out_map(void* map_out, float* mat, int np);
// Tensor-core trailing update of Gauss-Jordan step kb: grid (tile columns,
// ngroups row groups, surfaces), operands through the two tensor maps, the
// update reduce-added into each surface's matrix through maps_out (device
// array of one 128-byte map per surface, 64-byte aligned).
cudaError_t sfd_launch_gj_update_tc(const void* map_c, const void* map_r, const void* maps_out,
                                    const SurfaceDesc* surf, int nsurf, int kb, int max_np, int ngroups,
                                    const long long* poff, unsigned int* status, cudaStream_t st);
__global__ void k_gemv(const SurfaceDesc* surf, const int2* rowblk, const float* mat, const float* v, double* y,
                       float2* ydf, double* acc, float2* accdf, Gate gate);
