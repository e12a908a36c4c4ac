// sfd_solve.cu -- dense solvers for the second-kind system M a = phi'.
//
// Replaces MatrixSolver<N,B>::solve (CSH/MatrixSolver.cuh:113-172: cuSOLVER
// getrf/getrs, cuBLAS getrfBatched/getrsBatched).
//
// Storage: each surface's matrix is padded to n_pad = ceil(n / 128) * 128 with
// an identity block, [[M, 0], [0, I]], so every panel and tile is full.  The
// factorisation / inverse of the padded matrix is [[f(M), 0], [0, I]].
//
// Pivoting.  M = 1/2 I + K is a second-kind operator; on every configuration
// of this path it is column-diagonally dominant or keeps its pivots on the
// diagonal (helium adds a near-constant image block).  Both factorisations here
// run without row exchanges and record max |l_ij| (LU) or the analogous
// multiplier bound (Gauss-Jordan).  max |l_ij| <= 1 certifies that partial
// pivoting (getrf) would have chosen exactly the same pivots, so the result is
// the reference's factorisation; otherwise the SFD_ST_PIVOT_SWAP status bit is
// raised and accuracy rests on the refinement residual check.
//
//  * FP64 mode: blocked right-looking LU (nb = 64) + blocked triangular solves.
//  * mixed mode: FP32 matrix, blocked in-place Gauss-Jordan inverse (nb = 128),
//    applied as a GEMV inside the FP64-accurate refinement loop.
#include "sfd_engine.cuh"
#include "sfd_mbar.cuh"
#include "sfd_solve.cuh"

#include <cuda_fp16.h>

#include <algorithm>

#include <cuda_bf16.h>

// =============================================================== assembly
// M_kj = c1 Im(z'_k cot((z_k - z_j)/2)) - [image] (1/4pi) Im cot((z_k - conj z_j)/2 + ih)
// M_kk = mdiag_k - [image] (1/4pi) Im cot(i (y_k + h))          (createM.cuh:43-92)
// with cot via w = exp(i z) (see sfd_kernels.cu).  Padded rows/cols = identity.
// FP64 entries (the FP64 engine's matrix).
__global__ void k_assemble64(const SurfaceDesc* surf, const int4* tiles, const cd* w, const cd* p, const cd* zp,
                             const double* mdiag, double* mat) {
  const int4 t = tiles[blockIdx.x];  // (surface, row0, col0, -)
  const SurfaceDesc& S = surf[t.x];
  const int n = S.n, np = pad_n(n), off = S.off;
  double* A = mat + S.moff;
  const bool image = (S.physics == 1 && !S.infinite_depth);
  const double c1 = S.physics == 0 ? 0.25 * (1 - S.rho) / SFD_PI : 0.25 / SFD_PI;
  const double inv4pi = 0.25 / SFD_PI;
  for (int e = threadIdx.x; e < 64 * 64; e += blockDim.x) {
    int k = t.y + (e >> 6), j = t.z + (e & 63);
    double v;
    if (k >= n || j >= n) {
      v = (k == j) ? 1.0 : 0.0;
    } else {
      cd wk = w[off + k];
      if (k == j) {
        v = mdiag[off + k];
      } else {
        cd wj = w[off + j];
        cd cot = cmul_i(cdiv(wk + wj, wk - wj));
        v = c1 * (zp[off + k] * cot).im;
      }
      if (image) {
        cd pk = p[off + k], pj = p[off + j];
        cd q = pk * cconj(pj);
        cd r = cdiv(cd{1.0 + q.re, q.im}, cd{1.0 - q.re, -q.im});  // cot = -i r  ->  Im cot = -Re r
        v -= inv4pi * (-r.re);
      }
    }
    A[(long long)k * np + j] = v;
  }
}

// FP32 entries of the preconditioner's matrix, one 64 x 64 tile per CTA of 256
// threads.  The tile's 64 row nodes and 64 column nodes are staged in shared
// memory from the double-float copies (wdf, pdf) written by the node-data
// kernel, so the entry loop runs on the FP32 pipe alone: w_k - w_j as
// (hi_k - hi_j) + (lo_k - lo_j) keeps FP32 relative accuracy for neighbouring
// nodes, and 1/|w_k - w_j|^2 is the fast reciprocal (the matrix only feeds the
// FP16 preconditioner, whose error is far larger).  Each thread writes 4 rows
// x 4 consecutive columns as float4 stores, a warp two full 256-byte rows.
// Per tile: 16 KB written, 3 KB read.
__global__ void __launch_bounds__(256) k_assemble32(const SurfaceDesc* surf, const int4* tiles, const float4* wdf,
                                                    const float4* pdf, const cd* p, const cd* zp,
                                                    const double* mdiag, float* mat) {
  __shared__ float4 s_wj[64];  // (re.hi, re.lo, im.hi, im.lo)
  __shared__ float2 s_pj[64];
  __shared__ float4 s_wk[64];
  __shared__ float2 s_zk[64];
  __shared__ float2 s_pk[64];
  __shared__ float s_dk[64];
  const int4 t = tiles[blockIdx.x];  // (surface, row0, col0, -)
  const SurfaceDesc& S = surf[t.x];
  const int n = S.n, np = pad_n(n), off = S.off;
  const bool image = (S.physics == 1 && !S.infinite_depth);
  const double inv4pi = 0.25 / SFD_PI;
  const float c1 = (float)(S.physics == 0 ? 0.25 * (1 - S.rho) / SFD_PI : 0.25 / SFD_PI);
  {
    const int i = threadIdx.x & 63;
    const int part = threadIdx.x >> 6;  // 0: column nodes, 1: row nodes, 2: row diagonal
    if (part == 0) {
      const int j = t.z + i;
      const bool in = j < n;
      s_wj[i] = in ? wdf[off + j] : make_float4(0.f, 0.f, 0.f, 0.f);
      s_pj[i] = (in && image) ? make_float2(pdf[off + j].x, pdf[off + j].z) : make_float2(0.f, 0.f);
    } else if (part == 1) {
      const int k = t.y + i;
      const bool in = k < n;
      s_wk[i] = in ? wdf[off + k] : make_float4(0.f, 0.f, 0.f, 0.f);
      s_pk[i] = (in && image) ? make_float2(pdf[off + k].x, pdf[off + k].z) : make_float2(0.f, 0.f);
      s_zk[i] = in ? make_float2((float)zp[off + k].re, (float)zp[off + k].im) : make_float2(0.f, 0.f);
    } else if (part == 2) {
      const int k = t.y + i;
      double v = 1.0;
      if (k < n) {
        v = mdiag[off + k];
        if (image) {
          const double q = cabs2(p[off + k]);
          v += inv4pi * (1.0 + q) / (1.0 - q);
        }
      }
      s_dk[i] = (float)v;
    }
  }
  __syncthreads();
  const int cg = threadIdx.x & 15, rg = threadIdx.x >> 4;
  const int c0 = 4 * cg;
  float4 wj[4];
  float2 pj[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    wj[c] = s_wj[c0 + c];
    pj[c] = s_pj[c0 + c];
  }
  float* A = mat + S.moff;
  const float fi = (float)inv4pi;
#pragma unroll
  for (int rr = 0; rr < 4; ++rr) {
    const int r = rg + 16 * rr;
    const int k = t.y + r;
    const float4 wk = s_wk[r];
    const float2 zk = s_zk[r], pk = s_pk[r];
    float v[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const float dr = (wk.x - wj[c].x) + (wk.y - wj[c].y);
      const float di = (wk.z - wj[c].z) + (wk.w - wj[c].w);
      const float sr = wk.x + wj[c].x, si = wk.z + wj[c].z;
      const float den = __fdividef(1.0f, fmaf(dr, dr, di * di));
      const float qr = fmaf(sr, dr, si * di) * den, qi = fmaf(si, dr, -sr * di) * den;  // (w_k+w_j)/(w_k-w_j)
      // cot = i (qr + i qi);  Im(z'_k cot) = zr qr - zi qi
      float fv = c1 * fmaf(zk.x, qr, -zk.y * qi);
      if (image) {
        const float q_r = fmaf(pk.x, pj[c].x, pk.y * pj[c].y), q_i = fmaf(pk.y, pj[c].x, -pk.x * pj[c].y);
        const float er = 1.f - q_r, ei = -q_i;
        const float d2 = __fdividef(1.0f, fmaf(er, er, ei * ei));
        fv = fmaf(fi, fmaf(1.f + q_r, er, q_i * ei) * d2, fv);
      }
      v[c] = fv;
    }
    const int j0 = t.z + c0;
    if (k >= n || j0 + 3 >= n || (k >= j0 && k <= j0 + 3)) {  // padding or the diagonal: entry by entry
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int j = j0 + c;
        if (k >= n || j >= n) v[c] = (k == j) ? 1.f : 0.f;
        else if (k == j) v[c] = s_dk[r];
      }
    }
    *reinterpret_cast<float4*>(A + (long long)k * np + j0) = make_float4(v[0], v[1], v[2], v[3]);
  }
}

cudaError_t sfd_launch_assemble64(const SurfaceDesc* surf, const int4* tiles, int ntiles, const cd* w, const cd* p,
                                  const cd* zp, const double* mdiag, double* mat, cudaStream_t st) {
  k_assemble64<<<ntiles, 256, 0, st>>>(surf, tiles, w, p, zp, mdiag, mat);
  return cudaPeekAtLastError();  // the caller's launch check reads and clears it
}
cudaError_t sfd_launch_assemble32(const SurfaceDesc* surf, const int4* tiles, int ntiles, const float4* wdf,
                                  const float4* pdf, const cd* p, const cd* zp, const double* mdiag, float* mat,
                                  cudaStream_t st) {
  k_assemble32<<<ntiles, 256, 0, st>>>(surf, tiles, wdf, pdf, p, zp, mdiag, mat);
  return cudaPeekAtLastError();
}

// =============================================================== FP64 LU
// Step kb (block column k0 = 64 kb) of the right-looking LU without row
// exchanges.  One CTA per surface factors the 64x64 diagonal block in shared
// memory.
// Copy a rows x cols FP64 tile (row stride lds in the source) into shared
// memory with row stride ldd, NT threads, B loads in flight per thread before
// the stores (a dependent load-store loop would pay one memory latency per
// element).  With transpose, dst[c * ldd + r] = src[r * lds + c].
template <int NT, int B, bool TRANSPOSE = false>
__device__ __forceinline__ void load_tile(double* dst, int ldd, const double* src, long long lds, int rows, int cols) {
  const int total = rows * cols;
  for (int e0 = 0; e0 < total; e0 += NT * B) {
    double t[B];
#pragma unroll
    for (int b = 0; b < B; ++b) {
      const int e = e0 + b * NT + threadIdx.x;
      t[b] = e < total ? src[(long long)(e / cols) * lds + (e % cols)] : 0.0;
    }
#pragma unroll
    for (int b = 0; b < B; ++b) {
      const int e = e0 + b * NT + threadIdx.x;
      if (e < total) {
        if (TRANSPOSE) dst[(e % cols) * ldd + e / cols] = t[b];
        else dst[(e / cols) * ldd + (e % cols)] = t[b];
      }
    }
  }
}

__global__ void __launch_bounds__(256) k_lu64_diag(const SurfaceDesc* surf, int nsurf, int kb, double* mat,
                                                   unsigned int* status, double* lmax) {
  const int s = blockIdx.x;
  if (s >= nsurf) return;
  const SurfaceDesc& S = surf[s];
  const int np = pad_n(S.n), k0 = kb * 64;
  if (k0 >= np) return;
  double* A = mat + S.moff;
  __shared__ double D[64][65];
  load_tile<256, 16>(&D[0][0], 65, A + (long long)k0 * np + k0, np, 64, 64);
  __syncthreads();
  double lm = 0.0;
  for (int c = 0; c < 64; ++c) {
    double piv = D[c][c];
    if (threadIdx.x == 0 && !(fabs(piv) > 1e-300)) atomicOr(status + s, SFD_ST_ZERO_PIVOT);
    double inv = 1.0 / piv;
    __syncthreads();
    for (int i = c + 1 + threadIdx.x; i < 64; i += 256) {
      double l = D[i][c] * inv;
      D[i][c] = l;
      lm = fmax(lm, fabs(l));
    }
    __syncthreads();
    for (int e = threadIdx.x; e < (63 - c) * (63 - c); e += 256) {
      int i = c + 1 + e / (63 - c), j = c + 1 + e % (63 - c);
      D[i][j] -= D[i][c] * D[c][j];
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < 64 * 64; e += 256) A[(long long)(k0 + (e >> 6)) * np + k0 + (e & 63)] = D[e >> 6][e & 63];
  for (int o = 16; o > 0; o >>= 1) lm = fmax(lm, __shfl_xor_sync(0xffffffffu, lm, o));
  if ((threadIdx.x & 31) == 0 && lm > 0) atomicMax(reinterpret_cast<unsigned long long*>(lmax) + s, __double_as_longlong(lm));
}

// Triangular updates of step kb: blockIdx.y == 0 -> L21 row tiles
// (x U11 = a, row-wise); blockIdx.y == 1 -> U12 column tiles (L11 x = a).
__global__ void __launch_bounds__(64) k_lu64_trsm(const SurfaceDesc* surf, int nsurf, int kb, double* mat,
                                                  double* lmax) {
  const int s = blockIdx.z;
  const SurfaceDesc& S = surf[s];
  const int np = pad_n(S.n), k0 = kb * 64;
  const int tile = kb + 1 + blockIdx.x;
  if (tile * 64 >= np) return;
  double* A = mat + S.moff;
  extern __shared__ double trsm_smem[];  // 2 x 64 x 65 doubles (kTrsmSmem bytes)
  double(*D)[65] = reinterpret_cast<double(*)[65]>(trsm_smem);
  double(*X)[65] = reinterpret_cast<double(*)[65]>(trsm_smem + 64 * 65);  // X[t]: thread t's row / column
  load_tile<64, 16>(&D[0][0], 65, A + (long long)k0 * np + k0, np, 64, 64);
  const int t = threadIdx.x;
  if (blockIdx.y == 0)  // rows tile*64 + r: solve x U = a (U upper incl. diagonal)
    load_tile<64, 16>(&X[0][0], 65, A + (long long)(tile * 64) * np + k0, np, 64, 64);
  else  // columns tile*64 + c, stored as X[c][r]
    load_tile<64, 16, true>(&X[0][0], 65, A + (long long)k0 * np + tile * 64, np, 64, 64);
  __syncthreads();
  if (blockIdx.y == 0) {
    double lm = 0.0;
    for (int c = 0; c < 64; ++c) {
      double v = X[t][c];
      for (int q = 0; q < c; ++q) v -= X[t][q] * D[q][c];
      v = v / D[c][c];
      X[t][c] = v;
      lm = fmax(lm, fabs(v));
    }
    for (int o = 16; o > 0; o >>= 1) lm = fmax(lm, __shfl_xor_sync(0xffffffffu, lm, o));
    if ((t & 31) == 0 && lm > 0) atomicMax(reinterpret_cast<unsigned long long*>(lmax) + s, __double_as_longlong(lm));
  } else {
    // column tile*64 + t: solve L x = a (L unit lower)
    for (int r = 0; r < 64; ++r) {
      double v = X[t][r];
      for (int q = 0; q < r; ++q) v -= D[r][q] * X[t][q];
      X[t][r] = v;
    }
  }
  __syncthreads();
  if (blockIdx.y == 0) {
    for (int e = t; e < 64 * 64; e += 64) A[(long long)(tile * 64 + (e >> 6)) * np + k0 + (e & 63)] = X[e >> 6][e & 63];
  } else {
    for (int e = t; e < 64 * 64; e += 64) A[(long long)(k0 + (e >> 6)) * np + tile * 64 + (e & 63)] = X[e & 63][e >> 6];
  }
}

// Partial-pivoting panel of step kb (LAPACK getf2 on the tall panel): one CTA
// per surface walks the 64 columns of [k0, np) x [k0, k0 + 64) in global
// memory (L2-resident): pivot search (largest |a_ik|, first row on ties, as
// idamax), row exchange inside the panel, scaling by the pivot, rank-1 update
// of the panel's remaining columns.  The exchanges outside the panel are
// applied afterwards by k_lu64_swap.  A zero pivot sets SFD_ST_ZERO_PIVOT and
// an exchange SFD_ST_PIVOT_SWAP.  This is the fallback / reference-semantics
// path, so it favours simplicity over speed: the exchange-free LU above is the
// fast path.
__global__ void __launch_bounds__(1024) k_lu64_panel_piv(const SurfaceDesc* surf, int nsurf, int kb, double* mat,
                                                         int* piv, unsigned int* status) {
  const int s = blockIdx.x;
  if (s >= nsurf) return;
  const SurfaceDesc& S = surf[s];
  const int np = pad_n(S.n), k0 = kb * 64;
  if (k0 >= np) return;
  double* A = mat + S.moff;
  __shared__ double rv[32];
  __shared__ int ri[32];
  __shared__ int sp;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  for (int c = 0; c < 64; ++c) {
    const int k = k0 + c;
    // pivot search over rows [k, np)
    double best = -1.0;
    int bi = np;
    for (int i = k + tid; i < np; i += blockDim.x) {
      const double v = fabs(A[(long long)i * np + k]);
      if (v > best) { best = v; bi = i; }  // rows ascend per thread: first maximum kept
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
    }
    if (lane == 0) { rv[warp] = best; ri[warp] = bi; }
    __syncthreads();
    if (tid == 0) {
      double b = rv[0];
      int i0 = ri[0];
      for (int w = 1; w < nw; ++w)
        if (rv[w] > b || (rv[w] == b && ri[w] < i0)) { b = rv[w]; i0 = ri[w]; }
      if (i0 >= np) i0 = k;  // NaN column: keep the diagonal
      if (!(b > 0.0)) atomicOr(status + s, SFD_ST_ZERO_PIVOT);
      if (i0 != k) atomicOr(status + s, SFD_ST_PIVOT_SWAP);
      piv[(long long)s * np + k] = i0;
      sp = i0;
    }
    __syncthreads();
    const int p = sp;
    if (p != k && tid < 64) {
      double* rk = A + (long long)k * np + k0;
      double* rp = A + (long long)p * np + k0;
      const double t = rk[tid];
      rk[tid] = rp[tid];
      rp[tid] = t;
    }
    __syncthreads();
    const double inv = 1.0 / A[(long long)k * np + k];
    for (int i = k + 1 + tid; i < np; i += blockDim.x) A[(long long)i * np + k] *= inv;
    __syncthreads();
    const int w = 63 - c;  // remaining panel columns
    if (w > 0) {
      const double* rk = A + (long long)k * np + k + 1;
      for (long long e = tid; e < (long long)(np - k - 1) * w; e += blockDim.x) {
        const int i = k + 1 + (int)(e / w), j = (int)(e % w);
        double* ai = A + (long long)i * np + k;
        ai[1 + j] -= ai[0] * rk[j];
      }
    }
    __syncthreads();
  }
}

// Row exchanges of panel kb applied to the columns outside the panel, one
// thread per column, the panel's 64 exchanges in order.
__global__ void __launch_bounds__(256) k_lu64_swap(const SurfaceDesc* surf, int nsurf, int kb, double* mat,
                                                   const int* piv) {
  const int s = blockIdx.y;
  if (s >= nsurf) return;
  const SurfaceDesc& S = surf[s];
  const int np = pad_n(S.n), k0 = kb * 64;
  if (k0 >= np) return;
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= np - 64) return;
  if (j >= k0) j += 64;  // skip the panel's own columns
  double* A = mat + S.moff;
  const int* P = piv + (long long)s * np;
  for (int c = 0; c < 64; ++c) {
    const int k = k0 + c, p = P[k];
    if (p != k) {
      const double t = A[(long long)k * np + j];
      A[(long long)k * np + j] = A[(long long)p * np + j];
      A[(long long)p * np + j] = t;
    }
  }
}

// U12 tiles of step kb: columns tile*64 + t solve L11 x = a (L11 unit lower),
// the U12 branch of k_lu64_trsm on its own (the pivoted panel already holds L21).
__global__ void __launch_bounds__(64) k_lu64_trsm_u(const SurfaceDesc* surf, int nsurf, int kb, double* mat) {
  const int s = blockIdx.z;
  if (s >= nsurf) return;
  const SurfaceDesc& S = surf[s];
  const int np = pad_n(S.n), k0 = kb * 64;
  const int tile = kb + 1 + blockIdx.x;
  if (tile * 64 >= np) return;
  double* A = mat + S.moff;
  extern __shared__ double trsm_smem[];  // 2 x 64 x 65 doubles (kTrsmSmem bytes)
  double(*D)[65] = reinterpret_cast<double(*)[65]>(trsm_smem);
  double(*X)[65] = reinterpret_cast<double(*)[65]>(trsm_smem + 64 * 65);
  load_tile<64, 16>(&D[0][0], 65, A + (long long)k0 * np + k0, np, 64, 64);
  load_tile<64, 16, true>(&X[0][0], 65, A + (long long)k0 * np + tile * 64, np, 64, 64);
  __syncthreads();
  const int t = threadIdx.x;
  for (int r = 0; r < 64; ++r) {
    double v = X[t][r];
    for (int q = 0; q < r; ++q) v -= D[r][q] * X[t][q];
    X[t][r] = v;
  }
  __syncthreads();
  for (int e = t; e < 64 * 64; e += 64) A[(long long)(k0 + (e >> 6)) * np + tile * 64 + (e & 63)] = X[e & 63][e >> 6];
}

// Trailing update A22 -= L21 U12 for step kb: 32x32 output tiles (four per
// 64x64 block, so small matrices still fill the GPU), K = 64, 2x2 outputs per
// thread.  grid = (2 rem, 2 rem, surfaces).
__global__ void __launch_bounds__(256) k_lu64_gemm(const SurfaceDesc* surf, int nsurf, int kb, double* mat) {
  const int s = blockIdx.z;
  const SurfaceDesc& S = surf[s];
  const int np = pad_n(S.n), k0 = kb * 64;
  const int r0 = k0 + 64 + 32 * blockIdx.y, c0 = k0 + 64 + 32 * blockIdx.x;
  if (r0 >= np || c0 >= np) return;
  double* A = mat + S.moff;
  __shared__ double La[32][65];
  __shared__ double Ub[64][33];
  load_tile<256, 8>(&La[0][0], 65, A + (long long)r0 * np + k0, np, 32, 64);
  load_tile<256, 8>(&Ub[0][0], 33, A + (long long)k0 * np + c0, np, 64, 32);
  __syncthreads();
  const int tr = (threadIdx.x >> 4) * 2, tc = (threadIdx.x & 15) * 2;
  double a00 = 0, a01 = 0, a10 = 0, a11 = 0;
#pragma unroll 8
  for (int q = 0; q < 64; ++q) {
    const double x0 = La[tr][q], x1 = La[tr + 1][q], y0 = Ub[q][tc], y1 = Ub[q][tc + 1];
    a00 = fma(x0, y0, a00);
    a01 = fma(x0, y1, a01);
    a10 = fma(x1, y0, a10);
    a11 = fma(x1, y1, a11);
  }
  double* o = A + (long long)(r0 + tr) * np + c0 + tc;
  o[0] -= a00;
  o[1] -= a01;
  o[np] -= a10;
  o[np + 1] -= a11;
}

// Forward (unit L) then backward (U) substitution, one CTA per surface, in
// 64-row blocks: block dot products by all warps, then warp 0 finishes the
// 64x64 triangle.  x (length n) is overwritten with the solution.
__global__ void __launch_bounds__(256) k_lu64_solve(const SurfaceDesc* surf, const double* mat, const double* b,
                                                    double* x, double* acc, const int* piv, Gate gate,
                                                    const double* lmax, unsigned int* status) {
  const int s = blockIdx.x;
  if (!gate_open(gate, s)) return;
  const SurfaceDesc& S = surf[s];
  const int n = S.n, np = pad_n(n), off = S.off;
  const double* A = mat + S.moff;
  if (lmax && threadIdx.x == 0 && lmax[s] > 1.0) atomicOr(status + s, SFD_ST_PIVOT_SWAP);
  extern __shared__ double xs[];  // np doubles
  for (int i = threadIdx.x; i < np; i += 256) xs[i] = i < n ? b[off + i] : 0.0;
  __syncthreads();
  if (piv) {  // row exchanges of the factorisation, in order (getrs applies them to b first)
    if (threadIdx.x == 0) {
      const int* P = piv + (long long)s * np;
      for (int k = 0; k < n; ++k) {
        const int p = P[k];
        if (p != k && p >= 0 && p < np) {
          const double t = xs[k];
          xs[k] = xs[p];
          xs[p] = t;
        }
      }
    }
    __syncthreads();
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nblk = np / 64;
  // forward: x_i = b_i - sum_{j<i} L_ij x_j
  for (int B = 0; B < nblk; ++B) {
    int r0 = B * 64;
    for (int rr = warp; rr < 64; rr += 8) {
      const double* row = A + (long long)(r0 + rr) * np;
      double sacc = 0.0;
      for (int j = lane; j < r0; j += 32) sacc += row[j] * xs[j];
      for (int o = 16; o > 0; o >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, o);
      if (lane == 0) xs[r0 + rr] -= sacc;
    }
    __syncthreads();
    if (warp == 0) {
      for (int c = 0; c < 64; ++c) {
        double xc = xs[r0 + c];
        for (int r = c + 1 + lane; r < 64; r += 32) xs[r0 + r] -= A[(long long)(r0 + r) * np + r0 + c] * xc;
        __syncwarp();
      }
    }
    __syncthreads();
  }
  // backward: x_i = (x_i - sum_{j>i} U_ij x_j) / U_ii
  for (int B = nblk - 1; B >= 0; --B) {
    int r0 = B * 64;
    for (int rr = warp; rr < 64; rr += 8) {
      const double* row = A + (long long)(r0 + rr) * np;
      double sacc = 0.0;
      for (int j = r0 + 64 + lane; j < np; j += 32) sacc += row[j] * xs[j];
      for (int o = 16; o > 0; o >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, o);
      if (lane == 0) xs[r0 + rr] -= sacc;
    }
    __syncthreads();
    if (warp == 0) {
      for (int c = 63; c >= 0; --c) {
        double xc;
        if (lane == 0) xs[r0 + c] = xs[r0 + c] / A[(long long)(r0 + c) * np + r0 + c];
        __syncwarp();
        xc = xs[r0 + c];
        for (int r = lane; r < c; r += 32) xs[r0 + r] -= A[(long long)(r0 + r) * np + r0 + c] * xc;
        __syncwarp();
      }
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < n; i += 256) {
    if (x) x[off + i] = xs[i];
    if (acc) acc[off + i] += xs[i];
  }
}

// =============================================================== FP32 Gauss-Jordan inverse
// Step kb (block K = [128 kb, 128 kb + 128)):
//   P = inv(A_KK)                        k_gj_diag   (one CTA per surface)
//   R = P A_K,:  and  C = A_:,K  (copies) k_gj_panel
//   A_ij -= C_i R_j (i,j not in K); A_Kj = R_j; A_iK = -C_i P; A_KK = P   k_gj_update
// In-register Gauss-Jordan inverse of a 32 x 32 block held by one warp
// (lane l holds row l); the pivot row is broadcast with shuffles, so no block
// barrier is needed.  Returns false on a zero pivot.
__device__ __forceinline__ bool warp_gj32(float (&r)[32]) {
  const int lane = threadIdx.x & 31;
  bool ok = true;
#pragma unroll
  for (int c = 0; c < 32; ++c) {
    const float piv = __shfl_sync(0xffffffffu, r[c], c);
    ok &= fabsf(piv) > 1e-30f;
    const float pinv = 1.0f / piv;
    const float colc = r[c];
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const float rj = __shfl_sync(0xffffffffu, r[j], c) * pinv;
      if (lane == c) r[j] = (j == c) ? pinv : rj;
      else r[j] = (j == c) ? -colc * pinv : fmaf(-colc, rj, r[j]);
    }
  }
  return ok;
}

// P = inv(A_KK) for the 128 x 128 diagonal block, blocked Gauss-Jordan with
// 32-wide panels: warp 0 inverts the 32 x 32 pivot block in registers, then all
// threads apply the rank-32 update to the block in shared memory.
__global__ void __launch_bounds__(512) k_gj_diag(const SurfaceDesc* surf, int nsurf, int kb, float* mat, float* pbuf,
                                                 unsigned int* status) {
  const int s = blockIdx.x;
  const SurfaceDesc& S = surf[s];
  const int np = pad_n(S.n), k0 = kb * 128;
  if (k0 >= np) return;
  const float* A = mat + S.moff;
  extern __shared__ float dsm[];
  float* D = dsm;                // 128 x 129
  float* Cq = D + 128 * 129;     // 128 x 33: column panel (before the update)
  float* Rq = Cq + 128 * 33;     // 32 x 128: P * row panel (P itself inside the panel)
  float* Pq = Rq + 32 * 128;     // 32 x 33
  for (int e = threadIdx.x; e < 128 * 128; e += 512) D[(e >> 7) * 129 + (e & 127)] = A[(long long)(k0 + (e >> 7)) * np + k0 + (e & 127)];
  __syncthreads();
  bool ok = true;
  for (int q = 0; q < 4; ++q) {
    const int q0 = 32 * q;
    if (threadIdx.x < 32) {
      float r[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) r[j] = D[(q0 + threadIdx.x) * 129 + q0 + j];
      ok &= warp_gj32(r);
#pragma unroll
      for (int j = 0; j < 32; ++j) Pq[threadIdx.x * 33 + j] = r[j];
    }
    for (int e = threadIdx.x; e < 128 * 32; e += 512) Cq[(e >> 5) * 33 + (e & 31)] = D[(e >> 5) * 129 + q0 + (e & 31)];
    __syncthreads();
    // R = P * D[panel rows, :] (inside the panel: P itself); thread -> row i, 8 columns
    {
      const int i = threadIdx.x >> 4, jb = (threadIdx.x & 15) * 8;
      const bool jk = (jb >= q0 && jb < q0 + 32);
      float v[8];
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) v[jj] = jk ? Pq[i * 33 + jb + jj - q0] : 0.f;
      if (!jk) {
        for (int k = 0; k < 32; ++k) {
          const float pk = Pq[i * 33 + k];
          const float* drow = D + (q0 + k) * 129 + jb;
#pragma unroll
          for (int jj = 0; jj < 8; ++jj) v[jj] = fmaf(pk, drow[jj], v[jj]);
        }
      }
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) Rq[i * 128 + jb + jj] = v[jj];
    }
    __syncthreads();
    // D update; thread -> 4 rows x 8 columns (panel membership uniform per tile)
    {
      const int ib = (threadIdx.x >> 4) * 4, jb = (threadIdx.x & 15) * 8;
      const bool ik = (ib >= q0 && ib < q0 + 32), jk = (jb >= q0 && jb < q0 + 32);
      float v[4][8];
      if (ik) {
#pragma unroll
        for (int ii = 0; ii < 4; ++ii)
#pragma unroll
          for (int jj = 0; jj < 8; ++jj) v[ii][jj] = Rq[(ib + ii - q0) * 128 + jb + jj];
      } else {
        const float* bsrc = jk ? Pq : Rq;
        const int bld = jk ? 33 : 128, boff = jk ? jb - q0 : jb;
#pragma unroll
        for (int ii = 0; ii < 4; ++ii)
#pragma unroll
          for (int jj = 0; jj < 8; ++jj) v[ii][jj] = jk ? 0.f : D[(ib + ii) * 129 + jb + jj];
        for (int k = 0; k < 32; ++k) {
          float c[4], b[8];
#pragma unroll
          for (int ii = 0; ii < 4; ++ii) c[ii] = Cq[(ib + ii) * 33 + k];
#pragma unroll
          for (int jj = 0; jj < 8; ++jj) b[jj] = bsrc[k * bld + boff + jj];
#pragma unroll
          for (int ii = 0; ii < 4; ++ii)
#pragma unroll
            for (int jj = 0; jj < 8; ++jj) v[ii][jj] = fmaf(-c[ii], b[jj], v[ii][jj]);
        }
      }
      __syncthreads();  // every thread has read D / Cq / Rq / Pq before D is rewritten
#pragma unroll
      for (int ii = 0; ii < 4; ++ii)
#pragma unroll
        for (int jj = 0; jj < 8; ++jj) D[(ib + ii) * 129 + jb + jj] = v[ii][jj];
    }
    __syncthreads();
  }
  if (!ok && threadIdx.x == 0) atomicOr(status + s, SFD_ST_ZERO_PIVOT);
  float* P = pbuf + (long long)s * 128 * 128;
  for (int e = threadIdx.x; e < 128 * 128; e += 512) P[e] = D[(e >> 7) * 129 + (e & 127)];
}

// x = hi + mid + lo in bf16 (24 significant bits: exact for an FP32 value up to
// the last rounding); parts are `stride` elements apart.
__device__ __forceinline__ void split_bf16x3(float x, __nv_bfloat16* dst, long long stride) {
  __nv_bfloat16 hi = __float2bfloat16_rn(x);
  float r1 = x - __bfloat162float(hi);
  __nv_bfloat16 mid = __float2bfloat16_rn(r1);
  float r2 = r1 - __bfloat162float(mid);
  dst[0] = hi;
  dst[stride] = mid;
  dst[2 * stride] = __float2bfloat16_rn(r2);
}

__global__ void __launch_bounds__(256) k_gj_panel(const SurfaceDesc* surf, int nsurf, int kb, const float* mat,
                                                  const float* pbuf, float* rbuf, float* cbuf, const long long* poff,
                                                  __nv_bfloat16* cparts, __nv_bfloat16* rparts, long long pstride) {
  const int s = blockIdx.z;
  const SurfaceDesc& S = surf[s];
  const int np = pad_n(S.n), k0 = kb * 128;
  if (k0 >= np) return;
  const int t = blockIdx.x;  // tile index over np/64
  if (t * 64 >= np) return;
  const float* A = mat + S.moff;
  const float* P = pbuf + (long long)s * 128 * 128;
  float* R = rbuf + poff[s];  // 128 x np
  float* C = cbuf + poff[s];  // np x 128
  // C copy (rows t*64 .. +64, all 128 columns of K)
  for (int e = threadIdx.x; e < 64 * 128; e += 256) {
    int r = t * 64 + (e >> 7), c = e & 127;
    float v = A[(long long)r * np + k0 + c];
    C[(long long)r * 128 + c] = v;
    if (cparts) split_bf16x3(v, cparts + poff[s] + (long long)r * 128 + c, pstride);
  }
  if (t * 64 >= k0 && t * 64 < k0 + 128) return;  // columns inside K: R not needed
  // shared memory: the GEMM operands, then (reused) the transposed tile
  __shared__ float sm[64 * 129];
  float (*Pt)[33] = reinterpret_cast<float (*)[33]>(sm);            // 128 x 33
  float (*Bt)[65] = reinterpret_cast<float (*)[65]>(sm + 128 * 33);  // 32 x 65
  const int tr = (threadIdx.x >> 4) * 8, tc = (threadIdx.x & 15) * 4;  // 16 x 16 threads -> 128 x 64
  float acc[8][4] = {};
  for (int q0 = 0; q0 < 128; q0 += 32) {
    __syncthreads();
    for (int e = threadIdx.x; e < 128 * 32; e += 256) Pt[e >> 5][e & 31] = P[(e >> 5) * 128 + q0 + (e & 31)];
    for (int e = threadIdx.x; e < 32 * 64; e += 256) Bt[e >> 6][e & 63] = A[(long long)(k0 + q0 + (e >> 6)) * np + t * 64 + (e & 63)];
    __syncthreads();
    for (int q = 0; q < 32; ++q) {
      float b[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bt[q][tc + j];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        float a = Pt[tr + i][q];
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a, b[j], acc[i][j]);
      }
    }
  }
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) R[(long long)(tr + i) * np + t * 64 + tc + j] = acc[i][j];
  if (rparts) {
    // R^T (K-major) for the tensor-core update: transpose through shared memory,
    // then write each R^T row (128 values, three bf16 parts) coalesced
    __syncthreads();
    float (*Rs)[129] = reinterpret_cast<float (*)[129]>(sm);  // 64 x 129
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) Rs[tc + j][tr + i] = acc[i][j];
    __syncthreads();
    for (int e = threadIdx.x; e < 64 * 128; e += 256) {
      int jl = e >> 7, k = e & 127;
      split_bf16x3(Rs[jl][k], rparts + poff[s] + (long long)(t * 64 + jl) * 128 + k, pstride);
    }
  }
}

// Output tile 64 x 64 (ti, tj) over the whole padded matrix.
// k_lines_only != 0: grid.x enumerates only the 64x64 tiles of block row K and
// block column K (4 T - 4 of them, T = n_pad / 64); the tensor-core kernel
// updates the rest.  Otherwise grid (T, T) covers every tile.
__global__ void __launch_bounds__(256) k_gj_update(const SurfaceDesc* surf, int nsurf, int kb, float* mat,
                                                   const float* pbuf, const float* rbuf, const float* cbuf,
                                                   const long long* poff, int k_lines_only) {
  const int s = blockIdx.z;
  const SurfaceDesc& S = surf[s];
  const int np = pad_n(S.n), k0 = kb * 128;
  if (k0 >= np) return;
  int ti = blockIdx.y, tj = blockIdx.x;
  if (k_lines_only) {
    const int T = np / 64, K64 = k0 / 64, idx = blockIdx.x;
    if (idx >= 4 * T - 4) return;
    if (idx < 2 * T) {
      ti = K64 + idx / T;
      tj = idx % T;
    } else {
      const int i2 = idx - 2 * T, r = i2 % (T - 2);
      tj = K64 + i2 / (T - 2);
      ti = r < K64 ? r : r + 2;
    }
  }
  if (ti * 64 >= np || tj * 64 >= np) return;
  float* A = mat + S.moff;
  const float* P = pbuf + (long long)s * 128 * 128;
  const float* R = rbuf + poff[s];
  const float* C = cbuf + poff[s];
  const bool iK = (ti * 64 >= k0 && ti * 64 < k0 + 128);
  const bool jK = (tj * 64 >= k0 && tj * 64 < k0 + 128);
  if (iK && jK) {
    for (int e = threadIdx.x; e < 64 * 64; e += 256) {
      int r = e >> 6, c = e & 63;
      A[(long long)(ti * 64 + r) * np + tj * 64 + c] = P[(ti * 64 - k0 + r) * 128 + tj * 64 - k0 + c];
    }
    return;
  }
  if (iK) {
    for (int e = threadIdx.x; e < 64 * 64; e += 256) {
      int r = e >> 6, c = e & 63;
      A[(long long)(ti * 64 + r) * np + tj * 64 + c] = R[(long long)(ti * 64 - k0 + r) * np + tj * 64 + c];
    }
    return;
  }
  __shared__ float Ct[64][33];
  __shared__ float Bt[32][65];
  const int tr = (threadIdx.x >> 4) * 4, tc = (threadIdx.x & 15) * 4;
  float acc[4][4] = {};
  for (int q0 = 0; q0 < 128; q0 += 32) {
    __syncthreads();
    for (int e = threadIdx.x; e < 64 * 32; e += 256) Ct[e >> 5][e & 31] = C[(long long)(ti * 64 + (e >> 5)) * 128 + q0 + (e & 31)];
    if (jK) {
      for (int e = threadIdx.x; e < 32 * 64; e += 256) Bt[e >> 6][e & 63] = P[(q0 + (e >> 6)) * 128 + tj * 64 - k0 + (e & 63)];
    } else {
      for (int e = threadIdx.x; e < 32 * 64; e += 256) Bt[e >> 6][e & 63] = R[(long long)(q0 + (e >> 6)) * np + tj * 64 + (e & 63)];
    }
    __syncthreads();
    for (int q = 0; q < 32; ++q) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = Ct[tr + i][q];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bt[q][tc + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      float* dst = A + (long long)(ti * 64 + tr + i) * np + tj * 64 + tc + j;
      *dst = jK ? -acc[i][j] : *dst - acc[i][j];
    }
}

// =============================================================== GEMV
// y[off + i] = sum_j X_ij v[off + j]  (X float or half, v float, y double).  A
// CTA covers kGemvRows rows: v (an FP32 copy written by the producer of the
// vector, so no CTA converts from FP64) is staged in shared memory, and the
// warps walk their rows with 16-byte loads (rows are 16-byte aligned: n_pad is
// a multiple of 128, and X[i][j] = 0 for j >= n in the padded inverse).
// Stage an FP32 vector (n entries, zero-padded to n_stage) in shared memory.
template <int NT>
__device__ __forceinline__ void stage_vector_f(float* vs, const float* v, int n, int n_stage) {
  for (int j = threadIdx.x; j < n_stage; j += NT) vs[j] = j < n ? v[j] : 0.f;
}

// Epilogue of the products: y (FP64, nullable), its double-float copy ydf
// (nullable), and the in-place update acc += y with the double-float copy of
// the new value (both nullable).
__device__ __forceinline__ void gemv_store(float yr, int g, double* y, float2* ydf, double* acc, float2* accdf) {
  const double d = (double)yr;
  if (y) y[g] = d;
  if (ydf) ydf[g] = make_float2(yr, 0.f);
  if (acc) {
    const double v = acc[g] + d;
    acc[g] = v;
    if (accdf) {
      const float hi = __double2float_rn(v);
      accdf[g] = make_float2(hi, __double2float_rn(v - (double)hi));
    }
  }
}

__global__ void __launch_bounds__(256) k_gemv(const SurfaceDesc* surf, const int2* rowblk, const float* mat,
                                              const float* v, double* y, float2* ydf, double* accv, float2* accdf,
                                              Gate gate) {
  sfd_pdl_begin();
  const int2 rb = rowblk[blockIdx.x];  // (surface, first row)
  if (!gate_open(gate, rb.x)) return;
  const SurfaceDesc& S = surf[rb.x];
  const int n = S.n, np = pad_n(n), off = S.off;
  extern __shared__ float4 vs4[];
  float* vs = reinterpret_cast<float*>(vs4);
  const int n4 = (n + 3) & ~3;
  stage_vector_f<256>(vs, v + off, n, n4);
  __syncthreads();
  const float* X = mat + S.moff;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r0 = rb.y + 2 * warp, r1 = r0 + 1;
  if (r0 >= n) return;
  const float4* x0 = reinterpret_cast<const float4*>(X + (long long)r0 * np);
  const float4* x1 = reinterpret_cast<const float4*>(X + (long long)(r1 < n ? r1 : r0) * np);
  float acc0 = 0.f, acc1 = 0.f;
  const int nq = n4 / 4;
  int q = lane;
  for (; q + 96 < nq; q += 128) {  // four 16-byte loads per row in flight
    float4 a0 = __ldg(x0 + q), a1 = __ldg(x0 + q + 32), a2 = __ldg(x0 + q + 64), a3 = __ldg(x0 + q + 96);
    float4 b0 = __ldg(x1 + q), b1 = __ldg(x1 + q + 32), b2 = __ldg(x1 + q + 64), b3 = __ldg(x1 + q + 96);
    float4 v0 = vs4[q], v1 = vs4[q + 32], v2 = vs4[q + 64], v3 = vs4[q + 96];
    acc0 = fmaf(a0.x, v0.x, fmaf(a0.y, v0.y, fmaf(a0.z, v0.z, fmaf(a0.w, v0.w, acc0))));
    acc1 = fmaf(b0.x, v0.x, fmaf(b0.y, v0.y, fmaf(b0.z, v0.z, fmaf(b0.w, v0.w, acc1))));
    acc0 = fmaf(a1.x, v1.x, fmaf(a1.y, v1.y, fmaf(a1.z, v1.z, fmaf(a1.w, v1.w, acc0))));
    acc1 = fmaf(b1.x, v1.x, fmaf(b1.y, v1.y, fmaf(b1.z, v1.z, fmaf(b1.w, v1.w, acc1))));
    acc0 = fmaf(a2.x, v2.x, fmaf(a2.y, v2.y, fmaf(a2.z, v2.z, fmaf(a2.w, v2.w, acc0))));
    acc1 = fmaf(b2.x, v2.x, fmaf(b2.y, v2.y, fmaf(b2.z, v2.z, fmaf(b2.w, v2.w, acc1))));
    acc0 = fmaf(a3.x, v3.x, fmaf(a3.y, v3.y, fmaf(a3.z, v3.z, fmaf(a3.w, v3.w, acc0))));
    acc1 = fmaf(b3.x, v3.x, fmaf(b3.y, v3.y, fmaf(b3.z, v3.z, fmaf(b3.w, v3.w, acc1))));
  }
  for (; q < nq; q += 32) {
    float4 vv = vs4[q];
    float4 a = __ldg(x0 + q), b = __ldg(x1 + q);
    acc0 = fmaf(a.x, vv.x, fmaf(a.y, vv.y, fmaf(a.z, vv.z, fmaf(a.w, vv.w, acc0))));
    acc1 = fmaf(b.x, vv.x, fmaf(b.y, vv.y, fmaf(b.z, vv.z, fmaf(b.w, vv.w, acc1))));
  }
  for (int o = 16; o > 0; o >>= 1) {
    acc0 += __shfl_xor_sync(0xffffffffu, acc0, o);
    acc1 += __shfl_xor_sync(0xffffffffu, acc1, o);
  }
  if (lane == 0) {
    gemv_store(acc0, off + r0, y, ydf, accv, accdf);
    if (r1 < n) gemv_store(acc1, off + r1, y, ydf, accv, accdf);
  }
}

// FP16 copy of the preconditioner for the GEMVs: row r is scaled by a power of
// two 2^s_r so that its largest entry lies in [2^13, 2^14) (exact scaling, no
// subnormals for entries down to 2^-10 of the row maximum); rscale[row] =
// 2^-s_r undoes it.  Same CTA / warp layout as k_gemv: 16 rows per CTA.
__global__ void __launch_bounds__(256) k_precond_to_half(const SurfaceDesc* surf, const int2* rowblk,
                                                         const float* mat, __half* mat16, float* rscale) {
  const int2 rb = rowblk[blockIdx.x];
  const SurfaceDesc& S = surf[rb.x];
  const int n = S.n, np = pad_n(n), off = S.off;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int rr = 0; rr < 2; ++rr) {
    const int r = rb.y + 2 * warp + rr;
    if (r >= n) break;
    const float* X = mat + S.moff + (long long)r * np;
    __half* H = mat16 + S.moff + (long long)r * np;
    float m = 0.f;
    for (int j = lane; j < np; j += 32) m = fmaxf(m, fabsf(X[j]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    int ex = 0;
    frexpf(m > 0.f ? m : 1.f, &ex);  // m < 2^ex
    const float sc = ldexpf(1.f, 14 - ex);
    for (int j = lane; j < np; j += 32) H[j] = __float2half_rn(X[j] * sc);
    if (lane == 0) rscale[off + r] = ldexpf(1.f, ex - 14);
  }
}

// acc + (8 FP16 entries of a row, chunk q) . (v[8q .. 8q + 8) staged as float4s)
__device__ __forceinline__ float dot8h(uint4 h, const float4* vsh, int q, float acc) {
  const __half2* hp = reinterpret_cast<const __half2*>(&h);
  const float4 va = vsh[2 * q], vb = vsh[2 * q + 1];
  float2 f0 = __half22float2(hp[0]), f1 = __half22float2(hp[1]), f2 = __half22float2(hp[2]),
         f3 = __half22float2(hp[3]);
  acc = fmaf(f0.x, va.x, fmaf(f0.y, va.y, fmaf(f1.x, va.z, fmaf(f1.y, va.w, acc))));
  return fmaf(f2.x, vb.x, fmaf(f2.y, vb.y, fmaf(f3.x, vb.z, fmaf(f3.y, vb.w, acc))));
}

// y = X v with the FP16 copy (FP32 accumulation), y scaled back per row.
// 16 warps per CTA, one row per warp.  Each lane streams its 16-byte chunks
// (8 entries) of the row in batches of four, software-pipelined one batch
// ahead; the first batch is issued before v is staged, so the staging
// latency overlaps the first matrix loads.
// Row blocks (rowblk, nblk entries of (surface, first row), batches): the CTAs
// are persistent and take blocks blockIdx.x, blockIdx.x + gridDim.x, ...; a
// batch of small surfaces would otherwise run as tens of thousands of short
// CTAs.  rowblk null (one surface): rows interleaved over the grid,
// r = block + grid * warp, so every SM gets the same number of rows within one.
// prefetch != 0 (one surface, ungated launches whose immediate predecessor
// does not write the matrix): each warp loads its first batch of the row
// before the wait on the preceding kernel (programmatic dependent launch); by
// then every earlier kernel of the stream has completed.
__global__ void __launch_bounds__(512) k_gemv_h(const SurfaceDesc* surf, const int2* rowblk, int nblk,
                                                const __half* mat16, const float* rscale, const float* v, double* y,
                                                float2* ydf, double* accv, float2* accdf, Gate gate, int prefetch) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint4 cur[4], nxt[4];
  bool have = false;  // cur holds the first batch already
  if (prefetch && !rowblk) {
    const SurfaceDesc& S = surf[0];  // written once at set-up
    const int n = S.n, r = blockIdx.x + gridDim.x * warp, nq = ((n + 7) & ~7) / 8;
    const int per_lane = lane < nq ? (nq - lane + 31) / 32 : 0;
    const uint4* xr = reinterpret_cast<const uint4*>(mat16 + S.moff + (long long)(r < n ? r : 0) * pad_n(n)) + lane;
#pragma unroll
    for (int i = 0; i < 4; ++i) cur[i] = (r < n && i < per_lane) ? __ldg(xr + 32 * i) : make_uint4(0, 0, 0, 0);
    have = true;
  }
  sfd_pdl_begin();
  extern __shared__ float4 vsh[];
  const int nit = rowblk ? nblk : 1;
  for (int blk = rowblk ? (int)blockIdx.x : 0; blk < nit; blk += rowblk ? (int)gridDim.x : 1) {
    int sidx, r;
    if (rowblk) {
      const int2 rb = rowblk[blk];
      sidx = rb.x;
      r = rb.y + warp;
    } else {
      sidx = 0;
      r = blockIdx.x + gridDim.x * warp;
    }
    if (!gate_open(gate, sidx)) continue;  // uniform over the CTA
    const SurfaceDesc& S = surf[sidx];
    const int n = S.n, np = pad_n(n), off = S.off;
    const bool live = r < n;
    const int n8 = (n + 7) & ~7;
    const int nq = n8 / 8;
    const int per_lane = lane < nq ? (nq - lane + 31) / 32 : 0;  // chunks q = lane + 32 i, i < per_lane
    const uint4* xr = reinterpret_cast<const uint4*>(mat16 + S.moff + (long long)(live ? r : 0) * np) + lane;
    if (!have) {
#pragma unroll
      for (int i = 0; i < 4; ++i) cur[i] = (live && i < per_lane) ? __ldg(xr + 32 * i) : make_uint4(0, 0, 0, 0);
    }
    have = false;
    __syncthreads();  // the previous block's readers of vsh are done
    stage_vector_f<512>(reinterpret_cast<float*>(vsh), v + off, n, n8);
    __syncthreads();
    if (!live) continue;
    auto dot8 = [&](uint4 h, int q, float acc) { return dot8h(h, vsh, q, acc); };
    float acc0 = 0.f, acc1 = 0.f;
    for (int b = 0; 4 * b < per_lane; ++b) {
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int idx = 4 * (b + 1) + i;
        nxt[i] = idx < per_lane ? __ldg(xr + 32 * idx) : make_uint4(0, 0, 0, 0);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int idx = 4 * b + i;
        if (idx < per_lane) {
          if (i & 1) acc1 = dot8(cur[i], lane + 32 * idx, acc1);
          else acc0 = dot8(cur[i], lane + 32 * idx, acc0);
        }
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) cur[i] = nxt[i];
    }
    float acc = acc0 + acc1;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) gemv_store(acc * rscale[off + r], off + r, y, ydf, accv, accdf);
  }
}


// ------------------------------------------------ streamed product, one surface
// y = X v for one surface with the FP16 rows streamed into shared memory by
// the copy engine.  One persistent CTA per SM takes the rows r = block +
// grid * i; CTA row i belongs to warp i % 8, and each warp owns `spw` row
// slots: it keeps up to spw whole rows of its own in flight as bulk copies
// (cp.async.bulk, one mbarrier per slot) and refills a slot with its next row
// as soon as it has consumed the row in it.  At N = 4096 with the default two
// slots that is 16 rows (128 KB) in flight per SM, against the 2 KB per warp
// that the register-pipelined k_gemv_h keeps.  Stand-alone it is not faster
// (the copies arrive at about 2 TB/s from DRAM); its gain in the step comes
// from requesting the first rows before the wait on the preceding kernel
// (prefetch below), which a register pipeline can only do for one small
// batch.  The arithmetic is k_gemv_h's entry
// for entry (each lane's chunks in the same order, the same two accumulators,
// the same reduction), so both give the same bits.  A slot is only ever waited
// on and refilled by its own warp, so a wait is never more than one phase
// ahead of the barrier.  A wait that runs out (1 << 22 probes) sets
// SFD_ST_TIMEOUT in the surface status; the warp then stops, waits (bounded)
// for its copies in flight and returns.
// prefetch != 0: the first rows are requested before the wait on the
// preceding kernel of the stream (programmatic dependent launch), so they
// arrive while that kernel finishes.  Only for ungated launches whose
// immediate predecessor does not write the matrix: by then every earlier
// kernel of the stream has completed (each waits on its own predecessor
// before it lets the next one start).
__global__ void __launch_bounds__(32 * kGemvSWarps, 1)
    k_gemv_hs(const SurfaceDesc* surf, int spw, int prefetch, const __half* mat16, const float* rscale,
              const float* v, double* y, float2* ydf, double* accv, float2* accdf, Gate gate,
              unsigned int* status) {
  using namespace sfd_async;
  constexpr unsigned kSpin = 1u << 22;
  const SurfaceDesc& S = surf[0];  // written once at set-up
  const int n = S.n, np = pad_n(n), off = S.off, n8 = (n + 7) & ~7;
  const int G = gridDim.x, b = blockIdx.x;
  const int rows = b < n ? (n - 1 - b) / G + 1 : 0;  // CTA rows i: matrix rows b + G i < n
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wrows = warp < rows ? (rows - 1 - warp) / kGemvSWarps + 1 : 0;  // warp rows j: i = warp + 8 j
  const uint32_t rb = (uint32_t)n8 * 2u;  // bytes per row copy (a multiple of 16)
  extern __shared__ __align__(128) unsigned char gsm[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(gsm) + warp * kGemvSMaxSpw;
  float4* vsh = reinterpret_cast<float4*>(gsm + kGemvSHead);
  unsigned char* slots = gsm + kGemvSHead + ((n8 * 4 + 127) & ~127) + (size_t)warp * spw * rb;
  const char* xrow = reinterpret_cast<const char*>(mat16 + S.moff + (long long)b * np);
  const long long xstride = (long long)G * np * 2;  // bytes from one CTA row to the next
  auto issue = [&](int j) {
    const uint32_t mb = smem_u32(bar + j % spw);
    mbar_expect_tx(mb, rb);
    bulk_g2s(smem_u32(slots + (size_t)(j % spw) * rb), xrow + (long long)(warp + kGemvSWarps * j) * xstride, rb,
             mb);
  };
  const int first = min(spw, wrows);
  auto start = [&] {
    if (lane == 0 && first > 0) {
      for (int k = 0; k < first; ++k) mbar_init(smem_u32(bar + k), 1);
      mbar_init_fence();
      for (int j = 0; j < first; ++j) issue(j);
    }
  };
  if (prefetch) start();
  sfd_pdl_begin();
  if (rows == 0) return;
  if (!prefetch) {
    if (!gate_open(gate, 0)) return;  // uniform over the grid
    start();
  }
  // stage v (zero from n to n8) while the first rows are in flight
  {
    const float* vs = v + off;
    if ((n & 3) == 0 && (reinterpret_cast<uintptr_t>(vs) & 15) == 0) {
      const float4* v4 = reinterpret_cast<const float4*>(vs);
      for (int q = threadIdx.x; q < n8 / 4; q += blockDim.x)
        vsh[q] = 4 * q < n ? v4[q] : make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
      float* vf = reinterpret_cast<float*>(vsh);
      for (int q = threadIdx.x; q < n8; q += blockDim.x) vf[q] = q < n ? vs[q] : 0.f;
    }
  }
  __syncthreads();
  const int nq = n8 / 8;
  const int per_lane = lane < nq ? (nq - lane + 31) / 32 : 0;  // chunks q = lane + 32 t, t < per_lane
  int j = 0;
  for (; j < wrows; ++j) {
    const uint32_t mb = smem_u32(bar + j % spw);
    const uint32_t parity = (uint32_t)(j / spw) & 1u;
    unsigned it = 0;
    while (!mbar_try(mb, parity) && ++it < kSpin) {
    }
    if (!__all_sync(0xffffffffu, it < kSpin)) {
      if (lane == 0) atomicOr(status, SFD_ST_TIMEOUT);
      break;
    }
    const uint4* xs = reinterpret_cast<const uint4*>(slots + (size_t)(j % spw) * rb);
    float acc0 = 0.f, acc1 = 0.f;
    int t = 0;
#pragma unroll 4
    for (; t + 1 < per_lane; t += 2) {
      const int q0 = lane + 32 * t, q1 = q0 + 32;
      const uint4 h0 = xs[q0], h1 = xs[q1];
      acc0 = dot8h(h0, vsh, q0, acc0);
      acc1 = dot8h(h1, vsh, q1, acc1);
    }
    if (t < per_lane) acc0 = dot8h(xs[lane + 32 * t], vsh, lane + 32 * t, acc0);
    float acc = acc0 + acc1;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __syncwarp();  // every lane's reads of the slot are done
    if (lane == 0) {
      const int g = off + b + G * (warp + kGemvSWarps * j);
      gemv_store(acc * rscale[g], g, y, ydf, accv, accdf);
      if (j + spw < wrows) {
        fence_proxy_async_smem();
        issue(j + spw);
      }
    }
  }
  if (j < wrows && lane == 0) {
    // gave up at row j: let the copies in flight (rows j .. j + spw - 1 that
    // were issued) land before the CTA's shared memory is released
    for (int jj = j; jj < min(wrows, j + spw); ++jj) {
      const uint32_t mb = smem_u32(bar + jj % spw);
      for (unsigned w = 0; w < kSpin && !mbar_try(mb, (uint32_t)(jj / spw) & 1u); ++w) {
      }
    }
  }
}

// Plan of the streamed product for one surface of n nodes on `nsm` SMs with
// `smem_max` bytes of shared memory per CTA: row slots per warp (capped at
// cap, and at the rows a warp gets) and the dynamic shared memory; spw = 0
// when one row per warp does not fit.
void sfd_gemv_stream_plan(int n, int nsm, int smem_max, int cap, int* spw, int* smem) {
  *spw = 0;
  *smem = 0;
  if (n < 1 || nsm < 1) return;
  const long long n8 = (n + 7) & ~7, rb = 2 * n8, vbytes = (4 * n8 + 127) & ~127LL;
  const long long room = (long long)smem_max - kGemvSHead - vbytes;
  const int rows_cta = (n + nsm - 1) / nsm, rows_warp = (rows_cta + kGemvSWarps - 1) / kGemvSWarps;
  long long k = room / (kGemvSWarps * rb);
  k = std::min<long long>(k, std::min(kGemvSMaxSpw, std::min(cap, rows_warp)));
  if (k < 1) return;
  *spw = (int)k;
  *smem = (int)(kGemvSHead + vbytes + kGemvSWarps * k * rb);
}

cudaError_t sfd_launch_gemv_stream(const SurfaceDesc* surf, int nsm, int spw, int smem, bool prefetch,
                                   const __half* mat16, const float* rscale, const float* v, double* y, float2* ydf,
                                   double* acc, float2* accdf, const Gate& gate, unsigned int* status,
                                   cudaStream_t st) {
  if (prefetch && gate.slot) return cudaErrorInvalidValue;  // a gated launch may not prefetch
  return sfd_launch(k_gemv_hs, dim3(nsm), dim3(32 * kGemvSWarps), (size_t)smem, st, true, surf, spw,
                    prefetch ? 1 : 0, mat16, rscale, v, y, ydf, acc, accdf, gate, status);
}

cudaError_t sfd_gemv_stream_configure(int smem) {
  return cudaFuncSetAttribute(k_gemv_hs, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}
