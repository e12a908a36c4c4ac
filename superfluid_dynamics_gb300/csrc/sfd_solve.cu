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
#include "sfd_solve.cuh"

// =============================================================== assembly
// M_kj = c1 Im(z'_k cot((z_k - z_j)/2)) - [image] (1/4pi) Im cot((z_k - conj z_j)/2 + ih)
// M_kk = mdiag_k - [image] (1/4pi) Im cot(i (y_k + h))          (createM.cuh:43-92)
// with cot via w = exp(i z) (see sfd_kernels.cu).  Padded rows/cols = identity.
template <typename T>
__global__ void k_assemble(const SurfaceDesc* surf, const int4* tiles, const cd* w, const cd* p, const cd* zp,
                           const double* mdiag, T* mat) {
  const int4 t = tiles[blockIdx.x];  // (surface, row0, col0, -)
  const SurfaceDesc& S = surf[t.x];
  const int n = S.n, np = pad_n(n), off = S.off;
  T* A = mat + S.moff;
  const bool image = (S.physics == 1 && !S.infinite_depth);
  const double c1 = S.physics == 0 ? 0.25 * (1 - S.rho) / SFD_PI : 0.25 / SFD_PI;
  const double inv4pi = 0.25 / SFD_PI;
  for (int e = threadIdx.x; e < 64 * 64; e += blockDim.x) {
    int k = t.y + (e >> 6), j = t.z + (e & 63);
    double v;
    if (k >= n || j >= n) {
      v = (k == j) ? 1.0 : 0.0;
    } else if (sizeof(T) == 8) {
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
    } else {
      // FP32 entries for the preconditioner: w_k - w_j from hi/lo splits so the
      // near-diagonal difference keeps FP32 relative accuracy.
      if (k == j) {
        v = mdiag[off + k];
        if (image) {
          cd pk = p[off + k];
          double q = cabs2(pk);
          v -= inv4pi * (-(1.0 + q) / (1.0 - q));
        }
      } else {
        cd wk = w[off + k], wj = w[off + j];
        float kr = (float)wk.re, ki = (float)wk.im, jr = (float)wj.re, ji = (float)wj.im;
        float dr = (kr - jr) + ((float)(wk.re - (double)kr) - (float)(wj.re - (double)jr));
        float di = (ki - ji) + ((float)(wk.im - (double)ki) - (float)(wj.im - (double)ji));
        float sr = kr + jr, si = ki + ji;
        float den = 1.0f / (dr * dr + di * di);
        float qr = (sr * dr + si * di) * den, qi = (si * dr - sr * di) * den;  // (w_k+w_j)/(w_k-w_j)
        // cot = i (qr + i qi) = -qi + i qr
        float zr = (float)zp[off + k].re, zi = (float)zp[off + k].im;
        float imv = zr * qr + zi * (-qi);
        float fv = (float)c1 * imv;
        if (image) {
          cd pk = p[off + k], pj = p[off + j];
          float pkr = (float)pk.re, pki = (float)pk.im, pjr = (float)pj.re, pji = (float)pj.im;
          float q_r = pkr * pjr + pki * pji, q_i = pki * pjr - pkr * pji;
          float nr = 1.f + q_r, ni = q_i, er = 1.f - q_r, ei = -q_i;
          float d2 = 1.0f / (er * er + ei * ei);
          float rr = (nr * er + ni * ei) * d2;
          fv -= (float)inv4pi * (-rr);
        }
        v = fv;
      }
    }
    A[(long long)k * np + j] = (T)v;
  }
}
cudaError_t sfd_launch_assemble64(const SurfaceDesc* surf, const int4* tiles, int ntiles, const cd* w, const cd* p,
                                  const cd* zp, const double* mdiag, double* mat, cudaStream_t st) {
  k_assemble<double><<<ntiles, 256, 0, st>>>(surf, tiles, w, p, zp, mdiag, mat);
  return cudaGetLastError();
}
cudaError_t sfd_launch_assemble32(const SurfaceDesc* surf, const int4* tiles, int ntiles, const cd* w, const cd* p,
                                  const cd* zp, const double* mdiag, float* mat, cudaStream_t st) {
  k_assemble<float><<<ntiles, 256, 0, st>>>(surf, tiles, w, p, zp, mdiag, mat);
  return cudaGetLastError();
}

// =============================================================== FP64 LU
// Step kb (block column k0 = 64 kb) of the right-looking LU without row
// exchanges.  One CTA per surface factors the 64x64 diagonal block in shared
// memory.
__global__ void __launch_bounds__(256) k_lu64_diag(const SurfaceDesc* surf, int nsurf, int kb, double* mat,
                                                   unsigned int* status, double* lmax) {
  const int s = blockIdx.x;
  if (s >= nsurf) return;
  const SurfaceDesc& S = surf[s];
  const int np = pad_n(S.n), k0 = kb * 64;
  if (k0 >= np) return;
  double* A = mat + S.moff;
  __shared__ double D[64][65];
  for (int e = threadIdx.x; e < 64 * 64; e += 256) D[e >> 6][e & 63] = A[(long long)(k0 + (e >> 6)) * np + k0 + (e & 63)];
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
  __shared__ double D[64][65];
  for (int e = threadIdx.x; e < 64 * 64; e += 64) D[e >> 6][e & 63] = A[(long long)(k0 + (e >> 6)) * np + k0 + (e & 63)];
  __syncthreads();
  double x[64];
  const int t = threadIdx.x;
  if (blockIdx.y == 0) {
    // row r = tile*64 + t: solve x U = a (U upper incl. diagonal)
    double* row = A + (long long)(tile * 64 + t) * np + k0;
    double lm = 0.0;
    for (int c = 0; c < 64; ++c) {
      double v = row[c];
      for (int q = 0; q < c; ++q) v -= x[q] * D[q][c];
      x[c] = v / D[c][c];
    }
    for (int c = 0; c < 64; ++c) { row[c] = x[c]; lm = fmax(lm, fabs(x[c])); }
    for (int o = 16; o > 0; o >>= 1) lm = fmax(lm, __shfl_xor_sync(0xffffffffu, lm, o));
    if ((t & 31) == 0 && lm > 0) atomicMax(reinterpret_cast<unsigned long long*>(lmax) + s, __double_as_longlong(lm));
  } else {
    // column c = tile*64 + t: solve L x = a (L unit lower)
    double* col = A + (long long)k0 * np + tile * 64 + t;
    for (int r = 0; r < 64; ++r) {
      double v = col[(long long)r * np];
      for (int q = 0; q < r; ++q) v -= D[r][q] * x[q];
      x[r] = v;
    }
    for (int r = 0; r < 64; ++r) col[(long long)r * np] = x[r];
  }
}

// Trailing update A22 -= L21 U12 for step kb (64x64 output tiles, K = 64).
__global__ void __launch_bounds__(256) k_lu64_gemm(const SurfaceDesc* surf, int nsurf, int kb, double* mat) {
  const int s = blockIdx.z;
  const SurfaceDesc& S = surf[s];
  const int np = pad_n(S.n), k0 = kb * 64;
  const int ti = kb + 1 + blockIdx.y, tj = kb + 1 + blockIdx.x;
  if (ti * 64 >= np || tj * 64 >= np) return;
  double* A = mat + S.moff;
  __shared__ double La[64][33];
  __shared__ double Ub[32][65];
  const int tr = (threadIdx.x >> 4) * 4, tc = (threadIdx.x & 15) * 4;
  double acc[4][4] = {};
  for (int q0 = 0; q0 < 64; q0 += 32) {
    __syncthreads();
    for (int e = threadIdx.x; e < 64 * 32; e += 256) La[e >> 5][e & 31] = A[(long long)(ti * 64 + (e >> 5)) * np + k0 + q0 + (e & 31)];
    for (int e = threadIdx.x; e < 32 * 64; e += 256) Ub[e >> 6][e & 63] = A[(long long)(k0 + q0 + (e >> 6)) * np + tj * 64 + (e & 63)];
    __syncthreads();
    for (int q = 0; q < 32; ++q) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = La[tr + i][q];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Ub[q][tc + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) A[(long long)(ti * 64 + tr + i) * np + tj * 64 + tc + j] -= acc[i][j];
}

// Forward (unit L) then backward (U) substitution, one CTA per surface, in
// 64-row blocks: block dot products by all warps, then warp 0 finishes the
// 64x64 triangle.  x (length n) is overwritten with the solution.
__global__ void __launch_bounds__(256) k_lu64_solve(const SurfaceDesc* surf, const double* mat, const double* b,
                                                    double* x) {
  const SurfaceDesc& S = surf[blockIdx.x];
  const int n = S.n, np = pad_n(n), off = S.off;
  const double* A = mat + S.moff;
  extern __shared__ double xs[];  // np doubles
  for (int i = threadIdx.x; i < np; i += 256) xs[i] = i < n ? b[off + i] : 0.0;
  __syncthreads();
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
  for (int i = threadIdx.x; i < n; i += 256) x[off + i] = xs[i];
}

// =============================================================== FP32 Gauss-Jordan inverse
// Step kb (block K = [128 kb, 128 kb + 128)):
//   P = inv(A_KK)                        k_gj_diag   (one CTA per surface)
//   R = P A_K,:  and  C = A_:,K  (copies) k_gj_panel
//   A_ij -= C_i R_j (i,j not in K); A_Kj = R_j; A_iK = -C_i P; A_KK = P   k_gj_update
__global__ void __launch_bounds__(512) k_gj_diag(const SurfaceDesc* surf, int nsurf, int kb, float* mat, float* pbuf,
                                                 unsigned int* status) {
  const int s = blockIdx.x;
  const SurfaceDesc& S = surf[s];
  const int np = pad_n(S.n), k0 = kb * 128;
  if (k0 >= np) return;
  float* A = mat + S.moff;
  extern __shared__ float D[];  // 128 x 129
  const int ld = 129;
  for (int e = threadIdx.x; e < 128 * 128; e += 512) D[(e >> 7) * ld + (e & 127)] = A[(long long)(k0 + (e >> 7)) * np + k0 + (e & 127)];
  __syncthreads();
  __shared__ float colc[128], rowc[128];
  for (int c = 0; c < 128; ++c) {
    float piv = D[c * ld + c];
    if (threadIdx.x == 0 && !(fabsf(piv) > 1e-30f)) atomicOr(status + s, SFD_ST_ZERO_PIVOT);
    float pinv = 1.0f / piv;
    if (threadIdx.x < 128) colc[threadIdx.x] = D[threadIdx.x * ld + c];
    else if (threadIdx.x < 256) rowc[threadIdx.x - 128] = D[c * ld + threadIdx.x - 128];
    __syncthreads();
    // row c scaled, column c replaced, the rest updated with the staged row/column
    for (int e = threadIdx.x; e < 128 * 128; e += 512) {
      int i = e >> 7, j = e & 127;
      float v;
      if (i == c) v = (j == c) ? pinv : rowc[j] * pinv;
      else if (j == c) v = -colc[i] * pinv;
      else v = D[i * ld + j] - colc[i] * (rowc[j] * pinv);
      D[i * ld + j] = v;
    }
    __syncthreads();
  }
  float* P = pbuf + (long long)s * 128 * 128;
  for (int e = threadIdx.x; e < 128 * 128; e += 512) P[e] = D[(e >> 7) * ld + (e & 127)];
}

// R_j = P A_Kj (128 x 64 tiles over j not in K); C = A_iK copy (64-row tiles).
__global__ void __launch_bounds__(256) k_gj_panel(const SurfaceDesc* surf, int nsurf, int kb, const float* mat,
                                                  const float* pbuf, float* rbuf, float* cbuf, const long long* poff) {
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
    C[(long long)r * 128 + c] = A[(long long)r * np + k0 + c];
  }
  if (t * 64 >= k0 && t * 64 < k0 + 128) return;  // columns inside K: R not needed
  __shared__ float Pt[128][33];
  __shared__ float Bt[32][65];
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
}

// Output tile 64 x 64 (ti, tj) over the whole padded matrix.
__global__ void __launch_bounds__(256) k_gj_update(const SurfaceDesc* surf, int nsurf, int kb, float* mat,
                                                   const float* pbuf, const float* rbuf, const float* cbuf,
                                                   const long long* poff) {
  const int s = blockIdx.z;
  const SurfaceDesc& S = surf[s];
  const int np = pad_n(S.n), k0 = kb * 128;
  if (k0 >= np) return;
  const int ti = blockIdx.y, tj = blockIdx.x;
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
// y[off + i] = sum_j X_ij v[off + j]  (X float, v / y double); one warp per row.
__global__ void __launch_bounds__(256) k_gemv(const SurfaceDesc* surf, const int2* rowblk, const float* mat,
                                              const double* v, double* y) {
  const int2 rb = rowblk[blockIdx.x];  // (surface, first row)
  const SurfaceDesc& S = surf[rb.x];
  const int n = S.n, np = pad_n(n), off = S.off;
  const float* X = mat + S.moff;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row = rb.y + warp;
  if (row >= n) return;
  const float* xr = X + (long long)row * np;
  float acc = 0.f;
  for (int j = lane * 4; j < n; j += 128) {
    float4 q = *reinterpret_cast<const float4*>(xr + j);
    acc = fmaf(q.x, (float)v[off + j], acc);
    if (j + 1 < n) acc = fmaf(q.y, (float)v[off + j + 1], acc);
    if (j + 2 < n) acc = fmaf(q.z, (float)v[off + j + 2], acc);
    if (j + 3 < n) acc = fmaf(q.w, (float)v[off + j + 3], acc);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) y[off + row] = (double)acc;
}

// a += delta (and keep delta for the FP32 correction pass)
__global__ void k_axpy_inplace(int n, double* a, const double* d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] += d[i];
}
