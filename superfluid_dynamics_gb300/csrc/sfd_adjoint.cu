// sfd_adjoint.cu -- reverse mode (hand-written adjoint) of the FP64 boundary-
// integral RHS and of RK4 trajectories, for engines holding one surface (water
// with rho = 0, or helium with the standard van der Waals Bernoulli closure).
//
// Forward quantities of one RHS evaluation at Y = (x, y, phi), as computed by
// the FP64 path (createM.cuh:65-117, WaterVelocities.cuh:38-242,
// Derivatives.cuh:274-384, BaseBoundaryIntegrator.cuh:137-306):
//   Z = (x - xi) + i y,  z' = s1 R1(Z) + s1,  z'' = s2 R2(Z),  phi' = s1 Re R1(phi)
//     R1, R2: unscaled spectral first / second derivatives.  Their Fourier
//     multipliers (reference Nyquist rules included) are purely imaginary /
//     real, so R1^H = -R1 and R2^H = R2.
//   w = e^{i z}, p = e^{-h} w
//   C_k = sum_{j!=k} a_j cot((z_k - z_j)/2) = i (2 w_k S_k - (A - a_k)),  S_k = sum_{j!=k} a_j / (w_k - w_j)
//   D_k = sum_j a_j cot((z_k - conj z_j)/2 + i h) = -i (2 T_k - A),       T_k = sum_j a_j / (1 - p_k conj p_j)
//   (M a)_k = Mdiag_k a_k + c1 Im(z'_k C_k) - cI Im D_k = phi'_k,   Mdiag = 1/2 + c1 Im(z''/z')
//   a' = s1 R1(a)
//   E = V2 a' - (i/4pi) C + (i/4pi) [image] D + a V1,  V1 = -(i/4pi) z''/z'^2 + 1/(2 z'),  V2 = i / (2 pi z')
//   dx = Re E,  dy = -Im E,  dphi = vdw ((1 + y/h)^-3 - 1) + |E|^2 / 2   (helium)
//                            dphi = -g y + |E|^2 / 2                        (water)
// Complex cotangents follow g_q = dL/dRe q + i dL/dIm q; for q = beta r with a
// constant beta, g_r += conj(beta) g_q (and Re of that for a real r).
//
// Backward, for output cotangents (gdx, gdy, gdphi):
//   E:    gE = (gdx + gdphi dx) - i (gdy + gdphi dy)
//   a':   ga' = conj(V2) gE;  C (velocity part): gC = (i/4pi) gE;  D: gD = -(i/4pi) gE
//   a:    ga = Re(conj(V1) gE) - s1 Re R1(ga') + Re sum_{k!=j} conj(cot_kj) gC_k + Re sum_k conj(cotI_kj) gD_k
//         where sum_{k!=j} conj(cot_kj) gC_k = i (sum gC - gC_j) + 2 i conj(sum_{k!=j} b_k / (w_j - w_k)),
//         b = w conj(gC), and sum_k conj(cotI_kj) gD_k = -i sum gD + 2 i sum_k gD_k / (1 - p_j conj p_k)
//   solve: lambda = M^-T ga (stored LU, transposed triangular solves); gphi' = lambda;
//         with rho_k = -lambda_k the cotangent of (M a)_k at fixed a:
//         gC += i c1 conj(z') rho,  gD += -i cI rho,  gz' += i c1 conj(C) rho,  gMdiag = rho a
//   w, p: gw_k = -2 i conj(S_k - w_k S2_k) gC_k - 2 i a_k conj(Q_k)
//         gp_k =  2 i conj(T2_k) gD_k - 2 i a_k conj(U_k)
//         S2_k = sum_{j!=k} a_j / (w_k - w_j)^2,  Q_k = sum_{j!=k} w_j conj(gC_j) / (w_k - w_j)^2
//         T2_k = sum_j a_j conj p_j / (1 - p_k conj p_j)^2,  U_k = sum_j gD_j conj p_j / (1 - p_k conj p_j)^2
//   z:    gz = -i conj(w) gw - i conj(p) gp + spectral part;  gZ = -s1 R1(gz') + s2 R2(gz'')
//   state: gx = Re(gz + gZ),  gy = Im(gz + gZ) + Bernoulli part,  gphi = -s1 Re R1(lambda)
// RK4 (AutonomousRungeKuttaStepper.cuh:338-375) is reversed stage by stage from
// per-stage records made by recomputing each checkpoint segment.
//
// Two precisions, following the engine's:
//  * FP64 engines record the LU factors of M per stage and solve M^T lambda = ga
//    with them (U^T then L^T).
//  * Mixed engines record O(n) data only.  The transposed solve is iterative
//    refinement preconditioned by the transpose of the engine's approximate
//    inverse X (FP16, row-scaled: X = diag(s) H, so X^T r = H^T (s r)):
//      lambda_0 = X^T ga;  r = ga - M^T lambda (FP64, matrix-free);  lambda += X^T r
//    where, with gC = i c1 conj(z') lambda and gD = -i cI lambda,
//      (M^T lambda)_j = Mdiag_j lambda_j + Re(i (sum gC - gC_j) + 2 i conj(Sb_j)) + Re(-i sum gD + 2 i Tb_j)
//    (Sb, Tb as in the ga line above, here with b_k = -i c1 w_k z'_k lambda_k).
//    The iterations are gated on the residual (they return at once once
//    max |r| <= 1e-13 max |ga|); a final residual above the engine's
//    refine_tol raises SFD_ST_REFINE_STALL.  Every pair sum of one stage reads
//    the pair reciprocals R_jk = 1 / (w_j - w_k) and I_jk = 1 / (1 - p_j conj p_k),
//    computed once per stage in FP64 into two n x n complex matrices.
#include <algorithm>
#include <cstring>

#include "sfd_internal.cuh"
#include "sfd_solve.cuh"

// Per-stage record of one RHS evaluation (device pointers).
struct AdjStage {
  double* Y;   // stage state [x|y|phi]
  double* k;   // stage RHS [dx|dy|dphi]
  double* lu;  // LU factors of M (np x np, row-major, no row exchanges); null for mixed engines
  double* a;
  cd *ap, *zp, *zpp, *C, *D, *w, *p;
};

namespace {

constexpr int kAdjThreads = 256;

__device__ __forceinline__ cd cadd(cd a, cd b) { return {a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cd crcp(cd b) {
  double d = 1.0 / (b.re * b.re + b.im * b.im);
  return {b.re * d, -b.im * d};
}

struct AdjConst {
  int n, np;
  int physics;
  bool image;
  double c1, cI, depth, vdw, gravity, rho;
};

AdjConst adj_const(const SurfaceDesc& S) {
  AdjConst c;
  c.n = S.n;
  c.np = pad_n(S.n);
  c.physics = S.physics;
  c.image = (S.physics == 1 && !S.infinite_depth);
  c.c1 = S.physics == 0 ? 0.25 * (1 - S.rho) / SFD_PI : 0.25 / SFD_PI;
  c.cI = c.image ? 0.25 / SFD_PI : 0.0;
  c.depth = S.depth;
  c.vdw = S.vdw;
  c.gravity = S.gravity;
  c.rho = S.rho;
  return c;
}

// ---------------------------------------------------------------- kernels
// Output side: E, V1, V2 and the Bernoulli closure.
__global__ void k_adj_out(AdjConst K, AdjStage st, const double* gk, double* gY, double* apb_re, double* apb_im,
                          cd* cbar, cd* dbar, double* abar, double* zpb_re, double* zpb_im, double* zppb_re,
                          double* zppb_im, double* pbar) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = K.n;
  if (k >= n) return;
  const double inv4pi = 0.25 / SFD_PI;
  const double dx = st.k[k], dy = st.k[n + k], yk = st.Y[n + k];
  const double gphi = gk[2 * n + k];
  const double gxt = gk[k] + gphi * dx, gyt = gk[n + k] + gphi * dy;
  const cd Eb = {gxt, -gyt};
  const cd zp = st.zp[k], zpp = st.zpp[k];
  const cd izp = crcp(zp);
  const cd izp2 = izp * izp;
  const cd V2 = cmul_i((0.5 / SFD_PI) * izp);
  const cd V1 = cmul_i(-inv4pi * (zpp * izp2)) + 0.5 * izp;
  const cd apb = cconj(V2) * Eb;
  apb_re[k] = apb.re;
  apb_im[k] = apb.im;
  const cd V2b = cconj(st.ap[k]) * Eb;
  cbar[k] = cmul_i(inv4pi * Eb);
  dbar[k] = K.image ? cmul_i(-inv4pi * Eb) : cd{0.0, 0.0};
  const double ak = st.a[k];
  abar[k] = (cconj(V1) * Eb).re;
  const cd V1b = ak * Eb;
  // dV1/dz'' = -(i/4pi) / z'^2;  dV1/dz' = (i/2pi) z'' / z'^3 - 1 / (2 z'^2);  dV2/dz' = -i / (2 pi z'^2)
  const cd dV1_dzpp = cmul_i(-inv4pi * izp2);
  const cd dV1_dzp = cmul_i((0.5 / SFD_PI) * (zpp * izp2 * izp)) - 0.5 * izp2;
  const cd dV2_dzp = cmul_i((-0.5 / SFD_PI) * izp2);
  const cd zppb = cconj(dV1_dzpp) * V1b;
  const cd zpb = cconj(dV1_dzp) * V1b + cconj(dV2_dzp) * V2b;
  zpb_re[k] = zpb.re;
  zpb_im[k] = zpb.im;
  zppb_re[k] = zppb.re;
  zppb_im[k] = zppb.im;
  double gy_b, gpar;
  if (K.physics == 0) {
    gy_b = gphi * (-(1 + K.rho) * K.gravity);
    gpar = gphi * (-(1 + K.rho) * yk);                 // d dphi / d g
  } else {
    const double q = 1.0 + yk / K.depth;
    const double q3 = 1.0 / (q * q * q);
    gy_b = gphi * K.vdw * (-3.0 / K.depth) * q3 / q;
    gpar = gphi * (q3 - 1.0);                          // d dphi / d vdw
  }
  gY[k] = 0.0;
  gY[n + k] = gy_b;
  gY[2 * n + k] = 0.0;
  pbar[k] = gpar;
}

// sum of gC and gD over the surface (one CTA, fixed order)
__global__ void k_adj_sum_cd(int n, const cd* cbar, const cd* dbar, cd* out) {
  __shared__ cd sc[kAdjThreads], sd[kAdjThreads];
  cd c = {0, 0}, d = {0, 0};
  for (int k = threadIdx.x; k < n; k += kAdjThreads) {
    c = cadd(c, cbar[k]);
    d = cadd(d, dbar[k]);
  }
  sc[threadIdx.x] = c;
  sd[threadIdx.x] = d;
  __syncthreads();
  for (int s = kAdjThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sc[threadIdx.x] = cadd(sc[threadIdx.x], sc[threadIdx.x + s]);
      sd[threadIdx.x] = cadd(sd[threadIdx.x], sd[threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = sc[0];
    out[1] = sd[0];
  }
}

// sum of the per-node parameter cotangents (one CTA, fixed order), added to *acc
__global__ void k_adj_sum_param(int n, const double* pbar, double scale, double* acc) {
  __shared__ double s[kAdjThreads];
  double v = 0.0;
  for (int k = threadIdx.x; k < n; k += kAdjThreads) v += pbar[k];
  s[threadIdx.x] = v;
  __syncthreads();
  for (int h = kAdjThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) s[threadIdx.x] += s[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) *acc += scale * s[0];
}

__device__ __forceinline__ cd warp_sum(cd v) {
  for (int o = 16; o > 0; o >>= 1) {
    v.re += __shfl_xor_sync(0xffffffffu, v.re, o);
    v.im += __shfl_xor_sync(0xffffffffu, v.im, o);
  }
  return v;
}

// Pass 1 (one warp per target j): Sb_j = sum_{k!=j} b_k / (w_j - w_k) with
// b = w conj(gC), and Tb_j = sum_k gD_k / (1 - p_j conj p_k).
__global__ void k_adj_sums1(AdjConst K, const cd* w, const cd* p, const cd* cbar, const cd* dbar, cd* sb, cd* tb) {
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (j >= K.n) return;
  const cd wj = w[j];
  const cd pj = K.image ? p[j] : cd{0, 0};
  cd accS = {0, 0}, accT = {0, 0};
  for (int k = lane; k < K.n; k += 32) {
    const cd wk = w[k];
    if (k != j) accS = cadd(accS, (wk * cconj(cbar[k])) * crcp(wj - wk));
    if (K.image) {
      const cd e = cd{1.0, 0.0} - pj * cconj(p[k]);
      accT = cadd(accT, dbar[k] * crcp(e));
    }
  }
  accS = warp_sum(accS);
  accT = warp_sum(accT);
  if (lane == 0) {
    sb[j] = accS;
    tb[j] = accT;
  }
}

// ga_j += -s1 Re R1(ga')_j + Re(i (sum gC - gC_j) + 2 i conj(Sb_j)) + Re(-i sum gD + 2 i Tb_j)
__global__ void k_adj_a(AdjConst K, const cd* sums, const cd* r1apb, const cd* cbar, const cd* sb, const cd* tb,
                        double* abar) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= K.n) return;
  const double s1 = 2.0 * SFD_PI / K.n;
  double g = abar[j] - s1 * r1apb[j].re;
  const cd sc = sums[0], sd = sums[1];
  g += (cmul_i(sc - cbar[j]) + cmul_i(2.0 * cconj(sb[j]))).re;
  if (K.image) g += (cmul_i(cd{-sd.re, -sd.im}) + cmul_i(2.0 * tb[j])).re;
  abar[j] = g;
}

// lambda = M^-T b from the row-major LU factors (M = L U, L unit lower):
// U^T t = b (forward), then L^T lambda = t (backward).  One CTA.
__global__ void __launch_bounds__(kAdjThreads) k_lu_solve_t(int n, int np, const double* LU, const double* b,
                                                           double* x) {
  extern __shared__ double xs[];           // np values
  __shared__ double part[4][64];
  for (int i = threadIdx.x; i < np; i += kAdjThreads) xs[i] = i < n ? b[i] : 0.0;
  __syncthreads();
  const int nblk = np / 64;
  const int ii = threadIdx.x & 63, grp = threadIdx.x >> 6;  // 4 groups split the row range
  // forward: t_i = (b_i - sum_{j<i} U_ji t_j) / U_ii
  for (int B = 0; B < nblk; ++B) {
    const int r0 = B * 64;
    double s = 0.0;
    for (int j = grp; j < r0; j += 4) s += LU[(long long)j * np + r0 + ii] * xs[j];
    part[grp][ii] = s;
    __syncthreads();
    if (threadIdx.x < 64) xs[r0 + ii] -= ((part[0][ii] + part[1][ii]) + part[2][ii]) + part[3][ii];
    __syncthreads();
    if (threadIdx.x < 32) {
      for (int c = 0; c < 64; ++c) {
        if (threadIdx.x == 0) xs[r0 + c] = xs[r0 + c] / LU[(long long)(r0 + c) * np + r0 + c];
        __syncwarp();
        const double tc = xs[r0 + c];
        for (int i = c + 1 + threadIdx.x; i < 64; i += 32) xs[r0 + i] -= LU[(long long)(r0 + c) * np + r0 + i] * tc;
        __syncwarp();
      }
    }
    __syncthreads();
  }
  // backward: lambda_i = t_i - sum_{j>i} L_ji lambda_j
  for (int B = nblk - 1; B >= 0; --B) {
    const int r0 = B * 64;
    double s = 0.0;
    for (int j = r0 + 64 + grp; j < np; j += 4) s += LU[(long long)j * np + r0 + ii] * xs[j];
    part[grp][ii] = s;
    __syncthreads();
    if (threadIdx.x < 64) xs[r0 + ii] -= ((part[0][ii] + part[1][ii]) + part[2][ii]) + part[3][ii];
    __syncthreads();
    if (threadIdx.x < 32) {
      for (int c = 63; c >= 0; --c) {
        const double lc = xs[r0 + c];
        for (int i = threadIdx.x; i < c; i += 32) xs[r0 + i] -= LU[(long long)(r0 + c) * np + r0 + i] * lc;
        __syncwarp();
      }
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < n; i += kAdjThreads) x[i] = xs[i];
}

// M-part cotangents at fixed a (rho = -lambda); totals of gC, gD for pass 2.
// With rmax (mixed engines' transposed solve), thread 0 also raises the
// refinement-stall bit when the solve's final residual rmax[last] is above
// tol * rmax[0] (or NaN).
__global__ void k_adj_node2(AdjConst K, AdjStage st, const double* lambda, cd* cbar, cd* dbar, double* zpb_re,
                            double* zpb_im, double* zppb_re, double* zppb_im, const double* rmax, int last,
                            double tol, unsigned int* status) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (rmax && k == 0 && !(rmax[last] <= tol * rmax[0])) atomicOr(status, (unsigned int)SFD_ST_REFINE_STALL);
  if (k >= K.n) return;
  const double rho = -lambda[k];
  const cd zp = st.zp[k], zpp = st.zpp[k];
  const cd izp = crcp(zp);
  cbar[k] = cbar[k] + cmul_i(K.c1 * rho * cconj(zp));
  if (K.image) dbar[k] = dbar[k] + cmul_i(cd{-K.cI * rho, 0.0});
  // Mdiag = 1/2 + c1 Im(z''/z'):  gR = i c1 gMdiag,  gMdiag = rho a
  const cd Rb = cmul_i(cd{K.c1 * rho * st.a[k], 0.0});
  const cd zppb = cconj(izp) * Rb;
  const cd zpb = cmul_i(K.c1 * rho * cconj(st.C[k])) + cconj(cd{-1.0, 0.0} * (zpp * izp * izp)) * Rb;
  zpb_re[k] += zpb.re;
  zpb_im[k] += zpb.im;
  zppb_re[k] += zppb.re;
  zppb_im[k] += zppb.im;
}

// Pass 2 (one warp per target k): S, S2, Q, T2, U as defined above; writes
// the w / p contributions to gx, gy.
__global__ void k_adj_sums2(AdjConst K, AdjStage st, const cd* cbar, const cd* dbar, double* gY) {
  const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (k >= K.n) return;
  const cd* w = st.w;
  const cd* p = st.p;
  const double* a = st.a;
  const cd wk = w[k];
  const cd pk = K.image ? p[k] : cd{0, 0};
  cd S = {0, 0}, S2 = {0, 0}, Q = {0, 0}, T2 = {0, 0}, U = {0, 0};
  for (int j = lane; j < K.n; j += 32) {
    const double aj = a[j];
    const cd wj = w[j];
    if (j != k) {
      const cd inv = crcp(wk - wj);
      const cd inv2 = inv * inv;
      S = cadd(S, aj * inv);
      S2 = cadd(S2, aj * inv2);
      Q = cadd(Q, (wj * cconj(cbar[j])) * inv2);
    }
    if (K.image) {
      const cd cpj = cconj(p[j]);
      const cd ie = crcp(cd{1.0, 0.0} - pk * cpj);
      const cd ie2c = (ie * ie) * cpj;
      T2 = cadd(T2, aj * ie2c);
      U = cadd(U, dbar[j] * ie2c);
    }
  }
  S = warp_sum(S);
  S2 = warp_sum(S2);
  Q = warp_sum(Q);
  T2 = warp_sum(T2);
  U = warp_sum(U);
  if (lane == 0) {
    const double ak = a[k];
    const cd wb = cmul_i(-2.0 * (cconj(S - wk * S2) * cbar[k])) + cmul_i(-2.0 * ak * cconj(Q));
    cd zb = cmul_i(-1.0 * (cconj(wk) * wb));
    if (K.image) {
      const cd pb = cmul_i(2.0 * (cconj(T2) * dbar[k])) + cmul_i(-2.0 * ak * cconj(U));
      zb = zb + cmul_i(-1.0 * (cconj(pk) * pb));
    }
    gY[k] += zb.re;
    gY[K.n + k] += zb.im;
  }
}

// ------------------------------------------------ mixed-precision reverse sweep
// Pair reciprocals of one stage, row j = target: R_jk = 1 / (w_j - w_k)
// (0 on the diagonal) and, with the image, I_jk = 1 / (1 - p_j conj p_k).
// One thread per pair; consecutive threads write consecutive k.
__global__ void k_adj_pairs(AdjConst K, const cd* w, const cd* p, cd* R, cd* I) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nn = (long long)K.n * K.n;
  if (t >= nn) return;
  const int j = (int)(t / K.n), k = (int)(t - (long long)j * K.n);
  R[t] = j == k ? cd{0.0, 0.0} : crcp(w[j] - w[k]);
  if (K.image) I[t] = crcp(cd{1.0, 0.0} - p[j] * cconj(p[k]));
}

// k_adj_sums1 from the pair reciprocals (one warp per target j).
__global__ void k_adj_sums1m(AdjConst K, const cd* w, const cd* R, const cd* I, const cd* cbar, const cd* dbar,
                             cd* sb, cd* tb) {
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (j >= K.n) return;
  const cd* Rj = R + (long long)j * K.n;
  const cd* Ij = I + (long long)j * K.n;
  cd accS = {0, 0}, accT = {0, 0};
  for (int k = lane; k < K.n; k += 32) {
    accS = cadd(accS, (w[k] * cconj(cbar[k])) * Rj[k]);  // R_jj = 0
    if (K.image) accT = cadd(accT, dbar[k] * Ij[k]);
  }
  accS = warp_sum(accS);
  accT = warp_sum(accT);
  if (lane == 0) {
    sb[j] = accS;
    tb[j] = accT;
  }
}

// k_adj_sums2 from the pair reciprocals (one warp per target k): R_kj =
// 1 / (w_k - w_j), I_kj = 1 / (1 - p_k conj p_j).
__global__ void k_adj_sums2m(AdjConst K, AdjStage st, const cd* R, const cd* I, const cd* cbar, const cd* dbar,
                             double* gY) {
  const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (k >= K.n) return;
  const cd* w = st.w;
  const cd* p = st.p;
  const double* a = st.a;
  const cd* Rk = R + (long long)k * K.n;
  const cd* Ik = I + (long long)k * K.n;
  cd S = {0, 0}, S2 = {0, 0}, Q = {0, 0}, T2 = {0, 0}, U = {0, 0};
  for (int j = lane; j < K.n; j += 32) {
    const double aj = a[j];
    const cd inv = Rk[j];  // 0 for j = k
    const cd inv2 = inv * inv;
    S = cadd(S, aj * inv);
    S2 = cadd(S2, aj * inv2);
    Q = cadd(Q, (w[j] * cconj(cbar[j])) * inv2);
    if (K.image) {
      const cd cpj = cconj(p[j]);
      const cd ie = Ik[j];
      const cd ie2c = (ie * ie) * cpj;
      T2 = cadd(T2, aj * ie2c);
      U = cadd(U, dbar[j] * ie2c);
    }
  }
  S = warp_sum(S);
  S2 = warp_sum(S2);
  Q = warp_sum(Q);
  T2 = warp_sum(T2);
  U = warp_sum(U);
  if (lane == 0) {
    const double ak = a[k];
    const cd wk = w[k];
    const cd wb = cmul_i(-2.0 * (cconj(S - wk * S2) * cbar[k])) + cmul_i(-2.0 * ak * cconj(Q));
    cd zb = cmul_i(-1.0 * (cconj(wk) * wb));
    if (K.image) {
      const cd pk = p[k];
      const cd pb = cmul_i(2.0 * (cconj(T2) * dbar[k])) + cmul_i(-2.0 * ak * cconj(U));
      zb = zb + cmul_i(-1.0 * (cconj(pk) * pb));
    }
    gY[k] += zb.re;
    gY[K.n + k] += zb.im;
  }
}

// Transposed solve, set-up (one CTA): lambda = 0, v = s * ga (FP32, input of
// the first H^T product), bw = -i c1 w z' (per-node weight of M^T lambda),
// rmax[0] = max |ga|, residual slots rmax[1..] = 0.
constexpr int kAdjtIters = 6;   // residual checks (each followed by a gated correction)
constexpr double kAdjtGateTol = 1e-13;
__global__ void __launch_bounds__(1024) k_adjt_init(AdjConst K, AdjStage st, const double* ga, const float* rscale,
                                                   double* lam, float* v, cd* bw, double* rmax) {
  __shared__ double red[32];
  double m = 0.0;
  for (int j = threadIdx.x; j < K.n; j += blockDim.x) {
    const double g = ga[j];
    lam[j] = 0.0;
    v[j] = (float)((double)rscale[j] * g);
    bw[j] = cmul_i(-K.c1 * (st.w[j] * st.zp[j]));
    m = fmax(m, fabs(g));  // a NaN entry is caught by the residual slots
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) rmax[0] = m;
  }
  if (threadIdx.x >= 1 && threadIdx.x <= kAdjtIters) rmax[threadIdx.x] = 0.0;
}

__device__ __forceinline__ bool adjt_converged(const double* rmax, int it) {
  return it > 0 && rmax[it] <= kAdjtGateTol * rmax[0];  // NaN: not converged
}

// lambda += H^T v (FP32 accumulation) where the residual of slot `it` is above
// the gate (slot 0: the first product, always).  One CTA per 64 columns, 16
// warps over the rows, a lane owns 2 columns; fixed-order reduction over the
// warps in shared memory.
__global__ void __launch_bounds__(512) k_gemv_ht(int n, int np, const __half* H, const float* v, double* lam,
                                                 const double* rmax, int it) {
  if (adjt_converged(rmax, it)) return;
  __shared__ float2 part[16][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * 64 + 2 * lane;  // np is a multiple of 128: c + 1 < np
  float2 acc = make_float2(0.f, 0.f);
  for (int i = warp; i < n; i += 16) {
    const float2 h = __half22float2(*reinterpret_cast<const __half2*>(H + (long long)i * np + c));
    const float vi = v[i];
    acc.x = fmaf(h.x, vi, acc.x);
    acc.y = fmaf(h.y, vi, acc.y);
  }
  part[warp][lane] = acc;
  __syncthreads();
  if (warp == 0) {
    float2 t = part[0][lane];
#pragma unroll
    for (int w = 1; w < 16; ++w) {
      t.x += part[w][lane].x;
      t.y += part[w][lane].y;
    }
    if (c < n) lam[c] += (double)t.x;
    if (c + 1 < n) lam[c + 1] += (double)t.y;
  }
}

// r = ga - M^T lambda (FP64) into v = s * r (FP32) and max |r| into slot `it`
// (one warp per target j; every warp also forms the totals sum conj(z') lambda
// and sum lambda in its pass over the row).  Where slot it - 1 is converged,
// slot it inherits it and nothing else runs.
__global__ void k_adjt_resid(AdjConst K, AdjStage st, const cd* R, const cd* I, const cd* bw, const double* ga,
                             const double* lam, const float* rscale, float* v, double* rmax, int it) {
  if (adjt_converged(rmax, it - 1)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) rmax[it] = rmax[it - 1];
    return;
  }
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (j >= K.n) return;
  const cd* Rj = R + (long long)j * K.n;
  const cd* Ij = I + (long long)j * K.n;
  cd sb = {0, 0}, tb = {0, 0}, sz = {0, 0};
  double sl = 0.0;
  for (int k = lane; k < K.n; k += 32) {
    const double lk = lam[k];
    sb = cadd(sb, lk * (bw[k] * Rj[k]));  // R_jj = 0
    sz = cadd(sz, lk * cconj(st.zp[k]));
    if (K.image) {
      tb = cadd(tb, lk * Ij[k]);
      sl += lk;
    }
  }
  sb = warp_sum(sb);
  sz = warp_sum(sz);
  tb = warp_sum(tb);
  for (int o = 16; o > 0; o >>= 1) sl += __shfl_xor_sync(0xffffffffu, sl, o);
  if (lane == 0) {
    const double lj = lam[j];
    const cd zp = st.zp[j];
    const double mdiag = 0.5 + K.c1 * (st.zpp[j] * crcp(zp)).im;
    const cd gCj = cmul_i(K.c1 * lj * cconj(zp));
    const cd sumC = cmul_i(K.c1 * sz);
    double mt = mdiag * lj + (cmul_i(sumC - gCj) + cmul_i(2.0 * cconj(sb))).re;
    if (K.image) {
      // sum gD = -i cI sum lambda;  Tb = sum_k gD_k I_jk = -i cI tb
      const cd sumD = cmul_i(cd{-K.cI * sl, 0.0});
      const cd Tb = cmul_i(-K.cI * tb);
      mt += (cmul_i(-1.0 * sumD) + cmul_i(2.0 * Tb)).re;
    }
    const double r = ga[j] - mt;
    v[j] = (float)((double)rscale[j] * r);
    const double ar = fabs(r);
    atomicMax(reinterpret_cast<unsigned long long*>(rmax + it),
              (unsigned long long)__double_as_longlong(ar == ar ? ar : 1e300));
  }
}

// spectral part: gZ = -s1 R1(gz') + s2 R2(gz''); gphi = -s1 Re R1(lambda)
__global__ void k_adj_final(AdjConst K, const cd* r1zpb, const cd* r2zppb, const cd* r1lam, double* gY) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K.n) return;
  const double s1 = 2.0 * SFD_PI / K.n;
  const double s2 = s1 * s1;
  const cd gz = (-s1) * r1zpb[k] + s2 * r2zppb[k];
  gY[k] += gz.re;
  gY[K.n + k] += gz.im;
  gY[2 * K.n + k] = -s1 * r1lam[k].re;
}

// RK4 helpers: out = alpha a + beta b (b nullable); acc += a + b + c + d
__global__ void k_adj_lin(int n3, double* out, double alpha, const double* a, double beta, const double* b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n3) return;
  double v = alpha * a[i];
  if (b) v += beta * b[i];
  out[i] = v;
}
__global__ void k_adj_acc4(int n3, double* acc, const double* a, const double* b, const double* c, const double* d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n3) return;
  acc[i] = acc[i] + ((a[i] + b[i]) + (c[i] + d[i]));
}

inline int nblocks(long long n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

// ---------------------------------------------------------------- workspace
struct AdjWork {
  int n = 0, np = 0;
  int cap_steps = 0;           // slots hold this many steps (x 4 stages)
  std::vector<AdjStage> slots;
  void* slot_mem = nullptr;
  // recorded trajectory
  int steps = 0, every = 0, nckpt = 0;
  double dt = 0.0;
  double* ckpt = nullptr;      // nckpt x 3n
  int ckpt_cap = 0;
  // scratch
  double *y = nullptr, *kacc = nullptr, *ktmp = nullptr, *ys = nullptr;
  double *gY = nullptr, *gk = nullptr, *gYs[4] = {nullptr, nullptr, nullptr, nullptr};
  double *abar = nullptr, *lam = nullptr, *apb_re = nullptr, *apb_im = nullptr;
  double *zpb_re = nullptr, *zpb_im = nullptr, *zppb_re = nullptr, *zppb_im = nullptr, *pbar = nullptr;
  cd *cbar = nullptr, *dbar = nullptr, *sb = nullptr, *tb = nullptr, *t1 = nullptr, *t2 = nullptr, *t3 = nullptr;
  cd* sums = nullptr;
  double* gparam = nullptr;    // device accumulator
  // mixed engines: pair reciprocals of the current stage (n x n each; I with
  // the image only), the transposed solve's node weights, FP32 product input
  // and residual slots, and the engine state saved around a recording
  bool mixed = false;
  cd *R = nullptr, *I = nullptr, *bw = nullptr;
  float* v = nullptr;
  double* rmax = nullptr;
  double* ysave = nullptr;
  int2* jobs = nullptr;        // {0, RAW}, {0, RAW2}
  std::vector<void*> allocs;
};

void sfd_adjoint_free(sfd_engine* e) {
  if (!e || !e->adj) return;
  for (void* p : e->adj->allocs) cudaFree(p);
  if (e->adj->slot_mem) cudaFree(e->adj->slot_mem);
  if (e->adj->ckpt) cudaFree(e->adj->ckpt);
  delete e->adj;
  e->adj = nullptr;
}

// Why reverse mode does not cover the engine, or null when it does.
const char* sfd_adjoint_unsupported(const sfd_engine* e) {
  if (e->opt.precision == SFD_PRECISION_MIXED && (!e->m16 || !e->rscale))
    return "reverse mode of a mixed engine needs the FP16 preconditioner (precond_half = 1)";
  if (e->nsurf != 1) return "reverse mode supports engines with one surface";
  const SurfaceDesc& S = e->hs[0];
  if (S.physics == 0 && S.rho != 0.0) return "reverse mode supports water with rho = 0 only";
  if (S.physics == 1 && S.bern_variant != 0) return "reverse mode supports the standard helium Bernoulli closure only";
  if (S.U != 0.0) return "reverse mode supports U = 0 only";
  if (S.drive) return "reverse mode does not cover the optomechanical drive";
  return nullptr;
}

namespace {

template <typename T>
cudaError_t adj_alloc(AdjWork* W, T** p, size_t count) {
  cudaError_t err = cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
  if (err == cudaSuccess) W->allocs.push_back(*p);
  return err;
}

#define ACK(expr)                                 \
  do {                                            \
    cudaError_t _e = (expr);                      \
    if (_e != cudaSuccess) return sfd_internal_cuda(_e, #expr); \
  } while (0)

int check_engine(sfd_engine* e) {
  if (!e) return sfd_internal_error(SFD_ERR_INVALID, "null engine");
  const char* why = sfd_adjoint_unsupported(e);
  return why ? sfd_internal_error(SFD_ERR_INVALID, why) : 0;
}

// Workspace with room for `steps` recorded steps (4 stage slots each).
int ensure_work(sfd_engine* e, int steps) {
  AdjWork* W = e->adj;
  if (W && W->cap_steps >= steps) return 0;
  if (W) {
    if (W->slot_mem) cudaFree(W->slot_mem);
    W->slot_mem = nullptr;
    W->slots.clear();
  } else {
    W = e->adj = new AdjWork();
    const int n = e->hs[0].n;
    W->n = n;
    W->np = pad_n(n);
    const size_t n3 = 3 * (size_t)n;
    ACK(adj_alloc(W, &W->y, n3));
    ACK(adj_alloc(W, &W->kacc, n3));
    ACK(adj_alloc(W, &W->ktmp, n3));
    ACK(adj_alloc(W, &W->ys, n3));
    ACK(adj_alloc(W, &W->gY, n3));
    ACK(adj_alloc(W, &W->gk, n3));
    for (int s = 0; s < 4; ++s) ACK(adj_alloc(W, &W->gYs[s], n3));
    double** dv[] = {&W->abar, &W->lam, &W->apb_re, &W->apb_im, &W->zpb_re, &W->zpb_im, &W->zppb_re, &W->zppb_im, &W->pbar};
    for (double** p : dv) ACK(adj_alloc(W, p, (size_t)n));
    cd** cv[] = {&W->cbar, &W->dbar, &W->sb, &W->tb, &W->t1, &W->t2, &W->t3};
    for (cd** p : cv) ACK(adj_alloc(W, p, (size_t)n));
    ACK(adj_alloc(W, &W->sums, 2));
    ACK(adj_alloc(W, &W->gparam, 1));
    W->mixed = e->opt.precision == SFD_PRECISION_MIXED;
    if (W->mixed) {
      const AdjConst K = adj_const(e->hs[0]);
      ACK(adj_alloc(W, &W->R, (size_t)n * n));
      if (K.image) ACK(adj_alloc(W, &W->I, (size_t)n * n));
      ACK(adj_alloc(W, &W->bw, (size_t)n));
      ACK(adj_alloc(W, &W->v, (size_t)n));
      ACK(adj_alloc(W, &W->rmax, (size_t)kAdjtIters + 1));
      ACK(adj_alloc(W, &W->ysave, n3));
    }
    ACK(adj_alloc(W, &W->jobs, 2));
    int2 jobs[2] = {{0, SFD_JOB_RAW}, {0, SFD_JOB_RAW2}};
    ACK(cudaMemcpy(W->jobs, jobs, sizeof(jobs), cudaMemcpyHostToDevice));
    ACK(cudaFuncSetAttribute(k_lu_solve_t, cudaFuncAttributeMaxDynamicSharedMemorySize, 8192 * (int)sizeof(double)));
  }
  const size_t n = W->n, np = W->np;
  auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
  const size_t lu_bytes = W->mixed ? 0 : al(8 * np * np);
  const size_t per = 2 * al(24 * n) + lu_bytes + al(8 * n) + 7 * al(16 * n);
  const size_t nslot = 4 * (size_t)steps;
  ACK(cudaMalloc(&W->slot_mem, per * nslot));
  unsigned char* b = static_cast<unsigned char*>(W->slot_mem);
  W->slots.resize(nslot);
  for (size_t i = 0; i < nslot; ++i) {
    AdjStage& s = W->slots[i];
    auto take = [&](size_t bytes) {
      unsigned char* r = b;
      b += al(bytes);
      return r;
    };
    s.Y = reinterpret_cast<double*>(take(24 * n));
    s.k = reinterpret_cast<double*>(take(24 * n));
    s.lu = W->mixed ? nullptr : reinterpret_cast<double*>(take(8 * np * np));
    s.a = reinterpret_cast<double*>(take(8 * n));
    s.ap = reinterpret_cast<cd*>(take(16 * n));
    s.zp = reinterpret_cast<cd*>(take(16 * n));
    s.zpp = reinterpret_cast<cd*>(take(16 * n));
    s.C = reinterpret_cast<cd*>(take(16 * n));
    s.D = reinterpret_cast<cd*>(take(16 * n));
    s.w = reinterpret_cast<cd*>(take(16 * n));
    s.p = reinterpret_cast<cd*>(take(16 * n));
  }
  W->cap_steps = steps;
  return 0;
}

// RHS at st.Y into st.k, keeping the intermediates the reverse pass reads.
// On a mixed engine `refactor` rebuilds the preconditioner at this
// evaluation (an FP64 engine factors M at every evaluation anyway).
int record_rhs(sfd_engine* e, AdjWork* W, AdjStage& st, bool refactor = true) {
  int rc = sfd_internal_rhs_ex(e, st.Y, st.k, refactor);
  if (rc) return rc;
  const size_t n = W->n, np = W->np;
  cudaStream_t s = e->stream;
  if (st.lu) ACK(cudaMemcpyAsync(st.lu, e->m64, 8 * np * np, cudaMemcpyDeviceToDevice, s));
  ACK(cudaMemcpyAsync(st.a, e->a, 8 * n, cudaMemcpyDeviceToDevice, s));
  ACK(cudaMemcpyAsync(st.ap, e->ap, 16 * n, cudaMemcpyDeviceToDevice, s));
  ACK(cudaMemcpyAsync(st.zp, e->zp, 16 * n, cudaMemcpyDeviceToDevice, s));
  ACK(cudaMemcpyAsync(st.zpp, e->zpp, 16 * n, cudaMemcpyDeviceToDevice, s));
  ACK(cudaMemcpyAsync(st.C, e->cacc, 16 * n, cudaMemcpyDeviceToDevice, s));
  ACK(cudaMemcpyAsync(st.D, e->dacc, 16 * n, cudaMemcpyDeviceToDevice, s));
  ACK(cudaMemcpyAsync(st.w, e->nd.w, 16 * n, cudaMemcpyDeviceToDevice, s));
  ACK(cudaMemcpyAsync(st.p, e->nd.p, 16 * n, cudaMemcpyDeviceToDevice, s));
  return 0;
}

int spectral(sfd_engine* e, AdjWork* W, int job, const double* re, const double* im, cd* out) {
  DerivArgs D{e->d_surf, 1, re, im, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, out, nullptr};
  cudaError_t err = sfd_launch_spectral(D, W->jobs + job, 1, W->n, e->stream);
  if (err != cudaSuccess) return sfd_internal_cuda(err, "spectral derivative");
  return 0;
}

// gYout = J(st)^T gk; the parameter cotangent is added to W->gparam.
int rhs_vjp(sfd_engine* e, AdjWork* W, const AdjStage& st, const double* gk, double* gYout) {
  const AdjConst K = adj_const(e->hs[0]);
  const int n = K.n;
  cudaStream_t s = e->stream;
  const int nb = nblocks(n, kAdjThreads), nw = nblocks(32LL * n, kAdjThreads);
  k_adj_out<<<nb, kAdjThreads, 0, s>>>(K, st, gk, gYout, W->apb_re, W->apb_im, W->cbar, W->dbar, W->abar, W->zpb_re,
                                       W->zpb_im, W->zppb_re, W->zppb_im, W->pbar);
  ACK(cudaGetLastError());
  int rc = spectral(e, W, 0, W->apb_re, W->apb_im, W->t1);
  if (rc) return rc;
  k_adj_sum_cd<<<1, kAdjThreads, 0, s>>>(n, W->cbar, W->dbar, W->sums);
  if (!W->mixed) {
    k_adj_sums1<<<nw, kAdjThreads, 0, s>>>(K, st.w, st.p, W->cbar, W->dbar, W->sb, W->tb);
    k_adj_a<<<nb, kAdjThreads, 0, s>>>(K, W->sums, W->t1, W->cbar, W->sb, W->tb, W->abar);
    k_lu_solve_t<<<1, kAdjThreads, K.np * sizeof(double), s>>>(n, K.np, st.lu, W->abar, W->lam);
    k_adj_node2<<<nb, kAdjThreads, 0, s>>>(K, st, W->lam, W->cbar, W->dbar, W->zpb_re, W->zpb_im, W->zppb_re,
                                           W->zppb_im, nullptr, 0, 0.0, nullptr);
    k_adj_sums2<<<nw, kAdjThreads, 0, s>>>(K, st, W->cbar, W->dbar, gYout);
  } else {
    const long long nn = (long long)n * n;
    k_adj_pairs<<<nblocks(nn, kAdjThreads), kAdjThreads, 0, s>>>(K, st.w, st.p, W->R, W->I);
    k_adj_sums1m<<<nw, kAdjThreads, 0, s>>>(K, st.w, W->R, W->I, W->cbar, W->dbar, W->sb, W->tb);
    k_adj_a<<<nb, kAdjThreads, 0, s>>>(K, W->sums, W->t1, W->cbar, W->sb, W->tb, W->abar);
    // lambda = M^-T ga by refinement preconditioned with X^T
    k_adjt_init<<<1, 1024, 0, s>>>(K, st, W->abar, e->rscale, W->lam, W->v, W->bw, W->rmax);
    k_gemv_ht<<<K.np / 64, 512, 0, s>>>(n, K.np, e->m16, W->v, W->lam, W->rmax, 0);
    for (int it = 1; it <= kAdjtIters; ++it) {
      k_adjt_resid<<<nw, kAdjThreads, 0, s>>>(K, st, W->R, W->I, W->bw, W->abar, W->lam, e->rscale, W->v, W->rmax,
                                              it);
      if (it < kAdjtIters) k_gemv_ht<<<K.np / 64, 512, 0, s>>>(n, K.np, e->m16, W->v, W->lam, W->rmax, it);
    }
    k_adj_node2<<<nb, kAdjThreads, 0, s>>>(K, st, W->lam, W->cbar, W->dbar, W->zpb_re, W->zpb_im, W->zppb_re,
                                           W->zppb_im, W->rmax, kAdjtIters, e->opt.refine_tol, e->status);
    k_adj_sums2m<<<nw, kAdjThreads, 0, s>>>(K, st, W->R, W->I, W->cbar, W->dbar, gYout);
  }
  ACK(cudaGetLastError());
  rc = spectral(e, W, 0, W->zpb_re, W->zpb_im, W->t1);
  if (!rc) rc = spectral(e, W, 1, W->zppb_re, W->zppb_im, W->t2);
  if (!rc) rc = spectral(e, W, 0, W->lam, nullptr, W->t3);
  if (rc) return rc;
  k_adj_final<<<nb, kAdjThreads, 0, s>>>(K, W->t1, W->t2, W->t3, gYout);
  // parameter: d/dA3 = d/dvdw / h^3 (helium), d/dg (water)
  const double scale = K.physics == 1 ? 1.0 / (K.depth * K.depth * K.depth) : 1.0;
  k_adj_sum_param<<<1, kAdjThreads, 0, s>>>(n, W->pbar, scale, W->gparam);
  ACK(cudaGetLastError());
  return 0;
}

const double kW[4] = {1.0, 2.0, 2.0, 1.0};

// One RK4 step of W->y in place (the forward path's stage kernels, so the
// trajectory matches the engine's own steps bitwise).  With rec != nullptr
// the four stages are recorded in rec[0..3].
int adj_step(sfd_engine* e, AdjWork* W, double dt, AdjStage* rec, bool refactor = true) {
  const int n3 = 3 * W->n;
  const int nb = nblocks(n3, 256);
  const double cy[4] = {dt * 0.5, dt * 0.5, dt, 0.0};
  cudaStream_t s = e->stream;
  for (int st = 0; st < 4; ++st) {
    const double* in = st == 0 ? W->y : (rec ? rec[st].Y : W->ys);
    double* kout = rec ? rec[st].k : W->ktmp;
    if (rec) {
      if (st == 0) ACK(cudaMemcpyAsync(rec[0].Y, W->y, 8 * (size_t)n3, cudaMemcpyDeviceToDevice, s));
      int rc = record_rhs(e, W, rec[st], refactor && st == 0);
      if (rc) return rc;
    } else {
      int rc = sfd_internal_rhs_ex(e, in, kout, refactor && st == 0);
      if (rc) return rc;
    }
    double* ynext = st < 3 ? (rec ? rec[st + 1].Y : W->ys) : nullptr;
    k_rk4_stage<<<nb, 256, 0, s>>>(n3, W->y, kout, W->kacc, ynext, kW[st], cy[st], st == 0);
    ACK(cudaGetLastError());
  }
  k_rk4_final<<<nb, 256, 0, s>>>(n3, W->y, W->kacc, dt / 6.0);
  ACK(cudaGetLastError());
  return 0;
}

// Reverse one recorded step: W->gY <- (d y_{n+1} / d y_n)^T W->gY.
int adj_step_back(sfd_engine* e, AdjWork* W, double dt, const AdjStage* rec) {
  const int n3 = 3 * W->n;
  const int nb = nblocks(n3, 256);
  cudaStream_t s = e->stream;
  // stage 4: gk4 = dt/6 gY
  k_adj_lin<<<nb, 256, 0, s>>>(n3, W->gk, dt / 6.0, W->gY, 0.0, nullptr);
  int rc = rhs_vjp(e, W, rec[3], W->gk, W->gYs[3]);
  if (rc) return rc;
  k_adj_lin<<<nb, 256, 0, s>>>(n3, W->gk, dt / 3.0, W->gY, dt, W->gYs[3]);
  rc = rhs_vjp(e, W, rec[2], W->gk, W->gYs[2]);
  if (rc) return rc;
  k_adj_lin<<<nb, 256, 0, s>>>(n3, W->gk, dt / 3.0, W->gY, dt * 0.5, W->gYs[2]);
  rc = rhs_vjp(e, W, rec[1], W->gk, W->gYs[1]);
  if (rc) return rc;
  k_adj_lin<<<nb, 256, 0, s>>>(n3, W->gk, dt / 6.0, W->gY, dt * 0.5, W->gYs[1]);
  rc = rhs_vjp(e, W, rec[0], W->gk, W->gYs[0]);
  if (rc) return rc;
  k_adj_acc4<<<nb, 256, 0, s>>>(n3, W->gY, W->gYs[0], W->gYs[1], W->gYs[2], W->gYs[3]);
  ACK(cudaGetLastError());
  return 0;
}

}  // namespace

// ---------------------------------------------------------------- C ABI
extern "C" int sfd_rhs_vjp_device(sfd_engine* e, const void* state, const void* cotangent, void* grad_state,
                                  double* grad_param) {
  int rc = check_engine(e);
  if (rc) return rc;
  if (!state || !cotangent || !grad_state) return sfd_internal_error(SFD_ERR_INVALID, "null argument");
  ACK(cudaSetDevice(e->device));
  rc = ensure_work(e, 1);
  if (rc) return rc;
  AdjWork* W = e->adj;
  const size_t n3 = 3 * (size_t)W->n;
  AdjStage& st = W->slots[0];
  ACK(cudaMemcpyAsync(st.Y, state, 8 * n3, cudaMemcpyDeviceToDevice, e->stream));
  ACK(cudaMemsetAsync(W->gparam, 0, sizeof(double), e->stream));
  rc = record_rhs(e, W, st);
  if (rc) return rc;
  rc = rhs_vjp(e, W, st, static_cast<const double*>(cotangent), static_cast<double*>(grad_state));
  if (rc) return rc;
  double gp = 0.0;
  ACK(cudaMemcpyAsync(&gp, W->gparam, sizeof(double), cudaMemcpyDeviceToHost, e->stream));
  ACK(cudaStreamSynchronize(e->stream));
  if (grad_param) *grad_param = gp;
  return 0;
}

// Row i of J is J^T e_i: one reverse sweep per row over the recorded stage,
// scattered into the column-major Jacobian.
__global__ void k_jac_unit(int n3, int row, double* g) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n3) g[c] = c == row ? 1.0 : 0.0;
}
__global__ void k_jac_scatter_row(int n3, int row, const double* g, double* jac) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n3) jac[(long long)c * n3 + row] = g[c];
}

extern "C" int sfd_jacobian_device(sfd_engine* e, const void* state, void* jac) {
  int rc = check_engine(e);
  if (rc) return rc;
  if (!state || !jac) return sfd_internal_error(SFD_ERR_INVALID, "null argument");
  ACK(cudaSetDevice(e->device));
  rc = ensure_work(e, 1);
  if (rc) return rc;
  AdjWork* W = e->adj;
  const int n3 = 3 * W->n;
  cudaStream_t s = e->stream;
  AdjStage& st = W->slots[0];
  ACK(cudaMemcpyAsync(st.Y, state, 8 * (size_t)n3, cudaMemcpyDeviceToDevice, s));
  rc = record_rhs(e, W, st);
  if (rc) return rc;
  double* out = static_cast<double*>(jac);
  for (int row = 0; row < n3; ++row) {
    k_jac_unit<<<nblocks(n3, 256), 256, 0, s>>>(n3, row, W->gk);
    rc = rhs_vjp(e, W, st, W->gk, W->gYs[0]);
    if (rc) return rc;
    k_jac_scatter_row<<<nblocks(n3, 256), 256, 0, s>>>(n3, row, W->gYs[0], out);
    ACK(cudaGetLastError());
  }
  ACK(cudaStreamSynchronize(s));
  return 0;
}

extern "C" int sfd_rk4_record(sfd_engine* e, double dt, int steps, int checkpoint_every, const double* state0,
                              double* state_final) {
  int rc = check_engine(e);
  if (rc) return rc;
  if (!state0 || steps < 0 || checkpoint_every < 1) return sfd_internal_error(SFD_ERR_INVALID, "invalid argument");
  ACK(cudaSetDevice(e->device));
  rc = ensure_work(e, checkpoint_every);
  if (rc) return rc;
  AdjWork* W = e->adj;
  const size_t n3 = 3 * (size_t)W->n;
  const int nckpt = steps / checkpoint_every + 1;
  if (nckpt > W->ckpt_cap) {
    if (W->ckpt) cudaFree(W->ckpt);
    W->ckpt = nullptr;
    ACK(cudaMalloc(&W->ckpt, 8 * n3 * nckpt));
    W->ckpt_cap = nckpt;
  }
  W->steps = steps;
  W->every = checkpoint_every;
  W->nckpt = nckpt;
  W->dt = dt;
  if (W->mixed) {
    // The engine's own stepping (captured step graphs, preconditioner schedule
    // and background rebuilds as configured) on its resident state, which is
    // saved before and restored after.
    ACK(cudaStreamSynchronize(e->stream));
    ACK(cudaMemcpyAsync(W->ysave, e->y0, 8 * n3, cudaMemcpyDeviceToDevice, e->stream));
    ACK(cudaMemcpyAsync(e->y0, state0, 8 * n3, cudaMemcpyHostToDevice, e->stream));
    for (int i = 0; i < steps && !rc; i += checkpoint_every) {
      ACK(cudaMemcpyAsync(W->ckpt + n3 * (i / checkpoint_every), e->y0, 8 * n3, cudaMemcpyDeviceToDevice,
                          e->stream));
      rc = sfd_rk4_steps_async(e, dt, std::min(checkpoint_every, steps - i));
    }
    if (!rc && state_final) ACK(cudaMemcpyAsync(state_final, e->y0, 8 * n3, cudaMemcpyDeviceToHost, e->stream));
    ACK(cudaMemcpyAsync(e->y0, W->ysave, 8 * n3, cudaMemcpyDeviceToDevice, e->stream));
    ACK(cudaStreamSynchronize(e->stream));
    return rc;
  }
  ACK(cudaMemcpyAsync(W->y, state0, 8 * n3, cudaMemcpyHostToDevice, e->stream));
  for (int i = 0; i < steps; ++i) {
    if (i % checkpoint_every == 0)
      ACK(cudaMemcpyAsync(W->ckpt + n3 * (i / checkpoint_every), W->y, 8 * n3, cudaMemcpyDeviceToDevice, e->stream));
    rc = adj_step(e, W, dt, nullptr);
    if (rc) return rc;
  }
  if (state_final) ACK(cudaMemcpyAsync(state_final, W->y, 8 * n3, cudaMemcpyDeviceToHost, e->stream));
  ACK(cudaStreamSynchronize(e->stream));
  return 0;
}

extern "C" int sfd_rk4_vjp(sfd_engine* e, const double* cot_final, double* grad_state0, double* grad_param) {
  int rc = check_engine(e);
  if (rc) return rc;
  if (!e->adj || e->adj->every < 1) return sfd_internal_error(SFD_ERR_INVALID, "sfd_rk4_vjp: call sfd_rk4_record first");
  if (!cot_final || !grad_state0) return sfd_internal_error(SFD_ERR_INVALID, "null argument");
  ACK(cudaSetDevice(e->device));
  AdjWork* W = e->adj;
  const size_t n3 = 3 * (size_t)W->n;
  cudaStream_t s = e->stream;
  ACK(cudaMemcpyAsync(W->gY, cot_final, 8 * n3, cudaMemcpyHostToDevice, s));
  ACK(cudaMemsetAsync(W->gparam, 0, sizeof(double), s));
  const int nseg = (W->steps + W->every - 1) / W->every;
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int n0 = seg * W->every, n1 = std::min(W->steps, n0 + W->every);
    // recompute the segment from its checkpoint, recording every stage
    // (a mixed engine rebuilds its preconditioner at the segment's first
    // evaluation and keeps it for the segment's recomputation and reversal)
    ACK(cudaMemcpyAsync(W->y, W->ckpt + n3 * seg, 8 * n3, cudaMemcpyDeviceToDevice, s));
    for (int i = n0; i < n1; ++i) {
      rc = adj_step(e, W, W->dt, &W->slots[4 * (size_t)(i - n0)], i == n0);
      if (rc) return rc;
    }
    for (int i = n1 - 1; i >= n0; --i) {
      rc = adj_step_back(e, W, W->dt, &W->slots[4 * (size_t)(i - n0)]);
      if (rc) return rc;
    }
  }
  double gp = 0.0;
  ACK(cudaMemcpyAsync(grad_state0, W->gY, 8 * n3, cudaMemcpyDeviceToHost, s));
  ACK(cudaMemcpyAsync(&gp, W->gparam, sizeof(double), cudaMemcpyDeviceToHost, s));
  ACK(cudaStreamSynchronize(s));
  if (grad_param) *grad_param = gp;
  return 0;
}
