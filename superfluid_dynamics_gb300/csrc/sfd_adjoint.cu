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
//    refinement preconditioned by X^T, the transpose of the engine's FP32
//    approximate inverse X (kept as an FP32 transposed copy per block of
//    recomputed steps):
//      lambda_0 = X^T ga;  r = ga - M^T lambda (FP64, matrix-free);  lambda += X^T r
//    where, with gC = i c1 conj(z') lambda and gD = -i cI lambda,
//      (M^T lambda)_j = Mdiag_j lambda_j + Re(i (sum gC - gC_j) + 2 i conj(Sb_j)) + Re(-i sum gD + 2 i Tb_j)
//    (Sb, Tb as in the ga line above, here with b_k = -i c1 w_k z'_k lambda_k).
//    The corrections are gated on the residual (they return at once once
//    max |r| <= 1e-13 max |ga|, or once a correction gained less than a factor
//    4); a final residual above the engine's refine_tol raises
//    SFD_ST_REFINE_STALL.  Every pair sum of one stage reads the pair
//    reciprocals R_jk = 1 / (w_j - w_k), bw_k R_jk and I_jk = 1 / (1 - p_j conj p_k),
//    computed once per stage in FP64 into n x n complex matrices.
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
  const float* xt;  // mixed engines: X^T of the preconditioner rebuilt for this stage's block of steps
};

namespace {

constexpr int kAdjThreads = 256;
// Transposed solve of mixed engines: residual checks (each but the last
// followed by a correction, gated on the residual), and the relative residual
// below which the remaining checks and corrections return at once.  They also
// stop once a correction gained less than a factor 1 / kAdjtStagnation: the
// residual has reached the noise floor of its FP64 evaluation (about 3e-15
// relative on the fit film at n = 512), where further corrections change
// nothing.
constexpr int kAdjtIters = 5;
constexpr double kAdjtGateTol = 1e-13;
constexpr double kAdjtStagnation = 0.25;
// The reverse sweep of a mixed engine rebuilds the preconditioner every
// kXtEvery steps of a recomputed segment and keeps one X^T per block of steps:
// with X up to 50 steps old the transposed solve needs five products or more,
// with X fresh three.
constexpr int kXtEvery = 10;

// Whether the solve stopped at residual check `it` (NaN: not stopped).
__device__ __forceinline__ bool adjt_converged(const double* rmax, int it) {
  return it > 0 && (rmax[it] <= kAdjtGateTol * rmax[0] || (it >= 2 && rmax[it] > kAdjtStagnation * rmax[it - 1]));
}

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
// Output side: E, V1, V2 and the Bernoulli closure.  The output cotangent is
// alpha ga + beta gb (gb nullable: the RK4 reverse combines the step's
// cotangents here).  With rmax (mixed engines), thread 0 clears the
// transposed solve's residual slots 0..kAdjtIters.
__global__ void k_adj_out(AdjConst K, AdjStage st, double alpha, const double* ga, double beta, const double* gb,
                          double* gY, double* apb_re, double* apb_im, cd* cbar, cd* dbar, double* abar,
                          double* zpb_re, double* zpb_im, double* zppb_re, double* zppb_im, double* pbar,
                          double* rmax) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = K.n;
  if (rmax && k <= kAdjtIters) rmax[k] = 0.0;
  if (k >= n) return;
  const double inv4pi = 0.25 / SFD_PI;
  const double dx = st.k[k], dy = st.k[n + k], yk = st.Y[n + k];
  auto cot = [&](int i) { return gb ? alpha * ga[i] + beta * gb[i] : alpha * ga[i]; };
  const double gphi = cot(2 * n + k);
  const double gxt = cot(k) + gphi * dx, gyt = cot(n + k) + gphi * dy;
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
// With rmax (mixed engines' transposed solve, residual slots 0..last), thread
// 0 also raises the refinement-stall bit when the final residual rmax[last]
// is above tol * rmax[0] (or NaN), and records the final relative residual
// and the corrections the solve ran (maxima over the solves of a call).
__global__ void k_adj_node2(AdjConst K, AdjStage st, const double* lambda, cd* cbar, cd* dbar, double* zpb_re,
                            double* zpb_im, double* zppb_re, double* zppb_im, const double* rmax, int last,
                            double tol, unsigned int* status, double* diag_rel, unsigned int* diag_corr, cd* bq) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (rmax && k == 0) {
    const double b = rmax[0], rl = rmax[last];
    if (!(rl <= tol * b)) atomicOr(status, (unsigned int)SFD_ST_REFINE_STALL);
    const double rel = b > 0.0 ? rl / b : (rl > 0.0 ? 1e300 : 0.0);
    atomicMax(reinterpret_cast<unsigned long long*>(diag_rel),
              (unsigned long long)__double_as_longlong(rel == rel ? rel : 1e300));
    unsigned int corr = 1;  // the first product
    for (int it = 1; it < last; ++it) corr += adjt_converged(rmax, it) ? 0u : 1u;
    atomicMax(diag_corr, corr);
  }
  if (k >= K.n) return;
  const double rho = -lambda[k];
  const cd zp = st.zp[k], zpp = st.zpp[k];
  const cd izp = crcp(zp);
  const cd cb = cbar[k] + cmul_i(K.c1 * rho * cconj(zp));
  cbar[k] = cb;
  if (bq) bq[k] = st.w[k] * cconj(cb);  // the weight w_j conj(gC_j) of the second-order sums
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
// (0 on the diagonal), Rb_jk = bw_k R_jk with bw = -i c1 w z' (the weights of
// M^T lambda) and, with the image, I_jk = 1 / (1 - p_j conj p_k).  R is
// antisymmetric and I Hermitian, so one CTA computes the 32 x 32 block (J, K),
// J <= K, once and writes it and its mirror (K, J) (through shared memory, so
// that both writes are coalesced): half the FP64 divisions of a full pass.
// The mirrored R is bitwise the direct one; the mirrored I may differ from a
// direct evaluation in the last bit (p_k conj p_j and p_j conj p_k round
// separately).
__device__ __forceinline__ cd adj_bw(const AdjConst& K, cd w, cd zp) { return cmul_i(-K.c1 * (w * zp)); }
__global__ void __launch_bounds__(256) k_adj_pairs(AdjConst K, const cd* w, const cd* p, const cd* zp, cd* R,
                                                   cd* Rb, cd* I) {
  __shared__ cd sr[32][33], si[32][33];
  __shared__ cd wJ[32], wK[32], pJ[32], pK[32], bJ[32], bK[32];
  const int n = K.n;
  // triangular block index t = Kb (Kb + 1) / 2 + Jb, Jb <= Kb
  const int t = blockIdx.x;
  int Kb = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
  while ((Kb + 1) * (Kb + 2) / 2 <= t) ++Kb;
  while (Kb * (Kb + 1) / 2 > t) --Kb;
  const int Jb = t - Kb * (Kb + 1) / 2;
  const int j0 = 32 * Jb, k0 = 32 * Kb;
  if (threadIdx.x < 32) {
    const int i = threadIdx.x;
    const int j = min(j0 + i, n - 1), k = min(k0 + i, n - 1);
    wJ[i] = w[j];
    wK[i] = w[k];
    bJ[i] = adj_bw(K, w[j], zp[j]);
    bK[i] = adj_bw(K, w[k], zp[k]);
    pJ[i] = K.image ? p[j] : cd{0.0, 0.0};
    pK[i] = K.image ? p[k] : cd{0.0, 0.0};
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 32 * 32; e += 256) {
    const int jj = e >> 5, kk = e & 31;
    const int j = j0 + jj, k = k0 + kk;
    cd r = {0.0, 0.0}, q = {0.0, 0.0};
    if (j < n && k < n) {
      r = j == k ? cd{0.0, 0.0} : crcp(wJ[jj] - wK[kk]);
      const long long o = (long long)j * n + k;
      R[o] = r;
      Rb[o] = bK[kk] * r;
      if (K.image) {
        q = crcp(cd{1.0, 0.0} - pJ[jj] * cconj(pK[kk]));
        I[o] = q;
      }
    }
    sr[jj][kk] = r;
    si[jj][kk] = q;
  }
  if (Jb == Kb) return;  // uniform over the CTA
  __syncthreads();
  // mirror: row k = k0 + a, column j = j0 + b: R_kj = -R_jk, I_kj = conj I_jk
  for (int e = threadIdx.x; e < 32 * 32; e += 256) {
    const int a = e >> 5, b = e & 31;
    const int k = k0 + a, j = j0 + b;
    if (k < n && j < n) {
      const cd r = sr[b][a];
      const cd rr = {-r.re, -r.im};
      const long long o = (long long)k * n + j;
      R[o] = rr;
      Rb[o] = bJ[b] * rr;
      if (K.image) I[o] = cconj(si[b][a]);
    }
  }
}

// The pair sums below give each target kWpt warps (a CTA holds kTpc targets):
// warp w of a target takes the sources k = lane + 32 (w + kWpt i), and the
// warps' sums are combined in a fixed order through shared memory, so results
// are bitwise repeatable.  One warp per target would leave about three warps
// per SM at n = 512, too few to cover the FP64 latency.
constexpr int kWpt = 4;
constexpr int kTpc = 2;
constexpr int kPairThreads = 32 * kWpt * kTpc;

// Combine NV complex accumulators of the kWpt warps of each target; the
// result is returned to lane 0 of the target's first warp (others: zeros).
template <int NV>
__device__ __forceinline__ void pair_reduce(cd* acc, cd (*sh)[kWpt][NV]) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = warp / kWpt, w = warp % kWpt;
#pragma unroll
  for (int i = 0; i < NV; ++i) acc[i] = warp_sum(acc[i]);
  if (lane == 0)
#pragma unroll
    for (int i = 0; i < NV; ++i) sh[t][w][i] = acc[i];
  __syncthreads();
  if (w == 0 && lane == 0) {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      cd v = sh[t][0][i];
#pragma unroll
      for (int q = 1; q < kWpt; ++q) v = cadd(v, sh[t][q][i]);
      acc[i] = v;
    }
  }
}

// k_adj_sums1 from the pair reciprocals, with k_adj_a's combination and the
// transposed solve's set-up in the epilogue: ga_j = abar_j - s1 Re R1(ga')_j
// + Re(i (sum gC - gC_j) + 2 i conj(Sb_j)) + Re(-i sum gD + 2 i Tb_j) is the
// solve's right-hand side; lambda_j = 0, v_j = ga_j (FP32, input of the first
// X^T product) and max |ga| into rmax[0] (cleared by k_adj_out).
__global__ void __launch_bounds__(kPairThreads) k_adj_sums1m(AdjConst K, const cd* w, const cd* R, const cd* I,
                                                            const cd* cbar, const cd* dbar, const cd* sums,
                                                            const cd* r1apb, double* abar, double* lam, float* v,
                                                            double* rmax) {
  __shared__ cd sh[kTpc][kWpt][2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.x * kTpc + warp / kWpt;
  const int k0 = lane + 32 * (warp % kWpt);
  cd acc[2] = {{0, 0}, {0, 0}};
  if (j < K.n) {
    const cd* Rj = R + (long long)j * K.n;
    const cd* Ij = I + (long long)j * K.n;
    for (int k = k0; k < K.n; k += 32 * kWpt) {
      acc[0] = cadd(acc[0], (w[k] * cconj(cbar[k])) * Rj[k]);  // R_jj = 0
      if (K.image) acc[1] = cadd(acc[1], dbar[k] * Ij[k]);
    }
  }
  pair_reduce<2>(acc, sh);
  if (j < K.n && k0 == 0) {
    const double s1 = 2.0 * SFD_PI / K.n;
    double g = abar[j] - s1 * r1apb[j].re;
    const cd sc = sums[0], sd = sums[1];
    g += (cmul_i(sc - cbar[j]) + cmul_i(2.0 * cconj(acc[0]))).re;
    if (K.image) g += (cmul_i(cd{-sd.re, -sd.im}) + cmul_i(2.0 * acc[1])).re;
    abar[j] = g;
    lam[j] = 0.0;
    v[j] = (float)g;
    const double ag = fabs(g);
    atomicMax(reinterpret_cast<unsigned long long*>(rmax), (unsigned long long)__double_as_longlong(ag == ag ? ag : 1e300));
  }
}

// k_adj_sums2 from the pair reciprocals: R_kj = 1 / (w_k - w_j),
// I_kj = 1 / (1 - p_k conj p_j).
__global__ void __launch_bounds__(kPairThreads) k_adj_sums2m(AdjConst K, AdjStage st, const cd* R, const cd* I,
                                                            const cd* cbar, const cd* dbar, const cd* bq,
                                                            double* gY) {
  __shared__ cd sh[kTpc][kWpt][5];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = blockIdx.x * kTpc + warp / kWpt;
  const int j0 = lane + 32 * (warp % kWpt);
  const cd* w = st.w;
  const cd* p = st.p;
  const double* a = st.a;
  cd acc[5] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}};  // S, S2, Q, T2, U
  if (k < K.n) {
    const cd* Rk = R + (long long)k * K.n;
    const cd* Ik = I + (long long)k * K.n;
    for (int j = j0; j < K.n; j += 32 * kWpt) {
      const double aj = a[j];
      const cd inv = Rk[j];  // 0 for j = k
      const cd inv2 = inv * inv;
      acc[0] = cadd(acc[0], aj * inv);
      acc[1] = cadd(acc[1], aj * inv2);
      acc[2] = cadd(acc[2], bq[j] * inv2);  // bq = w conj(gC)
      if (K.image) {
        const cd ie = Ik[j];
        const cd ie2c = (ie * ie) * cconj(p[j]);
        acc[3] = cadd(acc[3], aj * ie2c);
        acc[4] = cadd(acc[4], dbar[j] * ie2c);
      }
    }
  }
  pair_reduce<5>(acc, sh);
  if (k < K.n && j0 == 0) {
    const cd S = acc[0], S2 = acc[1], Q = acc[2], T2 = acc[3], U = acc[4];
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

// X^T as a row-major FP32 matrix: xt[j][i] = X[i][j] for the np x np padded
// inverse (the padding keeps its identity).  32 x 32 tiles through shared memory.
// Record of one evaluation's node data into a stage slot (one launch in place
// of eight copies).
__global__ void k_adj_store(int n, const double* a, const cd* ap, const cd* zp, const cd* zpp, const cd* C,
                            const cd* D, const cd* w, const cd* p, AdjStage st) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  st.a[i] = a[i];
  st.ap[i] = ap[i];
  st.zp[i] = zp[i];
  st.zpp[i] = zpp[i];
  st.C[i] = C[i];
  st.D[i] = D[i];
  st.w[i] = w[i];
  st.p[i] = p[i];
}

__global__ void k_adj_transpose(int np, const float* X, float* xt) {
  __shared__ float tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) tile[r][threadIdx.x] = X[(long long)(by + r) * np + bx + threadIdx.x];
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) xt[(long long)(bx + r) * np + by + threadIdx.x] = tile[threadIdx.x][r];
}


// lambda += X^T v (FP32 products, FP64 update) where the residual of slot
// `it` is above the gate (slot 0: the first product, always): one warp per row
// j of xt = X^T, kGtRows rows per CTA.  The epilogue also writes the CTA's
// partial sums of conj(z'_j) lambda_j and lambda_j (fixed order), which the
// residual kernel totals: part[2 b] = sum conj(z') lambda, part[2 b + 1].re =
// sum lambda over the CTA's rows.
constexpr int kGtRows = 16;
__global__ void __launch_bounds__(32 * kGtRows) k_adjt_gemv(int n, int np, const float* xt, const float* v,
                                                           const cd* zp, double* lam, cd* part, const double* rmax,
                                                           int it) {
  if (adjt_converged(rmax, it)) return;
  extern __shared__ float4 vsh4[];
  __shared__ cd red[kGtRows][2];
  float* vsh = reinterpret_cast<float*>(vsh4);
  const int n4 = (n + 3) & ~3;
  for (int i = threadIdx.x; i < n4; i += blockDim.x) vsh[i] = i < n ? v[i] : 0.f;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.x * kGtRows + warp;
  cd pz = {0, 0}, pl = {0, 0};
  if (j < n) {
    const float4* row = reinterpret_cast<const float4*>(xt + (long long)j * np);
    float acc = 0.f;
    for (int q = lane; q < n4 / 4; q += 32) {
      const float4 a = __ldg(row + q), b = vsh4[q];
      acc = fmaf(a.x, b.x, fmaf(a.y, b.y, fmaf(a.z, b.z, fmaf(a.w, b.w, acc))));
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) {
      const double l = lam[j] + (double)acc;
      lam[j] = l;
      pz = l * cconj(zp[j]);
      pl = {l, 0.0};
    }
  }
  if (lane == 0) {
    red[warp][0] = pz;
    red[warp][1] = pl;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    cd a = red[0][0], b = red[0][1];
    for (int w = 1; w < kGtRows; ++w) {
      a = cadd(a, red[w][0]);
      b = cadd(b, red[w][1]);
    }
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
  }
}

// r = ga - M^T lambda (FP64) into v = r (FP32) and max |r| into slot `it`
// (sum conj(z') lambda and sum lambda from the product's partial sums,
// nparts CTAs).  Where slot it - 1 is converged, slot it inherits it and
// nothing else runs.
__global__ void __launch_bounds__(kPairThreads) k_adjt_resid(AdjConst K, AdjStage st, const cd* Rb, const cd* I,
                                                            const cd* part, int nparts, const double* ga,
                                                            const double* lam, float* v, double* rmax, int it) {
  if (adjt_converged(rmax, it - 1)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) rmax[it] = rmax[it - 1];
    return;
  }
  __shared__ cd sh[kTpc][kWpt][2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.x * kTpc + warp / kWpt;
  const int k0 = lane + 32 * (warp % kWpt);
  cd acc[2] = {{0, 0}, {0, 0}};  // sb = sum_k lambda_k bw_k R_jk, tb = sum_k lambda_k I_jk
  if (j < K.n) {
    const cd* Rj = Rb + (long long)j * K.n;
    const cd* Ij = I + (long long)j * K.n;
    for (int k = k0; k < K.n; k += 32 * kWpt) {
      const double lk = lam[k];
      const cd rb = Rj[k];
      acc[0].re = fma(lk, rb.re, acc[0].re);  // Rb_jj = 0
      acc[0].im = fma(lk, rb.im, acc[0].im);
      if (K.image) {
        const cd ie = Ij[k];
        acc[1].re = fma(lk, ie.re, acc[1].re);
        acc[1].im = fma(lk, ie.im, acc[1].im);
      }
    }
  }
  pair_reduce<2>(acc, sh);
  if (j < K.n && k0 == 0) {
    cd sz = {0, 0};
    double sl = 0.0;
    for (int b = 0; b < nparts; ++b) {
      sz = cadd(sz, part[2 * b]);
      sl += part[2 * b + 1].re;
    }
    const cd sb = acc[0], tb = acc[1];
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
    v[j] = (float)r;
    const double ar = fabs(r);
    atomicMax(reinterpret_cast<unsigned long long*>(rmax + it),
              (unsigned long long)__double_as_longlong(ar == ar ? ar : 1e300));
  }
}

// spectral part: gZ = -s1 R1(gz') + s2 R2(gz''); gphi = -s1 Re R1(lambda)
// Block 0 also adds scale * sum pbar to *acc (the parameter cotangent, summed
// in a fixed order).
__global__ void __launch_bounds__(kAdjThreads) k_adj_final(AdjConst K, const cd* r1zpb, const cd* r2zppb,
                                                          const cd* r1lam, double* gY, const double* pbar,
                                                          double scale, double* acc) {
  if (blockIdx.x == 0) {
    __shared__ double sp[kAdjThreads];
    double v = 0.0;
    for (int i = threadIdx.x; i < K.n; i += kAdjThreads) v += pbar[i];
    sp[threadIdx.x] = v;
    __syncthreads();
    for (int h = kAdjThreads / 2; h > 0; h >>= 1) {
      if (threadIdx.x < h) sp[threadIdx.x] += sp[threadIdx.x + h];
      __syncthreads();
    }
    if (threadIdx.x == 0) *acc += scale * sp[0];
  }
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K.n) return;
  const double s1 = 2.0 * SFD_PI / K.n;
  const double s2 = s1 * s1;
  const cd gz = (-s1) * r1zpb[k] + s2 * r2zppb[k];
  gY[k] += gz.re;
  gY[K.n + k] += gz.im;
  gY[2 * K.n + k] = -s1 * r1lam[k].re;
}

// RK4 helper: acc += a + b + c + d
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
  cd *R = nullptr, *Rb = nullptr, *I = nullptr, *bq = nullptr;
  cd* part = nullptr;          // per-CTA partial sums of the X^T product (2 per CTA)
  float* v = nullptr;
  float* xt = nullptr;         // transpose of the FP32 approximate inverse (np x np)
  double* rmax = nullptr;
  double* ysave = nullptr;
  double* diag_rel = nullptr;  // max final relative residual of the transposed solves of the last call
  unsigned int* diag_corr = nullptr;  // max corrections they ran
  // four-step transforms of the reverse sweep (power-of-two n in [512, 8192]):
  // plan a' (the a' cotangent) and plan 3 (z', z'' and lambda cotangents)
  F4Plan f4_ap, f4_3;
  cd* f4_scr = nullptr;
  // fork / join of the reverse sweep's independent branches onto the
  // engine's auxiliary stream (mixed engines)
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  int2* jobs = nullptr;        // {0, RAW}, {0, RAW2}
  std::vector<void*> allocs;
  // captured steps of sfd_rk4_vjp (engines with use_graphs): for step slot i
  // of a segment, g_rec[i] recomputes the step recording its stages into
  // slots 4i..4i+3 (slot 0 with the preconditioner rebuild) and g_rev[i]
  // reverses it; valid for g_dt and the current slots
  std::vector<cudaGraphExec_t> g_rec, g_rev;
  std::vector<long long> g_rec_nodes, g_rev_nodes;
  double g_dt = 0.0;
  AdjConst g_K{};  // surface constants the graphs' kernels were given
};

static bool same_const(const AdjConst& a, const AdjConst& b) {
  return a.n == b.n && a.np == b.np && a.physics == b.physics && a.image == b.image && a.c1 == b.c1 &&
         a.cI == b.cI && a.depth == b.depth && a.vdw == b.vdw && a.gravity == b.gravity && a.rho == b.rho;
}

static void adj_destroy_graphs(AdjWork* W) {
  for (auto* v : {&W->g_rec, &W->g_rev})
    for (cudaGraphExec_t& g : *v)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
}

void sfd_adjoint_free(sfd_engine* e) {
  if (!e || !e->adj) return;
  adj_destroy_graphs(e->adj);
  if (e->adj->xt) cudaFree(e->adj->xt);
  if (e->adj->ev_fork) cudaEventDestroy(e->adj->ev_fork);
  if (e->adj->ev_join) cudaEventDestroy(e->adj->ev_join);
  for (void* p : e->adj->allocs) cudaFree(p);
  if (e->adj->slot_mem) cudaFree(e->adj->slot_mem);
  if (e->adj->ckpt) cudaFree(e->adj->ckpt);
  delete e->adj;
  e->adj = nullptr;
}

// Why reverse mode does not cover the engine, or null when it does.
const char* sfd_adjoint_unsupported(const sfd_engine* e) {
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
    adj_destroy_graphs(W);  // captured with the old slots
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
      ACK(adj_alloc(W, &W->Rb, (size_t)n * n));
      ACK(adj_alloc(W, &W->bq, (size_t)n));
      if (K.image) ACK(adj_alloc(W, &W->I, (size_t)n * n));
      ACK(adj_alloc(W, &W->part, 2 * (size_t)((n + kGtRows - 1) / kGtRows)));
      ACK(adj_alloc(W, &W->v, (size_t)n));
      ACK(adj_alloc(W, &W->rmax, (size_t)kAdjtIters + 1));
      ACK(adj_alloc(W, &W->ysave, n3));

      ACK(cudaEventCreateWithFlags(&W->ev_fork, cudaEventDisableTiming));
      ACK(cudaEventCreateWithFlags(&W->ev_join, cudaEventDisableTiming));
      ACK(adj_alloc(W, &W->diag_rel, 1));
      ACK(adj_alloc(W, &W->diag_corr, 1));
    }
    if (sfd_f4_eligible(n)) {
      // jobs: a' cotangent -> t1; then z' -> t1, z'' -> t2, lambda -> t3
      const F4Job ja[1] = {{0, SFD_F4_RAW1, 0, 0, W->apb_re, W->apb_im, W->t1}};
      const F4Job j3[3] = {{0, SFD_F4_RAW1, 0, 0, W->zpb_re, W->zpb_im, W->t1},
                           {0, SFD_F4_RAW2, (long long)n, 0, W->zppb_re, W->zppb_im, W->t2},
                           {0, SFD_F4_RAW1, 2LL * n, 0, W->lam, nullptr, W->t3}};
      for (int pi = 0; pi < 2; ++pi) {
        F4Plan& P = pi == 0 ? W->f4_ap : W->f4_3;
        const F4Job* jl = pi == 0 ? ja : j3;
        const int nj = pi == 0 ? 1 : 3;
        std::vector<int2> ul[3];
        for (int j = 0; j < nj; ++j) {
          for (int u = 0; u < 64; ++u) ul[0].push_back({j, u});
          for (int u = 0; u < n / 64; ++u) ul[1].push_back({j, u});
          for (int u = 0; u < 64; ++u) ul[2].push_back({j, u});
        }
        ACK(adj_alloc(W, &P.jobs, (size_t)nj));
        ACK(cudaMemcpy(P.jobs, jl, nj * sizeof(F4Job), cudaMemcpyHostToDevice));
        for (int ph = 0; ph < 3; ++ph) {
          ACK(adj_alloc(W, &P.units[ph], ul[ph].size()));
          ACK(cudaMemcpy(P.units[ph], ul[ph].data(), ul[ph].size() * sizeof(int2), cudaMemcpyHostToDevice));
          P.nunits[ph] = (int)ul[ph].size();
        }
        P.njobs = nj;
      }
      ACK(adj_alloc(W, &W->f4_scr, 3 * (size_t)n));
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
  if (W->mixed) {
    if (W->xt) cudaFree(W->xt);
    W->xt = nullptr;
    ACK(cudaMalloc(&W->xt, sizeof(float) * np * np * (size_t)((steps + kXtEvery - 1) / kXtEvery)));
  }
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
    s.xt = W->mixed ? W->xt + np * np * (i / 4 / kXtEvery) : nullptr;
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
  k_adj_store<<<nblocks((long long)n, kAdjThreads), kAdjThreads, 0, s>>>((int)n, e->a, e->ap, e->zp, e->zpp, e->cacc,
                                                                          e->dacc, e->nd.w, e->nd.p, st);
  ACK(cudaGetLastError());
  return 0;
}

int spectral(sfd_engine* e, AdjWork* W, int job, const double* re, const double* im, cd* out,
             cudaStream_t st = nullptr) {
  DerivArgs D{e->d_surf, 1, re, im, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, out, nullptr};
  cudaError_t err = sfd_launch_spectral(D, W->jobs + job, 1, W->n, st ? st : e->stream);
  if (err != cudaSuccess) return sfd_internal_cuda(err, "spectral derivative");
  return 0;
}

// The jobs of a four-step plan (unscaled first / second derivatives of the
// jobs' own inputs) in its three launches.
int spectral_f4(sfd_engine* e, AdjWork* W, const F4Plan& P, cudaStream_t st = nullptr) {
  DerivArgs D{e->d_surf, 1, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  for (int ph = 1; ph <= 3; ++ph) {
    cudaError_t err = sfd_launch_f4(D, P, W->f4_scr, st ? st : e->stream, ph);
    if (err != cudaSuccess) return sfd_internal_cuda(err, "four-step transform");
  }
  return 0;
}

// Start of a reverse-mode call: clear the transposed-solve record.
int clear_diag(sfd_engine* e, AdjWork* W) {
  if (!W->mixed) return 0;
  ACK(cudaMemsetAsync(W->diag_rel, 0, sizeof(double), e->stream));
  ACK(cudaMemsetAsync(W->diag_corr, 0, sizeof(unsigned int), e->stream));
  return 0;
}

// Mixed engines: X^T from the FP32 inverse the last preconditioner rebuild
// left in e->m32, into the stage's block (call after every evaluation that
// rebuilt it).
int refresh_xt(sfd_engine* e, AdjWork* W, const AdjStage& st) {
  if (!W->mixed) return 0;
  k_adj_transpose<<<dim3(W->np / 32, W->np / 32), dim3(32, 8), 0, e->stream>>>(W->np, e->m32,
                                                                               const_cast<float*>(st.xt));
  ACK(cudaGetLastError());
  return 0;
}

// gYout = J(st)^T gk; the parameter cotangent is added to W->gparam.
// The output cotangent is alpha ga + beta gb (gb nullable).
int rhs_vjp(sfd_engine* e, AdjWork* W, const AdjStage& st, double alpha, const double* ga, double beta,
            const double* gb, double* gYout) {
  const AdjConst K = adj_const(e->hs[0]);
  const int n = K.n;
  cudaStream_t s = e->stream;
  const int nb = nblocks(n, kAdjThreads), nw = nblocks(32LL * n, kAdjThreads);
  k_adj_out<<<nb, kAdjThreads, 0, s>>>(K, st, alpha, ga, beta, gb, gYout, W->apb_re, W->apb_im, W->cbar, W->dbar,
                                       W->abar, W->zpb_re, W->zpb_im, W->zppb_re, W->zppb_im, W->pbar,
                                       W->mixed ? W->rmax : nullptr);
  ACK(cudaGetLastError());
  // Mixed engines fork independent work onto the auxiliary stream (captured
  // graphs keep the fork as parallel branches): the pair reciprocals and the
  // gC / gD totals beside the a' cotangent's transform, and later the
  // cotangents' transforms beside the second-order pair sums.
  const bool fork = W->mixed && e->aux && !e->profile;
  cudaStream_t x = fork ? e->aux : s;
  const int T = (n + 31) / 32;
  if (fork) {
    ACK(cudaEventRecord(W->ev_fork, s));
    ACK(cudaStreamWaitEvent(x, W->ev_fork, 0));
  }
  if (W->mixed) k_adj_pairs<<<T * (T + 1) / 2, 256, 0, x>>>(K, st.w, st.p, st.zp, W->R, W->Rb, W->I);
  k_adj_sum_cd<<<1, kAdjThreads, 0, x>>>(n, W->cbar, W->dbar, W->sums);
  if (fork) ACK(cudaEventRecord(W->ev_join, x));
  int rc = W->f4_ap.njobs ? spectral_f4(e, W, W->f4_ap) : spectral(e, W, 0, W->apb_re, W->apb_im, W->t1);
  if (rc) return rc;
  if (fork) ACK(cudaStreamWaitEvent(s, W->ev_join, 0));
  if (!W->mixed) {
    k_adj_sums1<<<nw, kAdjThreads, 0, s>>>(K, st.w, st.p, W->cbar, W->dbar, W->sb, W->tb);
    k_adj_a<<<nb, kAdjThreads, 0, s>>>(K, W->sums, W->t1, W->cbar, W->sb, W->tb, W->abar);
    k_lu_solve_t<<<1, kAdjThreads, K.np * sizeof(double), s>>>(n, K.np, st.lu, W->abar, W->lam);
    k_adj_node2<<<nb, kAdjThreads, 0, s>>>(K, st, W->lam, W->cbar, W->dbar, W->zpb_re, W->zpb_im, W->zppb_re,
                                           W->zppb_im, nullptr, 0, 0.0, nullptr, nullptr, nullptr, nullptr);
    k_adj_sums2<<<nw, kAdjThreads, 0, s>>>(K, st, W->cbar, W->dbar, gYout);
  } else {
    const int np_blocks = (n + kTpc - 1) / kTpc;
    const int gt_blocks = (n + kGtRows - 1) / kGtRows;
    const size_t gt_smem = (size_t)((n + 3) & ~3) * sizeof(float);
    // Sb, Tb and the solve's right-hand side ga (k_adj_a), lambda = 0, v = ga
    k_adj_sums1m<<<np_blocks, kPairThreads, 0, s>>>(K, st.w, W->R, W->I, W->cbar, W->dbar, W->sums, W->t1,
                                                    W->abar, W->lam, W->v, W->rmax);
    // lambda = M^-T ga by refinement preconditioned with X^T (the FP32
    // inverse's transpose, st.xt): lambda = X^T ga, then r = ga - M^T lambda,
    // lambda += X^T r while the residual is above the gate
    for (int it = 0; it < kAdjtIters; ++it) {
      if (it > 0)
        k_adjt_resid<<<np_blocks, kPairThreads, 0, s>>>(K, st, W->Rb, W->I, W->part, gt_blocks, W->abar, W->lam,
                                                        W->v, W->rmax, it);
      k_adjt_gemv<<<gt_blocks, 32 * kGtRows, gt_smem, s>>>(n, K.np, st.xt, W->v, st.zp, W->lam, W->part, W->rmax,
                                                           it);
    }
    k_adjt_resid<<<np_blocks, kPairThreads, 0, s>>>(K, st, W->Rb, W->I, W->part, gt_blocks, W->abar, W->lam, W->v,
                                                    W->rmax, kAdjtIters);
    k_adj_node2<<<nb, kAdjThreads, 0, s>>>(K, st, W->lam, W->cbar, W->dbar, W->zpb_re, W->zpb_im, W->zppb_re,
                                           W->zppb_im, W->rmax, kAdjtIters, e->opt.refine_tol, e->status,
                                           W->diag_rel, W->diag_corr, W->bq);
    if (fork) {
      ACK(cudaEventRecord(W->ev_fork, s));
      ACK(cudaStreamWaitEvent(x, W->ev_fork, 0));
    }
    k_adj_sums2m<<<np_blocks, kPairThreads, 0, x>>>(K, st, W->R, W->I, W->cbar, W->dbar, W->bq, gYout);
    if (fork) ACK(cudaEventRecord(W->ev_join, x));
  }
  ACK(cudaGetLastError());
  if (W->f4_3.njobs) {
    rc = spectral_f4(e, W, W->f4_3);
  } else {
    rc = spectral(e, W, 0, W->zpb_re, W->zpb_im, W->t1);
    if (!rc) rc = spectral(e, W, 1, W->zppb_re, W->zppb_im, W->t2);
    if (!rc) rc = spectral(e, W, 0, W->lam, nullptr, W->t3);
  }
  if (rc) return rc;
  if (fork) ACK(cudaStreamWaitEvent(s, W->ev_join, 0));
  // parameter: d/dA3 = d/dvdw / h^3 (helium), d/dg (water)
  const double scale = K.physics == 1 ? 1.0 / (K.depth * K.depth * K.depth) : 1.0;
  k_adj_final<<<nb, kAdjThreads, 0, s>>>(K, W->t1, W->t2, W->t3, gYout, W->pbar, scale, W->gparam);
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
  // stage cotangents: k4: dt/6 gY; k3: dt/3 gY + dt g(Y4); k2: dt/3 gY + dt/2 g(Y3); k1: dt/6 gY + dt/2 g(Y2)
  int rc = rhs_vjp(e, W, rec[3], dt / 6.0, W->gY, 0.0, nullptr, W->gYs[3]);
  if (rc) return rc;
  rc = rhs_vjp(e, W, rec[2], dt / 3.0, W->gY, dt, W->gYs[3], W->gYs[2]);
  if (rc) return rc;
  rc = rhs_vjp(e, W, rec[1], dt / 3.0, W->gY, dt * 0.5, W->gYs[2], W->gYs[1]);
  if (rc) return rc;
  rc = rhs_vjp(e, W, rec[0], dt / 6.0, W->gY, dt * 0.5, W->gYs[1], W->gYs[0]);
  if (rc) return rc;
  k_adj_acc4<<<nb, 256, 0, s>>>(n3, W->gY, W->gYs[0], W->gYs[1], W->gYs[2], W->gYs[3]);
  ACK(cudaGetLastError());
  return 0;
}

// Run `body` (which enqueues on the engine stream) through the cached graph
// *g, capturing it first if there is none; *nodes counts its nodes.
template <typename F>
int run_captured(sfd_engine* e, cudaGraphExec_t* g, long long* nodes, F&& body) {
  if (!*g) {
    cudaGraph_t graph = nullptr;
    const long long before = e->launches;
    ACK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    int rc = body();
    cudaError_t ce = cudaStreamEndCapture(e->stream, &graph);
    e->launches = before;
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (ce != cudaSuccess) return sfd_internal_cuda(ce, "adjoint step capture");
    size_t nn = 0;
    cudaGraphGetNodes(graph, nullptr, &nn);
    *nodes = (long long)nn;
    ce = cudaGraphInstantiate(g, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return sfd_internal_cuda(ce, "adjoint step graph");
  }
  ACK(cudaGraphLaunch(*g, e->stream));
  e->launches += *nodes;
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
  rc = clear_diag(e, W);
  if (!rc) rc = record_rhs(e, W, st);
  if (!rc) rc = refresh_xt(e, W, st);
  if (rc) return rc;
  rc = rhs_vjp(e, W, st, 1.0, static_cast<const double*>(cotangent), 0.0, nullptr, static_cast<double*>(grad_state));
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
  rc = clear_diag(e, W);
  if (!rc) rc = record_rhs(e, W, st);
  if (!rc) rc = refresh_xt(e, W, st);
  if (rc) return rc;
  double* out = static_cast<double*>(jac);
  for (int row = 0; row < n3; ++row) {
    k_jac_unit<<<nblocks(n3, 256), 256, 0, s>>>(n3, row, W->gk);
    rc = rhs_vjp(e, W, st, 1.0, W->gk, 0.0, nullptr, W->gYs[0]);
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
  rc = clear_diag(e, W);
  if (rc) return rc;
  const int nseg = (W->steps + W->every - 1) / W->every;
  // With graphs, each step of a segment (recomputation and reversal) is one
  // captured graph per step slot, replayed for every segment and call.
  const bool graphs = e->opt.use_graphs && !e->profile;
  if (graphs) {
    rc = sfd_internal_bg_flush(e);  // a pending background rebuild cannot be switched in during capture
    if (rc) return rc;
    // the reverse kernels take the surface constants (A3, g, ...) by value:
    // after sfd_set_problem the graphs are captured again
    const AdjConst K = adj_const(e->hs[0]);
    if (W->g_dt != W->dt || !same_const(W->g_K, K)) adj_destroy_graphs(W);
    W->g_dt = W->dt;
    W->g_K = K;
    const size_t cap = (size_t)W->cap_steps;
    W->g_rec.resize(cap, nullptr);
    W->g_rev.resize(cap, nullptr);
    W->g_rec_nodes.resize(cap, 0);
    W->g_rev_nodes.resize(cap, 0);
  }
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int n0 = seg * W->every, n1 = std::min(W->steps, n0 + W->every);
    // recompute the segment from its checkpoint, recording every stage
    // (a mixed engine rebuilds its preconditioner every kXtEvery steps of the
    // segment and keeps each X^T for the reversal of its block of steps)
    ACK(cudaMemcpyAsync(W->y, W->ckpt + n3 * seg, 8 * n3, cudaMemcpyDeviceToDevice, s));
    for (int i = n0; i < n1; ++i) {
      const int k = i - n0;
      AdjStage* rec = &W->slots[4 * (size_t)k];
      const bool rebuild = k % kXtEvery == 0;
      auto body = [&] {
        e->allow_warm = true;  // a recomputed RK4 trajectory: evaluations may start warm
        int r = adj_step(e, W, W->dt, rec, rebuild);
        e->allow_warm = false;
        return (!r && rebuild) ? refresh_xt(e, W, rec[0]) : r;
      };
      rc = graphs ? run_captured(e, &W->g_rec[k], &W->g_rec_nodes[k], body) : body();
      if (rc) return rc;
    }
    for (int i = n1 - 1; i >= n0; --i) {
      const int k = i - n0;
      const AdjStage* rec = &W->slots[4 * (size_t)k];
      auto body = [&] { return adj_step_back(e, W, W->dt, rec); };
      rc = graphs ? run_captured(e, &W->g_rev[k], &W->g_rev_nodes[k], body) : body();
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

extern "C" int sfd_adjoint_residual(sfd_engine* e, double* max_rel_residual, int* max_corrections) {
  if (!e) return sfd_internal_error(SFD_ERR_INVALID, "null engine");
  double rel = 0.0;
  unsigned int corr = 0;
  AdjWork* W = e->adj;
  if (W && W->mixed) {
    ACK(cudaSetDevice(e->device));
    ACK(cudaMemcpyAsync(&rel, W->diag_rel, sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    ACK(cudaMemcpyAsync(&corr, W->diag_corr, sizeof(unsigned int), cudaMemcpyDeviceToHost, e->stream));
    ACK(cudaStreamSynchronize(e->stream));
  }
  if (max_rel_residual) *max_rel_residual = rel;
  if (max_corrections) *max_corrections = (int)corr;
  return 0;
}
