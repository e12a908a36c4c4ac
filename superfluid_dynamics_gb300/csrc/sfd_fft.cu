// sfd_fft.cu -- spectral xi-derivatives of one RK stage.
//
// Replaces ZPhiDerivative::exec / FftDerivative::exec (CSH/Derivatives.cuh:
// 189-257, 310-384) and the multiplier kernels first_derivative_multiplication /
// second_derivative_fft (CSH/utilities.cuh:106-148, 178-200).  Instead of a
// cuFFT plan plus ~8 small kernels per derivative, one CTA per (surface,
// derivative) job holds the whole signal in shared memory (n <= 8192 complex
// doubles = 128 KB) and runs forward transform -> spectral multiply ->
// inverse transform -> scaling without leaving the SM.  Any n = 2^a * (odd
// factors) is supported (the batched helium case uses n = 32 m, m up to 64),
// so the transform is a mixed-radix Stockham FFT: radix-4/2 butterflies plus an
// output-parallel DFT stage for each odd prime factor.
#include <cooperative_groups.h>

#include "sfd_engine.cuh"
#include "sfd_kernels.cuh"

namespace {

constexpr int kFftThreads = 1024;
constexpr int kMaxPerThread = 8;  // n <= 8192 = 8 * 1024

__device__ __forceinline__ cd twid(const cd* tw, int e, int sign) {
  cd t = tw[e];  // shared-memory table in the cluster kernel, global (L1/L2) otherwise
  return sign < 0 ? t : cd{t.re, -t.im};
}

// multiply by -i (forward) or +i (inverse): the radix-4 rotation
__device__ __forceinline__ cd rot(cd a, int sign) { return sign < 0 ? cd{a.im, -a.re} : cd{-a.im, a.re}; }

// One Stockham pass with radix 2 or 4 over buf[0..n) by NT threads holding up
// to MPT values each; p = product of the radices already done.  Twiddles come
// from a table of a multiple of n: W_n^e = tw[e * ts].
template <int R, int NT, int MPT>
__device__ __forceinline__ void stockham_pass(cd* buf, int n, int p, const cd* tw, int ts, int sign) {
  const int T = n / R;
  const int stw = n / (p * R) * ts;
  constexpr int C = (MPT + R - 1) / R;  // butterflies per thread (T = n / R <= C * NT)
  cd u[C][R];
  const bool pow2 = (p & (p - 1)) == 0;
#pragma unroll
  for (int c = 0; c < C; ++c) {
    int i = threadIdx.x + c * NT;
    if (i < T) {
      int k = pow2 ? (i & (p - 1)) : i % p;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        cd v = buf[i + r * T];
        if (r > 0 && k > 0) v = v * twid(tw, r * k * stw, sign);
        u[c][r] = v;
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int c = 0; c < C; ++c) {
    int i = threadIdx.x + c * NT;
    if (i < T) {
      int k = pow2 ? (i & (p - 1)) : i % p;
      int j = (i - k) * R + k;
      if (R == 2) {
        buf[j] = u[c][0] + u[c][1];
        buf[j + p] = u[c][0] - u[c][1];
      } else {
        cd a0 = u[c][0] + u[c][2], a1 = u[c][0] - u[c][2];
        cd b0 = u[c][1] + u[c][3], b1 = rot(u[c][1] - u[c][3], sign);
        buf[j] = a0 + b0;
        buf[j + p] = a1 + b1;
        buf[j + 2 * p] = a0 - b0;
        buf[j + 3 * p] = a1 - b1;
      }
    }
  }
  __syncthreads();
}

// Odd-radix pass: every output y[j + q p] = sum_r x[i + r T] W_n^{r (k + q p) n/(pR)}
// is computed by one thread (R complex MACs), staged in registers, then stored.
template <int NT, int MPT>
__device__ __forceinline__ void odd_pass(cd* buf, int n, int p, int R, const cd* tw, int ts, int sign) {
  const int T = n / R;
  const int stw = n / (p * R);
  cd out[MPT];
#pragma unroll
  for (int c = 0; c < MPT; ++c) {
    int o = threadIdx.x + c * NT;
    if (o < n) {
      int blk = o / (p * R), rem = o - blk * (p * R);
      int q = rem / p, k = rem - q * p;
      int i = blk * p + k;
      int m = k + q * p;
      cd acc = buf[i];
      for (int r = 1; r < R; ++r) {
        int e = (int)(((long long)r * m * stw) % n);
        acc = acc + buf[i + r * T] * twid(tw, e * ts, sign);
      }
      out[c] = acc;
    }
  }
  __syncthreads();
#pragma unroll
  for (int c = 0; c < MPT; ++c) {
    int o = threadIdx.x + c * NT;
    if (o < n) buf[o] = out[c];
  }
  __syncthreads();
}

// Unnormalised in-place FFT of buf[0..n) (sign -1 forward as CUFFT_FORWARD,
// +1 inverse without the 1/n); radices rad[0..nrad), twiddles tw[e * ts].
template <int NT, int MPT>
__device__ void cta_fft_n(cd* buf, int n, const int* rad, int nrad, const cd* tw, int ts, int sign) {
  int p = 1;
  for (int s = 0; s < nrad; ++s) {
    int R = rad[s];
    if (R == 4) stockham_pass<4, NT, MPT>(buf, n, p, tw, ts, sign);
    else if (R == 2) stockham_pass<2, NT, MPT>(buf, n, p, tw, ts, sign);
    else odd_pass<NT, MPT>(buf, n, p, R, tw, ts, sign);
    p *= R;
  }
}

__device__ __forceinline__ void cta_fft(cd* buf, const SurfaceDesc& S, int sign) {
  cta_fft_n<kFftThreads, kMaxPerThread>(buf, S.n, S.rad, S.nrad, S.tw, 1, sign);
}

// Spectral multipliers, restated from utilities.cuh:106-148 (first) and
// :178-200 (second), including the reference's Nyquist treatment: the first
// derivative maps mode n/2 to i (pi/2) c and zeroes mode n/2 + 1.
// inv_n = 1 / n: the multipliers scale by a reciprocal instead of dividing
// (FP64 division is a long dependent sequence on the FP64 pipe).
__device__ __forceinline__ cd first_mult(cd c, int i, int n, double inv_n) {
  double f;
  if (i < n / 2) f = (double)i * inv_n;
  else if (i == n / 2) f = SFD_PI * i * inv_n;
  else if (i == n / 2 + 1) return {0.0, 0.0};
  else f = (double)(i - n) * inv_n;
  return {-f * c.im, f * c.re};
}
__device__ __forceinline__ cd second_mult(cd c, int i, int n, double inv_n) {
  const int kk = (i <= n / 2) ? -i * i : -(i - n) * (i - n);
  const double f = (double)kk * inv_n;
  return {f * c.re, f * c.im};
}
// xi_j = 2 pi j / n rounded exactly as the division of the reference
// (Derivatives.cuh:285) rounds it: the product 2 pi j, then its quotient by n
// from the correctly rounded reciprocal and one correction with the exact
// remainder (Markstein's quotient refinement), which gives the correctly
// rounded quotient.  x - xi is a near-cancellation for Eulerian nodes, so the
// abscissa must match the reference's bit for bit, not to within an ulp.
__device__ __forceinline__ double xi_node(int j, double dn, double inv_n) {
  const double a = 2.0 * SFD_PI * (double)j;
  const double q0 = a * inv_n;
  const double r = fma(-q0, dn, a);
  return fma(r, inv_n, q0);
}

}  // namespace

__global__ void __launch_bounds__(kFftThreads, 1) k_spectral_deriv(DerivArgs A, const int2* jobs) {
  sfd_pdl_begin();
  extern __shared__ double2 smem_raw[];
  cd* buf = reinterpret_cast<cd*>(smem_raw);
  const int2 job = jobs[blockIdx.x];
  if (!gate_open(A.gate, job.x)) return;
  const SurfaceDesc& S = A.surf[job.x];  // read in place: copying would put rad[] on the stack
  const int n = S.n, off = S.off, kind = job.y;
  const double rho = S.physics == 0 ? S.rho : 0.0;
  const double dn = (double)n, inv_n = 1.0 / dn;
  const double uq = -(1 + rho) * SFD_PI * S.U / n;  // linear part of phi per node (same rounding as per element)
  for (int j = threadIdx.x; j < n; j += kFftThreads) {
    cd v;
    if (kind == SFD_JOB_ZP || kind == SFD_JOB_ZPP) {
      v = {A.x[off + j] - xi_node(j, dn, inv_n), A.y[off + j]};                // Derivatives.cuh:285,317
    } else if (kind == SFD_JOB_PHIP) {
      v = {A.phi[off + j] - uq * (double)j,                                    // Derivatives.cuh:286,318
           A.phi_im ? A.phi_im[off + j] : 0.0};
    } else if (kind == SFD_JOB_RAW || kind == SFD_JOB_RAW2) {
      v = {A.x[off + j], A.y ? A.y[off + j] : 0.0};
    } else {
      v = {A.a[off + j], 0.0};                                                 // real_to_complex(a)
    }
    buf[j] = v;
  }
  __syncthreads();
  cta_fft(buf, S, -1);
  for (int i = threadIdx.x; i < n; i += kFftThreads)
    buf[i] = (kind == SFD_JOB_ZPP || kind == SFD_JOB_RAW2) ? second_mult(buf[i], i, n, inv_n)
                                                           : first_mult(buf[i], i, n, inv_n);
  __syncthreads();
  cta_fft(buf, S, +1);
  const double s1 = 2.0 * SFD_PI / n;
  const double s2 = 4.0 * SFD_PI * SFD_PI / (n * n);
  for (int j = threadIdx.x; j < n; j += kFftThreads) {
    cd v = buf[j];
    switch (kind) {
      case SFD_JOB_ZP: A.zp[off + j] = {v.re * s1 + s1, v.im * s1}; break;   // Derivatives.cuh:323,374
      case SFD_JOB_ZPP: A.zpp[off + j] = {v.re * s2, v.im * s2}; break;       // :321
      case SFD_JOB_PHIP: {
        double r = v.re * s1;                                                 // :324, complex_to_real
        if (S.U != 0) r += -(1 + rho) * SFD_PI * S.U / n;                     // :380-383
        A.phip[off + j] = r;
        if (A.phipf) A.phipf[off + j] = (float)r;
        break;
      }
      case SFD_JOB_RAW:                                                       // FftDerivative::exec, scale 1
      case SFD_JOB_RAW2: A.ap[off + j] = v; break;
      default: A.ap[off + j] = {v.re * s1, v.im * s1}; break;                 // BaseBoundaryIntegrator.cuh:203
    }
  }
}

// ===================================================================== cluster version
// One thread-block cluster of C = SFD_FFT_CLUSTER CTAs per job; the transform of
// length n = C M is split as (with k = k1 + M k2, j = C m + c):
//   forward:  Y_c = FFT_M(x[C m + c]);  Z_c[k1] = W_n^{c k1} Y_c[k1]          (CTA c)
//             X[k1 + M k2] = sum_c W_C^{c k2} Z_c[k1]            (CTA owning k1, via DSMEM)
//   multiply: X <- mult(X)  (reference Nyquist rules, global index k)
//   inverse:  V_c[k1] = W_n^{-c k1} sum_k2 W_C^{-c k2} X[k1 + M k2]   (CTA owning k1)
//             x[C m + c] = IFFT_M(V_c)[m]                        (CTA c, via DSMEM)
// so each SM does 1/C of the FP64 work and the exchange stays on chip.  GB300
// runs FP64 at 2 FMA per clock per SM, so the kernel counts FP64 operations:
// no division per element, and the exchange's 8-point transforms split over
// two lanes (one shuffle butterfly + a 4-point DFT each), which keeps one
// warp per SM sub-partition busy at R = 64 with close to the arithmetic of a
// single-lane transform.
namespace {
constexpr int kCT = 512;        // threads per CTA of the cluster kernel
constexpr int kCMPT = 2;        // values per thread in the M-point FFT (M <= 1024)
constexpr double kH = 0.70710678118654752440;

__device__ __forceinline__ cd shfl_xor_cd(cd a, int m) {
  return {__shfl_xor_sync(0xffffffffu, a.re, m), __shfl_xor_sync(0xffffffffu, a.im, m)};
}
// W_8^j for j < 4, sign -1 (forward, e^{-2 pi i j / 8}) or +1 (inverse)
__device__ __forceinline__ cd w8(int j, int sign) {
  const double sg = sign < 0 ? -1.0 : 1.0;
  switch (j) {
    case 0: return {1.0, 0.0};
    case 1: return {kH, sg * kH};
    case 2: return {0.0, sg};
    default: return {-kH, sg * kH};
  }
}
// 4-point DFT in registers, natural order in and out (sign -1 forward,
// +1 inverse without scaling).
__device__ __forceinline__ void dft4(cd* y, int sign) {
  const cd a0 = y[0] + y[2], a1 = y[0] - y[2];
  const cd b0 = y[1] + y[3], b1 = rot(y[1] - y[3], sign);
  y[0] = a0 + b0;
  y[1] = a1 + b1;
  y[2] = a0 - b0;
  y[3] = a1 - b1;
}
}  // namespace

__global__ void __cluster_dims__(SFD_FFT_CLUSTER, 1, 1) __launch_bounds__(kCT)
    k_spectral_cluster(DerivArgs A, const int2* jobs) {
  sfd_pdl_begin();
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  constexpr int C = SFD_FFT_CLUSTER;
  static_assert(C == 8, "the exchange step is written for 8-CTA clusters");
  extern __shared__ double2 csmem_raw[];
  const int2 job = jobs[blockIdx.y];
  if (!gate_open(A.gate, job.x)) return;  // every CTA of the cluster has the same job
  const SurfaceDesc& S = A.surf[job.x];
  const int n = S.n, off = S.off, kind = job.y;
  const int M = n / C, R = M / C;
  const int c = (int)cluster.block_rank();
  const bool second = (kind == SFD_JOB_ZPP);
  cd* buf = reinterpret_cast<cd*>(csmem_raw);  // M values
  cd* vbuf = buf + M;                          // C x R values
  cd* twm = vbuf + M;                          // W_M^e = W_n^{C e}, e < M
  const double2* twc = reinterpret_cast<const double2*>(S.ctw) + M + (size_t)c * 2 * M;  // W_n^{c k1}
  const double2* twq = twc + M;                                                          // W_n^{q (c R + t)}
  const double rho = S.physics == 0 ? S.rho : 0.0;
  const double dn = (double)n, inv_n = 1.0 / dn;
  const double uq = -(1 + rho) * SFD_PI * S.U / n;  // linear part of phi per node
  for (int e = threadIdx.x; e < M; e += kCT) {
    const double2 a = __ldg(reinterpret_cast<const double2*>(S.ctw) + e);
    twm[e] = {a.x, a.y};
  }
  // 1. decimated load x[C m + c]
  for (int m = threadIdx.x; m < M; m += kCT) {
    const int j = C * m + c;
    cd v;
    if (kind == SFD_JOB_ZP || kind == SFD_JOB_ZPP) v = {A.x[off + j] - xi_node(j, dn, inv_n), A.y[off + j]};
    else if (kind == SFD_JOB_PHIP) v = {A.phi[off + j] - uq * (double)j, A.phi_im ? A.phi_im[off + j] : 0.0};
    else if (kind == SFD_JOB_RAW) v = {A.x[off + j], A.y[off + j]};
    else v = {A.a[off + j], 0.0};
    buf[m] = v;
  }
  __syncthreads();
  cta_fft_n<kCT, kCMPT>(buf, M, S.rad_m, S.nrad_m, twm, 1, -1);
  // 2. Z_c[k1] = W_n^{c k1} Y_c[k1]
  if (c) {
    for (int k1 = threadIdx.x; k1 < M; k1 += kCT)
      if (k1) {
        const double2 w = __ldg(twc + k1);
        buf[k1] = buf[k1] * cd{w.x, w.y};
      }
  }
  cluster.sync();
  // 3. exchange across the cluster for this CTA's k1 range.  Two lanes per
  //    k1: lane h holds the values of CTAs 4h..4h+3; one shuffle butterfly
  //    (span 4) plus an in-register 4-point DFT per lane give X[k1 + M (2k + h)]
  //    in lane h, and the inverse runs the same two steps backwards.  A warp
  //    covers 16 k1 values and skips the loop when none of them is in range;
  //    inside a partly filled warp every lane shuffles and the idle ones only
  //    skip their loads and stores.
  {
    const int h = threadIdx.x & 1;
    const int warp_t = (threadIdx.x >> 5) * 16;
    for (int t0 = 0; t0 < R; t0 += kCT / 2) {
      if (t0 + warp_t >= R) break;
      const int t = t0 + (threadIdx.x >> 1);
      const bool act = t < R;
      const int k1 = c * R + t;
      cd v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] = act ? cluster.map_shared_rank(buf, 4 * h + q)[k1] : cd{0.0, 0.0};
      // forward, span 4: lane 0 keeps x_q + x_{q+4}, lane 1 (x_q - x_{q+4}) W_8^q
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const cd o = shfl_xor_cd(v[q], 1);
        const cd sq = h ? o - v[q] : v[q] + o;
        v[q] = (h && q) ? sq * w8(q, -1) : sq;
      }
      dft4(v, -1);  // lane h: X[k1 + M (2k + h)] in v[k]
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int kk = k1 + M * (2 * k + h);
        v[k] = second ? second_mult(v[k], kk, n, inv_n) : first_mult(v[k], kk, n, inv_n);
      }
      // inverse: 4-point inverse DFT per lane, then the span-4 butterfly with W_8^{+q}
      dft4(v, +1);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const cd wq = (h && q) ? v[q] * w8(q, +1) : v[q];
        const cd o = shfl_xor_cd(wq, 1);
        v[q] = h ? o - wq : wq + o;  // lane h: sum over k2 for target CTA 4h + q
      }
      if (act) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int qq = 4 * h + q;
          cd u = v[q];
          if (qq && k1) {
            const double2 w = __ldg(twq + qq * R + t);
            u = u * cd{w.x, -w.y};
          }
          vbuf[qq * R + t] = u;
        }
      }
    }
  }
  cluster.sync();
  // 4. gather V_c[k1] for all k1, inverse M-point FFT, write x[C m + c]
  const double s1 = 2.0 * SFD_PI / n;
  const double s2 = 4.0 * SFD_PI * SFD_PI / (n * n);
  {
    for (int k1 = threadIdx.x; k1 < M; k1 += kCT) {
      int owner = k1 / R, t = k1 - owner * R;
      buf[k1] = cluster.map_shared_rank(vbuf, owner)[c * R + t];
    }
    __syncthreads();
    cta_fft_n<kCT, kCMPT>(buf, M, S.rad_m, S.nrad_m, twm, 1, +1);
    for (int m = threadIdx.x; m < M; m += kCT) {
      const int j = off + C * m + c;
      cd x = buf[m];
      if (kind == SFD_JOB_ZPP) {
        A.zpp[j] = {x.re * s2, x.im * s2};               // Derivatives.cuh:321
      } else if (kind == SFD_JOB_ZP) {
        A.zp[j] = {x.re * s1 + s1, x.im * s1};           // :323,374
      } else if (kind == SFD_JOB_PHIP) {
        double r = x.re * s1;                           // :324, complex_to_real
        if (S.U != 0) r += uq;
        A.phip[j] = r;
        if (A.phipf) A.phipf[j] = (float)r;
      } else if (kind == SFD_JOB_RAW) {
        A.ap[j] = x;
      } else {
        A.ap[j] = {x.re * s1, x.im * s1};
      }
    }
    __syncthreads();
  }
  cluster.sync();  // keep this CTA's shared memory alive until every peer has read it
}

cudaError_t sfd_launch_spectral_cluster(const DerivArgs& A, const int2* jobs, int njobs, int max_n, cudaStream_t st) {
  if (njobs == 0) return cudaSuccess;
  const int M = max_n / SFD_FFT_CLUSTER;
  size_t smem = (size_t)3 * M * sizeof(cd);
  return sfd_launch(k_spectral_cluster, dim3(SFD_FFT_CLUSTER, njobs), dim3(kCT), smem, st, true, A, jobs);
}

cudaError_t sfd_fft_configure() {
  cudaError_t e = cudaFuncSetAttribute(k_spectral_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       3 * (8192 / SFD_FFT_CLUSTER) * (int)sizeof(cd));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_spectral_deriv, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              8192 * (int)sizeof(cd));
}

// Launch helper: one CTA per job, dynamic shared memory = max n * 16 bytes.
cudaError_t sfd_launch_spectral(const DerivArgs& A, const int2* jobs, int njobs, int max_n, cudaStream_t st) {
  if (njobs == 0) return cudaSuccess;
  size_t smem = (size_t)max_n * sizeof(cd);
  return sfd_launch(k_spectral_deriv, dim3(njobs), dim3(kFftThreads), smem, st, true, A, jobs);
}
