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
#include "sfd_engine.cuh"
#include "sfd_kernels.cuh"

namespace {

constexpr int kFftThreads = 1024;
constexpr int kMaxPerThread = 8;  // n <= 8192 = 8 * 1024

__device__ __forceinline__ cd twid(const cd* tw, int e, int sign) {
  double2 t = __ldg(reinterpret_cast<const double2*>(tw) + e);
  return sign < 0 ? cd{t.x, t.y} : cd{t.x, -t.y};
}

// multiply by -i (forward) or +i (inverse): the radix-4 rotation
__device__ __forceinline__ cd rot(cd a, int sign) { return sign < 0 ? cd{a.im, -a.re} : cd{-a.im, a.re}; }

// One Stockham pass with radix 2 or 4; p = product of the radices already done.
template <int R>
__device__ __forceinline__ void stockham_pass(cd* buf, int n, int p, const cd* tw, int sign) {
  const int T = n / R;
  const int stw = n / (p * R);
  constexpr int C = kMaxPerThread / R;
  cd u[C][R];
#pragma unroll
  for (int c = 0; c < C; ++c) {
    int i = threadIdx.x + c * kFftThreads;
    if (i < T) {
      int k = i % p;
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
    int i = threadIdx.x + c * kFftThreads;
    if (i < T) {
      int k = i % p;
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
__device__ __forceinline__ void odd_pass(cd* buf, int n, int p, int R, const cd* tw, int sign) {
  const int T = n / R;
  const int stw = n / (p * R);
  cd out[kMaxPerThread];
#pragma unroll
  for (int c = 0; c < kMaxPerThread; ++c) {
    int o = threadIdx.x + c * kFftThreads;
    if (o < n) {
      int blk = o / (p * R), rem = o - blk * (p * R);
      int q = rem / p, k = rem - q * p;
      int i = blk * p + k;
      int m = k + q * p;
      cd acc = buf[i];
      for (int r = 1; r < R; ++r) {
        int e = (int)(((long long)r * m * stw) % n);
        acc = acc + buf[i + r * T] * twid(tw, e, sign);
      }
      out[c] = acc;
    }
  }
  __syncthreads();
#pragma unroll
  for (int c = 0; c < kMaxPerThread; ++c) {
    int o = threadIdx.x + c * kFftThreads;
    if (o < n) buf[o] = out[c];
  }
  __syncthreads();
}

// Unnormalised in-place FFT of buf[0..n) (sign -1 forward as CUFFT_FORWARD,
// +1 inverse without the 1/n).
__device__ void cta_fft(cd* buf, const SurfaceDesc& S, int sign) {
  int p = 1;
  const int n = S.n, nrad = S.nrad;
  const cd* tw = S.tw;
  for (int s = 0; s < nrad; ++s) {
    int R = S.rad[s];
    if (R == 4) stockham_pass<4>(buf, n, p, tw, sign);
    else if (R == 2) stockham_pass<2>(buf, n, p, tw, sign);
    else odd_pass(buf, n, p, R, tw, sign);
    p *= R;
  }
}

// Spectral multipliers, restated from utilities.cuh:106-148 (first) and
// :178-200 (second), including the reference's Nyquist treatment: the first
// derivative maps mode n/2 to i (pi/2) c and zeroes mode n/2 + 1.
__device__ __forceinline__ cd first_mult(cd c, int i, int n) {
  double dn = (double)n;
  if (i < n / 2) return {(double)(-i) * c.im / dn, (double)i * c.re / dn};
  if (i == n / 2) return {-SFD_PI * i * c.im / dn, SFD_PI * i * c.re / dn};
  if (i == n / 2 + 1) return {0.0, 0.0};
  return {(double)(-(i - n)) * c.im / dn, (double)(i - n) * c.re / dn};
}
__device__ __forceinline__ cd second_mult(cd c, int i, int n) {
  int kk = (i <= n / 2) ? -i * i : -(i - n) * (i - n);
  return {(double)kk * c.re / (double)n, (double)kk * c.im / (double)n};
}

}  // namespace

__global__ void __launch_bounds__(kFftThreads, 1) k_spectral_deriv(DerivArgs A, const int2* jobs) {
  extern __shared__ double2 smem_raw[];
  cd* buf = reinterpret_cast<cd*>(smem_raw);
  const int2 job = jobs[blockIdx.x];
  const SurfaceDesc& S = A.surf[job.x];  // read in place: copying would put rad[] on the stack
  const int n = S.n, off = S.off, kind = job.y;
  const double rho = S.physics == 0 ? S.rho : 0.0;
  for (int j = threadIdx.x; j < n; j += kFftThreads) {
    cd v;
    if (kind == SFD_JOB_ZP || kind == SFD_JOB_ZPP) {
      v = {A.x[off + j] - 2 * SFD_PI * (double)j / n, A.y[off + j]};          // Derivatives.cuh:285,317
    } else if (kind == SFD_JOB_PHIP) {
      v = {A.phi[off + j] - (-(1 + rho) * SFD_PI * S.U / n * (double)j),      // Derivatives.cuh:286,318
           A.phi_im ? A.phi_im[off + j] : 0.0};
    } else if (kind == SFD_JOB_RAW) {
      v = {A.x[off + j], A.y[off + j]};
    } else {
      v = {A.a[off + j], 0.0};                                                 // real_to_complex(a)
    }
    buf[j] = v;
  }
  __syncthreads();
  cta_fft(buf, S, -1);
  for (int i = threadIdx.x; i < n; i += kFftThreads)
    buf[i] = kind == SFD_JOB_ZPP ? second_mult(buf[i], i, n) : first_mult(buf[i], i, n);
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
        break;
      }
      case SFD_JOB_RAW: A.ap[off + j] = v; break;                             // FftDerivative::exec, scale 1
      default: A.ap[off + j] = {v.re * s1, v.im * s1}; break;                 // BaseBoundaryIntegrator.cuh:203
    }
  }
}

cudaError_t sfd_fft_configure() {
  return cudaFuncSetAttribute(k_spectral_deriv, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              8192 * (int)sizeof(cd));
}

// Launch helper: one CTA per job, dynamic shared memory = max n * 16 bytes.
cudaError_t sfd_launch_spectral(const DerivArgs& A, const int2* jobs, int njobs, int max_n, cudaStream_t st) {
  if (njobs == 0) return cudaSuccess;
  size_t smem = (size_t)max_n * sizeof(cd);
  k_spectral_deriv<<<njobs, kFftThreads, smem, st>>>(A, jobs);
  return cudaGetLastError();
}
