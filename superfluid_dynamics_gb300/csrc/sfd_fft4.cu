// sfd_fft4.cu -- spectral xi-derivatives of power-of-two surfaces spread over
// the whole GPU.
//
// Same mathematics as the single-CTA and cluster transforms of sfd_fft.cu
// (ZPhiDerivative::exec / FftDerivative::exec, CSH/Derivatives.cuh:189-384,
// with the multipliers of first_derivative_multiplication /
// second_derivative_fft, CSH/utilities.cuh:106-200, Nyquist rules included):
// forward FFT, multiply, inverse FFT, scale.  GB300's FP64 pipe is narrow
// (about 2 FMA lanes per clock per SM), so a transform confined to one SM or
// one 8-SM cluster is bound by that SM's FP64 issue.  Here a transform of
// n = 64 N2 points (512 <= n <= 8192) is the four-step factorisation
//   x[n1 + 64 n2],  X[k2 + N2 k1]:
//   phase 1  column FFTs over n2 (length N2) for every n1, times W_n^{n1 k2}
//   phase 2  row FFTs over n1 (length 64) for every k2, the spectral
//            multiplier of the global mode k = k2 + N2 k1, the inverse row
//            FFTs (z' and z'' share the forward row FFT), times W_n^{-n1 k2}
//   phase 3  inverse column FFTs over k2, scaling, output
// Each FFT of length L (8 <= L <= 128) belongs to one warp: lane l holds the
// elements l + 32 q (q < L / 32; for L < 32 lanes l >= L idle), and the
// transform is radix-2 across lanes by shuffles (and across a lane's own
// elements for spans of 64 and more), so a lane's dependent chain is about
// 3 FP64 operations and one shuffle per pass.  The forward transform is the
// decimation in frequency (natural order in, bit-reversed out), the inverse
// the decimation in time (bit-reversed in, natural out), so the row phase
// runs forward, multiplier and inverse on the same registers.  Each CTA is
// one warp; its shared memory holds W_L^e.
// Intermediate rows and columns go through an L2-resident scratch (16 bytes
// per node and output).
#include "sfd_engine.cuh"
#include "sfd_kernels.cuh"

namespace {

__device__ __forceinline__ cd twid(const cd* tw, int e, int sign) {
  const cd t = tw[e];
  return sign < 0 ? t : cd{t.re, -t.im};
}
__device__ __forceinline__ cd shfl_xor_cd(cd a, int m) {
  return {__shfl_xor_sync(0xffffffffu, a.re, m), __shfl_xor_sync(0xffffffffu, a.im, m)};
}

// 1 / n for a power of two n, built from the exponent bits (no FP64 division)
__device__ __forceinline__ double inv_pow2(int n) {
  const int e = __ffs(n) - 1;
  return __longlong_as_double((long long)(1023 - e) << 52);
}

template <int L>
struct WF {
  static constexpr int Q = L >= 32 ? L / 32 : 1;  // elements per lane
  static constexpr int LOG = L == 8 ? 3 : L == 16 ? 4 : L == 32 ? 5 : L == 64 ? 6 : 7;
};
template <int L>
__device__ __forceinline__ int bitrev(int i) {
  return (int)(__brev((unsigned)i) >> (32 - WF<L>::LOG));
}

// Forward-direction decimation in frequency (sign -1) or its conjugate (+1):
// natural-order input, bit-reversed output.  twL[e] = W_L^e.
template <int L>
__device__ __forceinline__ void warp_dif(cd* v, const cd* twL, int lane, int sign) {
  constexpr int Q = WF<L>::Q;
#pragma unroll
  for (int half = L / 2; half >= 1; half >>= 1) {
    const int step = L / (2 * half);  // W_{2 half}^j = W_L^{j step}
    if (half >= 32) {
      const int h = half / 32;
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        if ((q / h) % 2 == 0) {
          const int j = (lane + 32 * q) % (2 * half);
          const cd a = v[q], b = v[q + h];
          v[q] = a + b;
          v[q + h] = (a - b) * twid(twL, j * step, sign);
        }
      }
    } else {
      const bool upper = (lane & half) != 0;
      const int j = upper ? (lane % (2 * half)) - half : 0;
      const cd w = upper ? twid(twL, j * step, sign) : cd{1.0, 0.0};
      const double sg = upper ? -1.0 : 1.0;
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        const cd own = v[q];
        const cd p = shfl_xor_cd(own, half);
        // upper lanes hold b and form (a - b) W, lower lanes a + b: one FMA per part
        const cd t = {fma(sg, own.re, p.re), fma(sg, own.im, p.im)};
        v[q] = t * w;
      }
    }
  }
}

// Decimation in time: bit-reversed input, natural-order output.
template <int L>
__device__ __forceinline__ void warp_dit(cd* v, const cd* twL, int lane, int sign) {
  constexpr int Q = WF<L>::Q;
#pragma unroll
  for (int half = 1; half < L; half <<= 1) {
    const int step = L / (2 * half);
    if (half >= 32) {
      const int h = half / 32;
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        if ((q / h) % 2 == 0) {
          const int j = (lane + 32 * q) % (2 * half);
          const cd a = v[q], b = v[q + h] * twid(twL, j * step, sign);
          v[q] = a + b;
          v[q + h] = a - b;
        }
      }
    } else {
      const bool upper = (lane & half) != 0;
      const int j = upper ? (lane % (2 * half)) - half : 0;
      const cd w = upper ? twid(twL, j * step, sign) : cd{1.0, 0.0};
      const double sg = upper ? -1.0 : 1.0;
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        const cd t = v[q] * w;  // upper lanes: b W; lower lanes: a
        const cd p = shfl_xor_cd(t, half);
        v[q] = {fma(sg, t.re, p.re), fma(sg, t.im, p.im)};  // upper: a - b W, lower: a + b W
      }
    }
  }
}

// spectral multipliers, as in sfd_fft.cu (utilities.cuh:106-148, :178-200)
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
// 2 pi j / n rounded as the reference's division rounds it (see sfd_fft.cu)
__device__ __forceinline__ double xi_node(int j, double dn, double inv_n) {
  const double a = 2.0 * SFD_PI * (double)j;
  const double q0 = a * inv_n;
  const double r = fma(-q0, dn, a);
  return fma(r, inv_n, q0);
}

// One warp (one unit: a row or column of one job) per CTA, so the units
// spread over as many SMs as there are units: GB300's FP64 pipe issues a
// warp's FP64 instruction about every 16 cycles, so an SM's FP64 pipe, not
// latency, bounds a CTA of several units.
constexpr int kWarpsPerCta = 1;
constexpr int kF4Threads = 32 * kWarpsPerCta;

}  // namespace

// Phase 1: forward column FFT over n2 for n1 = u, times W_n^{n1 k2}.
template <int L>
__device__ __forceinline__ void f4_phase1(const DerivArgs& A, const F4Job& J, const SurfaceDesc& S, int u,
                                          int lane, const cd* twL, cd* scr) {
  constexpr int Q = WF<L>::Q;
  const int n = S.n, off = S.off, n1 = u;
  const double dn = (double)n, inv_n = inv_pow2(n);
  const double rho = S.physics == 0 ? S.rho : 0.0;
  const double uq = -(1 + rho) * SFD_PI * S.U * inv_n;  // n a power of two: exact as the division
  cd v[Q], pw[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int i = lane + 32 * q;
    const int k2 = bitrev<L>(i & (L - 1));
    pw[q] = twid(S.tw, (n1 * k2) & (n - 1), -1);  // issued before the transform: its index is known
    if (i < L) {
      const int m = n1 + 64 * i;  // node index
      if (J.kind == SFD_F4_Z) v[q] = {A.x[off + m] - xi_node(m, dn, inv_n), A.y[off + m]};          // Derivatives.cuh:285,317
      else if (J.kind == SFD_F4_PHI) v[q] = {A.phi[off + m] - uq * (double)m, A.phi_im ? A.phi_im[off + m] : 0.0};  // :286,318
      else if (J.kind == SFD_F4_AP) v[q] = {A.a[off + m], 0.0};                                     // real_to_complex(a)
      else v[q] = {J.in_re[off + m], J.in_im ? J.in_im[off + m] : 0.0};                             // RAW jobs
    } else {
      v[q] = {0.0, 0.0};
    }
  }
  warp_dif<L>(v, twL, lane, -1);
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int i = lane + 32 * q;
    if (i < L) scr[J.scr0 + (long long)bitrev<L>(i) * 64 + n1] = v[q] * pw[q];
  }
}

// Phase 2: row k2 = u: forward 64-point FFT, multiplier of mode k2 + N2 k1,
// inverse FFT(s), times W_n^{-n1 k2}.
__device__ __forceinline__ void f4_phase2(const F4Job& J, const SurfaceDesc& S, int u, int lane, const cd* twL,
                                          cd* scr) {
  constexpr int Q = 2;
  const int n = S.n, N2 = n / 64, k2 = u;
  const double inv_n = inv_pow2(n);
  cd* row = scr + J.scr0 + (long long)k2 * 64;
  cd v[Q], w[Q], pw[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int i = lane + 32 * q;
    v[q] = row[i];
    pw[q] = twid(S.tw, (i * k2) & (n - 1), +1);
  }
  warp_dif<64>(v, twL, lane, -1);  // element i holds X[k2 + N2 bitrev(i)]
  const bool second_too = J.kind == SFD_F4_Z;
  const bool second_only = J.kind == SFD_F4_RAW2;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int k = k2 + N2 * bitrev<64>(lane + 32 * q);
    w[q] = second_too ? second_mult(v[q], k, n, inv_n) : v[q];
    v[q] = second_only ? second_mult(v[q], k, n, inv_n) : first_mult(v[q], k, n, inv_n);
  }
  warp_dit<64>(v, twL, lane, +1);  // element i holds Y'[n1 = i]
#pragma unroll
  for (int q = 0; q < Q; ++q) row[lane + 32 * q] = v[q] * pw[q];
  if (second_too) {
    warp_dit<64>(w, twL, lane, +1);
    cd* row2 = scr + J.scr1 + (long long)k2 * 64;
#pragma unroll
    for (int q = 0; q < Q; ++q) row2[lane + 32 * q] = w[q] * pw[q];
  }
}

// Phase 3: inverse column FFT over k2.  Unit u: output o = u / 64 (z' then
// z'' for the z job), column n1 = u % 64.
template <int L>
__device__ __forceinline__ void f4_phase3(const DerivArgs& A, const F4Job& J, const SurfaceDesc& S, int u,
                                          int lane, const cd* twL, const cd* scr) {
  constexpr int Q = WF<L>::Q;
  const int n = S.n, off = S.off;
  const int o = u >> 6, n1 = u & 63;
  const cd* col = scr + (o ? J.scr1 : J.scr0) + n1;
  cd v[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int i = lane + 32 * q;
    v[q] = i < L ? col[(long long)bitrev<L>(i) * 64] : cd{0.0, 0.0};  // bit-reversed input
  }
  warp_dit<L>(v, twL, lane, +1);
  // n is a power of two, so scaling by 1/n is exact and equals the division
  const double inv_n = inv_pow2(n);
  const double s1 = 2.0 * SFD_PI * inv_n;
  const double s2 = 4.0 * SFD_PI * SFD_PI * inv_n * inv_n;
  const double rho = S.physics == 0 ? S.rho : 0.0;
  const double uq = -(1 + rho) * SFD_PI * S.U * inv_n;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int i = lane + 32 * q;
    if (i >= L) continue;
    const int j = off + n1 + 64 * i;
    const cd x = v[q];
    if (J.kind == SFD_F4_Z) {
      if (o == 0) A.zp[j] = {x.re * s1 + s1, x.im * s1};  // Derivatives.cuh:323,374
      else A.zpp[j] = {x.re * s2, x.im * s2};           // :321
    } else if (J.kind == SFD_F4_PHI) {
      double r = x.re * s1;                             // :324, complex_to_real
      if (S.U != 0) r += uq;                            // :380-383
      A.phip[j] = r;
      if (A.phipf) A.phipf[j] = (float)r;
    } else if (J.kind == SFD_F4_AP) {
      A.ap[j] = {x.re * s1, x.im * s1};                 // BaseBoundaryIntegrator.cuh:203
    } else {
      J.out[j] = x;                                     // RAW jobs: unscaled
    }
  }
}

template <int PHASE, int L>
__device__ __forceinline__ void f4_run(const DerivArgs& A, const F4Job& J, const SurfaceDesc& S, int u, int lane,
                                       cd* twL, cd* scr) {
  // W_L^e for this CTA's transform length (the CTA's units share one job)
  for (int e = threadIdx.x; e < L; e += kF4Threads) twL[e] = S.tw[(long long)e * (S.n / L)];
  __syncthreads();
  if (PHASE == 1) f4_phase1<L>(A, J, S, u, lane, twL, scr);
  else if (PHASE == 2) f4_phase2(J, S, u, lane, twL, scr);
  else f4_phase3<L>(A, J, S, u, lane, twL, scr);
}

template <int PHASE>
__global__ void __launch_bounds__(kF4Threads) k_fft4(DerivArgs A, const F4Job* jobs, const int2* units, int nunits,
                                                     cd* scr) {
  sfd_pdl_begin();
  __shared__ cd twL[128];
  const int lane = threadIdx.x & 31;
  const int ui = blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5);  // grid = units / kWarpsPerCta: ui < nunits
  const int2 uw = units[ui];
  const F4Job J = jobs[uw.x];
  if (!gate_open(A.gate, J.surf)) return;  // uniform over the CTA
  const SurfaceDesc& S = A.surf[J.surf];
  if (PHASE == 2) {
    f4_run<2, 64>(A, J, S, uw.y, lane, twL, scr);
    return;
  }
  switch (S.n / 64) {
    case 8: f4_run<PHASE, 8>(A, J, S, uw.y, lane, twL, scr); break;
    case 16: f4_run<PHASE, 16>(A, J, S, uw.y, lane, twL, scr); break;
    case 32: f4_run<PHASE, 32>(A, J, S, uw.y, lane, twL, scr); break;
    case 64: f4_run<PHASE, 64>(A, J, S, uw.y, lane, twL, scr); break;
    default: f4_run<PHASE, 128>(A, J, S, uw.y, lane, twL, scr); break;
  }
}

bool sfd_f4_eligible(int n) { return n >= 512 && n <= 8192 && (n & (n - 1)) == 0; }

cudaError_t sfd_launch_f4(const DerivArgs& A, const F4Plan& p, cd* scr, cudaStream_t st, int phase) {
  const int nu = p.nunits[phase - 1];
  if (nu == 0) return cudaSuccess;
  const int grid = nu / kWarpsPerCta;  // every job contributes a multiple of 4 units
  const F4Job* jobs = p.jobs;
  const int2* units = p.units[phase - 1];
  if (phase == 1) return sfd_launch(k_fft4<1>, dim3(grid), dim3(kF4Threads), 0, st, true, A, jobs, units, nu, scr);
  if (phase == 2) return sfd_launch(k_fft4<2>, dim3(grid), dim3(kF4Threads), 0, st, true, A, jobs, units, nu, scr);
  return sfd_launch(k_fft4<3>, dim3(grid), dim3(kF4Threads), 0, st, true, A, jobs, units, nu, scr);
}
