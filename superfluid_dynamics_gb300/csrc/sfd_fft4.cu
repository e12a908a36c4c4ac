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
// Each FFT of length L = 8 P is one unit of 8 threads: thread t holds
// x[t + 8 j] (j < P), does a P-point DFT in registers, multiplies by
// W_L^{t ka}, exchanges through shared memory and finishes with 8-point DFTs
// (thread t then holds X[t + 8 q + P kb]).  The row phase needs no exchange
// between the forward and the inverse transform: the forward leaves thread t
// holding exactly the inputs its inverse needs.  Units of one job are
// contiguous and a multiple of 4, so a warp's four units share their length.
// Intermediate rows and columns go through an L2-resident scratch (16 bytes
// per node and output).
#include "sfd_engine.cuh"
#include "sfd_kernels.cuh"

namespace {

constexpr double kH = 0.70710678118654752440;          // cos(pi/4)
constexpr double kC8 = 0.92387953251128675613;         // cos(pi/8)
constexpr double kS8 = 0.38268343236508977173;         // sin(pi/8)

__device__ __forceinline__ cd rot(cd a, int sign) { return sign < 0 ? cd{a.im, -a.re} : cd{-a.im, a.re}; }

// Natural-order DFTs in registers (sign -1: exp(-2 pi i jk / P), +1: inverse
// without 1/P).
__device__ __forceinline__ void dft2(cd* v) {
  const cd a = v[0], b = v[1];
  v[0] = a + b;
  v[1] = a - b;
}
__device__ __forceinline__ void dft4(cd* v, int sign) {
  const cd a0 = v[0] + v[2], a1 = v[0] - v[2];
  const cd b0 = v[1] + v[3], b1 = rot(v[1] - v[3], sign);
  v[0] = a0 + b0;
  v[1] = a1 + b1;
  v[2] = a0 - b0;
  v[3] = a1 - b1;
}
// W_8^k (k < 4) times a, for the given sign
__device__ __forceinline__ cd w8mul(cd a, int k, int sign) {
  const double s = sign < 0 ? -1.0 : 1.0;
  switch (k) {
    case 0: return a;
    case 1: return cd{kH * (a.re - s * a.im), kH * (a.im + s * a.re)};
    case 2: return rot(a, sign);
    default: return cd{kH * (-a.re - s * a.im), kH * (-a.im + s * a.re)};
  }
}
__device__ __forceinline__ void dft8(cd* v, int sign) {
  cd e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
  dft4(e, sign);
  dft4(o, sign);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const cd t = w8mul(o[k], k, sign);
    v[k] = e[k] + t;
    v[k + 4] = e[k] - t;
  }
}
// W_16^k (k < 8) times a
__device__ __forceinline__ cd w16mul(cd a, int k, int sign) {
  if ((k & 1) == 0) return w8mul(a, k >> 1, sign);
  const double s = sign < 0 ? -1.0 : 1.0;
  double c, sn;  // cos and sin of 2 pi k / 16 for odd k
  switch (k) {
    case 1: c = kC8; sn = kS8; break;
    case 3: c = kS8; sn = kC8; break;
    case 5: c = -kS8; sn = kC8; break;
    default: c = -kC8; sn = kS8; break;
  }
  sn *= s;  // exp(s i 2 pi k / 16)
  return cd{a.re * c - a.im * sn, a.re * sn + a.im * c};
}
__device__ __forceinline__ void dft16(cd* v, int sign) {
  cd e[8], o[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    e[j] = v[2 * j];
    o[j] = v[2 * j + 1];
  }
  dft8(e, sign);
  dft8(o, sign);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const cd t = w16mul(o[k], k, sign);
    v[k] = e[k] + t;
    v[k + 8] = e[k] - t;
  }
}
template <int P>
__device__ __forceinline__ void dftP(cd* v, int sign) {
  if constexpr (P == 2) dft2(v);
  else if constexpr (P == 4) dft4(v, sign);
  else if constexpr (P == 8) dft8(v, sign);
  else if constexpr (P == 16) dft16(v, sign);
}

__device__ __forceinline__ cd twid(const cd* tw, long long e, int sign) {
  const cd t = tw[e];
  return sign < 0 ? t : cd{t.re, -t.im};
}

// Length L = 8 P FFT of one unit (8 threads, t = lane % 8).  In: v[j] =
// x[t + 8 j], j < P.  Out: v[q * 8 + kb] = X[ka + P kb] for ka = t + 8 q
// (q < max(1, P / 8); for P < 8 only threads t < P hold outputs).  tw: W_n^e
// with n = L * tws; sm: 8 P complex values of shared memory for this unit.
template <int P>
__device__ __forceinline__ void unit_fft(cd* v, cd* sm, int t, const cd* tw, int tws, int sign) {
  dftP<P>(v, sign);
#pragma unroll
  for (int ka = 1; ka < P; ++ka)
    if (t) v[ka] = v[ka] * twid(tw, (long long)t * ka * tws, sign);
#pragma unroll
  for (int ka = 0; ka < P; ++ka) sm[t * P + ka] = v[ka];
  __syncwarp();
  constexpr int Q = P >= 8 ? P / 8 : 1;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int ka = t + 8 * q;
    cd b[8];
#pragma unroll
    for (int tt = 0; tt < 8; ++tt) b[tt] = (ka < P) ? sm[tt * P + ka] : cd{0.0, 0.0};
    dft8(b, sign);
#pragma unroll
    for (int kb = 0; kb < 8; ++kb) v[q * 8 + kb] = b[kb];
  }
  __syncwarp();  // the unit's shared memory is reused by the caller
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

constexpr int kUnitsPerCta = 4;  // one warp
constexpr int kF4Threads = 8 * kUnitsPerCta;

}  // namespace

// Phase 1: column FFTs.  Unit u of a job: n1 = u (64 units).
template <int P>
__device__ __forceinline__ void f4_phase1(const DerivArgs& A, const F4Job& J, const SurfaceDesc& S, int u, int t,
                                          cd* sm, cd* scr) {
  const int n = S.n, off = S.off;
  const int n1 = u;
  const double dn = (double)n, inv_n = 1.0 / dn;
  const double rho = S.physics == 0 ? S.rho : 0.0;
  const double uq = -(1 + rho) * SFD_PI * S.U / n;
  cd v[P >= 8 ? P : 8];
#pragma unroll
  for (int j = 0; j < P; ++j) {
    const int m = n1 + 64 * (t + 8 * j);  // node index
    if (J.kind == SFD_F4_Z) v[j] = {A.x[off + m] - xi_node(m, dn, inv_n), A.y[off + m]};        // Derivatives.cuh:285,317
    else if (J.kind == SFD_F4_PHI) v[j] = {A.phi[off + m] - uq * (double)m, A.phi_im ? A.phi_im[off + m] : 0.0};  // :286,318
    else v[j] = {A.a[off + m], 0.0};                                                            // real_to_complex(a)
  }
  unit_fft<P>(v, sm, t, S.tw, n / (8 * P), -1);
  constexpr int Q = P >= 8 ? P / 8 : 1;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int ka = t + 8 * q;
    if (ka < P) {
#pragma unroll
      for (int kb = 0; kb < 8; ++kb) {
        const int k2 = ka + P * kb;
        scr[J.scr0 + (long long)k2 * 64 + n1] = v[q * 8 + kb] * twid(S.tw, ((long long)n1 * k2) % n, -1);
      }
    }
  }
}

// Phase 2: row k2 = u: forward 64-point FFT, multiplier, inverse FFT(s).
__device__ __forceinline__ void f4_phase2(const F4Job& J, const SurfaceDesc& S, int u, int t, cd* sm, cd* scr) {
  const int n = S.n, N2 = n / 64, k2 = u;
  const double inv_n = 1.0 / (double)n;
  cd* row = scr + J.scr0 + (long long)k2 * 64;
  cd v[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) v[j] = row[t + 8 * j];
  unit_fft<8>(v, sm, t, S.tw, n / 64, -1);  // v[kb] = X[k2 + N2 (t + 8 kb)]
  const bool second_too = J.kind == SFD_F4_Z;
  cd w[8];
#pragma unroll
  for (int kb = 0; kb < 8; ++kb) {
    const int k = k2 + N2 * (t + 8 * kb);
    w[kb] = second_too ? second_mult(v[kb], k, n, inv_n) : v[kb];
    v[kb] = first_mult(v[kb], k, n, inv_n);
  }
  // thread t holds the inverse transform's inputs m = t + 8 kb
  unit_fft<8>(v, sm, t, S.tw, n / 64, +1);  // v[kb] = Y'[n1 = t + 8 kb]
#pragma unroll
  for (int kb = 0; kb < 8; ++kb) {
    const int n1 = t + 8 * kb;
    row[n1] = v[kb] * twid(S.tw, ((long long)n1 * k2) % n, +1);
  }
  if (second_too) {
    unit_fft<8>(w, sm, t, S.tw, n / 64, +1);
    cd* row2 = scr + J.scr1 + (long long)k2 * 64;
#pragma unroll
    for (int kb = 0; kb < 8; ++kb) {
      const int n1 = t + 8 * kb;
      row2[n1] = w[kb] * twid(S.tw, ((long long)n1 * k2) % n, +1);
    }
  }
}

// Phase 3: inverse column FFTs.  Unit u: output o = u / 64 (z' then z''
// for the z job), column n1 = u % 64.
template <int P>
__device__ __forceinline__ void f4_phase3(const DerivArgs& A, const F4Job& J, const SurfaceDesc& S, int u, int t,
                                          cd* sm, const cd* scr) {
  const int n = S.n, off = S.off;
  const int o = u >> 6, n1 = u & 63;
  const cd* col = scr + (o ? J.scr1 : J.scr0) + n1;
  cd v[P >= 8 ? P : 8];
#pragma unroll
  for (int j = 0; j < P; ++j) v[j] = col[(long long)(t + 8 * j) * 64];
  unit_fft<P>(v, sm, t, S.tw, n / (8 * P), +1);
  const double s1 = 2.0 * SFD_PI / n;
  const double s2 = 4.0 * SFD_PI * SFD_PI / ((double)n * n);
  const double rho = S.physics == 0 ? S.rho : 0.0;
  const double uq = -(1 + rho) * SFD_PI * S.U / n;
  constexpr int Q = P >= 8 ? P / 8 : 1;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int ka = t + 8 * q;
    if (ka < P) {
#pragma unroll
      for (int kb = 0; kb < 8; ++kb) {
        const int j = off + n1 + 64 * (ka + P * kb);
        const cd x = v[q * 8 + kb];
        if (J.kind == SFD_F4_Z) {
          if (o == 0) A.zp[j] = {x.re * s1 + s1, x.im * s1};  // Derivatives.cuh:323,374
          else A.zpp[j] = {x.re * s2, x.im * s2};           // :321
        } else if (J.kind == SFD_F4_PHI) {
          double r = x.re * s1;                             // :324, complex_to_real
          if (S.U != 0) r += uq;                            // :380-383
          A.phip[j] = r;
          if (A.phipf) A.phipf[j] = (float)r;
        } else {
          A.ap[j] = {x.re * s1, x.im * s1};                 // BaseBoundaryIntegrator.cuh:203
        }
      }
    }
  }
}

template <int PHASE>
__global__ void __launch_bounds__(kF4Threads) k_fft4(DerivArgs A, const F4Job* jobs, const int2* units, int nunits,
                                                     cd* scr) {
  __shared__ cd sm_all[kUnitsPerCta][8 * 16];
  const int lane = threadIdx.x & 31, unit_in_cta = lane >> 3, t = lane & 7;
  const int ui = blockIdx.x * kUnitsPerCta + unit_in_cta;
  if (ui >= nunits) return;  // unit counts are multiples of 4: whole warps leave together
  const int2 uw = units[ui];
  const F4Job J = jobs[uw.x];
  if (!gate_open(A.gate, J.surf)) return;  // a job's units share the surface: whole warps leave together
  const SurfaceDesc& S = A.surf[J.surf];
  cd* sm = sm_all[unit_in_cta];
  if (PHASE == 2) {
    f4_phase2(J, S, uw.y, t, sm, scr);
    return;
  }
  const int P = (S.n / 64) / 8;
  switch (P) {
    case 1: PHASE == 1 ? f4_phase1<1>(A, J, S, uw.y, t, sm, scr) : f4_phase3<1>(A, J, S, uw.y, t, sm, scr); break;
    case 2: PHASE == 1 ? f4_phase1<2>(A, J, S, uw.y, t, sm, scr) : f4_phase3<2>(A, J, S, uw.y, t, sm, scr); break;
    case 4: PHASE == 1 ? f4_phase1<4>(A, J, S, uw.y, t, sm, scr) : f4_phase3<4>(A, J, S, uw.y, t, sm, scr); break;
    case 8: PHASE == 1 ? f4_phase1<8>(A, J, S, uw.y, t, sm, scr) : f4_phase3<8>(A, J, S, uw.y, t, sm, scr); break;
    default: PHASE == 1 ? f4_phase1<16>(A, J, S, uw.y, t, sm, scr) : f4_phase3<16>(A, J, S, uw.y, t, sm, scr); break;
  }
}

bool sfd_f4_eligible(int n) { return n >= 512 && n <= 8192 && (n & (n - 1)) == 0; }

cudaError_t sfd_launch_f4(const DerivArgs& A, const F4Plan& p, cd* scr, cudaStream_t st, int phase) {
  const int nu = p.nunits[phase - 1];
  if (nu == 0) return cudaSuccess;
  const int grid = (nu + kUnitsPerCta - 1) / kUnitsPerCta;
  if (phase == 1) k_fft4<1><<<grid, kF4Threads, 0, st>>>(A, p.jobs, p.units[0], nu, scr);
  else if (phase == 2) k_fft4<2><<<grid, kF4Threads, 0, st>>>(A, p.jobs, p.units[1], nu, scr);
  else k_fft4<3><<<grid, kF4Threads, 0, st>>>(A, p.jobs, p.units[2], nu, scr);
  return cudaPeekAtLastError();  // the caller's launch check reads and clears it
}
