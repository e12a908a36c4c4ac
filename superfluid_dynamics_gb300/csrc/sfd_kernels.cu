// sfd_kernels.cu -- node-level kernels and the O(N^2) boundary sums.
//
// The reference materialises three dense N x N matrices per RHS evaluation
// (M in createM.cuh:43-92; V1 twice in WaterVelocities.cuh:38-107) and reads V1
// back through two ZGEMVs.  Every one of those N^2 entries is an evaluation of
// cot((z_k - z_j)/2) (and, for finite depth, of cot((z_k - conj z_j)/2 + i h)).
// With w = exp(i z):
//     cot((z_k - z_j)/2)           = i (w_k + w_j) / (w_k - w_j)
//     cot((z_k - conj z_j)/2 + ih) = -i (1 + q_kj) / (1 - q_kj),
//                                    q_kj = p_k conj(p_j),  p = w e^{-h}
// and, because the vortex strength a is real, every product the reference forms
// (M a, V1 a, and the lower / upper velocity variants) is an affine function of
//     S_k = sum_{j != k} a_j / (w_k - w_j)        T_k = sum_j a_j / (1 - q_kj)
// (C_k = sum_{j!=k} a_j cot(.) = i (2 w_k S_k - (A - a_k)), D_k = -i (2 T_k - A),
//  A = sum_j a_j).  So the engine never stores V1: one streaming pass over the
// sources gives S (and T) for all targets, and O(N) epilogues give M a, the
// refinement residual and both velocities.  The transcendental count falls
// from N^2 complex tangents to N complex exponentials per pass.
//
// Three precisions of the same pass: FP64 (the plain FP64 mode), double-float
// pairs on the FP32 pipes (~48 bits, the accurate pass of the mixed mode) and
// FP32 (for small refinement corrections only).
#include "sfd_engine.cuh"
#include "sfd_kernels.cuh"

#include <type_traits>

// ----------------------------------------------------------------- node prep
// w = exp(i z) = e^{-y} (cos x + i sin x); p = w e^{-h} (helium);
// per-node diagonal data of M and of the velocity matrices.
__global__ void k_node_prep(const SurfaceDesc* surf, const int* node_surf, int ntot, const double* x,
                            const double* y, const cd* zp, const cd* zpp, NodeData nd) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ntot) return;
  const SurfaceDesc& S = surf[node_surf[g]];
  double s, c;
  sincos(x[g], &s, &c);
  double e = exp(-y[g]);
  cd w = {e * c, e * s};
  nd.w[g] = w;
  {
    df wr = df_from_double(w.re), wi = df_from_double(w.im);
    nd.wdf[g] = make_float4(wr.hi, wr.lo, wi.hi, wi.lo);
  }
  if (S.physics == 1 && !S.infinite_depth) {
    double eh = exp(-S.depth);
    cd p = {w.re * eh, w.im * eh};
    nd.p[g] = p;
    df pr = df_from_double(p.re), pi = df_from_double(p.im);
    nd.pdf[g] = make_float4(pr.hi, pr.lo, pi.hi, pi.lo);
  }
  cd z1 = zp[g], z2 = zpp[g];
  cd r = cdiv(z2, z1);
  const double inv4pi = 0.25 / SFD_PI;
  double mdiag;
  if (S.physics == 0) mdiag = 0.5 * (1 + S.rho) + 0.25 * (1 - S.rho) / SFD_PI * r.im;  // createM.cuh:56
  else mdiag = 0.5 + 0.25 / SFD_PI * r.im;                                               // createM.cuh:78
  nd.mdiag[g] = mdiag;
  // V1_kk (without the image term) = -(i/4pi) z''/z'^2 +- 1/(2 z')   (WaterVelocities.cuh:54-62,87-97)
  cd zz = z1 * z1;
  cd t = cmul_i(-inv4pi * cdiv(z2, zz));
  cd half_inv = cdiv(cd{1.0, 0.0}, 2.0 * z1);
  nd.v1low[g] = t + half_inv;
  nd.v1up[g] = t - half_inv;
  nd.v2[g] = cmul_i(cdiv(cd{1.0, 0.0}, 2.0 * SFD_PI * z1));  // i / (2 pi z')   (:63,98)
}

// ----------------------------------------------------------------- sums
// Work item = (surface, first target, first source, chunk index).  Each CTA
// stages one chunk of sources in shared memory and accumulates S (and T) for
// kSumTargets targets (two per thread), writing partials per chunk.  The last
// CTA to finish a target tile (arrival counter per tile) reduces that tile's
// chunks in a fixed order (bitwise reproducible) and applies the epilogue, so
// one launch does the whole pass.

namespace {

struct SrcDF {
  float wr_hi, wr_lo, wi_hi, wi_lo;  // w_j
  float pr_hi, pr_lo, pi_hi, pi_lo;  // conj(p_j) is formed on the fly
  float a_hi, a_lo;
};

// (sr, si) += a / (nr + i ni) = a (nr - i ni) / (nr^2 + ni^2), all double-float.
__device__ __forceinline__ void df_div_acc(df nr, df ni, df a, df& sr, df& si) {
  df t = df_mul(a, df_rcp(df_sqsum(nr, ni)));
  sr = df_add(sr, df_mul(t, nr));
  si = df_sub(si, df_mul(t, ni));
}

}  // namespace

struct Src64 {
  double wr, wi, pr, pi, a;
};

// Accumulators of one target.
template <int PREC>
struct Acc;
template <>
struct Acc<SFD_PREC_F64> {
  double sr = 0, si = 0, tr = 0, ti = 0;
};
template <>
struct Acc<SFD_PREC_DF> {
  df sr{0.f, 0.f}, si{0.f, 0.f}, tr{0.f, 0.f}, ti{0.f, 0.f};
};
template <>
struct Acc<SFD_PREC_F32> {
  float sr = 0.f, si = 0.f, tr = 0.f, ti = 0.f;
};

// Target data of one target.
template <int PREC>
struct Tgt;
template <>
struct Tgt<SFD_PREC_F64> {
  cd w, p;
  __device__ void load(cd w_, cd p_) { w = w_; p = p_; }
};
template <>
struct Tgt<SFD_PREC_DF> {
  df wr, wi, pr, pi;
  __device__ void load(float4 w_, float4 p_) {
    wr = {w_.x, w_.y}; wi = {w_.z, w_.w};
    pr = {p_.x, p_.y}; pi = {p_.z, p_.w};
  }
};
template <>
struct Tgt<SFD_PREC_F32> {
  float wr_hi, wr_lo, wi_hi, wi_lo, pr, pi;
  __device__ void load(float4 w_, float4 p_) {
    wr_hi = w_.x; wr_lo = w_.y; wi_hi = w_.z; wi_lo = w_.w;
    pr = p_.x; pi = p_.z;
  }
};

// One (target, source) pair.
__device__ __forceinline__ void pair_acc(const Tgt<SFD_PREC_F64>& t, const Src64& s, bool self, bool image,
                                         Acc<SFD_PREC_F64>& A) {
  if (!self) {
    double dr = t.w.re - s.wr, di = t.w.im - s.wi;
    double inv = s.a / (dr * dr + di * di);
    A.sr += inv * dr;
    A.si -= inv * di;
  }
  if (image) {  // 1 - pk conj(pj)
    double qr = t.p.re * s.pr + t.p.im * s.pi, qi = t.p.im * s.pr - t.p.re * s.pi;
    double dr = 1.0 - qr, di = -qi;
    double inv = s.a / (dr * dr + di * di);
    A.tr += inv * dr;
    A.ti -= inv * di;
  }
}
__device__ __forceinline__ void pair_acc(const Tgt<SFD_PREC_DF>& t, const SrcDF& s, bool self, bool image,
                                         Acc<SFD_PREC_DF>& A) {
  df aj{s.a_hi, s.a_lo};
  if (!self) {
    df dr = df_diff(t.wr, df{s.wr_hi, s.wr_lo});
    df di = df_diff(t.wi, df{s.wi_hi, s.wi_lo});
    df_div_acc(dr, di, aj, A.sr, A.si);
  }
  if (image) {
    df prj{s.pr_hi, s.pr_lo}, pij{s.pi_hi, s.pi_lo};
    df qr = df_add(df_mul(t.pr, prj), df_mul(t.pi, pij));
    df qi = df_sub(df_mul(t.pi, prj), df_mul(t.pr, pij));
    df_div_acc(df_sub(df{1.f, 0.f}, qr), df_neg(qi), aj, A.tr, A.ti);
  }
}
__device__ __forceinline__ void pair_acc(const Tgt<SFD_PREC_F32>& t, const SrcDF& s, bool self, bool image,
                                         Acc<SFD_PREC_F32>& A) {
  if (!self) {
    float dr = (t.wr_hi - s.wr_hi) + (t.wr_lo - s.wr_lo);
    float di = (t.wi_hi - s.wi_hi) + (t.wi_lo - s.wi_lo);
    float inv = s.a_hi * rcp_approx(fmaf(dr, dr, di * di));
    A.sr = fmaf(inv, dr, A.sr);
    A.si = fmaf(-inv, di, A.si);
  }
  if (image) {
    float qr = t.pr * s.pr_hi + t.pi * s.pi_hi, qi = t.pi * s.pr_hi - t.pr * s.pi_hi;
    float dr = 1.f - qr, di = -qi;
    float inv = s.a_hi * rcp_approx(fmaf(dr, dr, di * di));
    A.tr = fmaf(inv, dr, A.tr);
    A.ti = fmaf(-inv, di, A.ti);
  }
}
__device__ __forceinline__ cd acc_s(const Acc<SFD_PREC_F64>& A) { return {A.sr, A.si}; }
__device__ __forceinline__ cd acc_t(const Acc<SFD_PREC_F64>& A) { return {A.tr, A.ti}; }
__device__ __forceinline__ float4 acc_s(const Acc<SFD_PREC_DF>& A) { return make_float4(A.sr.hi, A.sr.lo, A.si.hi, A.si.lo); }
__device__ __forceinline__ float4 acc_t(const Acc<SFD_PREC_DF>& A) { return make_float4(A.tr.hi, A.tr.lo, A.ti.hi, A.ti.lo); }
__device__ __forceinline__ float4 acc_s(const Acc<SFD_PREC_F32>& A) { return make_float4(A.sr, 0.f, A.si, 0.f); }
__device__ __forceinline__ float4 acc_t(const Acc<SFD_PREC_F32>& A) { return make_float4(A.tr, 0.f, A.ti, 0.f); }

__device__ __forceinline__ df df_warp_sum(df v) {
  for (int o = 16; o > 0; o >>= 1) {
    df u = {__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
    v = df_add(v, u);
  }
  return v;
}

template <int PREC>
using SrcT = typename std::conditional<PREC == SFD_PREC_F64, Src64, SrcDF>::type;

// Epilogue of one target tile (run by the last CTA to finish it): reduce the
// chunk partials in fixed order (bitwise reproducible) and form, per node,
//   C_k = i (2 w_k S_k - (A - a_k)),   D_k = -i (2 T_k - A)
//   (M a)_k = Mdiag_k a_k + c1 Im(z'_k C_k) - [image] (1/4pi) Im D_k
// mode 0: C/D overwritten, r = phi' - M a; mode 1: C/D accumulated, r -= M a.
template <int PREC>
__device__ void sums_epilogue(const SumArgs& A, const SurfaceDesc& S, int sidx, int tile, int t0, bool image) {
  const int n = S.n, off = S.off;
  const int nchunk = (n + kSumChunk - 1) / kSumChunk;
  __shared__ double asum_sh;
  if (threadIdx.x == 0) {
    const long long ia = (long long)tile * A.max_chunks;
    if constexpr (PREC == SFD_PREC_F64) {
      double s = 0.0;
      for (int c = 0; c < nchunk; ++c) s += __ldcg(A.part_a + ia + c);
      asum_sh = s;
    } else {
      df s = {0.f, 0.f};
      const float2* pa = reinterpret_cast<const float2*>(A.part_a) + ia;
      for (int c = 0; c < nchunk; ++c) {
        float2 v = __ldcg(pa + c);
        s = df_add(s, df{v.x, v.y});
      }
      asum_sh = df_to_double(s);
    }
  }
  __syncthreads();
  const double asum = asum_sh;
  const double c1 = S.physics == 0 ? 0.25 * (1 - S.rho) / SFD_PI : 0.25 / SFD_PI;
  double rmax = 0.0;
  for (int q = 0; q < kSumTargets / kSumThreads; ++q) {
    const int tk = t0 + q * kSumThreads + threadIdx.x;
    if (tk >= n) continue;
    const int g = off + tk;
    cd sum_s, sum_t = {0, 0};
    if constexpr (PREC == SFD_PREC_F64) {
      double sr = 0, si = 0, tr = 0, ti = 0;
      for (int c = 0; c < nchunk; ++c) {
        const long long o = (long long)c * A.ntot + g;
        double2 v = __ldcg(reinterpret_cast<const double2*>(A.part_s) + o);
        sr += v.x;
        si += v.y;
        if (image) {
          double2 u = __ldcg(reinterpret_cast<const double2*>(A.part_t) + o);
          tr += u.x;
          ti += u.y;
        }
      }
      sum_s = {sr, si};
      sum_t = {tr, ti};
    } else {
      df sr = {0.f, 0.f}, si = {0.f, 0.f}, tr = {0.f, 0.f}, ti = {0.f, 0.f};
      for (int c = 0; c < nchunk; ++c) {
        const long long o = (long long)c * A.ntot + g;
        float4 v = __ldcg(reinterpret_cast<const float4*>(A.part_s) + o);
        sr = df_add(sr, df{v.x, v.y});
        si = df_add(si, df{v.z, v.w});
        if (image) {
          float4 u = __ldcg(reinterpret_cast<const float4*>(A.part_t) + o);
          tr = df_add(tr, df{u.x, u.y});
          ti = df_add(ti, df{u.z, u.w});
        }
      }
      sum_s = {df_to_double(sr), df_to_double(si)};
      sum_t = {df_to_double(tr), df_to_double(ti)};
    }
    const double ak = A.a[g];
    const cd wk = A.w[g];
    const cd C = cmul_i(2.0 * (wk * sum_s) - cd{asum - ak, 0.0});
    const cd D = image ? cmul_i(cd{-(2.0 * sum_t.re - asum), -(2.0 * sum_t.im)}) : cd{0, 0};
    double ma = A.mdiag[g] * ak + c1 * (A.zp[g] * C).im;
    if (image) ma -= 0.25 / SFD_PI * D.im;
    double rnew;
    if (A.mode == 0) {
      A.cacc[g] = C;
      if (image) A.dacc[g] = D;
      rnew = A.phip[g] - ma;
    } else {
      A.cacc[g] = A.cacc[g] + C;
      if (image) A.dacc[g] = A.dacc[g] + D;
      rnew = A.r[g] - ma;
    }
    A.r[g] = rnew;
    double rv = fabs(rnew);
    if (!(rv == rv)) rv = 1e300;
    rmax = fmax(rmax, rv);
  }
  if (A.rnorm) {
    // |r| max per surface: non-negative doubles order like their bit patterns
    unsigned long long m = (unsigned long long)__double_as_longlong(rmax);
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long v = __shfl_xor_sync(0xffffffffu, m, o);
      m = v > m ? v : m;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<unsigned long long*>(A.rnorm) + sidx, m);
  }
}

template <int PREC>
__global__ void __launch_bounds__(kSumThreads) k_boundary_sums(SumArgs A) {
  const int4 item = A.items[blockIdx.x];
  const SurfaceDesc& S = A.surf[item.x];
  const int n = S.n, off = S.off;
  const int t0 = item.y, j0 = item.z, chunk = item.w;
  const int jn = min(kSumChunk, n - j0);
  const bool image = (S.physics == 1 && !S.infinite_depth);
  __shared__ SrcT<PREC> src[kSumChunk];
  __shared__ double asum_warp[kSumThreads / 32];
  __shared__ float2 asum_warp_df[kSumThreads / 32];
  // stage the chunk's sources (and their weight sum, kept by the first target tile)
  double apart = 0.0;
  df apart_df = {0.f, 0.f};
  for (int jj = threadIdx.x; jj < jn; jj += kSumThreads) {
    int g = off + j0 + jj;
    if constexpr (PREC == SFD_PREC_F64) {
      cd w = A.w[g];
      double aj = A.a[g];
      apart += aj;
      cd p = image ? A.p[g] : cd{0.0, 0.0};
      src[jj] = Src64{w.re, w.im, p.re, p.im, aj};
    } else {
      float4 w = A.wdf[g];
      float2 ad = A.adf[g];
      float4 p = image ? A.pdf[g] : make_float4(0.f, 0.f, 0.f, 0.f);
      apart_df = df_add(apart_df, df{ad.x, ad.y});
      src[jj] = SrcDF{w.x, w.y, w.z, w.w, p.x, p.y, p.z, p.w, ad.x, PREC == SFD_PREC_DF ? ad.y : 0.f};
    }
  }
  {
    if constexpr (PREC == SFD_PREC_F64) {
      for (int o = 16; o > 0; o >>= 1) apart += __shfl_xor_sync(0xffffffffu, apart, o);
      if ((threadIdx.x & 31) == 0) asum_warp[threadIdx.x >> 5] = apart;
    } else {
      apart_df = df_warp_sum(apart_df);
      if ((threadIdx.x & 31) == 0) asum_warp_df[threadIdx.x >> 5] = make_float2(apart_df.hi, apart_df.lo);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {  // this chunk's weight sum, kept per (target tile, chunk)
    const long long ia = (long long)(S.tile_base + t0 / kSumTargets) * A.max_chunks + chunk;
    if constexpr (PREC == SFD_PREC_F64) {
      double s = 0.0;
      for (int i = 0; i < kSumThreads / 32; ++i) s += asum_warp[i];
      A.part_a[ia] = s;
    } else {
      df s = {0.f, 0.f};
      for (int i = 0; i < kSumThreads / 32; ++i) s = df_add(s, df{asum_warp_df[i].x, asum_warp_df[i].y});
      reinterpret_cast<float2*>(A.part_a)[ia] = make_float2(s.hi, s.lo);
    }
  }
  // two targets per thread: tk0 and tk0 + kSumThreads
  const int tk0 = t0 + threadIdx.x, tk1 = tk0 + kSumThreads;
  const bool a0 = tk0 < n, a1 = tk1 < n;
  const int g0 = off + (a0 ? tk0 : 0), g1 = off + (a1 ? tk1 : 0);
  Tgt<PREC> T0, T1;
  if constexpr (PREC == SFD_PREC_F64) {
    T0.load(A.w[g0], image ? A.p[g0] : cd{0, 0});
    T1.load(A.w[g1], image ? A.p[g1] : cd{0, 0});
  } else {
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    T0.load(A.wdf[g0], image ? A.pdf[g0] : z4);
    T1.load(A.wdf[g1], image ? A.pdf[g1] : z4);
  }
  const int self0 = a0 ? tk0 - j0 : -1, self1 = a1 ? tk1 - j0 : -1;
  Acc<PREC> R0, R1;
#pragma unroll 2
  for (int jj = 0; jj < jn; ++jj) {
    const SrcT<PREC> s = src[jj];
    pair_acc(T0, s, jj == self0, image, R0);
    pair_acc(T1, s, jj == self1, image, R1);
  }
  long long o = (long long)chunk * A.ntot + off;
  const int tile = S.tile_base + t0 / kSumTargets;
  if constexpr (PREC == SFD_PREC_F64) {
    if (a0) {
      A.part_s[o + tk0] = acc_s(R0);
      if (image) A.part_t[o + tk0] = acc_t(R0);
    }
    if (a1) {
      A.part_s[o + tk1] = acc_s(R1);
      if (image) A.part_t[o + tk1] = acc_t(R1);
    }
  } else {
    float4* ps = reinterpret_cast<float4*>(A.part_s);
    float4* pt = reinterpret_cast<float4*>(A.part_t);
    if (a0) {
      ps[o + tk0] = acc_s(R0);
      if (image) pt[o + tk0] = acc_t(R0);
    }
    if (a1) {
      ps[o + tk1] = acc_s(R1);
      if (image) pt[o + tk1] = acc_t(R1);
    }
  }
  // ---- arrival count: the last CTA of this target tile finishes it
  __shared__ int last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nchunk = (n + kSumChunk - 1) / kSumChunk;
    last = (atomicAdd(A.tile_count + tile, 1) == nchunk - 1);
    if (last) A.tile_count[tile] = 0;  // ready for the next pass
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  sums_epilogue<PREC>(A, S, item.x, tile, t0, image);
}

cudaError_t sfd_launch_sums(int prec, const SumArgs& A, int nitems, cudaStream_t st) {
  if (nitems == 0) return cudaSuccess;
  if (prec == SFD_PREC_F64) k_boundary_sums<SFD_PREC_F64><<<nitems, kSumThreads, 0, st>>>(A);
  else if (prec == SFD_PREC_DF) k_boundary_sums<SFD_PREC_DF><<<nitems, kSumThreads, 0, st>>>(A);
  else k_boundary_sums<SFD_PREC_F32><<<nitems, kSumThreads, 0, st>>>(A);
  return cudaGetLastError();
}

// Velocities and Bernoulli:
//   vel_k = conj(-(i/4pi) C_k + [image] (i/4pi) D_k + V1_kk a_k + V2_k a'_k)   (lower)
//   water:  dphi = -(1+rho) g y + |v|^2/2 + rho |v_up|^2/2 - rho (u_low[1] u_up + v_low v_up)
//   helium: dphi = vdw (1 + y/h)^-3 - vdw + |v|^2/2
// Output goes to the RHS slot (dx, dy, dphi).  Status bit on non-finite values.
__global__ void k_velocity_bernoulli(VelArgs V) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= V.ntot) return;
  const int s = V.node_surf[g];
  const SurfaceDesc& S = V.surf[s];
  const bool image = (S.physics == 1 && !S.infinite_depth);
  const double inv4pi = 1.0 / (4.0 * SFD_PI);
  cd C = V.cacc[g];
  cd base = cmul_i(-inv4pi * C);
  if (image) base = base + cmul_i(inv4pi * V.dacc[g]);
  double ak = V.a[g];
  cd apk = V.ap[g];
  cd v2a = V.v2[g] * apk;
  cd low = cconj(v2a + base + ak * V.v1low[g]);
  V.dx[g] = low.re;
  V.dy[g] = low.im;
  double yk = V.y[g];
  double out;
  if (S.physics == 0) {
    double v1 = low.re * low.re + low.im * low.im;
    out = -(1 + S.rho) * (S.gravity * yk) + 0.5 * v1;
    if (S.rho != 0.0) {
      cd up = cconj(v2a + base + ak * V.v1up[g]);
      double v2 = up.re * up.re + up.im * up.im;
      // createM.cuh:104 reads the lower velocity at (concatenated) node 1
      cd low1 = V.vel_low1[0];
      double v12 = low1.re * up.re + low.im * up.im;
      out += 0.5 * S.rho * v2 - S.rho * v12;
    }
  } else if (S.bern_variant == 1) {
    // series expansion of the van der Waals term (createM.cuh:171-193)
    double kin = 0.5 * low.re * low.re + 0.5 * low.im * low.im;
    double vdw = 0.0;
    const int o = S.expansion_order;  // switch fall-through of the reference: 3 -> 2 -> 1
    if (o == 3) vdw += -10.0 / 3.0 * pow(yk, 3.0) / (S.depth * S.depth);
    if (o == 3 || o == 2) vdw += 2.0 * pow(yk, 2.0) / S.depth;
    if (o >= 1 && o <= 3) vdw += -yk;
    out = vdw + kin;
  } else if (S.bern_variant == 2) {
    // surface-tension variant with the reference's fixed prefactor (createM.cuh:195-211)
    cd z1 = V.zp[g], z2 = V.zpp[g];
    double curv = (z1.re * z2.im - z1.im * z2.re) / pow(z1.re * z1.re + z1.im * z1.im, 1.5);
    double v1 = low.re * low.re + low.im * low.im;
    out = 20.447761896665416 * S.depth / 3.0 * (1.0 / pow(1.0 + yk / S.depth, 3) - 1) + 0.5 * v1 + S.kappa * curv;
  } else {
    double q = 1.0 + yk / S.depth;
    out = S.vdw * pow(q, -3.0) - S.vdw + 0.5 * low.re * low.re + 0.5 * low.im * low.im;
  }
  V.dphi[g] = out;
  if (!isfinite(out) || !isfinite(low.re) || !isfinite(low.im)) atomicOr(V.status + s, SFD_ST_NONFINITE);
}

// The water cross term reads the lower velocity of concatenated node 1
// (createM.cuh:104).  For rho != 0 that value is computed first (one thread).
__global__ void k_velocity_node1(VelArgs V) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  int g = V.ntot > 1 ? 1 : 0;
  const SurfaceDesc& S = V.surf[V.node_surf[g]];
  const bool image = (S.physics == 1 && !S.infinite_depth);
  const double inv4pi = 1.0 / (4.0 * SFD_PI);
  cd base = cmul_i(-inv4pi * V.cacc[g]);
  if (image) base = base + cmul_i(inv4pi * V.dacc[g]);
  V.vel_low1[0] = cconj(V.v2[g] * V.ap[g] + base + V.a[g] * V.v1low[g]);
}

// ----------------------------------------------------------------- RK4 pieces
// stage combine (AutonomousRungeKuttaStepper.cuh:338-375, utilities.cuh:78-83):
//   kacc = (first ? k : kacc + wk * k);  ystage = y0 + cy * k  (if cy != 0)
__global__ void k_rk4_stage(int n3, const double* __restrict__ y0, const double* __restrict__ k,
                            double* __restrict__ kacc, double* __restrict__ ystage, double wk, double cy, int first) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n3) return;
  double kv = k[i];
  kacc[i] = first ? kv : kacc[i] + wk * kv;
  if (ystage) ystage[i] = y0[i] + cy * kv;
}
__global__ void k_rk4_final(int n3, double* __restrict__ y0, const double* __restrict__ kacc, double c) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n3) return;
  y0[i] = y0[i] + c * kacc[i];
}

// ----------------------------------------------------------------- invariants
// Per surface (one CTA each), FP64, fixed-order warp-shuffle tree:
// [kinetic, potential, surface, flux, mass] with the Energies.cuh scalings.
__global__ void k_invariants(const SurfaceDesc* surf, const double* x, const double* y, const double* phi,
                             const cd* zp, const double* u, const double* v, double kappa, double* out) {
  const SurfaceDesc S = surf[blockIdx.x];
  double acc[5] = {0, 0, 0, 0, 0};
  for (int k = threadIdx.x; k < S.n; k += blockDim.x) {
    int g = S.off + k;
    double xp = zp[g].re, yp = zp[g].im;
    acc[0] += phi[g] * (-1.0 * yp * u[g] + xp * v[g]);
    if (S.physics == 0) acc[1] += y[g] * y[g] * xp;
    else acc[1] += (1.0 / pow(1.0 + y[g] / S.depth, 2) - 1.0);
    acc[2] += sqrt(xp * xp + yp * yp);
    acc[3] += v[g] * xp + u[g] * yp;
    acc[4] += y[g] * xp;
  }
  __shared__ double red[5][32];
  for (int q = 0; q < 5; ++q) {
    double t = acc[q];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double r[5];
    for (int q = 0; q < 5; ++q) {
      r[q] = 0;
      for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r[q] += red[q][i];
    }
    double* o = out + 5 * blockIdx.x;
    o[0] = r[0] * 0.25 / SFD_PI;
    o[1] = S.physics == 0 ? r[1] * 0.25 * (1.0 + S.rho) * S.gravity / SFD_PI : r[1] * S.depth * S.depth / 6.0;
    o[2] = (r[2] - 2.0 * SFD_PI) * kappa / (2.0 * SFD_PI);
    o[3] = r[3] * 0.5 / SFD_PI;
    o[4] = r[4];
  }
}
