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

#include <algorithm>
#include <cooperative_groups.h>
#include <type_traits>

// ----------------------------------------------------------------- node prep
// w = exp(i z) = e^{-y} (cos x + i sin x); p = w e^{-h} (helium);
// per-node diagonal data of M and of the velocity matrices.
// Two independent FP64 chains per node, one per warp of a 64-thread block of
// 32 nodes (GB300's FP64 pipe is narrow, so the chains' latency is the cost):
// warp 0 the exponentials (w, p), warp 1 the z' / z'' terms, which share one
// reciprocal 1 / z'.
// The thread of a surface's first node also clears the surface's residual
// slots and max |phi'| (rslot, bnorm nullable): every boundary-sum pass of the
// evaluation runs after this kernel.
__global__ void __launch_bounds__(64) k_node_prep(const SurfaceDesc* surf, const int* node_surf, int ntot,
                                                  const double* x, const double* y, const cd* zp, const cd* zpp,
                                                  NodeData nd, double* rslot, double* bnorm) {
  sfd_pdl_begin();
  const int g = blockIdx.x * 32 + (threadIdx.x & 31);
  if (g >= ntot) return;
  const int sidx = node_surf[g];
  const SurfaceDesc& S = surf[sidx];
  if (threadIdx.x >= 32 && g == S.off && rslot) {
#pragma unroll
    for (int i = 0; i < SFD_RSLOTS; ++i) rslot[(long long)sidx * SFD_RSLOTS + i] = 0.0;
    bnorm[sidx] = 0.0;
  }
  if (threadIdx.x < 32) {
    double s, c;
    sincos(x[g], &s, &c);
    const double e = exp(-y[g]);
    const cd w = {e * c, e * s};
    nd.w[g] = w;
    const df wr = df_from_double(w.re), wi = df_from_double(w.im);
    nd.wdf[g] = make_float4(wr.hi, wr.lo, wi.hi, wi.lo);
    if (S.physics == 1 && !S.infinite_depth) {
      const double eh = exp(-S.depth);
      const cd p = {w.re * eh, w.im * eh};
      nd.p[g] = p;
      const df pr = df_from_double(p.re), pi = df_from_double(p.im);
      nd.pdf[g] = make_float4(pr.hi, pr.lo, pi.hi, pi.lo);
    }
    return;
  }
  const cd z1 = zp[g], z2 = zpp[g];
  const cd iz = cdiv(cd{1.0, 0.0}, z1);  // 1 / z'
  const cd r = z2 * iz;                  // z'' / z'
  constexpr double inv4pi = 0.25 / SFD_PI;
  double mdiag;
  if (S.physics == 0) mdiag = 0.5 * (1 + S.rho) + inv4pi * (1 - S.rho) * r.im;  // createM.cuh:56
  else mdiag = 0.5 + inv4pi * r.im;                                             // createM.cuh:78
  nd.mdiag[g] = mdiag;
  // V1_kk (without the image term) = -(i/4pi) z''/z'^2 +- 1/(2 z')   (WaterVelocities.cuh:54-62,87-97)
  const cd t = cmul_i(-inv4pi * (r * iz));
  const cd half_inv = 0.5 * iz;
  nd.v1low[g] = t + half_inv;
  nd.v1up[g] = t - half_inv;
  nd.v2[g] = cmul_i((0.5 / SFD_PI) * iz);  // i / (2 pi z')   (:63,98)
}

// ----------------------------------------------------------------- sums
// One cluster of kSumCL CTAs per (surface, tile of kSumTile targets).  CTA r of
// the cluster stages sources [r per, (r+1) per) (per = ceil(n / kSumCL)) in
// shared memory; its kSumGroups groups of kSumTile threads (one target each)
// take every kSumGroups-th of those sources.  Group partials are summed in
// shared memory, the cluster's CTA partials over distributed shared memory, in
// a fixed order (bitwise reproducible), and CTA r finishes targets
// [r kSumPerRank, (r+1) kSumPerRank) of the tile with the epilogue (C, D, M a,
// residual).  One launch per pass; no partials leave the chip.  This is the
// FP64 engines' pass; the mixed engines' double-float and FP32 passes run on
// (tile, source slice) CTAs (k_sums_dfs, k_sums_f32 below).

namespace {

struct SrcDF {
  float wr_hi, wr_lo, wi_hi, wi_lo;  // w_j
  float pr_hi, pr_lo, pi_hi, pi_lo;  // conj(p_j) is formed on the fly
  float a_hi, a_lo;
};

// acc += x with the running high part tracked exactly by a two-sum and every
// low-order bit collected in acc.lo (cascaded summation, Ogita, Rump and
// Oishi's Sum2): as accurate as summing in twice the working precision, with
// one renormalisation at the end (df_acc_done) instead of one per term.
__device__ __forceinline__ void df_acc(df& acc, float xh, float xl) {
  const df s = two_sum(acc.hi, xh);
  acc.hi = s.hi;
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(s.lo, xl));
}
__device__ __forceinline__ df df_acc_done(df acc) { return two_sum(acc.hi, acc.lo); }
// a * b as an unnormalised pair (p + e == a b to double-float accuracy); the
// accumulator absorbs e, so the product needs no renormalisation.
__device__ __forceinline__ df df_mul_raw(df a, df b) {
  const df p = two_prod(a.hi, b.hi);
  return {p.hi, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo))};
}

// x^2 + y^2 and 1 / a as unnormalised pairs (low part within a few ulp of
// the high part), for operands that only enter df_mul_raw / df_rcp_raw.
__device__ __forceinline__ df df_sqsum_raw(df x, df y) {
  const df px = two_prod(x.hi, x.hi);
  const float ex = __fmaf_rn(2.0f * x.hi, x.lo, px.lo);
  const df py = two_prod(y.hi, y.hi);
  const float ey = __fmaf_rn(2.0f * y.hi, y.lo, py.lo);
  const df s = two_sum(px.hi, py.hi);
  return {s.hi, __fadd_rn(s.lo, __fadd_rn(ex, ey))};
}
__device__ __forceinline__ df df_rcp_raw(df a) {
  float r0;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(a.hi));
  const df p = two_prod(a.hi, r0);
  float e = __fsub_rn(__fsub_rn(1.0f, p.hi), p.lo);
  e = __fmaf_rn(-a.lo, r0, e);
  return {r0, __fmul_rn(r0, e)};
}

// (sr, si) += a / (nr + i ni) = a (nr - i ni) / (nr^2 + ni^2), all double-float.
__device__ __forceinline__ void df_div_acc(df nr, df ni, df a, df& sr, df& si) {
  const df t = df_mul_raw(a, df_rcp_raw(df_sqsum_raw(nr, ni)));
  const df pr = df_mul_raw(t, nr), pi = df_mul_raw(t, ni);
  df_acc(sr, pr.hi, pr.lo);
  df_acc(si, -pi.hi, -pi.lo);
}

// ---- packed double-float pairs.  GB300 issues one FP32x2 instruction
// (add / mul / fma .f32x2, each lane rounded to nearest as the scalar
// instruction) per pair of FP32 operations, so the double-float pass keeps
// the real and imaginary parts of a complex double-float side by side and
// runs the identical operation sequence on both at once: the error-free
// transforms stay exact per lane and the sums are bitwise those of the
// scalar sequence, with about half the instructions.
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, neg2(b)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// two double-float numbers: lane x and lane y
struct df2 {
  float2 hi, lo;
};
__device__ __forceinline__ df2 two_sum2(float2 a, float2 b) {
  const float2 s = add2(a, b);
  const float2 bb = sub2(s, a);
  return {s, add2(sub2(a, sub2(s, bb)), sub2(b, bb))};
}
__device__ __forceinline__ df2 quick_two_sum2(float2 a, float2 b) {
  const float2 s = add2(a, b);
  return {s, sub2(b, sub2(s, a))};
}
__device__ __forceinline__ df2 two_prod2(float2 a, float2 b) {
  const float2 p = mul2(a, b);
  return {p, fma2(a, b, neg2(p))};
}
// df_diff per lane, for the node differences w_k - w_j (k != j): the
// renormalisation is a quick two-sum, exact because |hi(w_k) - hi(w_j)| is at
// least the node spacing (about 2 pi / n), far above the low parts' sum
// (ulps of |w| ~ 1), whenever the two nodes are distinct in FP32
__device__ __forceinline__ df2 df_diff2(float2 a_hi, float2 a_lo, float2 b_hi, float2 b_lo) {
  const df2 s = two_sum2(a_hi, neg2(b_hi));
  return quick_two_sum2(s.hi, add2(s.lo, sub2(a_lo, b_lo)));
}
// df_mul per lane (normalised)
__device__ __forceinline__ df2 df_mul2(float2 a_hi, float2 a_lo, float2 b_hi, float2 b_lo) {
  const df2 p = two_prod2(a_hi, b_hi);
  return quick_two_sum2(p.hi, fma2(a_hi, b_lo, fma2(a_lo, b_hi, p.lo)));
}
// df_add per lane
__device__ __forceinline__ df2 df_add2(df2 a, df2 b) {
  const df2 s = two_sum2(a.hi, b.hi);
  return quick_two_sum2(s.hi, add2(s.lo, add2(a.lo, b.lo)));
}
// df_acc per lane
__device__ __forceinline__ void df_acc2(df2& acc, float2 xh, float2 xl) {
  const df2 s = two_sum2(acc.hi, xh);
  acc.hi = s.hi;
  acc.lo = add2(acc.lo, add2(s.lo, xl));
}
// (acc.x, acc.y) += (a d.x / |d|^2, a d.y / |d|^2): the packed form of
// df_div_acc for a / (d.x + i d.y) = (a d.x, -a d.y) / |d|^2, with the
// imaginary lane accumulated negated (no per-pair sign flips; negation is
// exact, so to_red's flip gives bitwise the sums of the unflipped sequence)
//   |d|^2: the two squares are non-negative, so ordered by size they need
//   only a quick two-sum; a / |d|^2: one FP32 quotient from the reciprocal
//   estimate and one correction from its remainder, formed exactly by FMAs
//   (the double-float division without a separate reciprocal refinement).
__device__ __forceinline__ void df_div_acc2(df2 d, df a, df2& acc) {
  const df2 P = two_prod2(d.hi, d.hi);
  const float2 E = fma2(mul2(d.hi, make_float2(2.f, 2.f)), d.lo, P.lo);
  const df s = quick_two_sum(fmaxf(P.hi.x, P.hi.y), fminf(P.hi.x, P.hi.y));
  const df q = {s.hi, __fadd_rn(s.lo, __fadd_rn(E.x, E.y))};
  float r0;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(q.hi));
  const float t0 = __fmul_rn(a.hi, r0);
  float rem = __fmaf_rn(-t0, q.hi, a.hi);  // a - t0 q, exact in the high parts
  rem = __fadd_rn(__fmaf_rn(-t0, q.lo, rem), a.lo);
  const df t = {t0, __fmul_rn(rem, r0)};
  const float2 th = make_float2(t.hi, t.hi), tl = make_float2(t.lo, t.lo);
  const df2 p = two_prod2(th, d.hi);
  const float2 e = fma2(th, d.lo, fma2(tl, d.hi, p.lo));
  df_acc2(acc, p.hi, e);
}

// double-float source of the packed pass: hi parts and lo parts of w (and p)
// as register pairs {re, im}
struct SrcDF2 {
  float4 w;  // w.re hi, w.im hi, w.re lo, w.im lo
  float4 p;  // p.re hi, p.im hi, p.re lo, p.im lo
  float a_hi, a_lo;
};

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
  df2 s{{0.f, 0.f}, {0.f, 0.f}};  // (S re, -S im)
  df2 t{{0.f, 0.f}, {0.f, 0.f}};  // (T re, -T im)
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
  float2 w_hi, w_lo;    // (re, im) of w
  float2 p_hi, p_lo;    // (re, im) of p
  float2 ps_hi, ps_lo;  // (im, re) of p
  __device__ void load(float4 w_, float4 p_) {
    w_hi = {w_.x, w_.z}; w_lo = {w_.y, w_.w};
    p_hi = {p_.x, p_.z}; p_lo = {p_.y, p_.w};
    ps_hi = {p_.z, p_.x}; ps_lo = {p_.w, p_.y};
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
__device__ __forceinline__ void pair_acc(const Tgt<SFD_PREC_DF>& t, const SrcDF2& s, bool self, bool image,
                                         Acc<SFD_PREC_DF>& A) {
  const df aj{s.a_hi, s.a_lo};
  if (!self) {
    // (w_k - w_j) as a packed pair, then a_j / (w_k - w_j) accumulated into S
    const df2 d = df_diff2(t.w_hi, t.w_lo, make_float2(s.w.x, s.w.y), make_float2(s.w.z, s.w.w));
    df_div_acc2(d, aj, A.s);
  }
  if (image) {
    // q = p_k conj(p_j): (qr, qi) = (pr prj + pi pij, pi prj - pr pij)
    const float2 prj_hi = make_float2(s.p.x, s.p.x), prj_lo = make_float2(s.p.z, s.p.z);
    const float2 pij_hi = make_float2(s.p.y, s.p.y), pij_lo = make_float2(s.p.w, s.p.w);
    const df2 m1 = df_mul2(t.p_hi, t.p_lo, prj_hi, prj_lo);    // (pr prj, pi prj)
    const df2 m2 = df_mul2(t.ps_hi, t.ps_lo, pij_hi, pij_lo);  // (pi pij, pr pij)
    const df2 q = df_add2(m1, df2{make_float2(m2.hi.x, -m2.hi.y), make_float2(m2.lo.x, -m2.lo.y)});
    // (1 - qr, -qi)
    const df2 d = df_add2(df2{make_float2(1.f, 0.f), make_float2(0.f, 0.f)}, df2{neg2(q.hi), neg2(q.lo)});
    df_div_acc2(d, aj, A.t);
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
template <int PREC>
using SrcT = typename std::conditional<PREC == SFD_PREC_F64, Src64,
                                       typename std::conditional<PREC == SFD_PREC_DF, SrcDF2, SrcDF>::type>::type;

// Fixed-order reduction values of one target: FP64 for the FP64 pass,
// double-float for the DF and FP32 passes.
template <int PREC>
struct Red {
  df sr{0.f, 0.f}, si{0.f, 0.f}, tr{0.f, 0.f}, ti{0.f, 0.f};
};
template <>
struct Red<SFD_PREC_F64> {
  double sr = 0, si = 0, tr = 0, ti = 0;
};
template <int PREC>
using WSum = typename std::conditional<PREC == SFD_PREC_F64, double, df>::type;

__device__ __forceinline__ Red<SFD_PREC_F64> to_red(const Acc<SFD_PREC_F64>& A) { return {A.sr, A.si, A.tr, A.ti}; }
__device__ __forceinline__ Red<SFD_PREC_DF> to_red(const Acc<SFD_PREC_DF>& A) {
  const df2 s = two_sum2(A.s.hi, A.s.lo), t = two_sum2(A.t.hi, A.t.lo);  // df_acc_done per lane
  return {df{s.hi.x, s.lo.x}, df{-s.hi.y, -s.lo.y}, df{t.hi.x, t.lo.x}, df{-t.hi.y, -t.lo.y}};
}
__device__ __forceinline__ Red<SFD_PREC_F32> to_red(const Acc<SFD_PREC_F32>& A) {
  return {df{A.sr, 0.f}, df{A.si, 0.f}, df{A.tr, 0.f}, df{A.ti, 0.f}};
}
__device__ __forceinline__ void red_add(Red<SFD_PREC_F64>& a, const Red<SFD_PREC_F64>& b) {
  a.sr += b.sr; a.si += b.si; a.tr += b.tr; a.ti += b.ti;
}
template <int PREC>
__device__ __forceinline__ void red_add(Red<PREC>& a, const Red<PREC>& b) {
  a.sr = df_add(a.sr, b.sr); a.si = df_add(a.si, b.si); a.tr = df_add(a.tr, b.tr); a.ti = df_add(a.ti, b.ti);
}
__device__ __forceinline__ double wsum_add(double a, double b) { return a + b; }
__device__ __forceinline__ df wsum_add(df a, df b) { return df_add(a, b); }
__device__ __forceinline__ double shfl_x(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ df shfl_x(df v, int o) {
  return {__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
}
__device__ __forceinline__ Red<SFD_PREC_F64> shfl_x(const Red<SFD_PREC_F64>& v, int o) {
  return {shfl_x(v.sr, o), shfl_x(v.si, o), shfl_x(v.tr, o), shfl_x(v.ti, o)};
}
template <int PREC>
__device__ __forceinline__ Red<PREC> shfl_x(const Red<PREC>& v, int o) {
  return {shfl_x(v.sr, o), shfl_x(v.si, o), shfl_x(v.tr, o), shfl_x(v.ti, o)};
}
__device__ __forceinline__ double to_d(double v) { return v; }
__device__ __forceinline__ double to_d(df v) { return df_to_double(v); }

// Epilogue of one target g (surface S) from its sums S_k, T_k and the weight
// sum A:
//   C_k = i (2 w_k S_k - (A - a_k)),   D_k = -i (2 T_k - A)
//   (M a)_k = Mdiag_k a_k + c1 Im(z'_k C_k) - [image] (1/4pi) Im D_k
// mode 0: C/D overwritten, r = phi' - M a; mode 1: C/D accumulated, r -= M a.
// Returns |r_k| (1e300 for NaN).
__device__ __forceinline__ double sums_finish(const SumArgs& A, const SurfaceDesc& S, int g, cd sum_s, cd sum_t,
                                              double asum, bool image) {
  constexpr double inv4pi = 0.25 / SFD_PI;
  const double c1 = S.physics == 0 ? inv4pi * (1 - S.rho) : inv4pi;
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
  if (A.rf) A.rf[g] = (float)rnew;
  double rv = fabs(rnew);
  return (rv == rv) ? rv : 1e300;
}

template <int PREC, int G>
__global__ void __cluster_dims__(kSumCL, 1, 1) __launch_bounds__(G * kSumTile, 1024 / (G * kSumTile))
    k_boundary_sums(SumArgs A) {
  sfd_pdl_begin();
  constexpr int kSumGroups = G;                  // source groups per CTA (tuned per engine)
  constexpr int kSumThreads = G * kSumTile;
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int2 item = A.items[blockIdx.x / kSumCL];
  const int sidx = item.x, t0 = item.y;
  if (!gate_open(A.gate, sidx)) return;  // every CTA of the cluster has the same surface
  const SurfaceDesc& S = A.surf[sidx];
  const int n = S.n, off = S.off;
  const bool image = (S.physics == 1 && !S.infinite_depth);
  const int per = (n + kSumCL - 1) / kSumCL;
  const int j_lo = min(n, rank * per), j_hi = min(n, j_lo + per);
  const int jn = j_hi - j_lo;
  extern __shared__ __align__(16) unsigned char sums_dyn[];
  SrcT<PREC>* src = reinterpret_cast<SrcT<PREC>*>(sums_dyn);
  __shared__ Red<PREC> gred[kSumGroups][kSumTile];
  __shared__ WSum<PREC> wwarp[kSumThreads / 32];
  __shared__ WSum<PREC> wcta;
  const int tid = threadIdx.x, lane = tid & 31;

  // ---- stage this CTA's sources and their weight sum
  WSum<PREC> wpart{};
  for (int jj = tid; jj < jn; jj += kSumThreads) {
    const int g = off + j_lo + jj;
    if constexpr (PREC == SFD_PREC_F64) {
      cd w = A.w[g];
      double aj = A.a[g];
      wpart += aj;
      cd p = image ? A.p[g] : cd{0.0, 0.0};
      src[jj] = Src64{w.re, w.im, p.re, p.im, aj};
    } else if constexpr (PREC == SFD_PREC_DF) {
      const float4 w = A.wdf[g];
      const float2 ad = A.adf[g];
      const float4 p = image ? A.pdf[g] : make_float4(0.f, 0.f, 0.f, 0.f);
      wpart = df_add(wpart, df{ad.x, ad.y});
      src[jj] = SrcDF2{make_float4(w.x, w.z, w.y, w.w), make_float4(p.x, p.z, p.y, p.w), ad.x, ad.y};
    } else {
      float4 w = A.wdf[g];
      float2 ad = A.adf[g];
      float4 p = image ? A.pdf[g] : make_float4(0.f, 0.f, 0.f, 0.f);
      wpart = df_add(wpart, df{ad.x, ad.y});
      src[jj] = SrcDF{w.x, w.y, w.z, w.w, p.x, p.y, p.z, p.w, ad.x, 0.f};
    }
  }
  for (int o = 16; o > 0; o >>= 1) wpart = wsum_add(wpart, shfl_x(wpart, o));
  if (lane == 0) wwarp[tid >> 5] = wpart;

  // ---- one target per thread of each group
  const int grp = tid / kSumTile, l = tid % kSumTile;
  const int tk = t0 + l;
  const bool active = tk < n;
  const int gt = off + (active ? tk : 0);
  Tgt<PREC> T;
  if constexpr (PREC == SFD_PREC_F64) {
    T.load(A.w[gt], image ? A.p[gt] : cd{0, 0});
  } else {
    T.load(A.wdf[gt], image ? A.pdf[gt] : make_float4(0.f, 0.f, 0.f, 0.f));
  }
  __syncthreads();
  if (tid == 0) {
    WSum<PREC> t = wwarp[0];
    for (int i = 1; i < kSumThreads / 32; ++i) t = wsum_add(t, wwarp[i]);
    wcta = t;
  }
  Acc<PREC> R;
  // Sources jj = grp, grp + G, ... in ascending order.  Only the block of
  // sources [lo, hi) that holds the tile's own nodes needs the j == k test;
  // the rest runs unchecked and unrolled, so the CTA holding the diagonal is
  // not the cluster's straggler.
  int lo = jn, hi = jn;
  if ((t0 < j_hi) && (t0 + kSumTile > j_lo)) {
    lo = max(0, t0 - j_lo);
    hi = min(jn, t0 + kSumTile - j_lo);
  }
  const int self = active ? tk - j_lo : -1;
  auto first = [&](int a) { return a + ((grp - a) % kSumGroups + kSumGroups) % kSumGroups; };
  int jj = grp;
#pragma unroll 4
  for (; jj < lo; jj += kSumGroups) pair_acc(T, src[jj], false, image, R);
  for (jj = first(lo); jj < hi; jj += kSumGroups) pair_acc(T, src[jj], jj == self, image, R);
#pragma unroll 4
  for (jj = first(hi); jj < jn; jj += kSumGroups) pair_acc(T, src[jj], false, image, R);
  gred[grp][l] = to_red(R);
  __syncthreads();
  if (grp == 0) {
    Red<PREC> v = gred[0][l];
#pragma unroll
    for (int q = 1; q < kSumGroups; ++q) red_add(v, gred[q][l]);
    gred[0][l] = v;
  }
  cluster.sync();

  // ---- CTA `rank` finishes targets [rank kSumPerRank, (rank+1) kSumPerRank)
  if (tid < kSumPerRank * kSumCL) {  // warps 0-1 entirely
    const int lt = rank * kSumPerRank + tid / kSumCL;
    const int q = tid % kSumCL;
    Red<PREC> v = cluster.map_shared_rank(&gred[0][0], q)[lt];
    WSum<PREC> aw = *cluster.map_shared_rank(&wcta, q);
#pragma unroll
    for (int o = 1; o < kSumCL; o <<= 1) {
      red_add(v, shfl_x(v, o));
      aw = wsum_add(aw, shfl_x(aw, o));
    }
    double rv = 0.0, bv = 0.0;
    const int tkk = t0 + lt;
    if (q == 0 && tkk < n) {
      const cd sum_s = {to_d(v.sr), to_d(v.si)};
      const cd sum_t = {to_d(v.tr), to_d(v.ti)};
      rv = sums_finish(A, S, off + tkk, sum_s, sum_t, to_d(aw), image);
      if (A.bnorm) {
        const double b = fabs(A.phip[off + tkk]);
        bv = (b == b) ? b : 1e300;
      }
    }
    // per-surface maxima: non-negative doubles order like their bit patterns
    auto warp_max_to = [&](double val, double* dst) {
      unsigned long long m = (unsigned long long)__double_as_longlong(val);
      for (int o = 16; o > 0; o >>= 1) {
        unsigned long long u = __shfl_xor_sync(0xffffffffu, m, o);
        m = u > m ? u : m;
      }
      if (lane == 0) atomicMax(reinterpret_cast<unsigned long long*>(dst), m);
    };
    if (A.rtrack) warp_max_to(rv, A.rtrack + (long long)sidx * SFD_RSLOTS);
    if (A.bnorm) warp_max_to(bv, A.bnorm + sidx);
  }
  cluster.sync();  // peers may still be reading this CTA's shared memory
}

size_t sfd_sums_smem(int prec, int max_n) {
  const size_t per = (size_t)(max_n + kSumCL - 1) / kSumCL;
  return per * (prec == SFD_PREC_F64 ? sizeof(Src64) : prec == SFD_PREC_DF ? sizeof(SrcDF2) : sizeof(SrcDF));
}

namespace {
template <int PREC>
cudaError_t configure_prec(int bytes) {
  cudaError_t e = cudaFuncSetAttribute(k_boundary_sums<PREC, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_boundary_sums<PREC, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_boundary_sums<PREC, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  return e;
}
template <int PREC>
cudaError_t launch_prec(const SumArgs& A, dim3 grid, int groups, size_t smem, cudaStream_t st) {
  if (groups == 2) return sfd_launch(k_boundary_sums<PREC, 2>, grid, dim3(2 * kSumTile), smem, st, true, A);
  if (groups == 8) return sfd_launch(k_boundary_sums<PREC, 8>, grid, dim3(8 * kSumTile), smem, st, true, A);
  return sfd_launch(k_boundary_sums<PREC, 4>, grid, dim3(4 * kSumTile), smem, st, true, A);
}
}  // namespace

template <int G>
__global__ void k_sums_dfs(SumArgs A, float4* dpart);

cudaError_t sfd_sums_configure() {
  // the largest staged source (the packed double-float one is 48 bytes) at n = 8192
  const int bytes = (int)std::max(std::max(sfd_sums_smem(SFD_PREC_F64, 8192), sfd_sums_smem(SFD_PREC_DF, 8192)),
                                  sfd_sums_smem(SFD_PREC_F32, 8192));
  cudaError_t e = configure_prec<SFD_PREC_F64>(bytes);
  if (e == cudaSuccess) e = configure_prec<SFD_PREC_F32>(bytes);
  // double-float pass on slices: slices of up to kF32MaxPer sources
  const int dfs = kF32MaxPer * (int)sizeof(SrcDF2);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_sums_dfs<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, dfs);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_sums_dfs<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, dfs);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_sums_dfs<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, dfs);
  return e;
}

cudaError_t sfd_launch_sums(int prec, const SumArgs& A, int nitems, int max_n, int groups, cudaStream_t st) {
  if (nitems == 0) return cudaSuccess;
  const dim3 grid(nitems * kSumCL);
  const size_t smem = sfd_sums_smem(prec, max_n);
  if (prec == SFD_PREC_F64) return launch_prec<SFD_PREC_F64>(A, grid, groups, smem, st);
  if (prec == SFD_PREC_DF) return cudaErrorInvalidValue;  // the double-float pass runs on slices (k_sums_dfs)
  return launch_prec<SFD_PREC_F32>(A, grid, groups, smem, st);
}

// ----------------------------------------------------------------- FP32 pass
// The FP32 correction passes move small weights (corrections delta ~ 1e-7 a
// and smaller), so their sums and epilogue only need FP32 accuracy.  Layout:
// one independent CTA per (64-target tile, slice of about 256 sources), two
// targets per thread (every shared-memory source read serves both), four
// source groups per CTA.  Each CTA writes its 64 partials and its weight-sum
// partial, then counts itself done on the tile's counter; the CTA that
// finishes last (no CTA ever waits) reduces the tile's slices in slice order,
// so the result does not depend on which CTA that is, and runs the epilogue in
// FP32 with only the final accumulations into C, D and r in FP64.
namespace {
constexpr int kF32Groups = 4;
constexpr int kF32Threads = 32 * kF32Groups;

// S part (sources j != k) and T part (image, every j) of one pair; sources
// are staged as {w.re hi, w.re lo, w.im hi, w.im lo} and {a, p.re, p.im, -}.
__device__ __forceinline__ void f32_s(const float (&t)[6], float4 s0, float a, float4& acc) {
  const float dr = (t[0] - s0.x) + (t[1] - s0.y);
  const float di = (t[2] - s0.z) + (t[3] - s0.w);
  const float inv = a * rcp_approx(fmaf(dr, dr, di * di));
  acc.x = fmaf(inv, dr, acc.x);
  acc.y = fmaf(-inv, di, acc.y);
}
__device__ __forceinline__ void f32_t(const float (&t)[6], float4 s1, float4& acc) {
  const float qr = t[4] * s1.y + t[5] * s1.z, qi = t[5] * s1.y - t[4] * s1.z;
  const float dr = 1.f - qr, di = -qi;
  const float inv = s1.x * rcp_approx(fmaf(dr, dr, di * di));
  acc.z = fmaf(inv, dr, acc.z);
  acc.w = fmaf(-inv, di, acc.w);
}

// Both targets of a thread as packed pairs (lane x: target t0, lane y:
// target t1), for the sources away from the tile's own nodes.
struct F32Pair {
  float2 wr_hi, wr_lo, wi_hi, wi_lo, pr, pi;
};
template <bool IMAGE>
__device__ __forceinline__ void f32_pair2(const F32Pair& T, float4 s0, float4 s1, float2& sr, float2& si,
                                          float2& tr, float2& ti) {
  const float2 dr = add2(sub2(T.wr_hi, make_float2(s0.x, s0.x)), sub2(T.wr_lo, make_float2(s0.y, s0.y)));
  const float2 di = add2(sub2(T.wi_hi, make_float2(s0.z, s0.z)), sub2(T.wi_lo, make_float2(s0.w, s0.w)));
  const float2 d2 = fma2(dr, dr, mul2(di, di));
  const float2 inv = mul2(make_float2(s1.x, s1.x), make_float2(rcp_approx(d2.x), rcp_approx(d2.y)));
  sr = fma2(inv, dr, sr);
  si = fma2(neg2(inv), di, si);
  if (IMAGE) {
    const float2 qr = fma2(T.pr, make_float2(s1.y, s1.y), mul2(T.pi, make_float2(s1.z, s1.z)));
    const float2 qi = fma2(T.pi, make_float2(s1.y, s1.y), neg2(mul2(T.pr, make_float2(s1.z, s1.z))));
    const float2 er = sub2(make_float2(1.f, 1.f), qr), ei = neg2(qi);
    const float2 e2 = fma2(er, er, mul2(ei, ei));
    const float2 inv2 = mul2(make_float2(s1.x, s1.x), make_float2(rcp_approx(e2.x), rcp_approx(e2.y)));
    tr = fma2(inv2, er, tr);
    ti = fma2(neg2(inv2), ei, ti);
  }
}

template <bool IMAGE>
__device__ __forceinline__ void f32_slice_loop(const float4* src, int jn, int grp, int lo, int hi, int self0,
                                               int self1, const float (&T0)[6], const float (&T1)[6], float4& acc0,
                                               float4& acc1) {
  auto first = [&](int a) { return a + ((grp - a) % kF32Groups + kF32Groups) % kF32Groups; };
  const F32Pair P{{T0[0], T1[0]}, {T0[1], T1[1]}, {T0[2], T1[2]}, {T0[3], T1[3]}, {T0[4], T1[4]}, {T0[5], T1[5]}};
  float2 sr = {acc0.x, acc1.x}, si = {acc0.y, acc1.y}, tr = {acc0.z, acc1.z}, ti = {acc0.w, acc1.w};
  int jj = grp;
#pragma unroll 4
  for (; jj < lo; jj += kF32Groups) f32_pair2<IMAGE>(P, src[2 * jj], src[2 * jj + 1], sr, si, tr, ti);
  acc0 = make_float4(sr.x, si.x, tr.x, ti.x);
  acc1 = make_float4(sr.y, si.y, tr.y, ti.y);
  // the tile's own nodes: j == k is skipped per target
  for (jj = first(lo); jj < hi; jj += kF32Groups) {
    const float4 s0 = src[2 * jj], s1 = src[2 * jj + 1];
    if (jj != self0) f32_s(T0, s0, s1.x, acc0);
    if (jj != self1) f32_s(T1, s0, s1.x, acc1);
    if (IMAGE) {
      f32_t(T0, s1, acc0);
      f32_t(T1, s1, acc1);
    }
  }
  sr = {acc0.x, acc1.x}; si = {acc0.y, acc1.y}; tr = {acc0.z, acc1.z}; ti = {acc0.w, acc1.w};
#pragma unroll 4
  for (jj = first(hi); jj < jn; jj += kF32Groups) f32_pair2<IMAGE>(P, src[2 * jj], src[2 * jj + 1], sr, si, tr, ti);
  acc0 = make_float4(sr.x, si.x, tr.x, ti.x);
  acc1 = make_float4(sr.y, si.y, tr.y, ti.y);
}

// Water (no image sums): the sources of a slice are staged in pairs (2m,
// 2m + 1) as {w.re hi, w.re hi', w.re lo, w.re lo'}, {w.im hi, w.im hi',
// w.im lo, w.im lo'} and {a, a'}, so one FP32x2 instruction works on two
// sources of one target with register pairs straight from the shared-memory
// loads (no per-source broadcasts), and the target's values are broadcast
// once, outside the loop.  Pairs holding a node of the tile itself take the
// per-source path with the j == k test.  The imaginary part is accumulated
// negated (exact) and the lanes summed at the end.
struct F32Tgt2 {
  float2 rh, rl, ih, il;  // the target's w parts, broadcast to both lanes
};
__device__ __forceinline__ void f32_pair_src2(const F32Tgt2& T, float4 A, float4 B, float2 a, float2& sr,
                                              float2& sin) {
  const float2 dr = add2(sub2(T.rh, make_float2(A.x, A.y)), sub2(T.rl, make_float2(A.z, A.w)));
  const float2 di = add2(sub2(T.ih, make_float2(B.x, B.y)), sub2(T.il, make_float2(B.z, B.w)));
  const float2 d2 = fma2(dr, dr, mul2(di, di));
  const float2 inv = mul2(a, make_float2(rcp_approx(d2.x), rcp_approx(d2.y)));
  sr = fma2(inv, dr, sr);
  sin = fma2(inv, di, sin);
}
__device__ __forceinline__ void f32_water_pairs(const float4* P0, const float4* P1, const float2* P2, int npairs,
                                                int grp, int plo, int phi, int jn, int self0, int self1,
                                                const float (&T0)[6], const float (&T1)[6], float4& acc0,
                                                float4& acc1) {
  auto first = [&](int a) { return a + ((grp - a) % kF32Groups + kF32Groups) % kF32Groups; };
  const F32Tgt2 U0{{T0[0], T0[0]}, {T0[1], T0[1]}, {T0[2], T0[2]}, {T0[3], T0[3]}};
  const F32Tgt2 U1{{T1[0], T1[0]}, {T1[1], T1[1]}, {T1[2], T1[2]}, {T1[3], T1[3]}};
  // the per-source path reads the targets from the broadcast pairs' first lanes
  const float V0[6] = {U0.rh.x, U0.rl.x, U0.ih.x, U0.il.x, 0.f, 0.f};
  const float V1[6] = {U1.rh.x, U1.rl.x, U1.ih.x, U1.il.x, 0.f, 0.f};
  float2 sr0 = {0.f, 0.f}, si0 = sr0, sr1 = sr0, si1 = sr0;
  int m = grp;
#pragma unroll 2
  for (; m < plo; m += kF32Groups) {
    const float4 A = P0[m], B = P1[m];
    const float2 a = P2[m];
    f32_pair_src2(U0, A, B, a, sr0, si0);
    f32_pair_src2(U1, A, B, a, sr1, si1);
  }
  // pairs holding a node of the tile: per source, j == k skipped per target
  for (m = first(plo); m < phi; m += kF32Groups) {
    const float4 A = P0[m], B = P1[m];
    const float2 a = P2[m];
    for (int e = 0; e < 2; ++e) {
      const int jj = 2 * m + e;
      if (jj >= jn) break;
      const float4 s0 = e ? make_float4(A.y, A.w, B.y, B.w) : make_float4(A.x, A.z, B.x, B.z);
      const float aj = e ? a.y : a.x;
      if (jj != self0) f32_s(V0, s0, aj, acc0);
      if (jj != self1) f32_s(V1, s0, aj, acc1);
    }
  }
#pragma unroll 2
  for (m = first(phi); m < npairs; m += kF32Groups) {
    const float4 A = P0[m], B = P1[m];
    const float2 a = P2[m];
    f32_pair_src2(U0, A, B, a, sr0, si0);
    f32_pair_src2(U1, A, B, a, sr1, si1);
  }
  acc0.x += sr0.x + sr0.y;
  acc0.y -= si0.x + si0.y;
  acc1.x += sr1.x + sr1.y;
  acc1.y -= si1.x + si1.y;
}

__device__ __forceinline__ void load_target(const SumArgs& A, int g, bool image, float (&T)[6]) {
  const float4 w = A.wdf[g];
  T[0] = w.x; T[1] = w.y; T[2] = w.z; T[3] = w.w;
  if (image) {
    const float4 p = A.pdf[g];
    T[4] = p.x; T[5] = p.z;
  } else {
    T[4] = 0.f; T[5] = 0.f;
  }
}
}  // namespace

// Asynchronous global -> shared copies (cp.async): the copy needs no
// register; the issuing thread waits for its own copies before reading them.
__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(sdst)),
               "l"(gsrc)
               : "memory");
}
__device__ __forceinline__ void cp_async8(void* sdst, const void* gsrc) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((unsigned)__cvta_generic_to_shared(sdst)),
               "l"(gsrc)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Epilogue operands of one target of the FP32 pass (16-byte aligned fields
// for the 16-byte copies).
struct __align__(16) F32Epi {
  float4 w;  // w as double-float pairs
  cd zp;     // z'
  double a, md, b;  // weight, M diagonal, phi' (first pass) or r (correction)
  double pad;
  cd c, d;   // corrections: the accumulated C and D
};

// 72 registers (7 CTAs per SM): the water pair loop spills under 64, and the
// 1024 CTAs of N = 4096 still fit one wave on 152 SMs.
__global__ void __launch_bounds__(kF32Threads, 7) k_sums_f32(SumArgs A) {
  const F32Work wk = A.swork[blockIdx.x];  // written once at set-up
  const int sidx = wk.sidx, t0 = wk.t0;
  const int n = wk.n, off = wk.off;
  const bool image = wk.image != 0;
  const int per = (n + wk.nsl - 1) / wk.nsl;
  const int j_lo = min(n, wk.slice * per), j_hi = min(n, j_lo + per), jn = j_hi - j_lo;
  extern __shared__ float4 f32_src[];  // 2 float4 per source
  __shared__ float4 red[kF32Groups][64];
  __shared__ df wred[kF32Groups];
  __shared__ int last;
  const int tid = threadIdx.x, lane = tid & 31, grp = tid >> 5;
  const int tk0 = t0 + lane, tk1 = t0 + 32 + lane;
  float T0[6], T1[6];
  // The node data (w, p) do not change during the solve: where the preceding
  // kernel does not write them, they are staged and the targets loaded
  // before the wait on that kernel, so they arrive while it finishes.
  const bool pre = A.prefetch && !A.gate.slot;
  // water: sources in pairs (P0, P1: w parts; P2: weights), see f32_water_pairs;
  // the second source of an odd slice's last pair is a far node of weight 0
  const int npairs = (jn + 1) >> 1;
  float4* P0 = f32_src;
  float4* P1 = f32_src + npairs;
  float2* P2 = reinterpret_cast<float2*>(f32_src + 2 * npairs);
  auto stage_w_pairs = [&] {
    for (int m = tid; m < npairs; m += kF32Threads) {
      const int g = off + j_lo + 2 * m;
      const float4 w0 = A.wdf[g];
      const float4 w1 = 2 * m + 1 < jn ? A.wdf[g + 1] : make_float4(1e4f, 0.f, 0.f, 0.f);
      P0[m] = make_float4(w0.x, w1.x, w0.y, w1.y);
      P1[m] = make_float4(w0.z, w1.z, w0.w, w1.w);
    }
  };
  if (pre) {
    if (image) {
      for (int jj = tid; jj < jn; jj += kF32Threads) cp_async16(&f32_src[2 * jj], A.wdf + off + j_lo + jj);
      cp_async_commit();
    } else {
      stage_w_pairs();
    }
    load_target(A, off + (tk0 < n ? tk0 : 0), image, T0);
    load_target(A, off + (tk1 < n ? tk1 : 0), image, T1);
  }
  sfd_pdl_begin();
  if (!gate_open(A.gate, sidx)) return;  // every slice of the tile skips together

  // ---- stage this slice's sources and its weight sum
  df wpart{0.f, 0.f};
  if (image) {
    for (int jj = tid; jj < jn; jj += kF32Threads) {
      const int g = off + j_lo + jj;
      const float2 ad = A.adf[g];
      const float4 p = A.pdf[g];
      wpart = df_add(wpart, df{ad.x, ad.y});
      if (!pre) f32_src[2 * jj] = A.wdf[g];
      f32_src[2 * jj + 1] = make_float4(ad.x, p.x, p.z, 0.f);
    }
  } else {
    if (!pre) stage_w_pairs();
    for (int m = tid; m < npairs; m += kF32Threads) {
      const int g = off + j_lo + 2 * m;
      const float2 a0 = A.adf[g];
      const float2 a1 = 2 * m + 1 < jn ? A.adf[g + 1] : make_float2(0.f, 0.f);
      wpart = df_add(wpart, df{a0.x, a0.y});
      wpart = df_add(wpart, df{a1.x, a1.y});
      P2[m] = make_float2(a0.x, a1.x);
    }
  }
  for (int o = 16; o > 0; o >>= 1)
    wpart = df_add(wpart, df{__shfl_xor_sync(0xffffffffu, wpart.hi, o), __shfl_xor_sync(0xffffffffu, wpart.lo, o)});
  if (lane == 0) wred[grp] = wpart;

  // ---- targets t0 + lane and t0 + 32 + lane
  if (!pre) {
    load_target(A, off + (tk0 < n ? tk0 : 0), image, T0);
    load_target(A, off + (tk1 < n ? tk1 : 0), image, T1);
  }
  if (pre) cp_async_wait_all();  // this thread's staged w; the barrier publishes them
  __syncthreads();
  // only the sources of the tile's own nodes need the j == k test
  int lo = jn, hi = jn;
  if (t0 < j_hi && t0 + 64 > j_lo) {
    lo = max(0, t0 - j_lo);
    hi = min(jn, t0 + 64 - j_lo);
  }
  const int self0 = tk0 < n ? tk0 - j_lo : -1, self1 = tk1 < n ? tk1 - j_lo : -1;
  float4 acc0 = make_float4(0.f, 0.f, 0.f, 0.f), acc1 = acc0;
  if (image) f32_slice_loop<true>(f32_src, jn, grp, lo, hi, self0, self1, T0, T1, acc0, acc1);
  else f32_water_pairs(P0, P1, P2, npairs, grp, lo >> 1, (hi + 1) >> 1, jn, self0, self1, T0, T1, acc0, acc1);
  red[grp][lane] = acc0;
  red[grp][32 + lane] = acc1;
  __syncthreads();

  // ---- this slice's partials (groups in order), then count the slice done
  const long long entry = wk.base + wk.slice;
  if (tid < 64) {
    float4 v = red[0][tid];
#pragma unroll
    for (int q = 1; q < kF32Groups; ++q) {
      const float4 u = red[q][tid];
      v.x += u.x; v.y += u.y; v.z += u.z; v.w += u.w;
    }
    A.spart[entry * 64 + tid] = v;
  }
  if (tid == 0) {
    df w = wred[0];
    for (int q = 1; q < kF32Groups; ++q) w = df_add(w, wred[q]);
    A.swsum[entry] = make_float2(w.hi, w.lo);
  }
  // Count the slice done with one acquire-release atomic instead of fences:
  // the barrier orders every thread's partial stores before thread 0's
  // release (release is cumulative), the counter's read-modify-writes form
  // one release sequence, so the last slice's acquire sees every slice's
  // partials, and its barrier orders them before its threads' loads.
  __syncthreads();
  if (tid == 0) {
    unsigned prev;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(prev) : "l"(A.scount + wk.item) : "memory");
    last = prev == (unsigned)(wk.nsl - 1);
  }
  __syncthreads();
  if (!last) return;

  // ---- the last slice of the tile: reduce in slice order, FP32 epilogue.
  // Two threads per target: half h loads slices [8h, 8h + 8) at once (one L2
  // round trip; at most kF32MaxSlices = 16 slices) and sums them in order;
  // half 1 hands its sum to half 0, which adds it last, so the order is fixed.
  if (tid == 0) A.scount[wk.item] = 0u;  // every slice has counted: ready for the next pass
  __shared__ float hsum[64][10];
  // epilogue operands of target t0 + tid: asynchronous copies into shared
  // memory, in flight together with the partial loads below (no registers
  // held across them)
  __shared__ F32Epi epi[64];
  const int tk = t0 + tid;
  const int ge = off + (tk < n ? tk : 0);
  if (tid < 64) {
    F32Epi& E = epi[tid];
    cp_async16(&E.w, A.wdf + ge);
    cp_async16(&E.zp, A.zp + ge);
    cp_async8(&E.a, A.a + ge);
    cp_async8(&E.md, A.mdiag + ge);
    cp_async8(&E.b, (A.mode == 0 ? A.phip : A.r) + ge);
    if (A.mode != 0) {
      cp_async16(&E.c, A.cacc + ge);
      if (image) cp_async16(&E.d, A.dacc + ge);
    }
    cp_async_commit();
  }
  df sr{0.f, 0.f}, si{0.f, 0.f}, tr{0.f, 0.f}, ti{0.f, 0.f}, aw{0.f, 0.f};
  {
    const int t = tid & 63, h = tid >> 6;
    float4 pv[8];
    float2 pw[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {  // slices [8h, 8h + 8): one L2 round trip
      const int sl = 8 * h + i;
      pv[i] = sl < wk.nsl ? __ldcg(A.spart + (wk.base + sl) * 64LL + t) : make_float4(0.f, 0.f, 0.f, 0.f);
      pw[i] = sl < wk.nsl ? __ldcg(A.swsum + wk.base + sl) : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if (8 * h + i < wk.nsl) {
        sr = df_add(sr, df{pv[i].x, 0.f});
        si = df_add(si, df{pv[i].y, 0.f});
        tr = df_add(tr, df{pv[i].z, 0.f});
        ti = df_add(ti, df{pv[i].w, 0.f});
        aw = df_add(aw, df{pw[i].x, pw[i].y});
      }
    }
    if (h == 1) {
      float* o = hsum[t];
      o[0] = sr.hi; o[1] = sr.lo; o[2] = si.hi; o[3] = si.lo; o[4] = tr.hi;
      o[5] = tr.lo; o[6] = ti.hi; o[7] = ti.lo; o[8] = aw.hi; o[9] = aw.lo;
    }
    __syncthreads();
    if (h == 1) return;
    const float* o = hsum[t];
    sr = df_add(sr, df{o[0], o[1]});
    si = df_add(si, df{o[2], o[3]});
    tr = df_add(tr, df{o[4], o[5]});
    ti = df_add(ti, df{o[6], o[7]});
    aw = df_add(aw, df{o[8], o[9]});
  }
  cp_async_wait_all();  // this thread's own copies: no barrier needed
  double rv = 0.0, bv = 0.0;
  if (tk < n) {
    const int g = ge;
    const F32Epi& E = epi[tid];
    const float4 ew = E.w;
    const cd ezp = E.zp;
    const double emd = E.md, eb = E.b;
    constexpr float inv4pi = (float)(0.25 / SFD_PI);
    const float c1 = wk.c1;
    const float wr = ew.x + ew.y, wi = ew.z + ew.w;
    const float ak = (float)E.a;
    const float Sr = sr.hi + sr.lo, Si = si.hi + si.lo, Af = aw.hi + aw.lo;
    // C = i (2 w S - (A - a_k)),  D = -i (2 T - A)
    const float ur = 2.f * (wr * Sr - wi * Si) - (Af - ak), ui = 2.f * (wr * Si + wi * Sr);
    const float Cr = -ui, Ci = ur;
    float Dr = 0.f, Di = 0.f;
    if (image) {
      Dr = 2.f * (ti.hi + ti.lo);
      Di = -(2.f * (tr.hi + tr.lo) - Af);
    }
    float ma = (float)emd * ak + c1 * ((float)ezp.re * Ci + (float)ezp.im * Cr);
    if (image) ma -= inv4pi * Di;
    double rnew;
    if (A.mode == 0) {
      A.cacc[g] = cd{(double)Cr, (double)Ci};
      if (image) A.dacc[g] = cd{(double)Dr, (double)Di};
      rnew = eb - (double)ma;
    } else {
      const cd c = E.c;
      A.cacc[g] = cd{c.re + (double)Cr, c.im + (double)Ci};
      if (image) {
        const cd d = E.d;
        A.dacc[g] = cd{d.re + (double)Dr, d.im + (double)Di};
      }
      rnew = eb - (double)ma;
    }
    A.r[g] = rnew;
    if (A.rf) A.rf[g] = (float)rnew;
    rv = fabs(rnew);
    rv = (rv == rv) ? rv : 1e300;
    if (A.bnorm) {  // mode 0: eb = phi'
      const double b = fabs(eb);
      bv = (b == b) ? b : 1e300;
    }
  }
  auto warp_max_to = [&](double val, double* dst) {
    unsigned long long m = (unsigned long long)__double_as_longlong(val);
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long u = __shfl_xor_sync(0xffffffffu, m, o);
      m = u > m ? u : m;
    }
    if (lane == 0) atomicMax(reinterpret_cast<unsigned long long*>(dst), m);
  };
  if (A.rtrack) warp_max_to(rv, A.rtrack + (long long)sidx * SFD_RSLOTS);
  if (A.bnorm) warp_max_to(bv, A.bnorm + sidx);
}

// two float4 per source (image layout), or per pair of sources two float4
// and one float2 (water layout: 40 bytes per pair, at most 32 per source
// from two sources on, plus the slack of a one-source slice)
static size_t f32_smem(int max_per) { return (size_t)std::max(1, max_per) * 2 * sizeof(float4) + 16; }

cudaError_t sfd_f32_ctas_per_sm(int max_per, int* ctas) {
  const size_t smem = f32_smem(max_per);
  cudaError_t e = cudaFuncSetAttribute(k_sums_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, k_sums_f32, kF32Threads, smem);
  return e;
}

cudaError_t sfd_launch_sums_f32(const SumArgs& A, int nwork, int max_per, cudaStream_t st) {
  if (nwork == 0) return cudaSuccess;
  return sfd_launch(k_sums_f32, dim3(nwork), dim3(kF32Threads), f32_smem(max_per), st, true, A);
}

// ------------------------------------------------- double-float pass on slices
// The accurate pass of a mixed solve (S_k, T_k in double-float, ~48 bits)
// with the FP32 pass's layout: one independent CTA per (64-target tile,
// source slice) work entry, sharing its work entries, tile counters and
// weight-sum partials (the passes run one after another on one stream).  G
// groups of 64 threads, one target per thread; group g takes the slice's
// sources g, g + G, ... in ascending order.  The CTA writes its 64 targets'
// double-float partials; the last slice of a tile to finish (acquire-release
// counter, as in the FP32 pass) reduces them in slice order and runs the FP64
// epilogue.  Compared with one 8-CTA cluster per tile, no CTA waits for its
// cluster peers, and small surfaces get slices sized to their work.
template <int G>
__global__ void __launch_bounds__(64 * G, 1024 / (64 * G)) k_sums_dfs(SumArgs A, float4* dpart) {
  sfd_pdl_begin();
  constexpr int NT = 64 * G;
  const F32Work wk = A.swork[blockIdx.x];
  const int sidx = wk.sidx, t0 = wk.t0;
  if (!gate_open(A.gate, sidx)) return;  // every slice of the tile skips together
  const int n = wk.n, off = wk.off;
  const bool image = wk.image != 0;
  const int per = (n + wk.nsl - 1) / wk.nsl;
  const int j_lo = min(n, wk.slice * per), j_hi = min(n, j_lo + per), jn = j_hi - j_lo;
  extern __shared__ __align__(16) unsigned char dfs_dyn[];
  SrcDF2* src = reinterpret_cast<SrcDF2*>(dfs_dyn);
  __shared__ Red<SFD_PREC_DF> gred[G][kSumTile];
  __shared__ df wred[NT / 32];
  __shared__ int last;
  const int tid = threadIdx.x, lane = tid & 31;

  // ---- stage this slice's sources and its weight sum
  df wpart{0.f, 0.f};
  for (int jj = tid; jj < jn; jj += NT) {
    const int g = off + j_lo + jj;
    const float4 w = A.wdf[g];
    const float2 ad = A.adf[g];
    const float4 p = image ? A.pdf[g] : make_float4(0.f, 0.f, 0.f, 0.f);
    wpart = df_add(wpart, df{ad.x, ad.y});
    src[jj] = SrcDF2{make_float4(w.x, w.z, w.y, w.w), make_float4(p.x, p.z, p.y, p.w), ad.x, ad.y};
  }
  for (int o = 16; o > 0; o >>= 1) wpart = df_add(wpart, shfl_x(wpart, o));
  if (lane == 0) wred[tid >> 5] = wpart;

  // ---- one target per thread of each group
  const int grp = tid / kSumTile, l = tid % kSumTile;
  const int tk = t0 + l;
  const int gt = off + (tk < n ? tk : 0);
  Tgt<SFD_PREC_DF> T;
  T.load(A.wdf[gt], image ? A.pdf[gt] : make_float4(0.f, 0.f, 0.f, 0.f));
  __syncthreads();
  Acc<SFD_PREC_DF> R;
  // only the sources of the tile's own nodes need the j == k test
  int lo = jn, hi = jn;
  if (t0 < j_hi && t0 + kSumTile > j_lo) {
    lo = max(0, t0 - j_lo);
    hi = min(jn, t0 + kSumTile - j_lo);
  }
  const int self = tk < n ? tk - j_lo : -1;
  auto first = [&](int a) { return a + ((grp - a) % G + G) % G; };
  int jj = grp;
#pragma unroll 4
  for (; jj < lo; jj += G) pair_acc(T, src[jj], false, image, R);
  for (jj = first(lo); jj < hi; jj += G) pair_acc(T, src[jj], jj == self, image, R);
#pragma unroll 4
  for (jj = first(hi); jj < jn; jj += G) pair_acc(T, src[jj], false, image, R);
  gred[grp][l] = to_red(R);
  __syncthreads();

  // ---- this slice's partials (groups in order), then count the slice done
  const long long entry = wk.base + wk.slice;
  if (tid < kSumTile) {
    Red<SFD_PREC_DF> v = gred[0][tid];
#pragma unroll
    for (int q = 1; q < G; ++q) red_add(v, gred[q][tid]);
    dpart[entry * 128 + 2 * tid] = make_float4(v.sr.hi, v.sr.lo, v.si.hi, v.si.lo);
    dpart[entry * 128 + 2 * tid + 1] = make_float4(v.tr.hi, v.tr.lo, v.ti.hi, v.ti.lo);
  }
  if (tid == 0) {
    df w = wred[0];
    for (int q = 1; q < NT / 32; ++q) w = df_add(w, wred[q]);
    A.swsum[entry] = make_float2(w.hi, w.lo);
  }
  // one acquire-release atomic per slice (see k_sums_f32)
  __syncthreads();
  if (tid == 0) {
    unsigned prev;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(prev) : "l"(A.scount + wk.item) : "memory");
    last = prev == (unsigned)(wk.nsl - 1);
  }
  __syncthreads();
  if (!last) return;

  // ---- the last slice of the tile: reduce in slice order, FP64 epilogue.
  // P parts of 64 threads: part h sums slices [h spp, (h + 1) spp) in order,
  // four loads in flight at a time; part 0 then adds parts 1 .. P - 1 in
  // order, so the order is fixed.
  if (tid == 0) A.scount[wk.item] = 0u;  // every slice has counted: ready for the next pass
  constexpr int P = G < 4 ? G : 4;
  constexpr int spp = (kF32MaxSlices + P - 1) / P;
  __shared__ float hsum[P][kSumTile][10];
  const int t = tid & 63, h = tid >> 6;
  Red<SFD_PREC_DF> v;
  df aw{0.f, 0.f};
  if (h < P) {
    for (int b = 0; b < spp; b += 4) {
      float4 pa[4], pb[4];
      float2 pw[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int sl = h * spp + b + i;
        const bool in = b + i < spp && sl < wk.nsl;
        pa[i] = in ? __ldcg(dpart + (wk.base + sl) * 128LL + 2 * t) : make_float4(0.f, 0.f, 0.f, 0.f);
        pb[i] = in ? __ldcg(dpart + (wk.base + sl) * 128LL + 2 * t + 1) : make_float4(0.f, 0.f, 0.f, 0.f);
        pw[i] = in ? __ldcg(A.swsum + wk.base + sl) : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        if (b + i < spp && h * spp + b + i < wk.nsl) {
          red_add(v, Red<SFD_PREC_DF>{df{pa[i].x, pa[i].y}, df{pa[i].z, pa[i].w}, df{pb[i].x, pb[i].y},
                                      df{pb[i].z, pb[i].w}});
          aw = df_add(aw, df{pw[i].x, pw[i].y});
        }
      }
    }
    if (h > 0) {
      float* o = hsum[h][t];
      o[0] = v.sr.hi; o[1] = v.sr.lo; o[2] = v.si.hi; o[3] = v.si.lo; o[4] = v.tr.hi;
      o[5] = v.tr.lo; o[6] = v.ti.hi; o[7] = v.ti.lo; o[8] = aw.hi; o[9] = aw.lo;
    }
  }
  __syncthreads();
  if (h != 0) return;
#pragma unroll
  for (int q = 1; q < P; ++q) {
    const float* o = hsum[q][t];
    red_add(v, Red<SFD_PREC_DF>{df{o[0], o[1]}, df{o[2], o[3]}, df{o[4], o[5]}, df{o[6], o[7]}});
    aw = df_add(aw, df{o[8], o[9]});
  }
  double rv = 0.0, bv = 0.0;
  if (tk < n) {
    const SurfaceDesc& S = A.surf[sidx];
    rv = sums_finish(A, S, off + tk, cd{to_d(v.sr), to_d(v.si)}, cd{to_d(v.tr), to_d(v.ti)}, to_d(aw), image);
    if (A.bnorm) {
      const double b = fabs(A.phip[off + tk]);
      bv = (b == b) ? b : 1e300;
    }
  }
  auto warp_max_to = [&](double val, double* dst) {
    unsigned long long m = (unsigned long long)__double_as_longlong(val);
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long u = __shfl_xor_sync(0xffffffffu, m, o);
      m = u > m ? u : m;
    }
    if (lane == 0) atomicMax(reinterpret_cast<unsigned long long*>(dst), m);
  };
  if (A.rtrack) warp_max_to(rv, A.rtrack + (long long)sidx * SFD_RSLOTS);
  if (A.bnorm) warp_max_to(bv, A.bnorm + sidx);
}

cudaError_t sfd_launch_sums_dfs(const SumArgs& A, float4* dpart, int nwork, int max_per, int groups,
                                cudaStream_t st) {
  if (nwork == 0) return cudaSuccess;
  const size_t smem = (size_t)std::max(1, max_per) * sizeof(SrcDF2);
  if (groups == 2) return sfd_launch(k_sums_dfs<2>, dim3(nwork), dim3(128), smem, st, true, A, dpart);
  if (groups == 8) return sfd_launch(k_sums_dfs<8>, dim3(nwork), dim3(512), smem, st, true, A, dpart);
  return sfd_launch(k_sums_dfs<4>, dim3(nwork), dim3(256), smem, st, true, A, dpart);
}

// Velocities and Bernoulli:
//   vel_k = conj(-(i/4pi) C_k + [image] (i/4pi) D_k + V1_kk a_k + V2_k a'_k)   (lower)
//   water:  dphi = -(1+rho) g y + |v|^2/2 + rho |v_up|^2/2 - rho (u_low[1] u_up + v_low v_up)
//   helium: dphi = vdw (1 + y/h)^-3 - vdw + |v|^2/2
//   driven helium adds damping * v + strength * I(y, x) [+ D, dD = beta I - D / tau]
// Output goes to the RHS slot (dx, dy, dphi [, dD]).  Status bit on non-finite values.
__global__ void k_velocity_bernoulli(VelArgs V) {
  sfd_pdl_begin();
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= V.ntot) return;
  const int s = V.node_surf[g];
  const SurfaceDesc& S = V.surf[s];
  const bool image = (S.physics == 1 && !S.infinite_depth);
  constexpr double inv4pi = 0.25 / SFD_PI;
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
    if (o == 3) vdw += -10.0 / 3.0 * (yk * yk * yk) / (S.depth * S.depth);
    if (o == 3 || o == 2) vdw += 2.0 * (yk * yk) / S.depth;
    if (o >= 1 && o <= 3) vdw += -yk;
    out = vdw + kin;
  } else if (S.bern_variant == 2) {
    // surface-tension variant with the reference's fixed prefactor (createM.cuh:195-211)
    cd z1 = V.zp[g], z2 = V.zpp[g];
    const double m2 = z1.re * z1.re + z1.im * z1.im;
    double curv = (z1.re * z2.im - z1.im * z2.re) / (m2 * sqrt(m2));
    double v1 = low.re * low.re + low.im * low.im;
    const double iq = S.depth / (S.depth + yk);  // (1 + y/h)^-1
    out = 20.447761896665416 * S.depth / 3.0 * (iq * iq * iq - 1) + 0.5 * v1 + S.kappa * curv;
  } else {
    const double iq = S.depth / (S.depth + yk);  // (1 + y/h)^-1: one division instead of pow
    out = S.vdw * (iq * iq * iq) - S.vdw + 0.5 * low.re * low.re + 0.5 * low.im * low.im;
  }
  if (S.drive) {
    // optomechanical drive (helium): damping of the vertical velocity, the
    // instantaneous intensity and, augmented, the delayed intensity D
    const double df = S.dr_detuning - S.dr_G * yk;
    const double dxk = V.x[g] - S.dr_x0;
    const double prof = exp(-(dxk * dxk) / (2.0 * S.dr_sigma * S.dr_sigma));
    const double inten =
        0.25 * S.dr_gamma * S.dr_gamma * S.dr_imax / (df * df + 0.25 * S.dr_gamma * S.dr_gamma) * prof;
    out += S.dr_damping * low.im;
    out += S.dr_strength * inten;
    if (S.drive_aug) {
      const double Dk = V.aux[g];
      out += Dk;
      V.daux[g] = S.dr_beta * inten - 1.0 / S.dr_tau * Dk;
    }
  }
  V.dphi[g] = out;
  if (V.daux && !S.drive_aug) V.daux[g] = 0.0;
  if (!isfinite(out) || !isfinite(low.re) || !isfinite(low.im)) atomicOr(V.status + s, SFD_ST_NONFINITE);
  if (V.rslot && g == S.off) {
    // Refinement summary of this evaluation: the final residual is the first
    // slot at or below tol * max |phi'| (the gated passes after it did not
    // run), else the last slot; a final residual above it is a stall.
    const double* sl = V.rslot + (long long)s * SFD_RSLOTS;
    const double b = V.bnorm[s];
    const double lim = V.tol * b;
    int i = 0;
    double fin = sl[0];
    if (V.tol > 0.0)
      while (!(fin <= lim) && i + 1 < V.nslots) fin = sl[++i];
    if (i > 0) atomicAdd(V.extra_count + s, (unsigned long long)i);
    atomicMax(reinterpret_cast<unsigned long long*>(V.rnorm) + s, (unsigned long long)__double_as_longlong(fin));
    const double rel = b > 0.0 ? fin / b : (fin > 0.0 ? 1e300 : 0.0);
    atomicMax(reinterpret_cast<unsigned long long*>(V.rrel) + s,
              (unsigned long long)__double_as_longlong(rel == rel ? rel : 1e300));
    if (V.tol > 0.0 && !(fin <= lim)) {
      atomicOr(V.status + s, SFD_ST_REFINE_STALL);
      if (V.stall_host) *reinterpret_cast<volatile unsigned int*>(V.stall_host) = 1u;
    }
    if (V.warm) V.warm[s] = (V.tol > 0.0 && fin <= lim) ? 0.0 : 1e300;
  }
}

// The water cross term reads the lower velocity of concatenated node 1
// (createM.cuh:104).  For rho != 0 that value is computed first (one thread).
__global__ void k_velocity_node1(VelArgs V) {
  sfd_pdl_begin();
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
  sfd_pdl_begin();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n3) return;
  double kv = k[i];
  kacc[i] = first ? kv : kacc[i] + wk * kv;
  if (ystage) ystage[i] = y0[i] + cy * kv;
}
__global__ void k_rk4_final(int n3, double* __restrict__ y0, const double* __restrict__ kacc, double c) {
  sfd_pdl_begin();
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
