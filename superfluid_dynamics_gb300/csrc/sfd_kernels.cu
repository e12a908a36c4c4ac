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
  if (S.physics == 1 && !S.infinite_depth) {
    double eh = exp(-S.depth);
    nd.p[g] = {w.re * eh, w.im * eh};
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
// kTargets targets (two per thread), writing FP64 partials per chunk; the
// epilogue reduces the chunks in a fixed order (bitwise reproducible).

namespace {

struct SrcDF {
  float wr_hi, wr_lo, wi_hi, wi_lo;  // w_j
  float pr_hi, pr_lo, pi_hi, pi_lo;  // conj(p_j) is formed on the fly
  float a_hi, a_lo;
};

__device__ __forceinline__ void df_div_acc(df nr, df ni, df a, df& sr, df& si) {
  // (sr, si) += a / (nr + i ni) = a (nr - i ni) / (nr^2 + ni^2)
  df den = df_add(df_mul(nr, nr), df_mul(ni, ni));
  df t = df_mul(a, df_rcp(den));
  sr = df_add(sr, df_mul(t, nr));
  si = df_sub(si, df_mul(t, ni));
}

}  // namespace

struct Src64 {
  double wr, wi, pr, pi, a;
};

template <int PREC>
__global__ void __launch_bounds__(kSumThreads) k_boundary_sums(SumArgs A) {
  const int4 item = A.items[blockIdx.x];
  const SurfaceDesc S = A.surf[item.x];
  const int n = S.n, off = S.off;
  const int t0 = item.y, j0 = item.z, chunk = item.w;
  const int jn = min(kSumChunk, n - j0);
  const bool image = (S.physics == 1 && !S.infinite_depth);
  // FP64 sources need exact doubles; the other precisions stage float pairs.
  __shared__ __align__(16) unsigned char src_raw[kSumChunk * (PREC == SFD_PREC_F64 ? sizeof(Src64) : sizeof(SrcDF))];
  Src64* src64 = reinterpret_cast<Src64*>(src_raw);
  SrcDF* src = reinterpret_cast<SrcDF*>(src_raw);
  __shared__ double asum_warp[kSumThreads / 32];
  double apart = 0.0;
  for (int jj = threadIdx.x; jj < jn; jj += kSumThreads) {
    int g = off + j0 + jj;
    cd w = A.w[g];
    double aj = A.a[g];
    apart += aj;
    cd p = image ? A.p[g] : cd{0.0, 0.0};
    if (PREC == SFD_PREC_F64) {
      src64[jj] = Src64{w.re, w.im, p.re, p.im, aj};
    } else {
      SrcDF s;
      if (PREC == SFD_PREC_F32) {
        // w split in hi/lo so that w_k - w_j keeps FP32 relative accuracy
        s.wr_hi = __double2float_rn(w.re); s.wr_lo = __double2float_rn(w.re - (double)s.wr_hi);
        s.wi_hi = __double2float_rn(w.im); s.wi_lo = __double2float_rn(w.im - (double)s.wi_hi);
        s.a_hi = __double2float_rn(aj); s.a_lo = 0.f;
      } else {
        df wr = df_from_double(w.re), wi = df_from_double(w.im), ad = df_from_double(aj);
        s.wr_hi = wr.hi; s.wr_lo = wr.lo; s.wi_hi = wi.hi; s.wi_lo = wi.lo; s.a_hi = ad.hi; s.a_lo = ad.lo;
      }
      df pr = df_from_double(p.re), pi = df_from_double(p.im);
      s.pr_hi = pr.hi; s.pr_lo = pr.lo; s.pi_hi = pi.hi; s.pi_lo = pi.lo;
      src[jj] = s;
    }
  }
  // per-chunk partial of A = sum a_j (written by the first target tile only)
  if (t0 == 0) {
    for (int o = 16; o > 0; o >>= 1) apart += __shfl_xor_sync(0xffffffffu, apart, o);
    if ((threadIdx.x & 31) == 0) asum_warp[threadIdx.x >> 5] = apart;
  }
  __syncthreads();
  if (t0 == 0 && threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < kSumThreads / 32; ++i) s += asum_warp[i];
    A.part_a[(long long)chunk * A.nsurf + item.x] = s;
  }

  for (int rep = 0; rep < kSumTargets / kSumThreads; ++rep) {
    const int tk = t0 + rep * kSumThreads + threadIdx.x;
    const bool active = tk < n;
    const int gk = off + (active ? tk : 0);
    const int self = active ? tk - j0 : -1;  // index of j == k inside this chunk (if any)
    cd wk = A.w[gk];
    cd pk = image ? A.p[gk] : cd{0, 0};
    cd outs = {0, 0}, outt = {0, 0};
    if (PREC == SFD_PREC_F64) {
      double sr = 0, si = 0, tr = 0, ti = 0;
      for (int jj = 0; jj < jn; ++jj) {
        const Src64 s = src64[jj];
        if (jj != self) {
          double dr = wk.re - s.wr, di = wk.im - s.wi;
          double inv = s.a / (dr * dr + di * di);
          sr += inv * dr;
          si -= inv * di;
        }
        if (image) {
          // 1 - pk conj(pj)
          double qr = pk.re * s.pr + pk.im * s.pi, qi = pk.im * s.pr - pk.re * s.pi;
          double dr = 1.0 - qr, di = -qi;
          double inv = s.a / (dr * dr + di * di);
          tr += inv * dr;
          ti -= inv * di;
        }
      }
      outs = {sr, si};
      outt = {tr, ti};
    } else if (PREC == SFD_PREC_DF) {
      df wkr = df_from_double(wk.re), wki = df_from_double(wk.im);
      df sr = {0.f, 0.f}, si = {0.f, 0.f}, tr = {0.f, 0.f}, ti = {0.f, 0.f};
      df pkr = df_from_double(pk.re), pki = df_from_double(pk.im);
      for (int jj = 0; jj < jn; ++jj) {
        const SrcDF s = src[jj];
        df aj = {s.a_hi, s.a_lo};
        if (jj != self) {
          df dr = df_sub(wkr, df{s.wr_hi, s.wr_lo});
          df di = df_sub(wki, df{s.wi_hi, s.wi_lo});
          df_div_acc(dr, di, aj, sr, si);
        }
        if (image) {
          df prj = {s.pr_hi, s.pr_lo}, pij = {s.pi_hi, s.pi_lo};
          df qr = df_add(df_mul(pkr, prj), df_mul(pki, pij));
          df qi = df_sub(df_mul(pki, prj), df_mul(pkr, pij));
          df dr = df_sub(df{1.f, 0.f}, qr);
          df di = df_neg(qi);
          df_div_acc(dr, di, aj, tr, ti);
        }
      }
      outs = {df_to_double(sr), df_to_double(si)};
      outt = {df_to_double(tr), df_to_double(ti)};
    } else {  // FP32: only for small corrections
      float wkr_hi = __double2float_rn(wk.re), wkr_lo = __double2float_rn(wk.re - (double)wkr_hi);
      float wki_hi = __double2float_rn(wk.im), wki_lo = __double2float_rn(wk.im - (double)wki_hi);
      float pkr = (float)pk.re, pki = (float)pk.im;
      float sr = 0.f, si = 0.f, tr = 0.f, ti = 0.f;
      for (int jj = 0; jj < jn; ++jj) {
        const SrcDF s = src[jj];
        if (jj != self) {
          float dr = (wkr_hi - s.wr_hi) + (wkr_lo - s.wr_lo);
          float di = (wki_hi - s.wi_hi) + (wki_lo - s.wi_lo);
          float inv = s.a_hi / (dr * dr + di * di);
          sr = fmaf(inv, dr, sr);
          si = fmaf(-inv, di, si);
        }
        if (image) {
          float prj = s.pr_hi, pij = s.pi_hi;
          float qr = pkr * prj + pki * pij, qi = pki * prj - pkr * pij;
          float dr = 1.f - qr, di = -qi;
          float inv = s.a_hi / (dr * dr + di * di);
          tr = fmaf(inv, dr, tr);
          ti = fmaf(-inv, di, ti);
        }
      }
      outs = {(double)sr, (double)si};
      outt = {(double)tr, (double)ti};
    }
    if (active) {
      long long o = (long long)chunk * A.ntot + gk;
      A.part_s[o] = outs;
      if (image) A.part_t[o] = outt;
    }
  }
}

cudaError_t sfd_launch_sums(int prec, const SumArgs& A, int nitems, cudaStream_t st) {
  if (nitems == 0) return cudaSuccess;
  if (prec == SFD_PREC_F64) k_boundary_sums<SFD_PREC_F64><<<nitems, kSumThreads, 0, st>>>(A);
  else if (prec == SFD_PREC_DF) k_boundary_sums<SFD_PREC_DF><<<nitems, kSumThreads, 0, st>>>(A);
  else k_boundary_sums<SFD_PREC_F32><<<nitems, kSumThreads, 0, st>>>(A);
  return cudaGetLastError();
}

// Reduce the chunk partials and form C, D, M a for every node:
//   C_k = i (2 w_k S_k - (A - a_k)),   D_k = -i (2 T_k - A)
//   (M a)_k = Mdiag_k a_k + c1 Im(z'_k C_k) - [image] (1/4pi) Im D_k
// mode 0: overwrite C/D accumulators and set r = phi' - M a
// mode 1: add to the accumulators and set r = r - M a  (correction pass)
__global__ void k_sum_epilogue(EpiArgs E, int mode) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= E.ntot) return;
  const int s = E.node_surf[g];
  const SurfaceDesc& S = E.surf[s];
  const int nchunk = (S.n + kSumChunk - 1) / kSumChunk;
  cd sum_s = {0, 0}, sum_t = {0, 0};
  double asum = 0.0;
  const bool image = (S.physics == 1 && !S.infinite_depth);
  for (int c = 0; c < nchunk; ++c) {
    long long o = (long long)c * E.ntot + g;
    sum_s = sum_s + E.part_s[o];
    if (image) sum_t = sum_t + E.part_t[o];
    asum += E.part_a[(long long)c * E.nsurf + s];
  }
  double ak = E.a[g];
  cd wk = E.w[g];
  cd C = cmul_i(2.0 * (wk * sum_s) - cd{asum - ak, 0.0});
  cd D = image ? cmul_i(cd{-(2.0 * sum_t.re - asum), -(2.0 * sum_t.im)}) : cd{0, 0};
  double c1 = S.physics == 0 ? 0.25 * (1 - S.rho) / SFD_PI : 0.25 / SFD_PI;
  double ma = E.mdiag[g] * ak + c1 * (E.zp[g] * C).im;
  if (image) ma -= 0.25 / SFD_PI * D.im;
  if (mode == 0) {
    E.cacc[g] = C;
    if (image) E.dacc[g] = D;
    E.r[g] = E.phip[g] - ma;
  } else {
    E.cacc[g] = E.cacc[g] + C;
    if (image) E.dacc[g] = E.dacc[g] + D;
    E.r[g] = E.r[g] - ma;
  }
  if (E.rnorm) {
    // |r| max per surface (for the refinement status); non-negative doubles
    // order like their bit patterns, so an integer atomicMax works.
    double rv = fabs(E.r[g]);
    if (!(rv == rv)) rv = 1e300;
    atomicMax(reinterpret_cast<unsigned long long*>(E.rnorm) + s, __double_as_longlong(rv));
  }
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
