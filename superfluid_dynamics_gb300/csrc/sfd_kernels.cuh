// sfd_kernels.cuh -- launch-argument structs and kernel declarations.
#pragma once
#include "sfd_engine.cuh"

enum : int { SFD_PREC_F64 = 0, SFD_PREC_DF = 1, SFD_PREC_F32 = 2 };

constexpr int kSumCL = 8;                          // CTAs per cluster (one target tile)
constexpr int kSumTile = 64;                       // targets per tile (one per thread of a group)
constexpr int kSumPerRank = kSumTile / kSumCL;     // targets finished by each CTA of the cluster
// Source groups per CTA (the CTA has groups * kSumTile threads): 2, 4 or 8,
// picked per engine and precision by timing (sfd_options.autotune); 4 otherwise.
constexpr int kSumGroupChoices[3] = {2, 4, 8};

struct NodeData {
  cd* w;        // exp(i z)
  cd* p;        // exp(i z) e^{-h} (helium image kernel)
  float4* wdf;  // w as double-float pairs (re.hi, re.lo, im.hi, im.lo)
  float4* pdf;  // p likewise
  double* mdiag;
  cd* v1low;    // V1_kk lower fluid (no image term)
  cd* v1up;     // V1_kk upper fluid
  cd* v2;       // V2_k
};

// One boundary-sum pass (one cluster per (surface, target tile)) with its
// epilogue (C, D, M a, residual) fused.
struct SumArgs {
  const SurfaceDesc* surf;
  const int2* items;    // (surface, first target) per cluster
  int nsurf;
  int ntot;
  const cd* w;
  const cd* p;
  const double* a;      // weights (FP64; every pass)
  const float4* wdf;    // double-float copies (DF / FP32 passes)
  const float4* pdf;
  const float2* adf;
  const double* mdiag;
  const cd* zp;
  const double* phip;
  cd* cacc;
  cd* dacc;
  double* r;
  double* rtrack;       // residual slot of this pass: per-surface max |r| at rtrack[s * SFD_RSLOTS] (nullable)
  int mode;             // 0: overwrite C/D and r = phi' - M a; 1: accumulate, r -= M a
  float* rf;            // FP32 copy of r for the preconditioner product (nullable)
  double* bnorm;        // mode 0: per-surface max |phi'| (nullable)
  Gate gate;            // extra corrections: skip surfaces whose previous residual is converged
  // FP32 pass (k_sums_f32): one CTA per (tile, source slice); the last CTA
  // of a tile to finish reduces the slices in order and runs the epilogue
  const struct F32Work* swork;  // one entry per CTA
  float4* spart;        // per work entry: 64 target partials (S re, S im, T re, T im)
  float2* swsum;        // per work entry: weight-sum partial (double-float)
  unsigned int* scount; // per item: slices finished (the last one resets it)
  // k_sums_f32, ungated: stage the node data (w, p: written by the node kernel
  // at the start of the evaluation) before the wait on the preceding kernel.
  // Only where that kernel is not the one that writes them.
  int prefetch;
};

// One CTA of the FP32 pass: everything it needs before its first source
// (no dependent loads of the item list or the surface descriptor).
struct F32Work {
  int item;    // index of the (surface, tile) item: its counter
  int slice;   // this CTA's slice of the sources
  int base;    // work entry of the item's slice 0 (partials are base + slice)
  int nsl;     // slices of the item
  int sidx;    // surface
  int t0;      // first target of the tile
  int n, off;  // surface nodes and node offset
  int image;   // finite-depth helium: image sums
  float c1;    // (1 - rho) / 4 pi (water), 1 / 4 pi (helium): factor of z' C in M a
  int pad[2];
};

// Source slices of the FP32 pass: at least kF32MinPer sources and at most
// kF32MaxSlices slices per tile (the last slice's reduction loads them in one
// round trip; SFD_F32_SLICES in the environment lowers the cap); slices
// above kF32MaxPer sources take a second wave rather than more shared memory
// (planned at engine creation).
constexpr int kF32MinPer = 64;
constexpr int kF32MaxPer = 512;
constexpr int kF32MaxSlices = 16;
// Resident CTAs per SM of the FP32 pass with slices of up to max_per sources.
cudaError_t sfd_f32_ctas_per_sm(int max_per, int* ctas);

struct VelArgs {
  const SurfaceDesc* surf;
  const int* node_surf;
  int nsurf;
  int ntot;
  const cd* cacc;
  const cd* dacc;
  const double* a;
  const cd* ap;
  const cd* v1low;
  const cd* v1up;
  const cd* v2;
  const double* y;
  const double* x;      // drive profile
  const double* aux;    // delayed intensity D (augmented drive; state block 4)
  double* daux;         // dD/dt (RHS block 4)
  const cd* zp;
  const cd* zpp;
  cd* vel_low1;
  double* dx;
  double* dy;
  double* dphi;
  unsigned int* status;
  // refinement bookkeeping of the solve (rslot null: none)
  const double* rslot;  // residual slots, SFD_RSLOTS per surface
  int nslots;           // slots the solve can fill: 1 + extra corrections
  const double* bnorm;  // per-surface max |phi'|
  double tol;           // relative residual tolerance (<= 0: no stall check)
  double* rnorm;        // per-surface max over evaluations of the final |r| (absolute)
  double* rrel;         // the same relative to max |phi'|
  unsigned long long* extra_count;  // per-surface count of extra corrections run
  unsigned int* stall_host;         // host-mapped word set on a refinement stall (nullable)
  double* warm;                     // mixed solves: per surface 0 when this solve converged (the next may
                                    // start from its solution), 1e300 otherwise (nullable)
};

__global__ void k_node_prep(const SurfaceDesc* surf, const int* node_surf, int ntot, const double* x,
                            const double* y, const cd* zp, const cd* zpp, NodeData nd, double* rslot,
                            double* bnorm);
cudaError_t sfd_launch_sums(int prec, const SumArgs& A, int nitems, int max_n, int groups, cudaStream_t st);
// FP32 pass over `nwork` (tile, slice) entries (A.swork), slices of at most
// max_per sources.
cudaError_t sfd_launch_sums_f32(const SumArgs& A, int nwork, int max_per, cudaStream_t st);
// Double-float pass on the FP32 pass's (tile, slice) work entries; dpart: 128
// float4 of double-float partials per work entry; groups: 2, 4 or 8 groups of
// 64 threads per CTA.
cudaError_t sfd_launch_sums_dfs(const SumArgs& A, float4* dpart, int nwork, int max_per, int groups,
                                cudaStream_t st);
cudaError_t sfd_sums_configure();
__global__ void k_velocity_bernoulli(VelArgs V);
__global__ void k_velocity_node1(VelArgs V);
__global__ void k_rk4_stage(int n3, const double* y0, const double* k, double* kacc, double* ystage, double wk,
                            double cy, int first);
__global__ void k_rk4_final(int n3, double* y0, const double* kacc, double c);
__global__ void k_invariants(const SurfaceDesc* surf, const double* x, const double* y, const double* phi,
                             const cd* zp, const double* u, const double* v, double kappa, double* out);

// Four-step transforms of power-of-two surfaces (sfd_fft4.cu): jobs write z'
// and z'' (from one forward transform), phi', or a'; the RAW jobs (reverse
// mode) transform their own input in_re + i in_im (in_im nullable) into out
// with the first (RAW1) or second (RAW2) derivative multiplier, unscaled (the
// d/dj of FftDerivative::exec).
enum : int { SFD_F4_Z = 0, SFD_F4_PHI = 1, SFD_F4_AP = 2, SFD_F4_RAW1 = 3, SFD_F4_RAW2 = 4 };
struct F4Job {
  int surf;
  int kind;
  long long scr0, scr1;  // scratch offsets (complex elements): rows of the job, and z'' rows for SFD_F4_Z
  const double* in_re;   // RAW jobs only
  const double* in_im;
  cd* out;
};
// The jobs of one spectral launch and their unit lists (job, unit) per phase.
struct F4Plan {
  F4Job* jobs = nullptr;
  int2* units[3] = {nullptr, nullptr, nullptr};
  int nunits[3] = {0, 0, 0};
  int njobs = 0;
};
bool sfd_f4_eligible(int n);
cudaError_t sfd_launch_f4(const DerivArgs& A, const F4Plan& p, cd* scr, cudaStream_t st, int phase);

cudaError_t sfd_launch_spectral(const DerivArgs& A, const int2* jobs, int njobs, int max_n, cudaStream_t st);
cudaError_t sfd_launch_spectral_cluster(const DerivArgs& A, const int2* jobs, int njobs, int max_n, cudaStream_t st);
cudaError_t sfd_fft_configure();
