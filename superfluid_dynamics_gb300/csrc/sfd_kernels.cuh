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
  double* rnorm;        // per-surface max |r| (nullable)
  int mode;             // 0: overwrite C/D and r = phi' - M a; 1: accumulate, r -= M a
  float* rf;            // FP32 copy of r for the preconditioner product (nullable)
};

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
};

__global__ void k_node_prep(const SurfaceDesc* surf, const int* node_surf, int ntot, const double* x,
                            const double* y, const cd* zp, const cd* zpp, NodeData nd);
cudaError_t sfd_launch_sums(int prec, const SumArgs& A, int nitems, int max_n, int groups, cudaStream_t st);
cudaError_t sfd_sums_configure();
__global__ void k_velocity_bernoulli(VelArgs V);
__global__ void k_velocity_node1(VelArgs V);
__global__ void k_rk4_stage(int n3, const double* y0, const double* k, double* kacc, double* ystage, double wk,
                            double cy, int first);
__global__ void k_rk4_final(int n3, double* y0, const double* kacc, double c);
__global__ void k_invariants(const SurfaceDesc* surf, const double* x, const double* y, const double* phi,
                             const cd* zp, const double* u, const double* v, double kappa, double* out);

cudaError_t sfd_launch_spectral(const DerivArgs& A, const int2* jobs, int njobs, int max_n, cudaStream_t st);
cudaError_t sfd_launch_spectral_cluster(const DerivArgs& A, const int2* jobs, int njobs, int max_n, cudaStream_t st);
cudaError_t sfd_fft_configure();
