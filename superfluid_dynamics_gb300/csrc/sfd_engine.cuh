// sfd_engine.cuh -- device-visible descriptors shared by the engine kernels.
#pragma once
#include "sfd_common.cuh"

#define SFD_MAX_RADICES 24

// One surface of a (possibly uneven) batch.  All node arrays of the batch are
// concatenated; surface s owns [off, off + n).  Dense per-surface matrices are
// concatenated too; surface s owns [moff, moff + n*n) stored row-major
// (row k = target node, column j = source node).
struct SurfaceDesc {
  int n;
  int off;
  long long moff;
  int physics;          // 0 water, 1 helium
  int infinite_depth;   // helium without image terms
  double rho;           // water density ratio
  double depth;         // helium film thickness h
  double vdw;           // A3 / h^3 (the reference fixes h / 3)
  double gravity;       // water g
  double U;             // uniform stream (only the linear part of phi uses it)
  double kappa;         // surface tension (helium Bernoulli variant)
  int bern_variant;     // 0 standard, 1 series expansion (createM.cuh:171-193), 2 surface tension (:200-211)
  int expansion_order;
  const cd* tw;         // forward FFT twiddles exp(-2 pi i e / n), e in [0, n)
  const cd* ctw;        // cluster transforms (nrad_m > 0): [W_n^{C e} | per CTA c: W_n^{c e}, W_n^{q (c R + t)}], M = n / C, R = M / C
  int nrad;
  int rad[SFD_MAX_RADICES];
  int nrad_m;           // radices of n / SFD_FFT_CLUSTER (cluster transforms; 0 = not eligible)
  int rad_m[SFD_MAX_RADICES];
  // optomechanical drive (helium; LightIntensity.cuh:19-37, DelayedIntensityIntegrator.cuh:22-36)
  int drive;            // 0 none, 1 drive terms in dphi/dt
  int drive_aug;        // delayed intensity D carried in the state
  double dr_detuning, dr_gamma, dr_G, dr_tau, dr_imax, dr_x0, dr_sigma, dr_beta, dr_damping, dr_strength;
};

// Cluster size of the distributed spectral-derivative kernel; surfaces with
// n % (SFD_FFT_CLUSTER^2) == 0 and n >= SFD_FFT_CLUSTER_MIN_N use it.
#define SFD_FFT_CLUSTER 8
#define SFD_FFT_CLUSTER_MIN_N 512

// Spectral-derivative job kinds (one CTA per job).
enum : int {
  SFD_JOB_ZP = 0,   // z' from x - 2 pi j/N + i y
  SFD_JOB_ZPP = 1,  // z''
  SFD_JOB_PHIP = 2, // phi' (real part kept)
  SFD_JOB_AP = 3,   // a' (complex kept)
  SFD_JOB_RAW = 4,  // d/dj of (x + i y) with no linear part and no 2 pi/N scale -> ap
  SFD_JOB_RAW2 = 5, // d^2/dj^2 of (x + i y), likewise unscaled -> ap (reverse mode)
};

// Residual slots of one RHS evaluation: slot 0 holds max |r| of the last
// regular pass of the solve, slot i the residual after extra correction i.
// k_node_prep clears them (and max |phi'|) for every evaluation.
#define SFD_MAX_EXTRA 4
#define SFD_RSLOTS (1 + SFD_MAX_EXTRA)

// Refinement gate.  A kernel given an open gate (slot != null) does its work
// only for the surfaces whose residual in `slot` is above tol * max |phi'|;
// for the others it returns at once.  This keeps the extra corrections inside
// a fixed launch sequence (and a fixed CUDA graph) while costing only a launch
// when they are not needed.  A NaN residual counts as above (slots store 1e300
// for NaN); a NaN scale counts as below.
struct Gate {
  const double* slot;   // rslot + (pass - 1): the previous tracked pass; null = ungated
  const double* bnorm;  // per-surface max |phi'|
  int stride;           // slots per surface (SFD_RSLOTS)
  double tol;           // relative residual tolerance
};
// Programmatic dependent launch.  A kernel launched with sfd_launch(..., pdl
// = true) may be scheduled while its predecessor in the stream still runs;
// every CTA calls sfd_pdl_begin() before its first global memory access: it
// waits until the predecessor grid has completed and its writes are visible,
// then lets the next kernel of the stream be scheduled in turn.  Every CTA
// waits, also one that returns early, so completion stays transitive along the
// stream.  In a launch without the attribute both instructions return at once.
__device__ __forceinline__ void sfd_pdl_begin() {
  cudaGridDependencySynchronize();
  cudaTriggerProgrammaticLaunchCompletion();
}

__device__ __forceinline__ bool gate_open(const Gate& G, int s) {
  return !G.slot || (G.slot[(long long)s * G.stride] > G.tol * G.bnorm[s]);
}

struct DerivArgs {
  const SurfaceDesc* surf;
  int nsurf;
  const double* x;
  const double* y;
  const double* phi;
  const double* phi_im;  // imaginary part of a complex phi input (nullable)
  const double* a;
  cd* zp;
  cd* zpp;
  double* phip;
  cd* ap;
  float* phipf;  // FP32 copy of phi' for the preconditioner product (nullable)
  Gate gate;     // jobs run only where the gate is open (ungated by default)
};

#ifdef __CUDACC__
#include <cstdlib>
#include <utility>
// Programmatic dependent launch is on unless SFD_PDL=0 is set in the
// environment (read once per process).
inline bool sfd_pdl_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("SFD_PDL");
    return !(v && v[0] == '0');
  }();
  return on;
}

// Launch `k` on `st`; with pdl (and sfd_pdl_enabled()) the launch carries the
// programmatic stream-serialization attribute (a programmatic edge when the
// stream is captured into a graph).  Only kernels that call sfd_pdl_begin()
// first may be launched with pdl.
template <typename... KArgs, typename... Args>
cudaError_t sfd_launch(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, bool pdl,
                       Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  if (pdl && sfd_pdl_enabled()) {
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
  }
  return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}
#endif
