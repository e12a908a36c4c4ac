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
