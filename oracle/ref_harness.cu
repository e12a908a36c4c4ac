// ref_harness.cu -- runs the reference's own FP64 CUDA path for one RHS
// evaluation and times its RK4 step.  TEST INFRASTRUCTURE ONLY: it generates
// the golden fixtures that pin the oracle's helium branch
// (tests/golden/make_ref_fixtures.py) and the context timing of the reference
// FP64 GPU step; nothing in the product links, loads or runs it.
//
// Built by oracle/ref_build.sh against the reference's headers where they lie
// (CuSuperHelium/CuSuperHelium/*.cuh), with a stub plotting header of this
// repository (oracle/ref_stub/matplotlibcpp.h) in place of the CPython-embedding
// one the reference includes for debug plots.  BaseBoundaryIntegralCalculator
// (BaseBoundaryIntegrator.cuh) is not compiled: its constructor initialises a
// base class it does not derive from (BaseBoundaryIntegrator.cuh:89), which
// nvcc rejects.  This file therefore restates its runTimeStep composition
// (BaseBoundaryIntegrator.cuh:137-273, calculateVorticities :275-306) over the
// reference's own classes and kernels:
//   ZPhiDerivative::exec -> BoundaryProblem::CreateMMatrix -> complex_to_real ->
//   MatrixSolver::solve -> real_to_complex -> FftDerivative::exec(a) ->
//   CalculateVelocities(lower) -> CalculateVelocities(upper) -> CalculateRhsPhi
//   -> energies and volume flux (CalculateEnergy), as the reference's RHS does.
// The RK4 step is AutonomousRungeKuttaStepper<std_complex,2N>::runStep's
// stage arithmetic (AutonomousRungeKuttaStepper.cuh:123-375): four RHS
// evaluations and cublasZaxpy stage updates.
//
// Usage:
//   ref_harness rhs  <water|helium> <N> <depth> <in.bin> <out.bin>
//       in.bin: x, y, phi (N doubles each); out.bin: vx, vy, dphi, a
//   ref_harness time <water|helium> <N> <depth> <in.bin> <steps> <dt>
//       prints "steps_per_s <value> ms_per_step <value>" (CUDA events)
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

// WaterBoundaryProblem.cuh first: it includes createM.cuh, whose kernels
// HeliumBoundaryProblem.cuh uses without including it.
#include "WaterBoundaryProblem.cuh"
#include "HeliumBoundaryProblem.cuh"
#include "MatrixSolver.cuh"

namespace {

#define HCK(expr)                                                                       \
  do {                                                                                  \
    cudaError_t _e = (expr);                                                            \
    if (_e != cudaSuccess) {                                                            \
      std::fprintf(stderr, "%s failed: %s\n", #expr, cudaGetErrorString(_e));          \
      std::exit(2);                                                                     \
    }                                                                                   \
  } while (0)

// One RHS evaluation of the reference on the complex state [Z | Phi].
template <int N>
struct RefRhs {
  ProblemProperties& props;
  BoundaryProblem<N, 1>& problem;
  VolumeFlux<N> volumeFlux;
  ZPhiDerivative<N, 1> zPhiDerivative;
  FftDerivative<N, 1> fftDerivative;
  MatrixSolver<N, 1> matrixSolver;
  std_complex *devZp, *devZpp, *devPhiPrimeComplex, *devaComplex, *devaprime, *devV1, *devV2, *devVelUpper;
  double *devPhiPrime, *devM, *deva;
  static constexpr int threads = 256, blocks = (N + threads - 1) / threads;

  RefRhs(ProblemProperties& p, BoundaryProblem<N, 1>& bp)
      : props(p), problem(bp), volumeFlux(p), zPhiDerivative(p) {
    HCK(cudaMalloc(&devZp, N * sizeof(std_complex)));
    HCK(cudaMalloc(&devZpp, N * sizeof(std_complex)));
    HCK(cudaMalloc(&devPhiPrimeComplex, N * sizeof(std_complex)));
    HCK(cudaMalloc(&devaComplex, N * sizeof(std_complex)));
    HCK(cudaMalloc(&devaprime, N * sizeof(std_complex)));
    HCK(cudaMalloc(&devV1, (size_t)N * N * sizeof(std_complex)));
    HCK(cudaMalloc(&devV2, N * sizeof(std_complex)));
    HCK(cudaMalloc(&devVelUpper, N * sizeof(std_complex)));
    HCK(cudaMalloc(&devPhiPrime, N * sizeof(double)));
    HCK(cudaMalloc(&devM, (size_t)N * N * sizeof(double)));
    HCK(cudaMalloc(&deva, N * sizeof(double)));
    fftDerivative.initialize();
  }

  void run(const std_complex* state, std_complex* rhs) {
    const std_complex* devZ = state;
    const std_complex* devPhi = state + N;
    std_complex* velLower = rhs;
    std_complex* rhsPhi = rhs + N;
    // calculateVorticities (BaseBoundaryIntegrator.cuh:275-306)
    zPhiDerivative.exec(devZ, devPhi, devZp, devPhiPrimeComplex, devZpp);
    problem.CreateMMatrix(devM, devZ, devZp, devZpp, props);
    complex_to_real<<<blocks, threads>>>(devPhiPrimeComplex, devPhiPrime, N);
    matrixSolver.solve(devM, devPhiPrime, deva);
    // runTimeStep (:137-273)
    real_to_complex<<<blocks, threads>>>(deva, devaComplex, N);
    fftDerivative.exec(devaComplex, devaprime, false, 2.0 * PI_d / N);
    problem.CalculateVelocities(devZ, devZp, devZpp, devaComplex, devaprime, devV1, devV2, velLower, props, true);
    problem.CalculateVelocities(devZ, devZp, devZpp, devaComplex, devaprime, devV1, devV2, devVelUpper, props, false);
    const ProblemPointers pp{devZ, devZp, devZpp, devPhi, devVelUpper, velLower};
    problem.CalculateRhsPhi(pp, rhsPhi, props);
    problem.CalculateEnergy({devZ, devZp, devZpp, devPhi, velLower}, cudaStreamPerThread);
    volumeFlux.CalculateEnergy(devZp, velLower, cudaStreamPerThread);
  }
};

std::vector<double> read_doubles(const char* path, size_t count) {
  std::vector<double> v(count);
  FILE* f = std::fopen(path, "rb");
  if (!f || std::fread(v.data(), sizeof(double), count, f) != count) {
    std::fprintf(stderr, "cannot read %zu doubles from %s\n", count, path);
    std::exit(2);
  }
  std::fclose(f);
  return v;
}

template <int N>
int run_case(int argc, char** argv, bool helium, double depth) {
  const bool timing = std::strcmp(argv[1], "time") == 0;
  ProblemProperties props;
  props.rho = 0.0;  // water: the configurations' rho = 0 (the default 1.0 would make M = I)
  props.depth = depth;
  props.kappa = 0.0;
  props.U = 0.0;
  props.use_expansions = false;
  props.infinite_depth = false;
  WaterBoundaryProblem<N, 1> water(props);
  HeliumBoundaryProblem<N, 1> heliumProblem(props);
  BoundaryProblem<N, 1>& bp = helium ? static_cast<BoundaryProblem<N, 1>&>(heliumProblem)
                                     : static_cast<BoundaryProblem<N, 1>&>(water);
  RefRhs<N> ref(props, bp);
  const std::vector<double> in = read_doubles(argv[5], 3 * (size_t)N);
  std::vector<std_complex> state(2 * N);
  for (int j = 0; j < N; ++j) {
    state[j] = std_complex(in[j], in[N + j]);
    state[N + j] = std_complex(in[2 * N + j], 0.0);
  }
  std_complex *dState, *dRhs;
  HCK(cudaMalloc(&dState, 2 * N * sizeof(std_complex)));
  HCK(cudaMalloc(&dRhs, 2 * N * sizeof(std_complex)));
  HCK(cudaMemcpy(dState, state.data(), 2 * N * sizeof(std_complex), cudaMemcpyHostToDevice));
  if (!timing) {
    ref.run(dState, dRhs);
    HCK(cudaDeviceSynchronize());
    std::vector<std_complex> rhs(2 * N);
    std::vector<double> a(N);
    HCK(cudaMemcpy(rhs.data(), dRhs, 2 * N * sizeof(std_complex), cudaMemcpyDeviceToHost));
    HCK(cudaMemcpy(a.data(), ref.deva, N * sizeof(double), cudaMemcpyDeviceToHost));
    std::vector<double> out(4 * (size_t)N);
    for (int j = 0; j < N; ++j) {
      out[j] = rhs[j].real();
      out[N + j] = rhs[j].imag();
      out[2 * N + j] = rhs[N + j].real();
      out[3 * N + j] = a[j];
    }
    FILE* f = std::fopen(argv[6], "wb");
    if (!f || std::fwrite(out.data(), sizeof(double), out.size(), f) != out.size()) return 2;
    std::fclose(f);
    return 0;
  }
  // RK4 (AutonomousRungeKuttaStepper.cuh:123-375): Y1 = Y0 + h/2 k1, Y2 = Y0 +
  // h/2 k2, Y3 = Y0 + h k3, Y0 += h/6 (k1 + 2 k2 + 2 k3 + k4), with
  // cublasZaxpy as the reference's step().
  const int steps = std::atoi(argv[6]);
  const double dt = std::atof(argv[7]);
  const int n2 = 2 * N;
  std_complex *Y1, *Y2, *Y3, *k1, *k2, *k3, *k4;
  for (std_complex** p : {&Y1, &Y2, &Y3, &k1, &k2, &k3, &k4}) HCK(cudaMalloc(p, n2 * sizeof(std_complex)));
  cublasHandle_t h;
  if (cublasCreate(&h) != CUBLAS_STATUS_SUCCESS) return 2;
  auto axpy = [&](double a, const std_complex* x, std_complex* y) {
    const cuDoubleComplex alpha = make_cuDoubleComplex(a, 0.0);
    cublasZaxpy(h, n2, &alpha, reinterpret_cast<const cuDoubleComplex*>(x), 1, reinterpret_cast<cuDoubleComplex*>(y), 1);
  };
  auto step = [&]() {
    ref.run(dState, k1);
    cudaMemcpy(Y1, dState, n2 * sizeof(std_complex), cudaMemcpyDeviceToDevice);
    axpy(dt / 2, k1, Y1);
    ref.run(Y1, k2);
    cudaMemcpy(Y2, dState, n2 * sizeof(std_complex), cudaMemcpyDeviceToDevice);
    axpy(dt / 2, k2, Y2);
    ref.run(Y2, k3);
    cudaMemcpy(Y3, dState, n2 * sizeof(std_complex), cudaMemcpyDeviceToDevice);
    axpy(dt, k3, Y3);
    ref.run(Y3, k4);
    axpy(dt / 6, k1, dState);
    axpy(dt / 3, k2, dState);
    axpy(dt / 3, k3, dState);
    axpy(dt / 6, k4, dState);
  };
  for (int s = 0; s < 2; ++s) step();  // warm-up (plans, handles, first launches)
  HCK(cudaDeviceSynchronize());
  cudaEvent_t e0, e1;
  HCK(cudaEventCreate(&e0));
  HCK(cudaEventCreate(&e1));
  HCK(cudaEventRecord(e0, 0));
  for (int s = 0; s < steps; ++s) step();
  HCK(cudaEventRecord(e1, 0));
  HCK(cudaDeviceSynchronize());
  float ms = 0.f;
  HCK(cudaEventElapsedTime(&ms, e0, e1));
  std::printf("steps_per_s %.6g ms_per_step %.6g\n", steps / (ms * 1e-3), ms / steps);
  cublasDestroy(h);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 7) {
    std::fprintf(stderr, "usage: ref_harness rhs|time water|helium N depth in.bin out.bin|steps [dt]\n");
    return 1;
  }
  const bool helium = std::strcmp(argv[2], "helium") == 0;
  const int n = std::atoi(argv[3]);
  const double depth = std::atof(argv[4]);
  switch (n) {
    case 128: return run_case<128>(argc, argv, helium, depth);
    case 256: return run_case<256>(argc, argv, helium, depth);
    case 1024: return run_case<1024>(argc, argv, helium, depth);
    case 4096: return run_case<4096>(argc, argv, helium, depth);
    default: std::fprintf(stderr, "N must be 128, 256, 1024 or 4096\n"); return 1;
  }
}
