// Drives the C++ facade (include/sfd.hpp) the way the reference's C++ apps
// drive their classes, and checks it against the engine's own C ABI:
//   BaseBoundaryIntegralCalculator::run  vs sfd_rhs_host (same state, SoA)
//   calculateVorticities / getDevA        vs the vortex strength of sfd_rhs_host
//   AutonomousRungeKuttaStepper, 10 steps vs sfd_rk4_steps; its TrajectoryLogger
//     record and initialize(devptr, true) in place vs the same steps
//   MatrixSolver<64, 3>                   vs Gaussian elimination on the host
//   RealBoundaryItegralCalculator and RK4 on it vs sfd_rhs_host / sfd_rk4_steps
//   GaussLegendre2                         vs sfd_gl2_evolve
//   the generic stepper on 256 rotations     vs the exact solution (10^4 steps of 1e-3)
// Prints the differences and exits 0 when all are within tolerance.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <random>
#include <vector>

#include "sfd.hpp"

using sfd::std_complex;

static double maxrel(const std::vector<double>& a, const std::vector<double>& b) {
  double d = 0, m = 0;
  for (size_t i = 0; i < a.size(); ++i) {
    d = std::fmax(d, std::fabs(a[i] - b[i]));
    m = std::fmax(m, std::fabs(b[i]));
  }
  return d / (m > 0 ? m : 1.0);
}

static void stage(const char* what) { std::fprintf(stderr, "facade_check: %s\n", what); }

int main() {
  constexpr int N = 128;
  const double PI = 3.14159265358979323846;
  sfd::ProblemProperties props;
  sfd::WaterBoundaryProblem<N, 1> water(props);
  sfd::BaseBoundaryIntegralCalculator<N, 1> calc(props, water);

  std::vector<std_complex> h(2 * N);
  std::vector<double> x(N), y(N), phi(N);
  for (int j = 0; j < N; ++j) {
    const double xi = 2 * PI * j / N;
    x[j] = xi;
    y[j] = 0.05 * std::cos(xi) + 0.01 * std::sin(3 * xi);
    phi[j] = 0.05 * std::sin(xi);
    h[j] = {x[j], y[j]};
    h[N + j] = {phi[j], 0.0};
  }
  std_complex *dS = nullptr, *dR = nullptr;
  cudaMalloc(&dS, sizeof(std_complex) * 2 * N);
  cudaMalloc(&dR, sizeof(std_complex) * 2 * N);
  cudaMemcpy(dS, h.data(), sizeof(std_complex) * 2 * N, cudaMemcpyHostToDevice);

  // reference values through the plain C ABI
  sfd_problem p;
  sfd_default_problem(&p);
  sfd_options o;
  sfd_default_options(&o);
  o.precision = SFD_PRECISION_FP64;
  int n = N;
  sfd_engine* e = nullptr;
  sfd::check(sfd_create(&n, 1, &p, 1, &o, &e));
  sfd::check(sfd_set_state_host(e, x.data(), y.data(), phi.data()));
  std::vector<double> dx(N), dy(N), dp(N), a(N);
  sfd::check(sfd_rhs_host(e, dx.data(), dy.data(), dp.data(), a.data(), nullptr, nullptr));

  // 1. run
  stage("run");
  calc.run(dS, dR);
  sfd::check(sfd_synchronize(calc.engine()));
  std::vector<std_complex> r(2 * N);
  cudaMemcpy(r.data(), dR, sizeof(std_complex) * 2 * N, cudaMemcpyDeviceToHost);
  std::vector<double> fr(3 * N), er(3 * N);
  for (int j = 0; j < N; ++j) {
    fr[j] = r[j].real(); fr[N + j] = r[j].imag(); fr[2 * N + j] = r[N + j].real();
    er[j] = dx[j]; er[N + j] = dy[j]; er[2 * N + j] = dp[j];
  }
  const double e_run = maxrel(fr, er);

  // 2. vorticities
  stage("vorticities");
  calc.calculateVorticities(dS);
  sfd::check(sfd_synchronize(calc.engine()));
  std::vector<double> fa(N);
  cudaMemcpy(fa.data(), calc.getDevA(), sizeof(double) * N, cudaMemcpyDeviceToHost);
  const double e_a = maxrel(fa, a);

  // 3. stepper
  stage("stepper");
  const double dt = 0.01;
  auto logger = std::make_shared<sfd::TrajectoryLogger<std_complex, 2 * N>>();
  std::vector<std_complex> ys(2 * N), ylast(2 * N), yadopt(2 * N);
  double* times = nullptr;
  std_complex* states = nullptr;
  size_t nt = 0, ns = 0;
  {
    sfd::AutonomousRungeKuttaStepper<std_complex, 2 * N> stepper(calc, dt, logger);
    stepper.initialize(h.data(), false);
    if (stepper.runEvolution(0.0, 10 * dt + 0.5 * dt) != sfd::OdeSolverResult::ReachedEndTime) return 2;
    cudaMemcpy(ys.data(), stepper.getY(), sizeof(std_complex) * 2 * N, cudaMemcpyDeviceToHost);
  }
  if (logger->copyTimesToHost(&times, &nt) || logger->copyStatesToHost(&states, &ns)) return 3;
  // the engine autotunes its boundary-sum split on first use, which may change
  // the summation order between the two runs: round-off level differences
  double e_log = (nt == 10 && ns == 10) ? 0.0 : 1.0;
  double tt = 0.0;  // the stepper accumulates its time step by step
  for (size_t i = 0; i < nt; ++i) {
    tt += dt;
    e_log = std::fmax(e_log, std::fabs(times[i] - tt));
  }
  if (ns == 10)
    for (int j = 0; j < 2 * N; ++j) e_log = std::fmax(e_log, std::abs(states[9 * 2 * N + j] - ys[j]));
  std::free(times);
  std::free(states);
  {  // initialize(devptr, true) advances the caller's array in place
    std_complex* dY = nullptr;
    cudaMalloc(&dY, sizeof(std_complex) * 2 * N);
    cudaMemcpy(dY, h.data(), sizeof(std_complex) * 2 * N, cudaMemcpyHostToDevice);
    sfd::AutonomousRungeKuttaStepper<std_complex, 2 * N> stepper(calc, dt);
    stepper.initialize(dY, true);
    for (int i = 0; i < 10; ++i) stepper.runStep(i);
    cudaDeviceSynchronize();
    if (stepper.getY() != dY) return 4;
    cudaMemcpy(yadopt.data(), dY, sizeof(std_complex) * 2 * N, cudaMemcpyDeviceToHost);
    cudaFree(dY);
  }
  for (int j = 0; j < 2 * N; ++j) e_log = std::fmax(e_log, std::abs(yadopt[j] - ys[j]));
  sfd::check(sfd_rk4_steps(e, dt, 10));
  std::vector<double> ex(N), ey(N), ep(N);
  sfd::check(sfd_get_state_host(e, ex.data(), ey.data(), ep.data()));
  std::vector<double> fs(3 * N), es(3 * N);
  for (int j = 0; j < N; ++j) {
    fs[j] = ys[j].real(); fs[N + j] = ys[j].imag(); fs[2 * N + j] = ys[N + j].real();
    es[j] = ex[j]; es[N + j] = ey[j]; es[2 * N + j] = ep[j];
  }
  const double e_step = maxrel(fs, es);

  stage("dense solver");
  // 4. dense solver on column-major, diagonally dominant systems
  constexpr int M = 64, B = 3;
  std::mt19937_64 rng(5);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  std::vector<double> Ah((size_t)B * M * M), bh((size_t)B * M), xh((size_t)B * M);
  for (int s = 0; s < B; ++s)
    for (int c = 0; c < M; ++c)
      for (int rr = 0; rr < M; ++rr) Ah[(size_t)s * M * M + (size_t)c * M + rr] = U(rng) / M + (rr == c ? 2.0 : 0.0);
  for (auto& v : bh) v = U(rng);
  double *dA = nullptr, *db = nullptr, *dxs = nullptr;
  cudaMalloc(&dA, sizeof(double) * Ah.size());
  cudaMalloc(&db, sizeof(double) * bh.size());
  cudaMalloc(&dxs, sizeof(double) * bh.size());
  cudaMemcpy(dA, Ah.data(), sizeof(double) * Ah.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(db, bh.data(), sizeof(double) * bh.size(), cudaMemcpyHostToDevice);
  sfd::MatrixSolver<M, B> solver;
  std::vector<unsigned int> st = solver.solveChecked(dA, db, dxs);
  cudaDeviceSynchronize();
  cudaMemcpy(xh.data(), dxs, sizeof(double) * xh.size(), cudaMemcpyDeviceToHost);
  double e_solve = 0;
  for (int s = 0; s < B; ++s) {  // host Gaussian elimination with partial pivoting
    std::vector<double> Ar((size_t)M * M), br(bh.begin() + (size_t)s * M, bh.begin() + (size_t)(s + 1) * M);
    for (int rr = 0; rr < M; ++rr)
      for (int c = 0; c < M; ++c) Ar[(size_t)rr * M + c] = Ah[(size_t)s * M * M + (size_t)c * M + rr];
    for (int k = 0; k < M; ++k) {
      int piv = k;
      for (int rr = k + 1; rr < M; ++rr)
        if (std::fabs(Ar[(size_t)rr * M + k]) > std::fabs(Ar[(size_t)piv * M + k])) piv = rr;
      for (int c = 0; c < M; ++c) std::swap(Ar[(size_t)k * M + c], Ar[(size_t)piv * M + c]);
      std::swap(br[k], br[piv]);
      for (int rr = k + 1; rr < M; ++rr) {
        const double l = Ar[(size_t)rr * M + k] / Ar[(size_t)k * M + k];
        for (int c = k; c < M; ++c) Ar[(size_t)rr * M + c] -= l * Ar[(size_t)k * M + c];
        br[rr] -= l * br[k];
      }
    }
    for (int k = M - 1; k >= 0; --k) {
      double v = br[k];
      for (int c = k + 1; c < M; ++c) v -= Ar[(size_t)k * M + c] * br[c];
      br[k] = v / Ar[(size_t)k * M + k];
    }
    std::vector<double> got(xh.begin() + (size_t)s * M, xh.begin() + (size_t)(s + 1) * M);
    e_solve = std::fmax(e_solve, maxrel(got, br));
  }
  unsigned int st_or = 0;
  for (unsigned int v : st) st_or |= v;

  // 5. real-state calculator, RK4 on it, and GL2, each against the engine's own entry points
  stage("real state, GL2");
  constexpr int M2 = 32;
  std::vector<double> s2(3 * M2);
  for (int j = 0; j < M2; ++j) {
    const double xi = 2 * PI * j / M2;
    s2[j] = xi;
    s2[M2 + j] = 0.05 * std::cos(xi);
    s2[2 * M2 + j] = 0.015 * std::sin(xi);
  }
  sfd::WaterBoundaryProblem<M2, 1> water2(props);
  sfd::BaseBoundaryIntegralCalculator<M2, 1> calc2(props, water2);
  sfd::RealBoundaryItegralCalculator<M2> real2(calc2);
  double *dS2 = nullptr, *dR2 = nullptr;
  cudaMalloc(&dS2, sizeof(double) * 3 * M2);
  cudaMalloc(&dR2, sizeof(double) * 3 * M2);
  cudaMemcpy(dS2, s2.data(), sizeof(double) * 3 * M2, cudaMemcpyHostToDevice);
  real2.run(dS2, dR2);
  sfd::check(sfd_synchronize(calc2.engine()));
  std::vector<double> r2(3 * M2), er2(3 * M2);
  cudaMemcpy(r2.data(), dR2, sizeof(double) * 3 * M2, cudaMemcpyDeviceToHost);
  int m2 = M2;
  sfd_engine* e2 = nullptr;
  sfd::check(sfd_create(&m2, 1, &p, 1, &o, &e2));
  sfd::check(sfd_set_state_host(e2, s2.data(), s2.data() + M2, s2.data() + 2 * M2));
  sfd::check(sfd_rhs_host(e2, er2.data(), er2.data() + M2, er2.data() + 2 * M2, nullptr, nullptr, nullptr));
  double e_real = maxrel(r2, er2);
  std::vector<double> y2(3 * M2), ey2(3 * M2);
  {
    sfd::AutonomousRungeKuttaStepper<double, 3 * M2> rk(real2, dt);
    rk.initialize(s2.data(), false);
    rk.runEvolution(0.0, 5 * dt + 0.5 * dt);
    cudaMemcpy(y2.data(), rk.getY(), sizeof(double) * 3 * M2, cudaMemcpyDeviceToHost);
  }
  sfd::check(sfd_set_state_host(e2, s2.data(), s2.data() + M2, s2.data() + 2 * M2));
  sfd::check(sfd_rk4_steps(e2, dt, 5));
  sfd::check(sfd_get_state_host(e2, ey2.data(), ey2.data() + M2, ey2.data() + 2 * M2));
  e_real = std::fmax(e_real, maxrel(y2, ey2));
  // GL2 through the facade and through the C entry point
  sfd::GaussLegendre2Options gopt;
  gopt.stepSize = 0.01;
  sfd::GaussLegendre2<M2> gl(calc2, gopt);
  gl.initialize(s2.data(), false);
  if (gl.runEvolution(0.0, 0.03) != sfd::OdeSolverResult::ReachedEndTime) return 5;
  double* gtimes = nullptr;
  double* gstates = nullptr;
  size_t gnt = 0, gns = 0;
  if (gl.copyTimesToHost(&gtimes, &gnt) || gl.copyStatesToHost(&gstates, &gns)) return 6;
  sfd::check(sfd_set_state_host(e2, s2.data(), s2.data() + M2, s2.data() + 2 * M2));
  sfd_gl2_options go;
  sfd_default_gl2_options(&go);
  go.step = 0.01;
  go.max_newton = 20;
  go.allow_simplified = 0;
  sfd_gl2_result gr;
  std::vector<double> ctimes(64);
  sfd::check(sfd_gl2_evolve(e2, 0.0, 0.03, &go, &gr, ctimes.data(), nullptr, 64));
  std::vector<double> gfin(3 * M2);
  sfd::check(sfd_get_state_host(e2, gfin.data(), gfin.data() + M2, gfin.data() + 2 * M2));
  double e_gl2 = (gnt == (size_t)gr.steps + 1 && gns == gnt && gtimes[0] == 0.0) ? 0.0 : 1.0;
  for (long long i = 0; i < gr.steps && e_gl2 == 0.0; ++i) e_gl2 = std::fabs(gtimes[i + 1] - ctimes[(size_t)i]);
  if (gns == gnt) {
    std::vector<double> last(gstates + (gns - 1) * 3 * M2, gstates + gns * 3 * M2);
    e_gl2 = std::fmax(e_gl2, maxrel(last, gfin));
  }
  std::free(gtimes);
  std::free(gstates);
  sfd_destroy(e2);
  cudaFree(dS2);
  cudaFree(dR2);

  // 6. the generic stepper on a user-defined problem: M rotations dx/dt = -y,
  //    dy/dt = x (ODE_Solvers.RK4, ODESolverTests.cuh:73-246), against cos / sin
  stage("rotation");
  double e_rot = 0.0;
  {
    constexpr int MR = 256;
    struct Rotation : sfd::AutonomousProblem<double, 2 * MR> {
      double *zeros = nullptr, *scratch = nullptr;
      cudaStream_t st = nullptr;
      Rotation() {
        cudaMalloc(&zeros, sizeof(double) * MR);
        cudaMalloc(&scratch, sizeof(double) * MR);
        cudaMemset(zeros, 0, sizeof(double) * MR);
      }
      ~Rotation() override {
        cudaFree(zeros);
        cudaFree(scratch);
      }
      // rhs = [-y | x]: -y as the stage combine 0 + (-1) y, x as a copy
      void run(double* state, double* rhs) override {
        sfd::check(sfd_rk4_stage_device(MR, zeros, state + MR, scratch, rhs, 1.0, -1.0, 1, st));
        cudaMemcpyAsync(rhs + MR, state, sizeof(double) * MR, cudaMemcpyDeviceToDevice, st);
      }
      void setStream(cudaStream_t s) override { st = s; }
    } rot;
    std::vector<double> r0(2 * MR), rT(2 * MR);
    for (int i = 0; i < MR; ++i) {
      const double th = 2 * PI * i / MR;
      r0[i] = std::cos(th);
      r0[MR + i] = std::sin(th);
    }
    const double h = 1e-3;
    const long long nsteps = 10000;
    sfd::AutonomousRungeKuttaStepper<double, 2 * MR> rk(rot, h);
    rk.initialize(r0.data(), false);
    rk.runEvolution(0.0, nsteps * h + 0.5 * h);
    cudaMemcpy(rT.data(), rk.getY(), sizeof(double) * 2 * MR, cudaMemcpyDeviceToHost);
    const double T = rk.getCurrentTime();
    for (int i = 0; i < MR; ++i) {
      const double th = 2 * PI * i / MR;
      e_rot = std::fmax(e_rot, std::fabs(rT[i] - std::cos(th + T)));
      e_rot = std::fmax(e_rot, std::fabs(rT[MR + i] - std::sin(th + T)));
    }
  }

  std::printf("run %.3e vorticity %.3e stepper %.3e logger/in-place %.3e solve %.3e real %.3e gl2 %.3e rotation %.3e "
              "status %u\n",
              e_run, e_a, e_step, e_log, e_solve, e_real, e_gl2, e_rot, st_or);
  std::fflush(stdout);
  sfd_destroy(e);
  for (void* p : {(void*)dS, (void*)dR, (void*)dA, (void*)db, (void*)dxs}) cudaFree(p);
  const bool ok = e_run < 1e-13 && e_a < 1e-13 && e_step < 1e-13 && e_log < 1e-14 && e_solve < 1e-12 &&
                  e_real < 1e-13 && e_gl2 < 1e-12 && e_rot < 1e-9 && st_or == 0;
  return ok ? 0 : 1;
}
