// sfd.hpp -- C++ facade over libsfd.so with the class names and call shapes
// of the reference's in-process interface (CuSuperHelium/CuSuperHelium):
//
//   AutonomousProblem<T, N>::run / setStream              (AutonomousProblem.h:9-28)
//   BoundaryProblem<N, B>, WaterBoundaryProblem<N, B>,
//   HeliumBoundaryProblem<N, B>                           (BoundaryProblem.cuh:47-62,
//                                                          WaterBoundaryProblem.cuh, HeliumBoundaryProblem.cuh)
//   BaseBoundaryIntegralCalculator<N, B>(properties, problem): run, runTimeStep,
//     calculateVorticities, getDevA / getDevZp / getDevZpp (BaseBoundaryIntegrator.cuh:14-33)
//   AutonomousRungeKuttaStepper<T, N>(problem, dt, logger): setTimeStep, initialize,
//     runStep, runEvolution, getY                         (AutonomousRungeKuttaStepper.cuh:24-44)
//   TrajectoryLogger<T, N>, OdeSolverResult               (TrajectoryLogger.cuh, OdeSolver.h)
//   MatrixSolver<N, B>::solve(M, b, a)                    (MatrixSolver.cuh:24-45)
//   RealBoundaryItegralCalculator<N>, GaussLegendre2<N>    (RealBoundaryIntegralCalculator.cuh,
//                                                          GaussLegendre.cuh:128-214)
//
// State layout is the reference's: device arrays of std_complex (two doubles,
// real then imaginary), [Z (N B) | Phi (N B)], with Phi's imaginary part
// ignored.  Everything runs on the GB300 engine behind the C ABI; errors throw
// std::runtime_error with sfd_last_error().  Header-only, C++17, builds with
// any host compiler (no CUDA code in here).
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdlib>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "sfd.h"

namespace sfd {

using std_complex = std::complex<double>;  // layout of cuda::std::complex<double>

inline void check(int rc) {
  if (rc != 0) throw std::runtime_error(std::string("sfd: ") + sfd_last_error());
}

// ProblemProperties.hpp:5-32 (nondimensional), plus the explicit constants
// the engine takes: A3 (helium; <= 0 selects h^4 / 3) and g (water).
struct ProblemProperties {
  double rho = 0.0;
  double depth = 1.0;
  double kappa = 0.0;
  double U = 0.0;
  bool infinite_depth = false;
  bool use_expansions = false;
  int expansion_order = 1;
  double A3 = 0.0;
  double gravity = 1.0;
};

template <typename T, int N>
class AutonomousProblem {
 public:
  virtual ~AutonomousProblem() = default;
  // rhs = f(initialState); both device pointers of N values of T
  virtual void run(T* initialState, T* rhs) = 0;
  virtual void setStream(cudaStream_t stream) = 0;
};

template <int N, size_t batchSize>
class BoundaryProblem {
 public:
  explicit BoundaryProblem(const ProblemProperties& p) : props(p) {}
  virtual ~BoundaryProblem() = default;
  virtual sfd_problem problem() const = 0;

 protected:
  ProblemProperties props;
};

template <int N, size_t batchSize>
class WaterBoundaryProblem : public BoundaryProblem<N, batchSize> {
 public:
  explicit WaterBoundaryProblem(const ProblemProperties& p) : BoundaryProblem<N, batchSize>(p) {}
  sfd_problem problem() const override {
    sfd_problem q;
    sfd_default_problem(&q);
    q.physics = SFD_WATER;
    q.rho = this->props.rho;
    q.gravity = this->props.gravity;
    q.U = this->props.U;
    return q;
  }
};

template <int N, size_t batchSize>
class HeliumBoundaryProblem : public BoundaryProblem<N, batchSize> {
 public:
  explicit HeliumBoundaryProblem(const ProblemProperties& p) : BoundaryProblem<N, batchSize>(p) {}
  sfd_problem problem() const override {
    sfd_problem q;
    sfd_default_problem(&q);
    q.physics = SFD_HELIUM;
    q.depth = this->props.depth;
    q.A3 = this->props.A3;
    q.kappa = this->props.kappa;
    q.U = this->props.U;
    q.infinite_depth = this->props.infinite_depth ? 1 : 0;
    q.use_expansions = this->props.use_expansions ? 1 : 0;
    q.expansion_order = this->props.expansion_order;
    return q;
  }
};

// One engine holding batchSize surfaces of N nodes.  FP64 by default like the
// reference; pass SFD_PRECISION_MIXED for the GB300 mixed-precision solve.
template <int N, size_t batchSize>
class BaseBoundaryIntegralCalculator : public AutonomousProblem<std_complex, 2 * N * (int)batchSize> {
 public:
  BaseBoundaryIntegralCalculator(const ProblemProperties& /*properties*/, const BoundaryProblem<N, batchSize>& bp,
                                 int precision = SFD_PRECISION_FP64) {
    sfd_options o;
    sfd_default_options(&o);
    o.precision = precision;
    std::vector<int> ns(batchSize, N);
    sfd_problem q = bp.problem();
    check(sfd_create(ns.data(), (int)batchSize, &q, 1, &o, &engine_));
  }
  ~BaseBoundaryIntegralCalculator() override { sfd_destroy(engine_); }
  BaseBoundaryIntegralCalculator(const BaseBoundaryIntegralCalculator&) = delete;
  BaseBoundaryIntegralCalculator& operator=(const BaseBoundaryIntegralCalculator&) = delete;

  void run(std_complex* initialState, std_complex* rhs) override { runTimeStep(initialState, rhs); }
  void runTimeStep(const std_complex* initialState, std_complex* rhs) {
    check(sfd_rhs_device_complex(engine_, initialState, rhs));
  }
  void calculateVorticities(const std_complex* initialState) {
    void *zp = nullptr, *zpp = nullptr;
    check(sfd_vorticities_device(engine_, initialState, &a_, &zp, &zpp));
    zp_ = static_cast<std_complex*>(zp);
    zpp_ = static_cast<std_complex*>(zpp);
  }
  double* getDevA() { return a_; }
  std_complex* getDevZp() { return zp_; }
  std_complex* getDevZpp() { return zpp_; }
  void setStream(cudaStream_t stream) override { check(sfd_set_stream(engine_, stream)); }
  sfd_engine* engine() { return engine_; }

 private:
  sfd_engine* engine_ = nullptr;
  double* a_ = nullptr;
  std_complex *zp_ = nullptr, *zpp_ = nullptr;
};

// Real-state view of a one-surface calculator (RealBoundaryIntegralCalculator.cuh:34-80,
// the reference's class name kept with its spelling): state and rhs are device
// arrays [x (N) | y (N) | phi (N)], which is the engine's own layout, so no
// conversion runs.
template <int N>
class RealBoundaryItegralCalculator : public AutonomousProblem<double, 3 * N> {
 public:
  explicit RealBoundaryItegralCalculator(BaseBoundaryIntegralCalculator<N, 1>& calculator) : calc_(calculator) {}
  void run(double* initialState, double* rhs) override { check(sfd_rhs_device(calc_.engine(), initialState, rhs)); }
  void setStream(cudaStream_t stream) override { calc_.setStream(stream); }

 private:
  BaseBoundaryIntegralCalculator<N, 1>& calc_;
};

// OdeSolver.h:2-5
enum class OdeSolverResult { ReachedEndTime, StiffnessDetected };

// GaussLegendre2Options (GaussLegendre.cuh:83-104), same fields and defaults.
struct GaussLegendre2Options {
  double stepSize = 0.01;
  double newtonTolerance = 1e-10;
  size_t maxNewtonIterations = 20;
  bool allowSimplifiedFallback = false;
  bool returnTrajectory = true;
  double armijo_c = 1e-4;
  double backtrack = 0.5;
  double minAlpha = 1e-6;
  size_t maxStepsHalves = 6;
};

// Implicit two-stage Gauss-Legendre (GaussLegendre.cuh:128-214) on the
// engine of a one-surface FP64 calculator; the stage Jacobians are the
// engine's (finite differences, or exact where reverse mode covers the
// problem), so no JacobianCalculator is passed.  States are [x | y | phi].
template <int N>
class GaussLegendre2 {
 public:
  explicit GaussLegendre2(BaseBoundaryIntegralCalculator<N, 1>& calculator,
                          GaussLegendre2Options options = GaussLegendre2Options())
      : calc_(calculator), opt_(options) {}
  // host (onDevice false) or device state [x | y | phi]
  void initialize(const double* initialState, bool onDevice = false) {
    if (onDevice) {
      const size_t b = 3 * (size_t)N * sizeof(double);
      std::vector<double> h(3 * (size_t)N);
      if (cudaMemcpy(h.data(), initialState, b, cudaMemcpyDeviceToHost) != cudaSuccess)
        throw std::runtime_error("sfd: initialize copy failed");
      set_(h.data());
    } else {
      set_(initialState);
    }
  }
  // throws std::runtime_error when a step fails to converge at every halving
  // (the reference throws as well)
  OdeSolverResult runEvolution(double startTime, double endTime) {
    sfd_gl2_options o;
    sfd_default_gl2_options(&o);
    o.step = opt_.stepSize;
    o.newton_tol = opt_.newtonTolerance;
    o.max_newton = (long long)opt_.maxNewtonIterations;
    o.allow_simplified = opt_.allowSimplifiedFallback ? 1 : 0;
    o.armijo_c = opt_.armijo_c;
    o.backtrack = opt_.backtrack;
    o.min_alpha = opt_.minAlpha;
    o.max_halvings = (long long)opt_.maxStepsHalves;
    if (opt_.returnTrajectory && times_.empty()) {
      times_.push_back(startTime);
      states_.insert(states_.end(), start_.begin(), start_.end());
    }
    sfd_gl2_result r;
    check(sfd_gl2_evolve_cb(calc_.engine(), startTime, endTime, &o, &r, opt_.returnTrajectory ? &record_ : nullptr,
                            this));
    if (r.status != 0)
      throw std::runtime_error("sfd: Gauss-Legendre 2nd Order method failed to converge at t=" + std::to_string(r.t));
    if (r.steps > 0) opt_.stepSize = std::fabs(r.h);  // the last accepted step carries over (GaussLegendre.cuh:318)
    last_.resize(3 * (size_t)N);
    check(sfd_get_state_host(calc_.engine(), last_.data(), last_.data() + N, last_.data() + 2 * N));
    start_ = last_;
    return OdeSolverResult::ReachedEndTime;
  }
  // std::malloc'd copies, released by the caller with std::free
  // (GaussLegendre.cuh:386-436); without returnTrajectory: no times, the last state
  int copyTimesToHost(double** hostTimes, size_t* countHost) const {
    if (!opt_.returnTrajectory) {
      *hostTimes = nullptr;
      *countHost = 0;
      return 0;
    }
    return copy_(times_, hostTimes, countHost, 1);
  }
  int copyStatesToHost(double** hostStates, size_t* countHost) const {
    return copy_(opt_.returnTrajectory ? states_ : last_, hostStates, countHost, 3 * (size_t)N);
  }
  void setStream(cudaStream_t stream) { calc_.setStream(stream); }

 private:
  void set_(const double* y) {
    check(sfd_set_state_host(calc_.engine(), y, y + N, y + 2 * N));
    start_.assign(y, y + 3 * (size_t)N);
    last_ = start_;
  }
  static void record_(void* self, double t, const double* state) {
    auto* g = static_cast<GaussLegendre2*>(self);
    g->times_.push_back(t);
    g->states_.insert(g->states_.end(), state, state + 3 * (size_t)N);
  }
  static int copy_(const std::vector<double>& v, double** out, size_t* count, size_t per) {
    double* p = static_cast<double*>(std::malloc(v.size() * sizeof(double) + 1));
    if (!p) return -1;
    std::copy(v.begin(), v.end(), p);
    *out = p;
    *count = v.size() / per;
    return 0;
  }
  BaseBoundaryIntegralCalculator<N, 1>& calc_;
  GaussLegendre2Options opt_;
  std::vector<double> times_, states_, start_, last_;
};

// Device-side trajectory record (TrajectoryLogger.cuh:8-79): one state of N
// values of T per logged time, appended on the logger's stream into a device
// buffer that doubles when full.  copyTimesToHost / copyStatesToHost return
// std::malloc'd arrays that the caller releases with std::free.
template <typename T, size_t N>
class TrajectoryLogger {
 public:
  TrajectoryLogger() = default;
  virtual ~TrajectoryLogger() { cudaFree(states_); }
  TrajectoryLogger(const TrajectoryLogger&) = delete;
  TrajectoryLogger& operator=(const TrajectoryLogger&) = delete;

  void logTrajectory(double currentTime, const T* devState) {
    if (!enabled_) return;
    if (times_.size() == cap_) grow();
    T* dst = states_ + times_.size() * N;
    if (cudaMemcpyAsync(dst, devState, sizeof(T) * N, cudaMemcpyDeviceToDevice, stream_) != cudaSuccess)
      throw std::runtime_error("sfd: TrajectoryLogger copy failed");
    times_.push_back(currentTime);
  }
  virtual int copyTimesToHost(double** times, size_t* count) {
    if (!enabled_ || !times || !count) return -1;
    double* t = static_cast<double*>(std::malloc(times_.size() * sizeof(double) + 1));
    if (!t) return -1;
    std::copy(times_.begin(), times_.end(), t);
    *times = t;
    *count = times_.size();
    return 0;
  }
  virtual int copyStatesToHost(T** hostStates, size_t* countHost) {
    if (!enabled_ || !hostStates || !countHost) return -1;
    const size_t bytes = times_.size() * N * sizeof(T);
    T* h = static_cast<T*>(std::malloc(bytes + 1));
    if (!h) return -1;
    if (bytes && (cudaMemcpyAsync(h, states_, bytes, cudaMemcpyDeviceToHost, stream_) != cudaSuccess ||
                  cudaStreamSynchronize(stream_) != cudaSuccess)) {
      std::free(h);
      return -1;
    }
    *hostStates = h;
    *countHost = times_.size();
    return 0;
  }
  bool isEnabled() const { return enabled_; }
  void setEnabled(bool on) { enabled_ = on; }
  void setStream(cudaStream_t s) { stream_ = s; }
  size_t size() const { return times_.size(); }

 private:
  void grow() {
    const size_t cap = cap_ ? 2 * cap_ : 64;
    T* p = nullptr;
    if (cudaMalloc(reinterpret_cast<void**>(&p), cap * N * sizeof(T)) != cudaSuccess)
      throw std::runtime_error("sfd: TrajectoryLogger allocation failed");
    if (cap_ && (cudaMemcpyAsync(p, states_, cap_ * N * sizeof(T), cudaMemcpyDeviceToDevice, stream_) != cudaSuccess ||
                 cudaStreamSynchronize(stream_) != cudaSuccess)) {
      cudaFree(p);
      throw std::runtime_error("sfd: TrajectoryLogger copy failed");
    }
    cudaFree(states_);
    states_ = p;
    cap_ = cap;
  }
  std::vector<double> times_;
  T* states_ = nullptr;
  size_t cap_ = 0;
  bool enabled_ = true;
  cudaStream_t stream_ = nullptr;
};

// Classic RK4 (AutonomousRungeKuttaStepper.cuh:123-375) on any
// AutonomousProblem<T, N>; T is double or std_complex.  The stage combines
// run on the device through the C ABI.
template <typename T, int N>
class AutonomousRungeKuttaStepper {
 public:
  // The stepper and the problem share one stream (created here, or the one
  // passed to setStream), so stage combines and RHS evaluations stay ordered.
  AutonomousRungeKuttaStepper(AutonomousProblem<T, N>& problem, double tstep = 1e-2,
                              std::shared_ptr<TrajectoryLogger<T, N>> logger = nullptr)
      : problem_(problem), dt_(tstep), logger_(std::move(logger)) {
    const size_t bytes = sizeof(T) * (size_t)N;
    for (double** p : {&own_y_, &ys_, &k_, &kacc_}) {
      if (cudaMalloc(reinterpret_cast<void**>(p), bytes) != cudaSuccess) {
        release();
        throw std::runtime_error("sfd: cudaMalloc failed in AutonomousRungeKuttaStepper");
      }
    }
    if (cudaStreamCreateWithFlags(&own_stream_, cudaStreamNonBlocking) != cudaSuccess) {
      release();
      throw std::runtime_error("sfd: cudaStreamCreate failed in AutonomousRungeKuttaStepper");
    }
    stream_ = own_stream_;
    problem_.setStream(stream_);
    if (logger_) logger_->setStream(stream_);
    y_ = own_y_;
  }
  ~AutonomousRungeKuttaStepper() { release(); }
  AutonomousRungeKuttaStepper(const AutonomousRungeKuttaStepper&) = delete;
  AutonomousRungeKuttaStepper& operator=(const AutonomousRungeKuttaStepper&) = delete;

  void setTimeStep(double tstep) { dt_ = tstep; }
  void setStream(cudaStream_t s) {
    stream_ = s;
    problem_.setStream(s);
    if (logger_) logger_->setStream(s);
  }
  // onDevice: adopt the caller's device array and advance it in place
  // (AutonomousRungeKuttaStepper.cuh:312-318); otherwise copy the host state
  // into the stepper's own array.
  void initialize(T* y0, bool onDevice = false) {
    if (onDevice) {
      y_ = reinterpret_cast<double*>(y0);
      return;
    }
    y_ = own_y_;
    if (cudaMemcpyAsync(y_, y0, sizeof(T) * (size_t)N, cudaMemcpyHostToDevice, stream_) != cudaSuccess)
      throw std::runtime_error("sfd: initialize copy failed");
  }
  void runStep(int /*step*/ = 0) {
    const long long n = (long long)(sizeof(T) / sizeof(double)) * N;
    const double wk[4] = {1.0, 2.0, 2.0, 1.0};
    const double cy[4] = {0.5 * dt_, 0.5 * dt_, dt_, 0.0};
    for (int s = 0; s < 4; ++s) {
      problem_.run(reinterpret_cast<T*>(s == 0 ? y_ : ys_), reinterpret_cast<T*>(k_));
      check(sfd_rk4_stage_device(n, y_, k_, kacc_, s < 3 ? ys_ : nullptr, wk[s], cy[s], s == 0, stream_));
    }
    check(sfd_rk4_final_device(n, y_, kacc_, dt_ / 6.0, stream_));
    time_ += dt_;
  }
  // floor((endTime - startTime) / dt) steps, logging the state after each
  // one when a logger is attached (AutonomousRungeKuttaStepper.cuh:417-437).
  // Returns ReachedEndTime once all steps ran.
  OdeSolverResult runEvolution(double startTime, double endTime) {
    time_ = startTime;
    const long long steps = (long long)((endTime - startTime) / dt_);
    for (long long i = 0; i < steps; ++i) {
      runStep((int)i);
      if (logger_) logger_->logTrajectory(time_, reinterpret_cast<const T*>(y_));
    }
    if (cudaStreamSynchronize(stream_) != cudaSuccess) throw std::runtime_error("sfd: runEvolution failed");
    return OdeSolverResult::ReachedEndTime;
  }
  T* getY() { return reinterpret_cast<T*>(y_); }
  double getCurrentTime() const { return time_; }

 private:
  void release() {
    if (stream_) cudaStreamSynchronize(stream_);
    for (double* p : {own_y_, ys_, k_, kacc_}) cudaFree(p);
    y_ = own_y_ = ys_ = k_ = kacc_ = nullptr;
    if (own_stream_) {
      // the problem and the logger outlive the stepper: hand them back their
      // default streams before the stepper's stream goes away
      if (stream_ == own_stream_) {
        try {
          problem_.setStream(nullptr);
        } catch (...) {
        }
        if (logger_) logger_->setStream(nullptr);
      }
      cudaStreamDestroy(own_stream_);
    }
    own_stream_ = nullptr;
  }
  AutonomousProblem<T, N>& problem_;
  double dt_;
  double time_ = 0.0;
  cudaStream_t stream_ = nullptr;
  cudaStream_t own_stream_ = nullptr;
  std::shared_ptr<TrajectoryLogger<T, N>> logger_;
  double* y_ = nullptr;  // the state advanced in place: own_y_ or an adopted caller array
  double *own_y_ = nullptr, *ys_ = nullptr, *k_ = nullptr, *kacc_ = nullptr;
};

// Batched dense FP64 solve of column-major N x N systems (MatrixSolver.cuh).
template <int N, size_t batchSize>
class MatrixSolver {
 public:
  MatrixSolver() { check(sfd_dense_solver_create(N, (int)batchSize, &d_)); }
  ~MatrixSolver() { sfd_dense_solver_destroy(d_); }
  MatrixSolver(const MatrixSolver&) = delete;
  MatrixSolver& operator=(const MatrixSolver&) = delete;
  // devM: batchSize column-major N x N matrices; devb, deva: batchSize x N
  void solve(double* devM, double* devb, double* deva) { check(sfd_dense_solve(d_, devM, devb, deva, nullptr)); }
  // as solve, returning the per-system status words (SFD_STATUS_*)
  std::vector<unsigned int> solveChecked(double* devM, double* devb, double* deva) {
    std::vector<unsigned int> st(batchSize);
    check(sfd_dense_solve(d_, devM, devb, deva, st.data()));
    return st;
  }
  void setStream(cudaStream_t stream) { check(sfd_dense_solver_set_stream(d_, stream)); }

 private:
  sfd_dense_solver* d_ = nullptr;
};

}  // namespace sfd
