/*
 * sfd.h -- C ABI of the GB300 boundary-integral engine (libsfd.so).
 *
 * Drop-in replacement for the CuSuperHelium Roberts-1983 boundary-integral
 * right-hand side and its RK4 time step.  Plain C types only: host pointers,
 * device pointers (as void*), sizes.  All functions return 0 on success and a
 * negative SFD_ERR_* code on failure; sfd_last_error() gives the message of the
 * calling thread's last failure.  Nothing here exits the process.
 *
 * Two groups of entry points:
 *  1. Reference-compatible exports: the exact signatures the reference's
 *     ctypes layer binds (CuSuperHelium/Python/integration/rhs.py:93-350),
 *     with the reference's SI-unit handling (adimensionalizeProperties,
 *     CuSuperHelium/CuSuperHelium/Export.cu:1222-1246) and finite-depth helium
 *     physics.  Each declaration cites the reference export it replaces.
 *  2. Engine API (sfd_*): a persistent handle that owns device buffers, so a
 *     time loop pays set-up once; nondimensional units; water or helium per
 *     surface; uneven-N batches; FP64 or mixed precision.
 */
#ifndef SFD_H
#define SFD_H

#include <stddef.h>

#ifdef __cplusplus
#define SFD_BOOL bool
extern "C" {
#else
#define SFD_BOOL _Bool
#endif

/* ------------------------------------------------------------ error codes */
#define SFD_OK 0
#define SFD_ERR_INVALID (-1)     /* bad argument (null pointer, unsupported size, ...) */
#define SFD_ERR_CUDA (-2)        /* a CUDA runtime call failed                          */
#define SFD_ERR_NUMERICS (-3)    /* non-finite values or solver breakdown (see status)  */
#define SFD_ERR_NO_DEVICE (-4)   /* no usable CUDA device                               */

/* ------------------------------------------------------------ physics */
#define SFD_WATER 0              /* WaterBoundaryProblem  (createMKernel path)          */
#define SFD_HELIUM 1             /* HeliumBoundaryProblem (createFiniteDepthMKernel)    */

#define SFD_PRECISION_FP64 0     /* every stage in FP64 (LU without exchanges, FP64
                                    refinement where its residual is above refine_tol)  */
#define SFD_PRECISION_MIXED 1    /* FP32 preconditioner + double-float/FP64 refinement  */

/* per-surface status bits (sfd_get_status) */
#define SFD_STATUS_NONFINITE 0x1u
#define SFD_STATUS_PIVOT_SWAP 0x2u      /* engine: an FP64 factorisation had |l_ij| > 1, so partial
                                           pivoting would have exchanged rows (the residual check
                                           and FP64 refinement then carry the accuracy); dense
                                           solver: rows were exchanged */
#define SFD_STATUS_ZERO_PIVOT 0x4u
#define SFD_STATUS_REFINE_STALL 0x8u    /* the solve's final residual stayed above refine_tol */
#define SFD_STATUS_TIMEOUT 0x20u        /* a bounded in-kernel wait ran out; that work was skipped */

/* Nondimensional physics of one surface; mirrors the fields of
 * ProblemProperties (CuSuperHelium/CuSuperHelium/ProblemProperties.hpp:5-32)
 * that the hot path reads, plus explicit A3 and g. */
typedef struct sfd_problem {
    int physics;          /* SFD_WATER or SFD_HELIUM                                     */
    int infinite_depth;   /* helium: drop the image terms (ProblemProperties.infinite_depth) */
    double rho;           /* water density ratio (the configs use 0)                     */
    double depth;         /* helium film thickness h                                     */
    double A3;            /* helium van der Waals constant; <= 0 selects the reference's h^4/3 */
    double gravity;       /* water g; <= 0 selects 1                                     */
    double U;             /* uniform stream (linear part of phi only; the configs use 0) */
    double kappa;         /* surface tension (helium Bernoulli variant; 0 = off)         */
    int use_expansions;   /* helium Bernoulli as a series in y (createM.cuh:171-193)      */
    int expansion_order;  /* 1..3                                                        */
} sfd_problem;

typedef struct sfd_options {
    int precision;        /* SFD_PRECISION_FP64 or SFD_PRECISION_MIXED                   */
    int refine_iters;     /* mixed: FP32 corrections after the accurate pass (default 2) */
    int refactor_every;   /* mixed: rebuild the preconditioner every k RK4 steps (1)     */
    int use_graphs;       /* capture one RK4 step in a CUDA graph (1)                    */
    int device;           /* CUDA device ordinal (0)                                     */
    int tensor_cores;     /* mixed: preconditioner update on tcgen05 tensor cores (1)    */
    int pre_iters;        /* mixed: FP32 full-residual iterations before it (default 1)  */
    int precond_half;     /* mixed: apply the preconditioner from an FP16 copy (1)       */
    int autotune;         /* time the boundary-sum CTA shapes on the first steps and keep
                             the fastest per precision (1)                               */
    int refactor_lag;     /* mixed, sfd_rk4_steps: 0 rebuilds the preconditioner inside the
                             step it is due (default); k > 0 rebuilds it on a low-priority
                             side stream from the state at that step and switches to it k
                             steps later (k < refactor_every), so the rebuild overlaps the
                             stepping.  Deterministic: the switch step is fixed.          */
    int extra_iters;      /* 0..4 (default 2): extra corrections of the solve, each run only
                             for surfaces whose residual after the regular passes (or the
                             previous extra one) is above refine_tol * max |phi'|; FP64 mode
                             corrects with the LU factors and FP64 sums, mixed mode with the
                             preconditioner and FP32 sums.  A final residual still above the
                             tolerance raises SFD_STATUS_REFINE_STALL; in mixed mode the next
                             step enqueued after the host sees it rebuilds the preconditioner */
    double refine_tol;    /* relative residual tolerance max |phi' - M a| / max |phi'| of
                             the solve (default 1e-10); <= 0 turns the check off          */
} sfd_options;

/* Optomechanical drive of a helium film, nondimensional (the reference's
 * OptomechanicalVariables after adimensionalizeOptomechanicalVariables,
 * Export.cu:1248-1270).  Per node, with the intensity
 *   I(y, x) = gamma^2 max_intensity / 4 / ((detuning - G y)^2 + (gamma/2)^2)
 *             * exp(-(x - x0)^2 / (2 sigma^2))      (LightIntensity.cuh:25-31)
 * the helium Bernoulli gains damping * v + strength * I
 * (HeliumDrivenAutonomousProblem.cuh:20-26, createM.cuh:141-158), and with
 * augmented != 0 the state carries the delayed intensity D as a fourth block:
 * dphi += D, dD/dt = beta I - D / tau (DelayedIntensityIntegrator.cuh:22-36). */
typedef struct sfd_drive {
    double detuning, gamma, G, tau, max_intensity, x0, sigma, beta, damping;
    double strength;      /* prefactor of I in dphi/dt (LightIntensity.cuh:34-37)     */
    int augmented;        /* 1: state [x | y | phi | D], RHS [dx | dy | dphi | dD]    */
} sfd_drive;

typedef struct sfd_engine sfd_engine;

/* ------------------------------------------------------------ engine API */
void sfd_default_options(sfd_options* opts);
void sfd_default_problem(sfd_problem* prob);   /* water, rho = 0, g = 1 */

/* Create an engine for `nsurf` surfaces with n[s] nodes each (1 <= n <= 8192).
 * `problems` holds one entry per surface (or one entry for all when
 * `shared_problem` != 0).  Replaces the constructor chain
 * BoundaryProblem -> BaseBoundaryIntegralCalculator<N,batch> ->
 * AutonomousRungeKuttaStepper<std_complex,2N>
 * (BaseBoundaryIntegrator.cuh:88-108, AutonomousRungeKuttaStepper.cuh:91-105). */
int sfd_create(const int* n, int nsurf, const sfd_problem* problems, int shared_problem,
               const sfd_options* opts, sfd_engine** out);
/* As sfd_create, with an optomechanical drive per surface (`drives` follows
 * `shared_problem` like `problems`; NULL = no drive).  Drives need helium
 * surfaces with the standard Bernoulli closure.  If any drive is augmented
 * the engine state gains the delayed-intensity block D (zero for undriven
 * surfaces), set and read with sfd_set_aux_host / sfd_get_aux_host. */
int sfd_create_driven(const int* n, int nsurf, const sfd_problem* problems, const sfd_drive* drives,
                      int shared_problem, const sfd_options* opts, sfd_engine** out);
int sfd_destroy(sfd_engine* e);
/* Use a caller stream (0 = the engine's own). */
int sfd_set_stream(sfd_engine* e, void* cuda_stream);
/* Source groups per CTA of the boundary sums chosen by the autotuner (or the
 * default 4), for the FP64, double-float and FP32 passes. */
int sfd_get_tuning(const sfd_engine* e, int* groups_f64_df_f32);
/* Replace the physical parameters of one surface (A3, g, depth, ...) on an
 * existing engine; physics, the depth mode and whether rho is zero must stay.
 * (The reference fixes these in the BoundaryProblem constructor,
 * BoundaryProblem.cuh:47-62; this setter serves parameter fits.) */
int sfd_set_problem(sfd_engine* e, int surface, const sfd_problem* problem);
int sfd_total_nodes(const sfd_engine* e);

/* State = concatenated per-surface nodes, SoA: x[ntot], y[ntot], phi[ntot]. */
int sfd_set_state_host(sfd_engine* e, const double* x, const double* y, const double* phi);
int sfd_get_state_host(sfd_engine* e, double* x, double* y, double* phi);
/* Delayed-intensity block D[ntot] of an augmented engine. */
int sfd_set_aux_host(sfd_engine* e, const double* D);
int sfd_get_aux_host(sfd_engine* e, double* D);
/* Same with device pointers (each ntot doubles). */
int sfd_set_state_device(sfd_engine* e, const void* x, const void* y, const void* phi);
int sfd_get_state_device(sfd_engine* e, void* x, void* y, void* phi);
/* Device address of the engine's resident state [x | y | phi] (3 * ntot doubles). */
int sfd_state_device_ptr(sfd_engine* e, void** state);

/* One RHS evaluation of the current state (BaseBoundaryIntegralCalculator::run,
 * BaseBoundaryIntegrator.cuh:137-314): dx, dy = lower-fluid velocity
 * (dz/dt), dphi = Bernoulli right-hand side.  Optional diagnostics (nullable):
 * a = vortex strength, zp / zpp = interleaved complex z', z'' (per index). */
int sfd_rhs_host(sfd_engine* e, double* dx, double* dy, double* dphi, double* a, double* zp, double* zpp);
/* Same on device pointers: state_in and rhs_out are [x|y|phi] / [dx|dy|dphi]. */
int sfd_rhs_device(sfd_engine* e, const void* state_in, void* rhs_out);

/* `steps` classic RK4 steps of size dt on the resident state
 * (AutonomousRungeKuttaStepper<std_complex,2N>::runStep, :123-307). */
int sfd_rk4_steps(sfd_engine* e, double dt, int steps);
/* Host-buffer stepping in one call: copy the state [x | y | phi] (ntot each)
 * in, run `steps` RK4 steps, copy it back out into the same arrays, with one
 * synchronisation.  Pinned host arrays make the copies asynchronous; arrays
 * that are consecutive parts of one buffer (y = x + ntot, phi = y + ntot)
 * move in one copy each way. */
int sfd_rk4_steps_host(sfd_engine* e, double* x, double* y, double* phi, double dt, int steps);
/* Enqueue without waiting for completion (timed loops). */
int sfd_rk4_steps_async(sfd_engine* e, double dt, int steps);
int sfd_synchronize(sfd_engine* e);
/* Make the engine stream wait for the work in flight on its background
 * rebuild stream (refactor_lag > 0), without switching to the rebuilt
 * preconditioner and without blocking the host. */
int sfd_join_background(sfd_engine* e);

/* Invariants of the current state, 5 doubles per surface: kinetic, potential
 * (gravitational or van der Waals), surface, volume flux (Energies.cuh:136-204)
 * and mass = sum y x'.  `kappa` scales the surface energy as in the reference. */
int sfd_invariants(sfd_engine* e, double kappa, double* out);

/* Per-surface status words (SFD_STATUS_* bits), max |l_ij| over the FP64
 * factorisations and max over RHS evaluations of the final solve residual
 * max |phi' - M a| (each nullable), all since the last sfd_clear_status. */
int sfd_get_status(sfd_engine* e, unsigned int* status, double* lmax, double* rnorm);
int sfd_clear_status(sfd_engine* e);
/* Refinement record since the last sfd_clear_status (each nullable):
 * rel_residual[s] = max over RHS evaluations of the final relative residual
 * max |phi' - M a| / max |phi'|, extra_iters[s] = extra corrections run for
 * surface s, *stall_rebuilds = preconditioner rebuilds that a refinement
 * stall triggered (since creation). */
int sfd_get_refinement(sfd_engine* e, double* rel_residual, long long* extra_iters, long long* stall_rebuilds);

/* Number of kernel launches the engine issued since creation (graph replays
 * count every kernel node). */
long long sfd_kernel_launches(const sfd_engine* e);

/* Per-kernel-class device time: while enabled, RK4 steps run eagerly (no
 * graph) and every kernel launch is bracketed by CUDA events on the engine
 * stream; sfd_profile_read returns accumulated milliseconds and launch counts
 * per class (names from sfd_profile_class_name; 23 classes).  The gated extra
 * corrections, the a' transform repeated after them and the starting product
 * a0 = X phi' (which returns at once on warm starts) have classes of their
 * own ("extra_corrections", "ap_redo", "start_product"), so the other classes
 * hold working launches only; the a' transform, which stepping on graphs runs
 * beside the last boundary-sum pass, is "ap_transform". */
#define SFD_PROFILE_CLASSES 23
int sfd_profile(sfd_engine* e, int enable);
int sfd_profile_read(sfd_engine* e, double* ms, long long* counts, int nclass);
const char* sfd_profile_class_name(int cls);

const char* sfd_last_error(void);
const char* sfd_version(void);

/* One FP64 RHS evaluation of a single surface that allocates no device memory.
 * No counterpart in the reference.  For callers that cannot call cudaMalloc:
 * code that runs inside another framework's memory pool, real-time loops that
 * must not allocate after start-up, hosts that forbid runtime allocation.
 * state_in = [x | y | phi] and rhs_out = [dx | dy | dphi] are device arrays of
 * 3n doubles (same results as sfd_rhs_device on an FP64 engine).  Scratch is
 * one static device array of about 8.7 MB, held by every GPU that loads the
 * library until exit; n is limited to 1..1024 (larger n returns
 * SFD_ERR_INVALID).  The call issues its kernels on `stream` (NULL = legacy
 * default stream) and returns without waiting for them; it makes no host to
 * device copy (its descriptors are written by a kernel).  Its first call on a
 * device resolves the array's device address (cudaGetSymbolAddress) and sets
 * the kernels' shared-memory limits, so make that first call before any stream
 * capture.  All calls share the array, so calls that overlap on the GPU
 * (different streams or threads) race; serialise them.  No status words are
 * reported: a non-finite input or a breakdown shows as non-finite entries of
 * rhs_out. */
int sfd_rhs_device_noalloc(const sfd_problem* problem, int n, const void* state_in, void* rhs_out, void* stream);

/* ------------------------------------------------------------ adaptive RKF45
 * Runge-Kutta-Fehlberg 4(5) with the reference's error norm and step control
 * (RK45Base, RK45.cuh:195-345; RK45_Options :21-27) on the engine's resident
 * state, from t0 to t1.  One 8-byte device-to-host read per trial step. */
typedef struct sfd_rkf45_options {
    double atol, rtol;    /* 1e-6, 1e-3 */
    double h_min, h_max;  /* 1e-16, 1e10 */
    double h0;            /* first trial step (1e-2) */
    long long max_rejected; /* per step, then status 1 (500) */
} sfd_rkf45_options;
typedef struct sfd_rkf45_result {
    int status;           /* 0 reached t1, 1 too many rejections (stiffness) */
    long long accepted, rejected;
    double t;             /* time reached */
    double h;             /* next step size */
} sfd_rkf45_result;
void sfd_default_rkf45_options(sfd_rkf45_options* o);
/* times (nullable, capacity cap) receives the time after each accepted step. */
int sfd_rkf45_evolve(sfd_engine* e, double t0, double t1, const sfd_rkf45_options* opts, sfd_rkf45_result* res,
                     double* times, long long cap);

/* ------------------------------------------------------------ implicit Gauss-Legendre 2
 * Two-stage Gauss-Legendre (order 4, A-stable) with damped Newton on the
 * stage equations (GaussLegendre2, GaussLegendre.cuh:216-605): an FP64
 * engine with one surface and no drive, from t0 to t1, step halving on
 * Newton failure.  The two stage states are evaluated as one two-surface
 * batch; the stage Jacobians come from central differences over a batched
 * FP64 engine (JacobianCalculator.cuh:223-284) or from the exact reverse-mode
 * Jacobian; the 6n x 6n Newton system is solved by the FP64 blocked LU. */
#define SFD_GL2_JACOBIAN_AUTO 0   /* exact where reverse mode covers the engine and n >= 384, else FD */
#define SFD_GL2_JACOBIAN_FD 1
#define SFD_GL2_JACOBIAN_EXACT 2
typedef struct sfd_gl2_options {
    double step;            /* first (and largest) step, 0.01 */
    double newton_tol;      /* converged when |R| <= tol (1 + |k|), 1e-10 */
    long long max_newton;   /* Newton iterations per attempt, 20 */
    int allow_simplified;   /* after a failed line search, continue once with J(y) frozen (0) */
    double armijo_c;        /* 1e-4 */
    double backtrack;       /* 0.5 */
    double min_alpha;       /* 1e-6 */
    long long max_halvings; /* step halvings per step, 6 */
    double fd_eps;          /* central-difference step, 1e-6 */
    int jacobian;           /* SFD_GL2_JACOBIAN_* */
} sfd_gl2_options;
typedef struct sfd_gl2_result {
    int status;             /* 0 reached t1; 1 Newton failed at every halving (state left at t) */
    long long steps, newton_iters, rhs_evals, jacobians, halvings;
    double t;               /* time reached */
    double h;               /* last accepted step */
    double residual;        /* Newton residual norm of the last attempt */
} sfd_gl2_result;
void sfd_default_gl2_options(sfd_gl2_options* o);
/* Advances the engine's resident state.  times (capacity cap, nullable)
 * receives the time after each accepted step, states (cap x 3n, nullable)
 * the state after it. */
int sfd_gl2_evolve(sfd_engine* e, double t0, double t1, const sfd_gl2_options* opts, sfd_gl2_result* res,
                   double* times, double* states, long long cap);
/* As sfd_gl2_evolve, calling fn(user, t, state) after each accepted step with
 * the time reached and the state (host, 3n doubles, valid during the call). */
typedef void (*sfd_gl2_step_fn)(void* user, double t, const double* state);
int sfd_gl2_evolve_cb(sfd_engine* e, double t0, double t1, const sfd_gl2_options* opts, sfd_gl2_result* res,
                      sfd_gl2_step_fn fn, void* user);

/* ------------------------------------------------------------ reverse mode (adjoint)
 * Hand-written adjoint of the RHS and of RK4 trajectories.  The reference
 * has no reverse mode (it differentiates by finite differences in
 * Python/integration/jacobian_tests.py:10-150); these entry points are new.
 * Requirements: an engine holding one surface, water with rho = 0 or helium
 * with the standard Bernoulli closure, U = 0.  The parameter derivative is
 * d/dA3 for helium and d/dg for water.
 * On an FP64 engine the per-stage records hold the LU factors of M and the
 * transposed solve M^T lambda = g uses them.  On a mixed engine the records
 * hold O(n) data; the transposed solve is FP64 refinement preconditioned by
 * the transpose of the engine's FP32 approximate inverse, rebuilt at the
 * first evaluation of each recomputed checkpoint segment (and of each
 * sfd_rhs_vjp_device / sfd_jacobian_device call); a final relative residual
 * above the engine's refine_tol raises SFD_STATUS_REFINE_STALL. */
/* grad_state = J(state)^T cotangent for the RHS state -> [dx|dy|dphi]; device
 * arrays of 3n doubles; synchronous. */
int sfd_rhs_vjp_device(sfd_engine* e, const void* state, const void* cotangent, void* grad_state,
                       double* grad_param);
/* Integrate `steps` RK4 steps of size dt from state0 (host, 3n) keeping a
 * checkpoint every `checkpoint_every` steps on the device; the final state is
 * written to state_final (host, 3n; nullable).  FP64 engines: same arithmetic
 * as sfd_rk4_steps with the same boundary-sum shape (bitwise equal with
 * autotune off, or once the autotuning first sfd_rk4_steps call has run: it
 * may keep another shape, which changes the summation order).  Mixed engines:
 * the engine's own stepping (sfd_rk4_steps, its graphs and preconditioner
 * schedule) on its resident state, which is saved before and restored after. */
int sfd_rk4_record(sfd_engine* e, double dt, int steps, int checkpoint_every, const double* state0,
                   double* state_final);
/* Reverse the recorded trajectory: grad_state0 = (d state_final / d state0)^T
 * cot_final and *grad_param = the parameter derivative of <cot_final,
 * state_final>.  Each checkpoint segment is recomputed once with every stage
 * recorded, then reversed stage by stage.  With use_graphs, each step of a
 * segment (recomputation and reversal) runs as a CUDA graph captured on first
 * use and kept for later calls with the same dt and problem. */
int sfd_rk4_vjp(sfd_engine* e, const double* cot_final, double* grad_state0, double* grad_param);
/* Record of the mixed transposed solves of the last sfd_rhs_vjp_device,
 * sfd_jacobian_device or sfd_rk4_vjp call (each nullable): the largest final
 * relative residual max |g - M^T lambda| / max |g| and the largest number of
 * preconditioner products one solve ran.  Zeros for FP64 engines. */
int sfd_adjoint_residual(sfd_engine* e, double* max_rel_residual, int* max_corrections);
/* Exact Jacobian of the RHS at `state` (device, 3n) from 3n reverse sweeps
 * over one recorded forward evaluation: jac (device, 9 n^2 doubles) in the
 * column-major layout of calculateJacobian. */
int sfd_jacobian_device(sfd_engine* e, const void* state, void* jac);

/* ------------------------------------------------------------ C++ facade support (include/sfd.hpp)
 * Interleaved complex state as the reference's calculators take it:
 * state = [Z (ntot complex) | Phi (ntot complex, imaginary part ignored)],
 * rhs = [dZ/dt | dPhi/dt (imaginary part 0)], device pointers, asynchronous on
 * the engine stream (BaseBoundaryIntegralCalculator::run,
 * BaseBoundaryIntegrator.cuh:137-262). */
int sfd_rhs_device_complex(sfd_engine* e, const void* state, void* rhs);
/* calculateVorticities (BaseBoundaryIntegrator.cuh:275-306): solves for the
 * vortex sheet strength a of the complex state and returns device pointers
 * to the engine's a (double[ntot]), z' and z'' (complex[ntot]); they stay
 * valid until the next call on the engine. */
int sfd_vorticities_device(sfd_engine* e, const void* state, double** a, void** zp, void** zpp);
/* RK4 stage combines on n doubles (AutonomousRungeKuttaStepper.cuh:338-375):
 * kacc = first ? k : kacc + wk k; ystage = y0 + cy k (ystage nullable);
 * final: y0 += c kacc. */
int sfd_rk4_stage_device(long long n, const void* y0, const void* k, void* kacc, void* ystage, double wk,
                         double cy, int first, void* stream);
int sfd_rk4_final_device(long long n, void* y0, const void* kacc, double c, void* stream);
/* MatrixSolver::solve (MatrixSolver.cuh:113-172): `batch` column-major n x n
 * systems M a = b on the device, FP64 blocked LU with partial pivoting (the
 * pivot choice of cusolverDnDgetrf, MatrixSolver.cuh:123-125); the optional
 * host status words get SFD_STATUS_PIVOT_SWAP where rows were exchanged and
 * SFD_STATUS_ZERO_PIVOT on a zero pivot (the call then waits for the device). */
typedef struct sfd_dense_solver sfd_dense_solver;
int sfd_dense_solver_create(int n, int batch, sfd_dense_solver** out);
int sfd_dense_solver_set_stream(sfd_dense_solver* d, void* stream);
int sfd_dense_solve(sfd_dense_solver* d, const double* M, const double* b, double* x, unsigned int* status);
int sfd_dense_solver_destroy(sfd_dense_solver* d);

/* Precision used by the reference-compatible exports below (default FP64). */
int sfd_set_default_precision(int precision);

/* ------------------------------------------------------------ reference-compatible exports */
/* CuSuperHelium/CuSuperHelium/Export.cuh:31 (Export.cu:560-599, :194-265). */
int calculateRHSFromVectors(const double* x, const double* y, const double* phi, double* vx, double* vy,
                            double* rhsPhi, double L, double rho, double kappa, double depth, size_t N);
/* Export.cuh:30 */
int calculateRHS256FromVectors(const double* x, const double* y, const double* phi, double* vx, double* vy,
                               double* rhsPhi, double L, double rho, double kappa, double depth);
/* Export.cuh:33 */
int calculateRHS2048FromVectors(const double* x, const double* y, const double* phi, double* vx, double* vy,
                                double* rhsPhi, double L, double rho, double kappa, double depth);
/* Export.cuh:51 (Export.cu:520-557): inputs concatenated per surface (256 each). */
int calculateRHS256FromVectorsBatched(const double* x, const double* y, const double* phi, double* vx, double* vy,
                                      double* rhsPhi, double L, double rho, double kappa, double depth,
                                      int batchSize);
/* Export.cuh:48 (Export.cu:279-349): complex Z, phi (interleaved re, im);
 * Zp / Zpp may be NULL. */
int calculateVorticities256FromVectors(const double* Z, const double* phi, double* a, double* Zp, double* Zpp,
                                       double L, double rho, double kappa, double depth);
/* Export.cuh:49 (Export.cu:351-384): spectral first derivative of 256 complex
 * samples (no linear part, no 2 pi / N scale). */
int calculateDerivativeFFT256(const double* input, double* output);

/* SimProperties / RK4SolverOptions (CuSuperHelium/CuSuperHelium/ExportTypes.cuh:8-40). */
typedef struct SimProperties {
    double L;
    double rho;
    double kappa;
    double depth;
    SFD_BOOL use_expansions;
    int expansion_order;
    SFD_BOOL infinite_depth;
} SimProperties;
typedef struct RK4SolverOptions {
    double timeStep;
    double t0;
    double t1;
    SFD_BOOL returnTrajectory;
} RK4SolverOptions;

/* Export.cuh:69 (Export.cu:767-770 is a stub there that returns 0 without
 * integrating; this one integrates).  initialState = [x | y | phi] (3N);
 * statesOut receives the initial state and the state after every step when
 * returnTrajectory, else only the final state; free with the next function. */
int integrateSimulationRK4(double* initialState, double** statesOut, size_t* statesCount, double** timesOut,
                           size_t* timesCount, SimProperties* simProperties, RK4SolverOptions* rkOptions, size_t N);
/* Export.cuh:70 */
int integrateSimulationRK4_freeMemory(double* statesOut, double* timesOut);

/* Export.cuh:50 (Export.cu:393-519): central-difference Jacobian of the
 * helium RHS (SI inputs as calculateRHSFromVectors), jac[col * 3N + row] =
 * d rhs_row / d state_col, rows and columns ordered [x | y | phi]; jac holds
 * 9 N^2 doubles.  All 6N perturbed states run as one batched FP64 engine
 * (in chunks of at most 8 GB of matrices). */
int calculateJacobian(const double* state, double* jac, double L, double rho, double kappa, double depth,
                      double epsilon, size_t N);
/* Export.cuh:53 (Export.cu:601-662, JacobianCalculator.cuh:11-75): the 3N
 * perturbed complex states [Z | Phi] of the finite-difference Jacobian at
 * N = 256.  Zperturbed holds 6 N^2 complex values (interleaved re, im):
 * positions of perturbation b at [b N, (b+1) N), potentials at
 * [3 N^2 + b N, ...); b / N perturbs x, y or phi by epsilon at node b % N.
 * Written on the host; L, rho, kappa and depth are unused, as in the reference. */
int calculatePerturbedStates256(const double* x, const double* y, const double* phi, double* Zperturbed, double L,
                                double rho, double kappa, double depth, double epsilon);
/* Export.cuh:28 (Export.cu:42-113): read a state file of N = 256 nodes
 * (`interface`, `potential`; y scaled by 2 pi / L), evaluate the helium RHS
 * and write it to outputFile as a state file (`interface` = (dx, dy),
 * `potential` = dphi) with attributes rho, kappa, U, depth (nondimensional),
 * initial_amplitude = (max y - min y) / 2 and rhs = true. */
int calculateRHS256FromFile(const char* inputFile, const char* outputFile, double L, double rho, double kappa,
                            double depth);

/* GaussLegendreOptions (ExportTypes.cuh:21-34). */
typedef struct GaussLegendreOptions {
    double t0;
    double t1;
    double stepSize;
    double newtonTolerance;
    size_t maxNewtonIterations;
    SFD_BOOL allowSimplifiedFallback;
    SFD_BOOL returnTrajectory;
    double armijo_c;
    double backtrack;
    double minAlpha;
    size_t maxStepsHalves;
} GaussLegendreOptions;
/* Export.cuh:66 (Export.cu:665-738): GL2 integration of the helium problem
 * (SI properties as the other exports; initial state [x | y | phi], t0, t1
 * and stepSize nondimensional as the reference takes them).  statesOut gets
 * the initial state and the state after every accepted step when
 * returnTrajectory (times likewise), else only the final state and no times.
 * Returns -1 when a step fails to converge at every halving. */
int integrateSimulationGL2(double* initialState, double** statesOut, size_t* statesCount, double** timesOut,
                           size_t* timesCount, SimProperties* simProperties, GaussLegendreOptions* glCOptions,
                           size_t N);
/* Export.cuh:67 */
int integrateSimulationGL2_freeMemory(double* statesOut, double* timesOut);

/* COptomechanicalVariables (ExportTypes.cuh:41-63), SI units. */
typedef struct COptomechanicalVariables {
    double detuning;
    double gamma;
    double G;
    double tau;
    double max_intensity;
    double initial_time;
    double location_x0_mode;
    double sigma_optical_mode;
    double beta;
    double damping_strength;
} COptomechanicalVariables;
/* Export.cuh:79 (Export.cu:1108-1181): RHS of the augmented driven helium
 * problem; state = [x | y | phi | D] (4N), rhs likewise. */
int calculateRhsAugmentedOptomechanical(double* state, double* rhs, SimProperties* simProperties,
                                        COptomechanicalVariables* optomechanicalVariables, size_t N);
/* Export.cuh:75 (Export.cu:980-1092): RK4 of the augmented driven helium
 * problem from t0 to t1; initialState and every returned state = [x | y | phi | D]. */
int integrateAugmentedOptomechanicalSimulationRK4(double* initialState, double** statesOut, size_t* statesCount,
                                                  double** timesOut, size_t* timesCount,
                                                  SimProperties* simProperties, RK4SolverOptions* rkOptions,
                                                  COptomechanicalVariables* optomechanicalVariables, size_t N);
/* Export.cuh:76 */
int integrateAugmentedOptomechanicalSimulationRK4_freeMemory(double* statesOut, double* timesOut);

#ifdef __cplusplus
}
#endif

#endif /* SFD_H */
