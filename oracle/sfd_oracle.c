/*
 * sfd_oracle.c -- CPU FP64 restatement of the CuSuperHelium boundary-integral
 * right-hand side and RK4 step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker (and the timed
 * CPU baseline of bench.py).  Nothing in the product library links or calls
 * it.  Every function below restates one reference routine and cites it
 * (paths relative to the reference project, CSH = CuSuperHelium/CuSuperHelium).
 *
 * Layout conventions of this file:
 *   - a surface is N nodes with real arrays x[N], y[N], phi[N];
 *   - complex values use C99 `double complex`;
 *   - dense matrices are row-major, M[k*N + j] = row k, column j
 *     (the reference stores the same entry column-major at k + j*N).
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.14159265358979323846

typedef double complex cplx;

/* Physics selector and parameters of one surface (nondimensional).
 * Mirrors ProblemProperties (CSH/ProblemProperties.hpp:5-32) restricted to
 * the fields the hot path reads, plus the explicit A3 / g the configs use. */
typedef struct {
    int physics;      /* 0 = water (WaterBoundaryProblem), 1 = helium (HeliumBoundaryProblem) */
    double rho;       /* density ratio (water only)                                          */
    double depth;     /* h: film thickness (helium)                                          */
    double vdw;       /* A3 / h^3; the reference fixes this at h/3 (CSH/createM.cuh:113)    */
    double gravity;   /* g (water); the reference uses 1                                     */
    double U;         /* uniform stream; only the linear-part handling of phi uses it        */
    int infinite_depth; /* helium: drop the image terms (CSH/createM.cuh:79,85)              */
} orc_problem;

/* ------------------------------------------------------------------ */
/* FFT: unnormalised complex DFT, forward sign exp(-2 pi i jk/N) like   */
/* cufftExecZ2Z(CUFFT_FORWARD); inverse exp(+...) and NOT divided by N  */
/* (CSH/Derivatives.cuh:197,243).  Recursive mixed radix on the         */
/* smallest prime factor; twiddles from one accurate table of size N.   */
/* ------------------------------------------------------------------ */
static int smallest_factor(int n) {
    if (n % 2 == 0) return 2;
    for (int p = 3; p * p <= n; p += 2)
        if (n % p == 0) return p;
    return n;
}

/* exp(sign * 2 pi i e / N) with the angle reduced by symmetry first. */
static cplx twiddle(long e, long N, int sign) {
    e %= N;
    if (e < 0) e += N;
    /* reduce to [0, N/8] using octant symmetries where N divisible by 8 */
    double ang = 2.0 * ORC_PI * (double)e / (double)N;
    double c = cos(ang), s = sin(ang);
    if (4 * e == N) { c = 0.0; s = 1.0; }
    else if (2 * e == N) { c = -1.0; s = 0.0; }
    else if (4 * e == 3 * N) { c = 0.0; s = -1.0; }
    else if (e == 0) { c = 1.0; s = 0.0; }
    return c + sign * s * I;
}

static void fft_rec(int n, const cplx* in, long stride, cplx* out, const cplx* tw, long N, cplx* scratch) {
    if (n == 1) { out[0] = in[0]; return; }
    int p = smallest_factor(n);
    int m = n / p;
    for (int r = 0; r < p; ++r)
        fft_rec(m, in + r * stride, stride * p, out + (long)r * m, tw, N, scratch);
    /* combine: X[k + q m] = sum_r W_n^{r (k + q m)} Y_r[k] */
    long step = N / n;
    for (int k = 0; k < m; ++k) {
        for (int q = 0; q < p; ++q) {
            cplx acc = 0.0;
            long idx = k + (long)q * m;
            for (int r = 0; r < p; ++r) {
                long e = ((long)r * idx) % n;
                acc += tw[e * step] * out[(long)r * m + k];
            }
            scratch[q] = acc;
        }
        for (int q = 0; q < p; ++q) out[k + (long)q * m] = scratch[q];
    }
}

/* In-place unnormalised FFT of length n; sign -1 forward, +1 inverse. */
void orc_fft(int n, cplx* data, int sign) {
    cplx* tw = (cplx*)malloc(sizeof(cplx) * n);
    cplx* tmp = (cplx*)malloc(sizeof(cplx) * n);
    cplx* scratch = (cplx*)malloc(sizeof(cplx) * n);
    for (long e = 0; e < n; ++e) tw[e] = twiddle(e, n, sign);
    fft_rec(n, data, 1, tmp, tw, n, scratch);
    memcpy(data, tmp, sizeof(cplx) * n);
    free(tw); free(tmp); free(scratch);
}

/* ------------------------------------------------------------------ */
/* Spectral multipliers.                                               */
/* ------------------------------------------------------------------ */

/* first_derivative_multiplication (CSH/utilities.cuh:106-148):
 *   i <  n/2      : c <- i*k*c/n
 *   i == n/2      : c <- i*(pi/2)*c   (Nyquist treated as exp(i pi j))
 *   i == n/2 + 1  : c <- 0
 *   otherwise     : c <- i*(k-n)*c/n                                    */
void orc_first_derivative_coeffs(int n, cplx* c) {
    for (int i = 0; i < n; ++i) {
        double x = creal(c[i]), y = cimag(c[i]);
        double rx, ry;
        if (i < n / 2) {
            rx = -i * y / (double)n;
            ry = i * x / (double)n;
        } else if (i == n / 2) {
            rx = -ORC_PI * i * y / (double)n;
            ry = ORC_PI * i * x / (double)n;
        } else if (i == n / 2 + 1) {
            rx = 0.0;
            ry = 0.0;
        } else {
            rx = -(i - n) * y / (double)n;
            ry = (i - n) * x / (double)n;
        }
        c[i] = rx + ry * I;
    }
}

/* second_derivative_fft (CSH/utilities.cuh:178-200): c <- -k^2 c / n,
 * with k = i for i <= n/2 and k = i - n above.                          */
void orc_second_derivative_coeffs(int n, cplx* c) {
    for (int i = 0; i < n; ++i) {
        double x = creal(c[i]), y = cimag(c[i]);
        long kk = (i <= n / 2) ? (long)i * i : (long)(i - n) * (i - n);
        c[i] = (-(double)kk * x / n) + (-(double)kk * y / n) * I;
    }
}

/* FftDerivative::exec (CSH/Derivatives.cuh:189-257): forward FFT, spectral
 * multiply, unnormalised inverse FFT, then multiply by `scale`.          */
void orc_fft_derivative(int n, const cplx* in, cplx* out, int second, double scale) {
    cplx* c = (cplx*)malloc(sizeof(cplx) * n);
    memcpy(c, in, sizeof(cplx) * n);
    orc_fft(n, c, -1);
    if (second) orc_second_derivative_coeffs(n, c);
    else orc_first_derivative_coeffs(n, c);
    orc_fft(n, c, +1);
    for (int i = 0; i < n; ++i) out[i] = (scale != 1.0) ? c[i] * scale : c[i];
    free(c);
}

/* ZPhiDerivative::exec (CSH/Derivatives.cuh:310-384) for one surface:
 * remove the linear parts 2 pi j / N from Z and -(1+rho) pi U j / N from
 * Phi, take z'' (x 4 pi^2/N^2), z' (x 2 pi/N, + 2 pi/N) and phi' (x 2 pi/N,
 * + the linear slope when U != 0).  All derivatives are per index j.     */
void orc_zphi_derivative(int n, const cplx* Z, const cplx* Phi, double rho, double U,
                         cplx* Zp, cplx* PhiP, cplx* Zpp) {
    cplx* zper = (cplx*)malloc(sizeof(cplx) * n);
    cplx* pper = (cplx*)malloc(sizeof(cplx) * n);
    for (int j = 0; j < n; ++j) {
        double zlin = 2 * ORC_PI * (double)j / n;                    /* Derivatives.cuh:285 */
        double plin = -(1 + rho) * ORC_PI * U / n * (double)j;        /* Derivatives.cuh:286 */
        zper[j] = Z[j] - zlin;
        pper[j] = Phi[j] - plin;
    }
    orc_fft_derivative(n, zper, Zpp, 1, 4.0 * ORC_PI * ORC_PI / ((double)n * n));
    orc_fft_derivative(n, zper, Zp, 0, 2.0 * ORC_PI / n);
    orc_fft_derivative(n, pper, PhiP, 0, 2.0 * ORC_PI / n);
    for (int j = 0; j < n; ++j) Zp[j] += 2.0 * ORC_PI / n;           /* Derivatives.cuh:374 */
    if (U != 0)
        for (int j = 0; j < n; ++j) PhiP[j] += -(1 + rho) * ORC_PI * U / n; /* :380-383 */
    free(zper); free(pper);
}

/* cot(0.5 (Zk - Zj)) as the reference evaluates it: 1 / tan(.)
 * (cotangent_green_function, CSH/utilities.cuh:312-315,347-350).        */
static cplx cot_green(cplx zk, cplx zj) { return 1.0 / ctan(0.5 * (zk - zj)); }
static cplx cot_c(cplx z) { return 1.0 / ctan(z); }

/* createMKernel (CSH/createM.cuh:43-63), water with density ratio rho. */
void orc_create_M_water(int n, const cplx* Z, const cplx* Zp, const cplx* Zpp, double rho, double* M) {
    #pragma omp parallel for schedule(static)
    for (int k = 0; k < n; ++k) {
        for (int j = 0; j < n; ++j) {
            double v;
            if (k == j) v = 0.5 * (1 + rho) + 0.25 * (1 - rho) / ORC_PI * cimag(Zpp[k] / Zp[k]);
            else v = 0.25 * (1 - rho) / ORC_PI * cimag(Zp[k] * cot_green(Z[k], Z[j]));
            M[(long)k * n + j] = v;
        }
    }
}

/* createFiniteDepthMKernel (CSH/createM.cuh:65-92), helium of depth h. */
void orc_create_M_helium(int n, const cplx* Z, const cplx* Zp, const cplx* Zpp, double h, int infinite_depth, double* M) {
    #pragma omp parallel for schedule(static)
    for (int k = 0; k < n; ++k) {
        for (int j = 0; j < n; ++j) {
            double v;
            if (k == j) {
                v = 0.5 + 0.25 / ORC_PI * cimag(Zpp[k] / Zp[k]);
                if (!infinite_depth) v -= 0.25 / ORC_PI * cimag(cot_c(0.0 + (cimag(Z[k]) + h) * I));
            } else {
                v = 0.25 / ORC_PI * cimag(Zp[k] * cot_green(Z[k], Z[j]));
                if (!infinite_depth) {
                    cplx t = 0.5 * (Z[k] - conj(Z[j])) + h * I;
                    v -= 0.25 / ORC_PI * cimag(cot_c(t));
                }
            }
            M[(long)k * n + j] = v;
        }
    }
}

/* ------------------------------------------------------------------ */
/* Dense LU with partial pivoting and solve (getrf + getrs semantics,  */
/* MatrixSolver::solve, CSH/MatrixSolver.cuh:113-126).  Right-looking,  */
/* blocked, with the trailing update threaded.  Returns 0 or k+1 for a  */
/* zero pivot at step k (the LAPACK `info` convention).                */
/* ------------------------------------------------------------------ */
int orc_lu_factor(int n, double* A, int* piv) {
    const int nb = 64;
    int info = 0;
    for (int k0 = 0; k0 < n; k0 += nb) {
        int kb = (n - k0 < nb) ? n - k0 : nb;
        /* unblocked panel factorisation of columns k0..k0+kb-1 (all rows) */
        for (int k = k0; k < k0 + kb; ++k) {
            int p = k;
            double best = fabs(A[(long)k * n + k]);
            for (int i = k + 1; i < n; ++i) {
                double v = fabs(A[(long)i * n + k]);
                if (v > best) { best = v; p = i; }
            }
            piv[k] = p;
            if (p != k) {
                double* rk = A + (long)k * n;
                double* rp = A + (long)p * n;
                for (int j = 0; j < n; ++j) { double t = rk[j]; rk[j] = rp[j]; rp[j] = t; }
            }
            double d = A[(long)k * n + k];
            if (d == 0.0) { if (!info) info = k + 1; continue; }
            double inv = 1.0 / d;
            int jend = k0 + kb;
            for (int i = k + 1; i < n; ++i) {
                double* ri = A + (long)i * n;
                double l = ri[k] * inv;
                ri[k] = l;
                const double* rk = A + (long)k * n;
                for (int j = k + 1; j < jend; ++j) ri[j] -= l * rk[j];
            }
        }
        int j0 = k0 + kb;
        if (j0 >= n) break;
        /* U12 = L11^{-1} A12 (unit lower triangular forward substitution) */
        for (int k = k0; k < k0 + kb; ++k) {
            const double* rk = A + (long)k * n;
            for (int i = k + 1; i < k0 + kb; ++i) {
                double* ri = A + (long)i * n;
                double l = ri[k];
                for (int j = j0; j < n; ++j) ri[j] -= l * rk[j];
            }
        }
        /* A22 -= L21 U12 */
        #pragma omp parallel for schedule(static)
        for (int i = j0; i < n; ++i) {
            double* ri = A + (long)i * n;
            for (int k = k0; k < k0 + kb; ++k) {
                double l = ri[k];
                const double* rk = A + (long)k * n;
                for (int j = j0; j < n; ++j) ri[j] -= l * rk[j];
            }
        }
    }
    return info;
}

void orc_lu_solve(int n, const double* LU, const int* piv, double* b) {
    for (int k = 0; k < n; ++k)
        if (piv[k] != k) { double t = b[k]; b[k] = b[piv[k]]; b[piv[k]] = t; }
    for (int i = 0; i < n; ++i) {
        double s = b[i];
        const double* ri = LU + (long)i * n;
        for (int j = 0; j < i; ++j) s -= ri[j] * b[j];
        b[i] = s;
    }
    for (int i = n - 1; i >= 0; --i) {
        double s = b[i];
        const double* ri = LU + (long)i * n;
        for (int j = i + 1; j < n; ++j) s -= ri[j] * b[j];
        b[i] = s / ri[i];
    }
}

/* ------------------------------------------------------------------ */
/* Velocities: vel = conj(V1 a + V2 o a')  (VelocityCalculator,        */
/* CSH/WaterVelocities.cuh:205-242) with V1, V2 from                   */
/* createVelocityMatrices (:38-70) or createHeliumVelocityMatrices      */
/* (:72-107).  V1 is never stored here: row k is summed on the fly.     */
/* ------------------------------------------------------------------ */
void orc_velocities(int n, const cplx* Z, const cplx* Zp, const cplx* Zpp, const double* a, const cplx* ap,
                    int helium, double h, int infinite_depth, int lower, cplx* vel) {
    #pragma omp parallel for schedule(static)
    for (int k = 0; k < n; ++k) {
        cplx acc = 0.0;
        for (int j = 0; j < n; ++j) {
            cplx v1;
            if (k == j) {
                v1 = I * (-1.0 / (4.0 * ORC_PI) * Zpp[k] / (Zp[k] * Zp[k]));
                if (helium && !infinite_depth)
                    v1 += I * (1.0 / (4.0 * ORC_PI) * cot_c(0.0 + (cimag(Z[k]) + h) * I));
                if (lower) v1 += 1.0 / (2.0 * Zp[k]);
                else v1 -= 0.5 / Zp[k];
            } else {
                v1 = I * (-1.0 / (4.0 * ORC_PI) * cot_green(Z[k], Z[j]));
                if (helium && !infinite_depth)
                    v1 += I * (1.0 / (4.0 * ORC_PI) * cot_c(0.5 * (Z[k] - conj(Z[j])) + h * I));
            }
            acc += v1 * a[j];
        }
        cplx v2 = I * (1.0 / (2.0 * ORC_PI * Zp[k]));
        vel[k] = conj(v2 * ap[k] + acc);
    }
}

/* ------------------------------------------------------------------ */
/* Bernoulli right-hand sides.                                         */
/* ------------------------------------------------------------------ */

/* compute_rhs_phi_expression (CSH/createM.cuh:96-107).  The reference
 * reads V1[1] (not V1[i]) in the cross term; with rho = 0 it vanishes.
 * That read is kept so results match for rho != 0 as well.             */
void orc_rhs_phi_water(int n, const cplx* Z, const cplx* vlow, const cplx* vup, double rho, double g, double* out) {
    for (int i = 0; i < n; ++i) {
        double yi = cimag(Z[i]);
        double v1 = creal(vlow[i]) * creal(vlow[i]) + cimag(vlow[i]) * cimag(vlow[i]);
        double v2 = creal(vup[i]) * creal(vup[i]) + cimag(vup[i]) * cimag(vup[i]);
        double v12 = creal(vlow[n > 1 ? 1 : 0]) * creal(vup[i]) + cimag(vlow[i]) * cimag(vup[i]);
        out[i] = -(1 + rho) * (g * yi) + 0.5 * v1 + 0.5 * rho * v2 - rho * v12;
    }
}

/* compute_rhs_helium_phi_expression (CSH/createM.cuh:109-117):
 * vdw (1 + y/h)^-3 - vdw + |v|^2 / 2 with vdw = A3 / h^3 (= h/3 there).   */
void orc_rhs_phi_helium(int n, const cplx* Z, const cplx* vlow, double h, double vdw, double* out) {
    for (int i = 0; i < n; ++i) {
        double q = 1.0 + cimag(Z[i]) / h;
        out[i] = vdw * pow(q, -3.0) - vdw + 0.5 * creal(vlow[i]) * creal(vlow[i]) + 0.5 * cimag(vlow[i]) * cimag(vlow[i]);
    }
}

/* ------------------------------------------------------------------ */
/* One RHS evaluation (BaseBoundaryIntegralCalculator::runTimeStep,    */
/* CSH/BaseBoundaryIntegrator.cuh:137-306).                            */
/* Outputs dx, dy (= Re/Im of the lower velocity) and dphi; optional    */
/* diagnostics: a (vortex strength), zp, zpp (complex, interleaved).    */
/* Returns the LU info (0 = fine).                                     */
/* ------------------------------------------------------------------ */
int orc_rhs(const orc_problem* P, int n, const double* x, const double* y, const double* phi,
            double* dx, double* dy, double* dphi, double* a_out, double* zp_out, double* zpp_out) {
    cplx* Z = (cplx*)malloc(sizeof(cplx) * n);
    cplx* Ph = (cplx*)malloc(sizeof(cplx) * n);
    cplx* Zp = (cplx*)malloc(sizeof(cplx) * n);
    cplx* Zpp = (cplx*)malloc(sizeof(cplx) * n);
    cplx* PhP = (cplx*)malloc(sizeof(cplx) * n);
    cplx* ac = (cplx*)malloc(sizeof(cplx) * n);
    cplx* ap = (cplx*)malloc(sizeof(cplx) * n);
    cplx* vlow = (cplx*)malloc(sizeof(cplx) * n);
    cplx* vup = (cplx*)malloc(sizeof(cplx) * n);
    double* M = (double*)malloc(sizeof(double) * (size_t)n * n);
    double* a = (double*)malloc(sizeof(double) * n);
    int* piv = (int*)malloc(sizeof(int) * n);
    for (int j = 0; j < n; ++j) { Z[j] = x[j] + y[j] * I; Ph[j] = phi[j]; }

    double rho = P->physics == 0 ? P->rho : 0.0;
    orc_zphi_derivative(n, Z, Ph, rho, P->U, Zp, PhP, Zpp);
    if (P->physics == 0) orc_create_M_water(n, Z, Zp, Zpp, P->rho, M);
    else orc_create_M_helium(n, Z, Zp, Zpp, P->depth, P->infinite_depth, M);
    for (int j = 0; j < n; ++j) a[j] = creal(PhP[j]);               /* complex_to_real */
    int info = orc_lu_factor(n, M, piv);
    orc_lu_solve(n, M, piv, a);
    for (int j = 0; j < n; ++j) ac[j] = a[j];                       /* real_to_complex */
    orc_fft_derivative(n, ac, ap, 0, 2.0 * ORC_PI / n);              /* a' */
    int helium = P->physics == 1;
    orc_velocities(n, Z, Zp, Zpp, a, ap, helium, P->depth, P->infinite_depth, 1, vlow);
    if (P->physics == 0) {
        if (P->rho != 0.0) orc_velocities(n, Z, Zp, Zpp, a, ap, 0, 0.0, 1, 0, vup);
        else for (int j = 0; j < n; ++j) vup[j] = 0.0;  /* multiplied by rho = 0 */
        orc_rhs_phi_water(n, Z, vlow, vup, P->rho, P->gravity, dphi);
    } else {
        orc_rhs_phi_helium(n, Z, vlow, P->depth, P->vdw, dphi);
    }
    for (int j = 0; j < n; ++j) { dx[j] = creal(vlow[j]); dy[j] = cimag(vlow[j]); }
    if (a_out) memcpy(a_out, a, sizeof(double) * n);
    if (zp_out) memcpy(zp_out, Zp, sizeof(cplx) * n);
    if (zpp_out) memcpy(zpp_out, Zpp, sizeof(cplx) * n);
    free(Z); free(Ph); free(Zp); free(Zpp); free(PhP); free(ac); free(ap);
    free(vlow); free(vup); free(M); free(a); free(piv);
    return info;
}

/* ------------------------------------------------------------------ */
/* Classic RK4 on the state [x, y, phi]                                 */
/* (AutonomousRungeKuttaStepper<std_complex,2N>::runStep,              */
/* CSH/AutonomousRungeKuttaStepper.cuh:123-307,338-375 and add_k_vectors */
/* CSH/utilities.cuh:78-83): Y1 = Y0 + h/2 k1, Y2 = Y0 + h/2 k2,         */
/* Y3 = Y0 + h k3, k = k1 + 2 k2 + 2 k3 + k4, Y0 += h/6 k.              */
/* ------------------------------------------------------------------ */
int orc_rk4_step(const orc_problem* P, int n, double dt, double* x, double* y, double* phi) {
    size_t sz = sizeof(double) * 3 * (size_t)n;
    double* Y0 = (double*)malloc(sz);
    double* Y = (double*)malloc(sz);
    double* k[4];
    for (int s = 0; s < 4; ++s) k[s] = (double*)malloc(sz);
    memcpy(Y0, x, sizeof(double) * n);
    memcpy(Y0 + n, y, sizeof(double) * n);
    memcpy(Y0 + 2 * n, phi, sizeof(double) * n);
    int info = 0;
    const double half = dt * 0.5, full = dt, sixth = dt / 6.0;
    const double coef[3] = {half, half, full};
    memcpy(Y, Y0, sz);
    for (int s = 0; s < 4; ++s) {
        int r = orc_rhs(P, n, Y, Y + n, Y + 2 * n, k[s], k[s] + n, k[s] + 2 * n, NULL, NULL, NULL);
        if (r && !info) info = r;
        if (s < 3)
            for (int i = 0; i < 3 * n; ++i) Y[i] = Y0[i] + coef[s] * k[s][i];
    }
    for (int i = 0; i < 3 * n; ++i) {
        double kk = k[0][i] + 2.0 * k[1][i] + 2.0 * k[2][i] + k[3][i];
        Y0[i] = Y0[i] + sixth * kk;
    }
    memcpy(x, Y0, sizeof(double) * n);
    memcpy(y, Y0 + n, sizeof(double) * n);
    memcpy(phi, Y0 + 2 * n, sizeof(double) * n);
    free(Y0); free(Y);
    for (int s = 0; s < 4; ++s) free(k[s]);
    return info;
}

int orc_rk4_steps(const orc_problem* P, int n, double dt, int steps, double* x, double* y, double* phi) {
    int info = 0;
    for (int s = 0; s < steps; ++s) {
        int r = orc_rk4_step(P, n, dt, x, y, phi);
        if (r && !info) info = r;
    }
    return info;
}

/* ------------------------------------------------------------------ */
/* Optomechanical drive of a helium film (nondimensional parameters).   */
/*   intensity (CSH/LightIntensity.cuh:25-31):                          */
/*     I(y, x) = gamma^2 I_max / 4 / ((detuning - G y)^2 + (gamma/2)^2)  */
/*               * exp(-(x - x0)^2 / (2 sigma^2))                        */
/*   dphi += damping * v + strength * I      (CSH/createM.cuh:141-158,   */
/*           HeliumDrivenAutonomousProblem.cuh:20-26; v = Im of the      */
/*           lower velocity)                                            */
/*   augmented state D (CSH/DelayedIntensityIntegrator.cuh:22-36,        */
/*           CSH/createM.cuh:160-178): dphi += D, dD = beta I - D / tau  */
/* ------------------------------------------------------------------ */
typedef struct {
    double detuning, gamma, G, tau, max_intensity, x0, sigma, beta, damping, strength;
    int augmented;
} orc_drive;

double orc_intensity(const orc_drive* D, double y, double x) {
    double df = D->detuning - D->G * y;
    double prof = exp(-pow(x - D->x0, 2.0) / (2.0 * pow(D->sigma, 2.0)));
    return 0.25 * pow(D->gamma, 2.0) * D->max_intensity / (pow(df, 2.0) + pow(D->gamma / 2.0, 2.0)) * prof;
}

/* Driven RHS on [x, y, phi (, D)] -> [dx, dy, dphi (, dD)] (dl / ddl used  */
/* only when augmented).                                                 */
int orc_rhs_driven(const orc_problem* P, const orc_drive* D, int n, const double* x, const double* y,
                   const double* phi, const double* dl, double* dx, double* dy, double* dphi, double* ddl) {
    int info = orc_rhs(P, n, x, y, phi, dx, dy, dphi, NULL, NULL, NULL);
    for (int i = 0; i < n; ++i) {
        double inten = orc_intensity(D, y[i], x[i]);
        dphi[i] += D->damping * dy[i];
        dphi[i] += D->strength * inten;
        if (D->augmented) {
            dphi[i] += dl[i];
            ddl[i] = D->beta * inten - 1.0 / D->tau * dl[i];
        }
    }
    return info;
}

/* Classic RK4 of the driven problem on [x, y, phi (, D)] (same stage     */
/* formula as orc_rk4_step).                                             */
int orc_rk4_steps_driven(const orc_problem* P, const orc_drive* D, int n, double dt, int steps, double* x,
                         double* y, double* phi, double* dl) {
    const int nb = D->augmented ? 4 : 3;
    size_t sz = sizeof(double) * nb * (size_t)n;
    double* Y0 = (double*)malloc(sz);
    double* Y = (double*)malloc(sz);
    double* k[4];
    for (int s = 0; s < 4; ++s) k[s] = (double*)calloc((size_t)nb * n, sizeof(double));
    memcpy(Y0, x, sizeof(double) * n);
    memcpy(Y0 + n, y, sizeof(double) * n);
    memcpy(Y0 + 2 * n, phi, sizeof(double) * n);
    if (D->augmented) memcpy(Y0 + 3 * n, dl, sizeof(double) * n);
    int info = 0;
    const double half = dt * 0.5, full = dt, sixth = dt / 6.0;
    const double coef[3] = {half, half, full};
    for (int st = 0; st < steps; ++st) {
        memcpy(Y, Y0, sz);
        for (int s = 0; s < 4; ++s) {
            int r = orc_rhs_driven(P, D, n, Y, Y + n, Y + 2 * n, Y + 3 * n, k[s], k[s] + n, k[s] + 2 * n,
                                   D->augmented ? k[s] + 3 * n : NULL);
            if (r && !info) info = r;
            if (s < 3)
                for (int i = 0; i < nb * n; ++i) Y[i] = Y0[i] + coef[s] * k[s][i];
        }
        for (int i = 0; i < nb * n; ++i) {
            double kk = k[0][i] + 2.0 * k[1][i] + 2.0 * k[2][i] + k[3][i];
            Y0[i] = Y0[i] + sixth * kk;
        }
    }
    memcpy(x, Y0, sizeof(double) * n);
    memcpy(y, Y0 + n, sizeof(double) * n);
    memcpy(phi, Y0 + 2 * n, sizeof(double) * n);
    if (D->augmented) memcpy(dl, Y0 + 3 * n, sizeof(double) * n);
    free(Y0); free(Y);
    for (int s = 0; s < 4; ++s) free(k[s]);
    return info;
}

/* ------------------------------------------------------------------ */
/* Adaptive Runge-Kutta-Fehlberg 4(5) (CSH/RK45.cuh:195-345,             */
/* CSH/RK45_Kernels.cuh:15-106): Fehlberg's 1969 tableau, the 5th-order  */
/* solution is kept, error = h sum (b - b*) k.  The error norm runs over */
/* the 2N complex state entries (z = x + i y, then phi):                 */
/*   err = sqrt(mean(|e|^2 / (atol + rtol max(|y|, |y5|))^2))            */
/* step factor 0.9 err^(-1/5), clamped to [0.2, 5] on acceptance and     */
/* [0.2, 1] on rejection, then to [h_min, h_max]; err == 0 grows 5x.     */
/* k1 is reused after a rejection.  The step is cut to the remaining     */
/* interval.  Returns 0 at t1, 1 after more than max_rejected rejections */
/* of one step; *accepted / *rejected count steps, times[] (if non-NULL, */
/* capacity cap) receives the time after each accepted step.            */
/* ------------------------------------------------------------------ */
static const double RKF_A[6][5] = {
    {0, 0, 0, 0, 0},
    {1.0 / 4.0, 0, 0, 0, 0},
    {3.0 / 32.0, 9.0 / 32.0, 0, 0, 0},
    {1932.0 / 2197.0, -7200.0 / 2197.0, 7296.0 / 2197.0, 0, 0},
    {439.0 / 216.0, -8.0, 3680.0 / 513.0, -845.0 / 4104.0, 0},
    {-8.0 / 27.0, 2.0, -3544.0 / 2565.0, 1859.0 / 4104.0, -11.0 / 40.0}};
static const double RKF_B[6] = {16.0 / 135.0, 0.0, 6656.0 / 12825.0, 28561.0 / 56430.0, -9.0 / 50.0, 2.0 / 55.0};
static const double RKF_BS[6] = {25.0 / 216.0, 0.0, 1408.0 / 2565.0, 2197.0 / 4104.0, -1.0 / 5.0, 0.0};

int orc_rkf45_evolve(const orc_problem* P, int n, double t0, double t1, double atol, double rtol, double h_min,
                     double h_max, double h0, long long max_rejected, double* x, double* y, double* phi,
                     double* t_out, double* h_out, long long* accepted, long long* rejected, double* times,
                     long long cap) {
    const size_t n3 = 3 * (size_t)n;
    double* Y = (double*)malloc(sizeof(double) * n3);
    double* T = (double*)malloc(sizeof(double) * n3);
    double* Y5 = (double*)malloc(sizeof(double) * n3);
    double* k[6];
    for (int s = 0; s < 6; ++s) k[s] = (double*)malloc(sizeof(double) * n3);
    memcpy(Y, x, sizeof(double) * n);
    memcpy(Y + n, y, sizeof(double) * n);
    memcpy(Y + 2 * n, phi, sizeof(double) * n);
    double t = t0, h = h0;
    int have_k1 = 0, status = 0;
    long long acc = 0, rej = 0;
    while (t < t1) {
        if (t1 - t < h) h = t1 - t;
        long long rej_here = 0;
        for (;;) {
            if (!have_k1) {
                orc_rhs(P, n, Y, Y + n, Y + 2 * n, k[0], k[0] + n, k[0] + 2 * n, NULL, NULL, NULL);
                have_k1 = 1;
            }
            for (int s = 1; s < 6; ++s) {
                for (size_t i = 0; i < n3; ++i) {
                    double v = Y[i];
                    for (int j = 0; j < s; ++j) v += (RKF_A[s][j] * h) * k[j][i];
                    T[i] = v;
                }
                orc_rhs(P, n, T, T + n, T + 2 * n, k[s], k[s] + n, k[s] + 2 * n, NULL, NULL, NULL);
            }
            double sumsq = 0.0;
            for (int i = 0; i < 2 * n; ++i) {
                double e2 = 0.0, y2 = 0.0, y52 = 0.0;
                int comps = i < n ? 2 : 1;
                for (int c = 0; c < comps; ++c) {
                    size_t idx = i < n ? (size_t)i + (size_t)c * n : (size_t)(2 * n + (i - n));
                    double y5v = Y[idx], ev = 0.0;
                    for (int j = 0; j < 6; ++j) {
                        y5v += (h * RKF_B[j]) * k[j][idx];
                        ev += (h * (RKF_B[j] - RKF_BS[j])) * k[j][idx];
                    }
                    Y5[idx] = y5v;
                    e2 += ev * ev;
                    y2 += Y[idx] * Y[idx];
                    y52 += y5v * y5v;
                }
                double sc = atol + rtol * fmax(sqrt(y2), sqrt(y52));
                if (sc < 1e-300) sc = 1e-300;
                sumsq += e2 / (sc * sc);
            }
            double err = sqrt(sumsq / (2.0 * n));
            int ok = err <= 1.0;
            double fac;
            if (err == 0.0) fac = ok ? 5.0 : 1.0;
            else {
                fac = 0.9 * pow(err, -0.2);
                fac = fmin(fmax(fac, 0.2), ok ? 5.0 : 1.0);
            }
            double hn = fmin(fmax(h * fac, h_min), h_max);
            if (err == 0.0) hn = h * fac;
            if (ok) {
                memcpy(Y, Y5, sizeof(double) * n3);
                have_k1 = 0;
                t += h;
                if (times && acc < cap) times[acc] = t;
                ++acc;
                h = hn;
                break;
            }
            h = hn;
            ++rej;
            if (++rej_here > max_rejected) { status = 1; break; }
        }
        if (status) break;
    }
    memcpy(x, Y, sizeof(double) * n);
    memcpy(y, Y + n, sizeof(double) * n);
    memcpy(phi, Y + 2 * n, sizeof(double) * n);
    *t_out = t;
    *h_out = h;
    *accepted = acc;
    *rejected = rej;
    free(Y); free(T); free(Y5);
    for (int s = 0; s < 6; ++s) free(k[s]);
    return status;
}

/* ------------------------------------------------------------------ */
/* Invariants (CSH/Energies.cuh:136-204 and scalings :61-128), with U=0 */
/* out[0] kinetic   = (1/4pi) sum phi (x' v - y' u)                     */
/* out[1] potential = water (1+rho) g/(4pi) sum y^2 x'  |  helium       */
/*                    h^2/6 sum [(1 + y/h)^-2 - 1]                       */
/* out[2] surface   = (sum |z'| - 2 pi) kappa / (2 pi) (kappa given)    */
/* out[3] flux      = (1/2pi) sum (v x' + u y')                          */
/* out[4] mass      = sum y x'  (not in the reference)                  */
/* Derivatives are per index (already scaled by 2 pi / N).               */
/* ------------------------------------------------------------------ */
void orc_invariants(const orc_problem* P, int n, const double* x, const double* y, const double* phi,
                    const double* u, const double* v, double kappa, double* out) {
    cplx* Z = (cplx*)malloc(sizeof(cplx) * n);
    cplx* Ph = (cplx*)malloc(sizeof(cplx) * n);
    cplx* Zp = (cplx*)malloc(sizeof(cplx) * n);
    cplx* Zpp = (cplx*)malloc(sizeof(cplx) * n);
    cplx* PhP = (cplx*)malloc(sizeof(cplx) * n);
    for (int j = 0; j < n; ++j) { Z[j] = x[j] + y[j] * I; Ph[j] = phi[j]; }
    double rho = P->physics == 0 ? P->rho : 0.0;
    orc_zphi_derivative(n, Z, Ph, rho, P->U, Zp, PhP, Zpp);
    double ke = 0, pe = 0, se = 0, fl = 0, ms = 0;
    for (int k = 0; k < n; ++k) {
        double xp = creal(Zp[k]), yp = cimag(Zp[k]);
        ke += phi[k] * (-1.0 * yp * u[k] + xp * v[k]);
        if (P->physics == 0) pe += y[k] * y[k] * xp;
        else pe += (1.0 / pow(1.0 + y[k] / P->depth, 2) - 1.0);
        se += sqrt(xp * xp + yp * yp);
        fl += v[k] * xp + u[k] * yp;
        ms += y[k] * xp;
    }
    out[0] = ke * 0.25 / ORC_PI;
    if (P->physics == 0) out[1] = pe * 0.25 * (1.0 + P->rho) * P->gravity / ORC_PI;
    else out[1] = pe * pow(P->depth, 2) / 6.0;
    out[2] = (se - 2.0 * ORC_PI) * kappa / (2.0 * ORC_PI);
    out[3] = fl * 0.5 / ORC_PI;
    out[4] = ms;
    free(Z); free(Ph); free(Zp); free(Zpp); free(PhP);
}

/* Thread count control for the timed CPU baseline. */
int orc_set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
    return omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

/* cot(0.5 (zk - zj)) exactly as cotangent_green_function evaluates it
 * (CSH/utilities.cuh:347-350); exposed for the known-answer test. */
void orc_cot_green(double zkr, double zki, double zjr, double zji, double* out) {
    cplx v = cot_green(zkr + zki * I, zjr + zji * I);
    out[0] = creal(v);
    out[1] = cimag(v);
}
