/* CPU restatement of the 2-D periodic Brusselator semi-discretisation and its fixed-step
 * SSPRK33 solve, in C with OpenMP: the timed CPU baseline of the headline workload
 * (test infrastructure; the product never links it).
 *
 * What it restates:
 *  - the semi-discretisation MethodOfLines generates for the reference's Brusselator test
 *    (test/Brusselator/brusselator_eq.jl:8-58; the same equations as the test's hand-written
 *    loop, brusselator_eq.jl:80-105):
 *      du = 1 + v u^2 - 4.4 u + alpha (Dxx u + Dyy u) + f(x, y, t)
 *      dv = 3.4 u - v u^2 + alpha (Dxx v + Dyy v)
 *    with f = 5 where (x - 0.3)^2 + (y - 0.6)^2 <= 0.1^2 and t >= 1.1 (brusselator_eq.jl:19),
 *    each second derivative the three-point centered stencil of its own dimension
 *    (centered_difference.jl:5-30) on a periodic grid whose unknowns are the points 2..l
 *    (u[1] == u[l], interface_boundary.jl:33-42);
 *  - the Shu-Osher SSPRK33 stages in OrdinaryDiffEq's evaluation order:
 *      u1 = u + dt f(u, t)
 *      u2 = (3 u + u1 + dt f(u1, t + dt)) / 4
 *      u' = (u + 2 u2 + 2 dt f(u2, t + dt/2)) / 3
 * The interior weights w[0..2] of the two second-derivative operators and the coordinates
 * of the unknowns are inputs, so the arithmetic uses the same doubles as the oracle.
 *
 * Layout: per field x fastest, u then v (2 * nx * ny doubles).
 */
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int64_t nx, ny;
    double wx[3], wy[3];   /* Dxx and Dyy interior weights (taps -1, 0, +1) */
    double alpha;
    const double* x;       /* nx coordinates of the unknowns along x */
    const double* y;       /* ny coordinates along y */
} bruss_grid;

static void rhs(const bruss_grid* g, const double* s, double* out, double t) {
    const int64_t nx = g->nx, ny = g->ny, n = nx * ny;
    const double* u = s;
    const double* v = s + n;
    const double fon = t >= 1.1 ? 1.0 : 0.0;
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < ny; ++j) {
        const int64_t jm = j == 0 ? ny - 1 : j - 1, jp = j == ny - 1 ? 0 : j + 1;
        const double dy = g->y[j] - 0.6;
        for (int64_t i = 0; i < nx; ++i) {
            const int64_t im = i == 0 ? nx - 1 : i - 1, ip = i == nx - 1 ? 0 : i + 1;
            const int64_t c = j * nx + i;
            const double uc = u[c], vc = v[c];
            const double lxu = g->wx[0] * u[j * nx + im] + g->wx[1] * uc + g->wx[2] * u[j * nx + ip];
            const double lyu = g->wy[0] * u[jm * nx + i] + g->wy[1] * uc + g->wy[2] * u[jp * nx + i];
            const double lxv = g->wx[0] * v[j * nx + im] + g->wx[1] * vc + g->wx[2] * v[j * nx + ip];
            const double lyv = g->wy[0] * v[jm * nx + i] + g->wy[1] * vc + g->wy[2] * v[jp * nx + i];
            const double dx = g->x[i] - 0.3;
            const double mask = (dx * dx + dy * dy <= 0.1 * 0.1) ? 1.0 : 0.0;
            const double u2v = vc * (uc * uc);
            out[c] = (((1.0 + u2v) - 4.4 * uc) + g->alpha * (lxu + lyu)) + (mask * fon) * 5.0;
            out[n + c] = (3.4 * uc - u2v) + g->alpha * (lxv + lyv);
        }
    }
}

/* Stage scratch kept between calls (grown on demand), so a timed call does not pay for
 * allocating and first-touching 3 state-sized arrays: the reference's integrator cache
 * likewise lives in its integrator, not in each step. */
static double* g_scratch = NULL;
static size_t g_scratch_len = 0;

static double* scratch(size_t n) {
    if (g_scratch_len < n) {
        free(g_scratch);
        g_scratch = (double*)malloc(sizeof(double) * n);
        g_scratch_len = g_scratch ? n : 0;
        if (g_scratch) {
#pragma omp parallel for schedule(static)
            for (int64_t q = 0; q < (int64_t)n; ++q) g_scratch[q] = 0.0;  /* first touch by the workers */
        }
    }
    return g_scratch;
}

void bruss_release(void) {
    free(g_scratch);
    g_scratch = NULL;
    g_scratch_len = 0;
}

/* nsteps SSPRK33 steps of size dt from t0, in place on s (2 nx ny doubles).  nthreads <= 0
 * keeps the OpenMP default.  Returns 0, or -1 when scratch memory cannot be allocated. */
int bruss_ssprk33(int64_t nx, int64_t ny, const double* wx, const double* wy, double alpha, const double* x,
                  const double* y, double* s, double t0, double dt, int64_t nsteps, int nthreads) {
    bruss_grid g;
    g.nx = nx;
    g.ny = ny;
    memcpy(g.wx, wx, sizeof(g.wx));
    memcpy(g.wy, wy, sizeof(g.wy));
    g.alpha = alpha;
    g.x = x;
    g.y = y;
#ifdef _OPENMP
    const int prev_threads = omp_get_max_threads();   /* restored on return */
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    const int64_t n2 = 2 * nx * ny;
    double* k = scratch(3 * (size_t)n2);
    if (!k) {
#ifdef _OPENMP
        omp_set_num_threads(prev_threads);
#endif
        return -1;
    }
    double* u1 = k + n2;
    double* u2 = u1 + n2;
    double t = t0;
    for (int64_t step = 0; step < nsteps; ++step) {
        rhs(&g, s, k, t);
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < n2; ++q) u1[q] = s[q] + dt * k[q];
        rhs(&g, u1, k, t + dt);
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < n2; ++q) u2[q] = ((3.0 * s[q] + u1[q]) + dt * k[q]) * 0.25;
        rhs(&g, u2, k, t + dt / 2);
        const double dt2 = 2.0 * dt;
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < n2; ++q) s[q] = ((s[q] + 2.0 * u2[q]) + dt2 * k[q]) / 3.0;
        t = t + dt;
    }
#ifdef _OPENMP
    omp_set_num_threads(prev_threads);
#endif
    return 0;
}

/* One right-hand side evaluation (for the parity tests). */
void bruss_rhs(int64_t nx, int64_t ny, const double* wx, const double* wy, double alpha, const double* x,
               const double* y, const double* s, double* out, double t) {
    bruss_grid g;
    g.nx = nx;
    g.ny = ny;
    memcpy(g.wx, wx, sizeof(g.wx));
    memcpy(g.wy, wy, sizeof(g.wy));
    g.alpha = alpha;
    g.x = x;
    g.y = y;
    rhs(&g, s, out, t);
}

int bruss_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
