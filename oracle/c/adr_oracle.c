/* CPU restatement of the 3-D advection-diffusion-reaction semi-discretisation and its
 * fixed-step SSPRK33 solve, in C with OpenMP: the timed CPU baseline and reference arm of
 * the 3-D workload (test infrastructure; the product never links it).
 *
 * The system (one field u on [0,1]^3, x and y periodic, z Dirichlet u = 0):
 *   du = Dx(K Dx u) + Dy(K Dy u) + Dz(K Dz u) + cmix Dx(Dy(u)) - cx Dx(u) - cy Dy(u) - lam u^2
 * discretised as MethodOfLines does it:
 *  - each Dj(K Dj u) by cartesian_nonlinear_laplacian (nonlinear_laplacian.jl:28-103): the
 *    outer half-offset first derivative over the two half points around the cell,
 *    wo[0] F(I - 1/2) + wo[1] F(I + 1/2), F = K(x~) (wi[0] u[Ih] + wi[1] u[Ih + 1]) with the
 *    inner half-offset first derivative wi (half_offset_centred_difference.jl:9-37) and K at
 *    the interpolated half-point coordinate x~ (nonlinear_laplacian.jl:74-83), which the
 *    caller passes as one array per dimension (K_j, one value per face of every line);
 *  - cmix Dx(Dy(u)) by mixed_central_difference (2nd_order_mixed_deriv.jl:5-22): the sum over
 *    the 3 x 3 tap pairs of (wmx[a] wmy[b]) u[i + a - 1, j + b - 1] (zero products skipped),
 *    both dimensions wrapped;
 *  - the first-order advection terms by upwinding (upwind_difference.jl:184-199): with the
 *    left-hand-side coefficient cx > 0 the backward stencil, wbx[0] u[i-1] + wbx[1] u[i];
 *  - the periodic unknowns are points 2..l (u[1] == u[l], interface_boundary.jl:33-42); the
 *    Dirichlet boundary points along z hold the observed value 0 (generate_bc_eqs.jl:238-328);
 *  - terms summed left to right in the equation's order, as the numpy oracle does;
 *  - SSPRK33 in OrdinaryDiffEq's evaluation order (see bruss_oracle.c).
 *
 * Layout: x fastest, then y, then z (nx * ny * nz doubles).  Face arrays:
 *   Kx[f + (nx+1) (j + ny k)], Ky[i + nx (f + (ny+1) k)], Kz[i + nx (j + ny f)],
 * f = 0 the left face of the first cell.
 */
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int64_t nx, ny, nz;
    double wi[3][2], wo[3][2];   /* inner and outer half-offset first-derivative weights     */
    double wmx[3], wmy[3];       /* centered first-derivative weights of the mixed term      */
    double wbx[2], wby[2];       /* backward first-order upwind weights (taps -1, 0)         */
    double cmix, cx, cy, lam;
    const double* K[3];
} adr_grid;

static void rhs(const adr_grid* g, const double* u, double* out) {
    const int64_t nx = g->nx, ny = g->ny, nz = g->nz;
    const int64_t sy = nx, sz = nx * ny;
    double wab[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) wab[a][b] = g->wmx[a] * g->wmy[b];
    const double* Kx = g->K[0];
    const double* Ky = g->K[1];
    const double* Kz = g->K[2];
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < nz; ++k) {
        for (int64_t j = 0; j < ny; ++j) {
            const int64_t jm = j == 0 ? ny - 1 : j - 1, jp = j == ny - 1 ? 0 : j + 1;
            const int64_t jj[3] = {jm, j, jp};
            for (int64_t i = 0; i < nx; ++i) {
                const int64_t im = i == 0 ? nx - 1 : i - 1, ip = i == nx - 1 ? 0 : i + 1;
                const int64_t ii[3] = {im, i, ip};
                const int64_t c = i + sy * j + sz * k;
                const double uc = u[c];
                /* x: faces i (left) and i + 1 (right) */
                const double fxl = Kx[i + (nx + 1) * (j + ny * k)] *
                                   (g->wi[0][0] * u[im + sy * j + sz * k] + g->wi[0][1] * uc);
                const double fxr = Kx[i + 1 + (nx + 1) * (j + ny * k)] *
                                   (g->wi[0][0] * uc + g->wi[0][1] * u[ip + sy * j + sz * k]);
                const double tx = g->wo[0][0] * fxl + g->wo[0][1] * fxr;
                const double fyl = Ky[i + nx * (j + (ny + 1) * k)] *
                                   (g->wi[1][0] * u[i + sy * jm + sz * k] + g->wi[1][1] * uc);
                const double fyr = Ky[i + nx * (j + 1 + (ny + 1) * k)] *
                                   (g->wi[1][0] * uc + g->wi[1][1] * u[i + sy * jp + sz * k]);
                const double ty = g->wo[1][0] * fyl + g->wo[1][1] * fyr;
                const double ulo = k == 0 ? 0.0 : u[c - sz];
                const double uhi = k == nz - 1 ? 0.0 : u[c + sz];
                const double fzl = Kz[i + nx * (j + ny * k)] * (g->wi[2][0] * ulo + g->wi[2][1] * uc);
                const double fzr = Kz[i + nx * (j + ny * (k + 1))] * (g->wi[2][0] * uc + g->wi[2][1] * uhi);
                const double tz = g->wo[2][0] * fzl + g->wo[2][1] * fzr;
                double mixed = 0.0;
                int started = 0;
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) {
                        if (wab[a][b] == 0.0) continue;
                        const double term = wab[a][b] * u[ii[a] + sy * jj[b] + sz * k];
                        mixed = started ? mixed + term : term;
                        started = 1;
                    }
                const double ax = g->wbx[0] * u[im + sy * j + sz * k] + g->wbx[1] * uc;
                const double ay = g->wby[0] * u[i + sy * jm + sz * k] + g->wby[1] * uc;
                double acc = tx + ty;
                acc = acc + tz;
                acc = acc + g->cmix * mixed;
                acc = acc + -(g->cx * ax);
                acc = acc + -(g->cy * ay);
                acc = acc + -(g->lam * (uc * uc));
                out[c] = acc;
            }
        }
    }
}

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

static void fill(adr_grid* g, const int64_t* n, const double* wi, const double* wo, const double* wm,
                 const double* wb, const double* coef, const double* Kx, const double* Ky, const double* Kz) {
    g->nx = n[0];
    g->ny = n[1];
    g->nz = n[2];
    for (int d = 0; d < 3; ++d)
        for (int q = 0; q < 2; ++q) {
            g->wi[d][q] = wi[2 * d + q];
            g->wo[d][q] = wo[2 * d + q];
        }
    memcpy(g->wmx, wm, 3 * sizeof(double));
    memcpy(g->wmy, wm + 3, 3 * sizeof(double));
    memcpy(g->wbx, wb, 2 * sizeof(double));
    memcpy(g->wby, wb + 2, 2 * sizeof(double));
    g->cmix = coef[0];
    g->cx = coef[1];
    g->cy = coef[2];
    g->lam = coef[3];
    g->K[0] = Kx;
    g->K[1] = Ky;
    g->K[2] = Kz;
}

/* One right-hand side evaluation.  n: unknowns per dimension; wi, wo: 3 x 2 weights;
 * wm: the x then y centered weights (3 each); wb: x then y backward weights (2 each);
 * coef: cmix, cx, cy, lambda. */
void adr_rhs(const int64_t* n, const double* wi, const double* wo, const double* wm, const double* wb,
             const double* coef, const double* Kx, const double* Ky, const double* Kz, const double* u,
             double* out) {
    adr_grid g;
    fill(&g, n, wi, wo, wm, wb, coef, Kx, Ky, Kz);
    rhs(&g, u, out);
}

/* nsteps SSPRK33 steps of size dt, in place on s.  nthreads <= 0 keeps the OpenMP default.
 * Returns 0, or -1 when scratch memory cannot be allocated. */
int adr_ssprk33(const int64_t* n, const double* wi, const double* wo, const double* wm, const double* wb,
                const double* coef, const double* Kx, const double* Ky, const double* Kz, double* s, double dt,
                int64_t nsteps, int nthreads) {
    adr_grid g;
    fill(&g, n, wi, wo, wm, wb, coef, Kx, Ky, Kz);
#ifdef _OPENMP
    const int prev_threads = omp_get_max_threads();   /* restored on return */
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    const int64_t m = n[0] * n[1] * n[2];
    double* k = scratch(3 * (size_t)m);
    if (!k) {
#ifdef _OPENMP
        omp_set_num_threads(prev_threads);
#endif
        return -1;
    }
    double* u1 = k + m;
    double* u2 = u1 + m;
    for (int64_t step = 0; step < nsteps; ++step) {
        rhs(&g, s, k);
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < m; ++q) u1[q] = s[q] + dt * k[q];
        rhs(&g, u1, k);
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < m; ++q) u2[q] = ((3.0 * s[q] + u1[q]) + dt * k[q]) * 0.25;
        rhs(&g, u2, k);
        const double dt2 = 2.0 * dt;
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < m; ++q) s[q] = ((s[q] + 2.0 * u2[q]) + dt2 * k[q]) / 3.0;
    }
#ifdef _OPENMP
    omp_set_num_threads(prev_threads);
#endif
    return 0;
}
