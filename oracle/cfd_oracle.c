/*
 * cfd_oracle.c -- CPU FP64 restatement of the CFD_NSsolver_forHPC time step.
 *
 * TEST INFRASTRUCTURE ONLY: this file is the checker for the CUDA library.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * it; the product path never does.
 *
 * Each function restates one reference function and cites the file:line it
 * follows (paths relative to the reference project root).  Floating-point
 * expressions keep the reference's evaluation order; the file is compiled
 * with -ffp-contract=off so that no multiply-add is fused behind our back.
 * Reductions use a fixed blocked order (og_dot), so results do not depend on
 * the OpenMP thread count.
 *
 * Parity is pinned by oracle/build_ref.py + oracle/ref_harness.cpp (the
 * reference's own headers compiled from a patched scratch copy) and by the
 * golden fixtures under tests/golden/.
 */
#include "cfd_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define GC 2
#define OG_BLK 4096

static inline long long icel(const og_grid *g, long long i, long long j, long long k)
{
    return i * (long long)g->ny * g->nz + j * g->nz + k;
}
static inline long long icelcal(const og_grid *g, long long i, long long j, long long k)
{
    return (i - GC) * (long long)g->nyc * g->nzc + (j - GC) * g->nzc + (k - GC);
}
static inline long long n_cal(const og_grid *g)
{
    return (long long)g->nxc * g->nyc * g->nzc;
}

/* ------------------------------------------------------------------------ */
/* Deterministic blocked dot product: per-block partial sums in index order,
 * then the partials summed in block order.  Stands in for math::dot
 * (inc/solver/math.hpp:38-52), whose OpenMP reduction order is unspecified. */
double og_dot(const double *a, const double *b, long long n)
{
    long long nb = (n + OG_BLK - 1) / OG_BLK;
    if (nb == 0) return 0.0;
    double *part = (double *)malloc((size_t)nb * sizeof(double));
#pragma omp parallel for schedule(static)
    for (long long blk = 0; blk < nb; ++blk) {
        long long lo = blk * OG_BLK, hi = lo + OG_BLK < n ? lo + OG_BLK : n;
        double s = 0.0;
        for (long long i = lo; i < hi; ++i) s += a[i] * b[i];
        part[blk] = s;
    }
    double r = 0.0;
    for (long long blk = 0; blk < nb; ++blk) r += part[blk];
    free(part);
    return r;
}

/* ------------------------------------------------------------------------ */
/* grid::init_uniform (inc/grid/structureGrid.hpp:409-440) */
void og_grid_uniform(int nxc, int nyc, int nzc, double lx, double ly, double lz,
                     double *X, double *Y, double *Z, double *Dx, double *Dy, double *Dz,
                     double *Dxs, double *Dys, double *Dzs)
{
    int nx = nxc + 2 * GC, ny = nyc + 2 * GC, nz = nzc + 2 * GC;
    double dx = lx / (nx - 2.0 * GC);
    double dy = ly / (ny - 2.0 * GC);
    double dz = lz / (nz - 2.0 * GC);
    X[0] = 0.0 - 2.0 * dx;
    for (int i = 1; i < nx + 1; ++i) X[i] = X[i - 1] + dx;
    Y[0] = 0.0 - 2.0 * dy;
    for (int j = 1; j < ny + 1; ++j) Y[j] = Y[j - 1] + dy;
    Z[0] = 0.0 - 2.0 * dz;
    for (int k = 1; k < nz + 1; ++k) Z[k] = Z[k - 1] + dz;
    for (int i = 0; i < nx; ++i) { Dx[i] = dx; Dxs[i] = dx; }
    for (int j = 0; j < ny; ++j) { Dy[j] = dy; Dys[j] = dy; }
    for (int k = 0; k < nz; ++k) { Dz[k] = dz; Dzs[k] = dz; }
}

/* ------------------------------------------------------------------------ */
/* QuickUnitA (inc/source/convection_and_difussion.hpp:20-49): QUICK face
 * values along the component's own axis.  Di = cell widths, Ds = staggered
 * widths, I = index of the current face. */
static inline void quick_a(double Up, double Un, const double *phi, long long pp, long long p,
                           long long ic, long long n, long long nn, const double *Di,
                           const double *Ds, int I, double *phiP, double *phiN)
{
    if (Up > 0.0)
        *phiP = 0.5 * (phi[ic] + phi[p])
              - 0.125 * Di[I + 1] * Di[I + 1] / Ds[I]
                    * ((phi[p] - phi[ic]) / Di[I + 1] - (phi[ic] - phi[n]) / Di[I]);
    else
        *phiP = 0.5 * (phi[ic] + phi[p])
              - 0.125 * Di[I + 1] * Di[I + 1] / Ds[I + 1]
                    * ((phi[pp] - phi[p]) / Di[I + 2] - (phi[p] - phi[ic]) / Di[I + 1]);
    if (Un > 0.0)
        *phiN = 0.5 * (phi[n] + phi[ic])
              - 0.125 * Di[I] * Di[I] / Ds[I - 1]
                    * ((phi[ic] - phi[n]) / Di[I] - (phi[n] - phi[nn]) / Di[I - 1]);
    else
        *phiN = 0.5 * (phi[n] + phi[ic])
              - 0.125 * Di[I] * Di[I] / Ds[I]
                    * ((phi[p] - phi[ic]) / Di[I + 1] - (phi[ic] - phi[n]) / Di[I]);
}

/* QuickUnitB (convection_and_difussion.hpp:53-84): QUICK face values across
 * the component's axis (roles of Di and Ds exchanged). */
static inline void quick_b(double Up, double Un, const double *phi, long long pp, long long p,
                           long long ic, long long n, long long nn, const double *Di,
                           const double *Ds, int I, double *phiP, double *phiN)
{
    if (Up > 0.0)
        *phiP = 0.5 * (phi[ic] + phi[p])
              - 0.125 * Ds[I] * Ds[I] / Di[I]
                    * ((phi[p] - phi[ic]) / Ds[I] - (phi[ic] - phi[n]) / Ds[I - 1]);
    else
        *phiP = 0.5 * (phi[ic] + phi[p])
              - 0.125 * Ds[I] * Ds[I] / Di[I + 1]
                    * ((phi[pp] - phi[p]) / Ds[I + 1] - (phi[p] - phi[ic]) / Ds[I]);
    if (Un > 0.0)
        *phiN = 0.5 * (phi[n] + phi[ic])
              - 0.125 * Ds[I - 1] * Ds[I - 1] / Di[I - 1]
                    * ((phi[ic] - phi[n]) / Ds[I - 1] - (phi[n] - phi[nn]) / Ds[I - 2]);
    else
        *phiN = 0.5 * (phi[n] + phi[ic])
              - 0.125 * Ds[I - 1] * Ds[I - 1] / Di[I]
                    * ((phi[p] - phi[ic]) / Ds[I] - (phi[ic] - phi[n]) / Ds[I - 1]);
}

/* ConvectionDifussion (convection_and_difussion.hpp:168-446), QUICK scheme,
 * first-order Euler, single domain (calDomain = [2, n-2) on every axis).
 * The normal component skips its last face (d = 1, lines 193, 274, 357). */
void og_convdiff(const og_grid *g, double dt, double nu,
                 const double *u0, const double *v0, const double *w0,
                 double *u1, double *v1, double *w1)
{
    og_convdiff_les(g, dt, nu, NULL, u0, v0, w0, u1, v1, w1);
}

/* With vis != NULL the diffusion of every face of cell (i,j,k) uses
   nu + vis[icelCal(i,j,k)] (the TERBULENCE_SMAGORINSKY branches of
   convection_and_difussion.hpp:246-250, 330-334, 413-417). */
void og_convdiff_les(const og_grid *g, double dt, double nu_mol, const double *vis,
                     const double *u0, const double *v0, const double *w0,
                     double *u1, double *v1, double *w1)
{
    const int nx = g->nx, ny = g->ny, nz = g->nz;
    const long long sx = (long long)ny * nz, sy = nz, sz = 1;
    const double *Dx = g->Dx, *Dy = g->Dy, *Dz = g->Dz;
    const double *Dxs = g->Dxs, *Dys = g->Dys, *Dzs = g->Dzs;

    /* u: lines 196-269 */
#pragma omp parallel for schedule(static)
    for (int i = GC; i < nx - GC - 1; ++i)
        for (int j = GC; j < ny - GC; ++j)
            for (int k = GC; k < nz - GC; ++k) {
                long long ic = icel(g, i, j, k);
                long long xm = ic - sx, xp = ic + sx, ym = ic - sy, yp = ic + sy, zm = ic - sz,
                          zp = ic + sz;
                double IT = (Dxs[i] * 0.5) / Dx[i];
                double Up = 0.5 * (u0[xp] + u0[ic]);
                double Un = 0.5 * (u0[xm] + u0[ic]);
                double Vp = v0[ic] + (v0[xp] - v0[ic]) * IT;
                double Vn = v0[ym] + (v0[ym + sx] - v0[ym]) * IT;
                double Wp = w0[ic] + (w0[xp] - w0[ic]) * IT;
                double Wn = w0[zm] + (w0[zm + sx] - w0[zm]) * IT;
                double uPx, uNx, uPy, uNy, uPz, uNz;
                quick_a(Up, Un, u0, ic + 2 * sx, xp, ic, xm, ic - 2 * sx, Dx, Dxs, i, &uPx, &uNx);
                quick_b(Vp, Vn, u0, ic + 2 * sy, yp, ic, ym, ic - 2 * sy, Dy, Dys, j, &uPy, &uNy);
                quick_b(Wp, Wn, u0, ic + 2 * sz, zp, ic, zm, ic - 2 * sz, Dz, Dzs, k, &uPz, &uNz);
                double convection = -dt * ((uPx * uPx - uNx * uNx) / Dxs[i]
                                           + (uPy * Vp - uNy * Vn) / Dy[j]
                                           + (uPz * Wp - uNz * Wn) / Dz[k]);
                const double nu = vis ? nu_mol + vis[icelcal(g, i, j, k)] : nu_mol;
                double difussion = nu * dt
                    * (((u0[xp] - u0[ic]) / Dx[i + 1] - (u0[ic] - u0[xm]) / Dx[i]) / Dxs[i]
                       + ((u0[yp] - u0[ic]) / Dys[j] - (u0[ic] - u0[ym]) / Dys[j - 1]) / Dy[j]
                       + ((u0[zp] - u0[ic]) / Dzs[k] - (u0[ic] - u0[zm]) / Dzs[k - 1]) / Dz[k]);
                u1[ic] = u0[ic] + convection + difussion;
            }

    /* v: lines 278-351 */
#pragma omp parallel for schedule(static)
    for (int i = GC; i < nx - GC; ++i)
        for (int j = GC; j < ny - GC - 1; ++j)
            for (int k = GC; k < nz - GC; ++k) {
                long long ic = icel(g, i, j, k);
                long long xm = ic - sx, xp = ic + sx, ym = ic - sy, yp = ic + sy, zm = ic - sz,
                          zp = ic + sz;
                double IT = (Dys[j] * 0.5) / Dy[j];
                double Vp = 0.5 * (v0[yp] + v0[ic]);
                double Vn = 0.5 * (v0[ym] + v0[ic]);
                double Up = u0[ic] + (u0[yp] - u0[ic]) * IT;
                double Un = u0[xm] + (u0[xm + sy] - u0[xm]) * IT;
                double Wp = w0[ic] + (w0[yp] - w0[ic]) * IT;
                double Wn = w0[zm] + (w0[zm + sy] - w0[zm]) * IT;
                double vPx, vNx, vPy, vNy, vPz, vNz;
                quick_b(Up, Un, v0, ic + 2 * sx, xp, ic, xm, ic - 2 * sx, Dx, Dxs, i, &vPx, &vNx);
                quick_a(Vp, Vn, v0, ic + 2 * sy, yp, ic, ym, ic - 2 * sy, Dy, Dys, j, &vPy, &vNy);
                quick_b(Wp, Wn, v0, ic + 2 * sz, zp, ic, zm, ic - 2 * sz, Dz, Dzs, k, &vPz, &vNz);
                double convection = -dt * ((Up * vPx - Un * vNx) / Dx[i]
                                           + (vPy * vPy - vNy * vNy) / Dys[j]
                                           + (Wp * vPz - Wn * vNz) / Dz[k]);
                const double nu = vis ? nu_mol + vis[icelcal(g, i, j, k)] : nu_mol;
                double difussion = nu * dt
                    * (((v0[xp] - v0[ic]) / Dxs[i] - (v0[ic] - v0[xm]) / Dxs[i - 1]) / Dx[i]
                       + ((v0[yp] - v0[ic]) / Dy[j + 1] - (v0[ic] - v0[ym]) / Dy[j]) / Dys[j]
                       + ((v0[zp] - v0[ic]) / Dzs[k] - (v0[ic] - v0[zm]) / Dzs[k - 1]) / Dz[k]);
                v1[ic] = v0[ic] + convection + difussion;
            }

    /* w: lines 360-434 (periodic z: also the top face, the same face as the bottom one) */
    const int wkend = nz - GC - (g->periodic_z ? 0 : 1);
#pragma omp parallel for schedule(static)
    for (int i = GC; i < nx - GC; ++i)
        for (int j = GC; j < ny - GC; ++j)
            for (int k = GC; k < wkend; ++k) {
                long long ic = icel(g, i, j, k);
                long long xm = ic - sx, xp = ic + sx, ym = ic - sy, yp = ic + sy, zm = ic - sz,
                          zp = ic + sz;
                double IT = (Dzs[k] * 0.5) / Dz[k];
                double Wp = 0.5 * (w0[zp] + w0[ic]);
                double Wn = 0.5 * (w0[zm] + w0[ic]);
                double Up = u0[ic] + (u0[zp] - u0[ic]) * IT;
                double Un = u0[xm] + (u0[xm + sz] - u0[xm]) * IT;
                double Vp = v0[ic] + (v0[zp] - v0[ic]) * IT;
                double Vn = v0[ym] + (v0[ym + sz] - v0[ym]) * IT;
                double wPx, wNx, wPy, wNy, wPz, wNz;
                quick_b(Up, Un, w0, ic + 2 * sx, xp, ic, xm, ic - 2 * sx, Dx, Dxs, i, &wPx, &wNx);
                quick_b(Vp, Vn, w0, ic + 2 * sy, yp, ic, ym, ic - 2 * sy, Dy, Dys, j, &wPy, &wNy);
                quick_a(Wp, Wn, w0, ic + 2 * sz, zp, ic, zm, ic - 2 * sz, Dz, Dzs, k, &wPz, &wNz);
                double convection = -dt * ((Up * wPx - Un * wNx) / Dx[i]
                                           + (Vp * wPy - Vn * wNy) / Dy[j]
                                           + (wPz * wPz - wNz * wNz) / Dzs[k]);
                const double nu = vis ? nu_mol + vis[icelcal(g, i, j, k)] : nu_mol;
                double difussion = nu * dt
                    * (((w0[xp] - w0[ic]) / Dxs[i] - (w0[ic] - w0[xm]) / Dxs[i - 1]) / Dx[i]
                       + ((w0[yp] - w0[ic]) / Dys[j] - (w0[ic] - w0[ym]) / Dys[j - 1]) / Dy[j]
                       + ((w0[zp] - w0[ic]) / Dz[k + 1] - (w0[ic] - w0[zm]) / Dz[k]) / Dzs[k]);
                w1[ic] = w0[ic] + convection + difussion;
            }
}

/* ------------------------------------------------------------------------ */
/* Source coupling of the predictor-corrector driver
 * (inc/run/RUN_CPU_PC_METHOD.hpp:309-316 and 460-467).  The reference indexes
 * the GHOSTED velocity array with the compact index icelCal(i,j,k), so
 * element m of u1 receives src[m] for m in [0, N).  aligned != 0 applies the
 * source at the cell it belongs to instead. */
void og_src_add(const og_grid *g, int aligned, double *u1, double *v1, double *w1,
                const double *src)
{
    long long N = n_cal(g);
    if (!aligned) {
#pragma omp parallel for schedule(static)
        for (long long m = 0; m < N; ++m) {
            u1[m] += src[m];
            v1[m] += src[N + m];
            w1[m] += src[2 * N + m];
        }
        return;
    }
#pragma omp parallel for schedule(static)
    for (int i = GC; i < g->nx - GC; ++i)
        for (int j = GC; j < g->ny - GC; ++j)
            for (int k = GC; k < g->nz - GC; ++k) {
                long long ic = icel(g, i, j, k), m = icelcal(g, i, j, k);
                u1[ic] += src[m];
                v1[ic] += src[N + m];
                w1[ic] += src[2 * N + m];
            }
}

/* source_termF += dt * Dfib.f (RUN_CPU_PC_METHOD.hpp:393-401) */
void og_src_accumulate(const og_grid *g, double dt, double *src, const double *f)
{
    long long n3 = 3 * n_cal(g);
#pragma omp parallel for schedule(static)
    for (long long m = 0; m < n3; ++m) src[m] += dt * f[m];
}

/* ------------------------------------------------------------------------ */
/* createBMatrix_omp (inc/matrix/b_matrix.hpp:51-80), JACOBI_PC variant */
void og_rhs(const og_grid *g, double dt, const double *jp,
            const double *u1, const double *v1, const double *w1, double *b)
{
    const double ddt = 1.0 / dt;
    const long long sx = (long long)g->ny * g->nz, sy = g->nz;
#pragma omp parallel for schedule(static)
    for (int i = GC; i < g->nx - GC; ++i)
        for (int j = GC; j < g->ny - GC; ++j)
            for (int k = GC; k < g->nz - GC; ++k) {
                long long ic = icel(g, i, j, k), row = icelcal(g, i, j, k);
                b[row] = -jp[row] * ddt
                       * ((u1[ic] - u1[ic - sx]) / g->Dx[i] + (v1[ic] - v1[ic - sy]) / g->Dy[j]
                          + (w1[ic] - w1[ic - 1]) / g->Dz[k]);
            }
}

/* The reference's all-Neumann pressure system is singular and its right-hand
 * side is not compatible (zero-gradient outflow does not conserve mass), so
 * tight tolerances break down (NaN / iteration cap).  This extension builds
 * the reference RHS and then removes the volume-weighted mean of the unscaled
 * RHS d = -(1/dt) div u*:  b <- b - jp * (sum(dV d) / sum(dV)).
 * Returns the removed mean.  Not part of the reference. */
double og_rhs_compat(const og_grid *g, double dt, const double *jp,
                     const double *u1, const double *v1, const double *w1, double *b)
{
    og_rhs(g, dt, jp, u1, v1, w1, b);
    const double ddt = 1.0 / dt;
    const long long N = n_cal(g);
    const long long sx = (long long)g->ny * g->nz, sy = g->nz;
    double *dvd = (double *)malloc((size_t)N * sizeof(double));
    double *dv = (double *)malloc((size_t)N * sizeof(double));
    double *one = (double *)malloc((size_t)N * sizeof(double));
#pragma omp parallel for schedule(static)
    for (int i = GC; i < g->nx - GC; ++i)
        for (int j = GC; j < g->ny - GC; ++j)
            for (int k = GC; k < g->nz - GC; ++k) {
                long long ic = icel(g, i, j, k), row = icelcal(g, i, j, k);
                double vol = g->Dx[i] * g->Dy[j] * g->Dz[k];
                double d = -ddt * ((u1[ic] - u1[ic - sx]) / g->Dx[i]
                                   + (v1[ic] - v1[ic - sy]) / g->Dy[j]
                                   + (w1[ic] - w1[ic - 1]) / g->Dz[k]);
                dvd[row] = vol * d;
                dv[row] = vol;
                one[row] = 1.0;
            }
    double mean = og_dot(dvd, one, N) / og_dot(dv, one, N);
#pragma omp parallel for schedule(static)
    for (long long r = 0; r < N; ++r) b[r] = b[r] - jp[r] * mean;
    free(dvd);
    free(dv);
    free(one);
    return mean;
}

/* ------------------------------------------------------------------------ */
/* SPE_matrix1::setupPressure + set_Jp_pc
 * (inc/matrix/SPE_sparseMatrix1.hpp:40-121).  xm..zp have the interior
 * length of their axis; val and jp are compact (N). */
void og_spe_setup(const og_grid *g, double *xm, double *xp, double *ym, double *yp,
                  double *zm, double *zp, double *val, double *jp)
{
    const int nx = g->nxc, ny = g->nyc, nz = g->nzc;
    for (int i = 0; i < nx; ++i) {
        xp[i] = 1.0 / g->Dx[i + GC] / g->Dxs[i + GC];
        xm[i] = 1.0 / g->Dx[i + GC] / g->Dxs[i + GC - 1];
    }
    for (int j = 0; j < ny; ++j) {
        yp[j] = 1.0 / g->Dy[j + GC] / g->Dys[j + GC];
        ym[j] = 1.0 / g->Dy[j + GC] / g->Dys[j + GC - 1];
    }
    for (int k = 0; k < nz; ++k) {
        zp[k] = 1.0 / g->Dz[k + GC] / g->Dzs[k + GC];
        zm[k] = 1.0 / g->Dz[k + GC] / g->Dzs[k + GC - 1];
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                long long ic = k + (long long)j * nz + (long long)i * ny * nz;
                double ijk = xm[i] + ym[j] + zm[k] + xp[i] + yp[j] + zp[k];
                if (i == 0) ijk -= xm[i];
                if (i == nx - 1) ijk -= xp[i];
                if (j == 0) ijk -= ym[j];
                if (j == ny - 1) ijk -= yp[j];
                if (k == 0 && !g->periodic_z) ijk -= zm[k];
                if (k == nz - 1 && !g->periodic_z) ijk -= zp[k];
                val[ic] = ijk;
                jp[ic] = 1.0 / ijk;
            }
}

/* SPE_matrix1::spmv_ompJP (SPE_sparseMatrix1.hpp:126-144); periodic_z wraps
   the z neighbours of the first and last k (extension) */
static void spe_spmv_ex(int nx, int ny, int nz, const double *xm, const double *xp, const double *ym,
                        const double *yp, const double *zm, const double *zp, const double *jp,
                        const double *x, double *r, int periodic_z)
{
    const long long nynz = (long long)ny * nz;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                long long ic = k + (long long)j * nz + (long long)i * nynz;
                double sum = 0.0;
                if (i != 0) sum += -xm[i] * jp[ic] * x[ic - nynz];
                if (j != 0) sum += -ym[j] * jp[ic] * x[ic - nz];
                if (k != 0) sum += -zm[k] * jp[ic] * x[ic - 1];
                else if (periodic_z) sum += -zm[k] * jp[ic] * x[ic + nz - 1];
                sum += x[ic];
                if (k != nz - 1) sum += -zp[k] * jp[ic] * x[ic + 1];
                else if (periodic_z) sum += -zp[k] * jp[ic] * x[ic - (nz - 1)];
                if (j != ny - 1) sum += -yp[j] * jp[ic] * x[ic + nz];
                if (i != nx - 1) sum += -xp[i] * jp[ic] * x[ic + nynz];
                r[ic] = sum;
            }
}

void og_spe_spmv(int nx, int ny, int nz, const double *xm, const double *xp, const double *ym,
                 const double *yp, const double *zm, const double *zp, const double *jp,
                 const double *x, double *r)
{
    const long long nynz = (long long)ny * nz;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                long long ic = k + (long long)j * nz + (long long)i * nynz;
                double sum = 0.0;
                if (i != 0) sum += -xm[i] * jp[ic] * x[ic - nynz];
                if (j != 0) sum += -ym[j] * jp[ic] * x[ic - nz];
                if (k != 0) sum += -zm[k] * jp[ic] * x[ic - 1];
                sum += x[ic];
                if (k != nz - 1) sum += -zp[k] * jp[ic] * x[ic + 1];
                if (j != ny - 1) sum += -yp[j] * jp[ic] * x[ic + nz];
                if (i != nx - 1) sum += -xp[i] * jp[ic] * x[ic + nynz];
                r[ic] = sum;
            }
}

/* ------------------------------------------------------------------------ */
/* createPressureMatrix (inc/matrix/PressureMatrix.hpp:5-117) with all six
 * faces Neumann (P_NEUMANN.hpp), stored the way ELL_matrix::set builds it
 * (ELL_sparseMatrix.hpp:147-160, 246-320): per row 7 slots, diagonal first,
 * then -x, +x, -y, +y, -z, +z neighbours that exist, padding (col = N-1,
 * val = 0).  cols/vals are row-major [row*7 + slot] like the reference. */
void og_ell_assemble(const og_grid *g, int *cols, double *vals, double *jp)
{
    const long long N = n_cal(g);
    const int xBeg = GC, yBeg = GC, zBeg = GC;
    const int xEnd = g->nx - GC - 1, yEnd = g->ny - GC - 1, zEnd = g->nz - GC - 1;
    const double *Dx = g->Dx, *Dy = g->Dy, *Dz = g->Dz;
    const double *Dxs = g->Dxs, *Dys = g->Dys, *Dzs = g->Dzs;
#pragma omp parallel for schedule(static)
    for (int i = xBeg; i <= xEnd; ++i)
        for (int j = yBeg; j <= yEnd; ++j)
            for (int k = zBeg; k <= zEnd; ++k) {
                double xp = 1.0 / Dx[i] / Dxs[i], yp = 1.0 / Dy[j] / Dys[j],
                       zp = 1.0 / Dz[k] / Dzs[k];
                double xm = 1.0 / Dx[i] / Dxs[i - 1], ym = 1.0 / Dy[j] / Dys[j - 1],
                       zm = 1.0 / Dz[k] / Dzs[k - 1];
                double aa = 0.0, bb = 0.0, cc = 0.0;
                if (i == xBeg) aa = -xm;
                if (i == xEnd) aa = -xp;
                if (j == yBeg) bb = -ym;
                if (j == yEnd) bb = -yp;
                if (k == zBeg && !g->periodic_z) cc = -zm;
                if (k == zEnd && !g->periodic_z) cc = -zp;
                long long row = icelcal(g, i, j, k);
                double val = xm + xp + ym + yp + zm + zp + aa + bb + cc;
                double jpr = 1. / val;
                jp[row] = jpr;
                int s = 0;
                int *c = cols + row * 7;
                double *v = vals + row * 7;
                c[s] = (int)row; v[s++] = val * jpr;
                if (i != xBeg) { c[s] = (int)icelcal(g, i - 1, j, k); v[s++] = -xm * jpr; }
                if (i != xEnd) { c[s] = (int)icelcal(g, i + 1, j, k); v[s++] = -xp * jpr; }
                if (j != yBeg) { c[s] = (int)icelcal(g, i, j - 1, k); v[s++] = -ym * jpr; }
                if (j != yEnd) { c[s] = (int)icelcal(g, i, j + 1, k); v[s++] = -yp * jpr; }
                if (k != zBeg) { c[s] = (int)icelcal(g, i, j, k - 1); v[s++] = -zm * jpr; }
                else if (g->periodic_z) { c[s] = (int)icelcal(g, i, j, zEnd); v[s++] = -zm * jpr; }
                if (k != zEnd) { c[s] = (int)icelcal(g, i, j, k + 1); v[s++] = -zp * jpr; }
                else if (g->periodic_z) { c[s] = (int)icelcal(g, i, j, zBeg); v[s++] = -zp * jpr; }
                for (; s < 7; ++s) { c[s] = (int)(N - 1); v[s] = 0.0; }
            }
}

/* ELL_matrix::multiply_omp (ELL_sparseMatrix.hpp:477-492): all 7 slots,
 * padding included, accumulated in slot order. */
void og_ell_spmv(long long n, const int *cols, const double *vals, const double *x, double *r)
{
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) {
        double s = 0.0;
        for (int j = 0; j < 7; ++j) s += vals[i * 7 + j] * x[cols[i * 7 + j]];
        r[i] = s;
    }
}

/* ------------------------------------------------------------------------ */
/* bicgstabRe2 (inc/solver/bicgstabRe2.hpp:13-189).  The solver object is
 * persistent: timestep_ counts solves (restarts are only allowed from the
 * 10th solve on), px1/px2 keep the last two initial guesses for the NaN
 * reset at the iteration cap. */
struct og_bicg {
    long long n;
    int kind;
    double tol, restart_tol;
    int maxit;
    int timestep, total_iters, resets, restarts, acc_reset_members;
    double *r0, *r1, *p1, *s1, *ap, *as, *px1, *px2;
    /* operator */
    int nxc, nyc, nzc;
    const double *xm, *xp, *ym, *yp, *zm, *zp, *jp;
    const int *cols;
    const double *vals;
    int periodic_z;  /* the SPE operator wraps in z */
};

og_bicg *og_bicg_create(long long n, double tol, int maxit)
{
    og_bicg *s = (og_bicg *)calloc(1, sizeof(og_bicg));
    s->n = n;
    s->tol = tol;
    s->restart_tol = 1e-7 * tol; /* pRestartFactor_ = 1e-7, lines 39-42, 60-62 */
    s->maxit = maxit;
    double **v[8] = {&s->r0, &s->r1, &s->p1, &s->s1, &s->ap, &s->as, &s->px1, &s->px2};
    for (int q = 0; q < 8; ++q) *v[q] = (double *)calloc((size_t)n, sizeof(double));
    return s;
}

void og_bicg_destroy(og_bicg *s)
{
    if (!s) return;
    free(s->r0); free(s->r1); free(s->p1); free(s->s1);
    free(s->ap); free(s->as); free(s->px1); free(s->px2);
    free(s);
}

void og_bicg_set_spe(og_bicg *s, int nxc, int nyc, int nzc, const double *xm, const double *xp,
                     const double *ym, const double *yp, const double *zm, const double *zp,
                     const double *jp)
{
    s->kind = 0;
    s->nxc = nxc; s->nyc = nyc; s->nzc = nzc;
    s->xm = xm; s->xp = xp; s->ym = ym; s->yp = yp; s->zm = zm; s->zp = zp; s->jp = jp;
}

void og_bicg_set_ell(og_bicg *s, const int *cols, const double *vals)
{
    s->kind = 1;
    s->cols = cols;
    s->vals = vals;
}

void og_bicg_set_periodic_z(og_bicg *s, int periodic_z) { s->periodic_z = periodic_z; }

static void bicg_apply(og_bicg *s, const double *x, double *r)
{
    if (s->kind == 0)
        spe_spmv_ex(s->nxc, s->nyc, s->nzc, s->xm, s->xp, s->ym, s->yp, s->zm, s->zp, s->jp, x, r,
                    s->periodic_z);
    else
        og_ell_spmv(s->n, s->cols, s->vals, x, r);
}

void og_bicg_counters(const og_bicg *s, int *timestep, int *total_iters, int *restarts,
                      int *resets)
{
    *timestep = s->timestep;
    *total_iters = s->total_iters;
    *restarts = s->restarts;
    *resets = s->resets;
}

/* bicgstabRe2<matrixT>::solve (bicgstabRe2.hpp:93-189).  Returns 0 on
 * convergence, 1 when the iteration cap was hit. */
int og_bicg_solve(og_bicg *s, const double *b, double *x, int *iters, double *relres)
{
    const long long n = s->n;
    s->timestep++;
    double r1r0, pre_r1r0, a, w, bet, norm0 = sqrt(og_dot(b, b, n));
    bicg_apply(s, x, s->r0);
    memcpy(s->px2, s->px1, (size_t)n * sizeof(double));
    memcpy(s->px1, x, (size_t)n * sizeof(double));
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) s->r0[i] = b[i] - s->r0[i];
    memcpy(s->r1, s->r0, (size_t)n * sizeof(double));
    memcpy(s->p1, s->r0, (size_t)n * sizeof(double));
    r1r0 = og_dot(s->r1, s->r0, n);
    int numIter = 0, capped = 0;
    for (;;) {
        bicg_apply(s, s->p1, s->ap);
        a = r1r0 / og_dot(s->ap, s->r0, n);
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < n; ++i) s->s1[i] = s->r1[i] - a * s->ap[i];
        bicg_apply(s, s->s1, s->as);
        w = og_dot(s->as, s->s1, n) / og_dot(s->as, s->as, n);
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < n; ++i) {
            x[i] += a * s->p1[i] + w * s->s1[i];
            s->r1[i] = s->s1[i] - w * s->as[i];
        }
        if ((sqrt(og_dot(s->r1, s->r1, n)) / norm0) < s->tol) break;
        if (numIter >= s->maxit) {
            /* NaN/Inf reset (lines 143-163) */
            long long reset = 0;
            for (long long i = 0; i < n; ++i)
                if (isnan(x[i]) || isinf(x[i])) { x[i] = s->px1[i]; ++reset; }
            if (reset > n * 0.1) {
                memcpy(x, s->px2, (size_t)n * sizeof(double));
                s->acc_reset_members += (int)n;
                ++s->resets;
            } else if (reset != 0) {
                s->acc_reset_members += (int)reset;
                ++s->resets;
            }
            capped = 1;
            break;
        }
        pre_r1r0 = r1r0;
        r1r0 = og_dot(s->r1, s->r0, n);
        bet = (a / w) * (r1r0 / pre_r1r0);
        if (s->timestep < 10 || fabs(pre_r1r0) > s->restart_tol) {
#pragma omp parallel for schedule(static)
            for (long long i = 0; i < n; ++i) s->p1[i] = s->r1[i] + bet * (s->p1[i] - w * s->ap[i]);
        } else {
            memcpy(s->r0, s->r1, (size_t)n * sizeof(double));
            memcpy(s->p1, s->r1, (size_t)n * sizeof(double));
            ++s->restarts;
        }
        ++numIter;
        ++s->total_iters;
    }
    *iters = numIter;
    *relres = sqrt(og_dot(s->r1, s->r1, n)) / norm0;
    return capped;
}

/* ------------------------------------------------------------------------ */
/* SOR coefficients (SorPipeLine.seq.hpp:30-43, SorPipeLine.omp.hpp:34-50,
 * grid::coef structureGrid.hpp:278-287).  cf[8*row + 0..5] = face area /
 * staggered distance towards +x,-x,+y,-y,+z,-z; cf[8*row+7] = -1/sum. */
void og_sor_coef(const og_grid *g, double *cf)
{
    const double *Dx = g->Dx, *Dy = g->Dy, *Dz = g->Dz;
    const double *Dxs = g->Dxs, *Dys = g->Dys, *Dzs = g->Dzs;
#pragma omp parallel for schedule(static)
    for (int i = GC; i < g->nx - GC; ++i)
        for (int j = GC; j < g->ny - GC; ++j)
            for (int k = GC; k < g->nz - GC; ++k) {
                long long ii = icelcal(g, i, j, k);
                cf[ii * 8] = Dy[j] * Dz[k] / Dxs[i];
                cf[ii * 8 + 1] = Dy[j] * Dz[k] / Dxs[i - 1];
                cf[ii * 8 + 2] = Dx[i] * Dz[k] / Dys[j];
                cf[ii * 8 + 3] = Dx[i] * Dz[k] / Dys[j - 1];
                cf[ii * 8 + 4] = Dx[i] * Dy[j] / Dzs[k];
                cf[ii * 8 + 5] = Dx[i] * Dy[j] / Dzs[k - 1];
                double coef = Dy[j] * Dz[k] / Dxs[i] + Dy[j] * Dz[k] / Dxs[i - 1]
                            + Dx[i] * Dz[k] / Dys[j] + Dx[i] * Dz[k] / Dys[j - 1]
                            + Dx[i] * Dy[j] / Dzs[k] + Dx[i] * Dy[j] / Dzs[k - 1];
                cf[ii * 8 + 7] = -1.0 / (coef);
            }
}

/* SOR right-hand side cf[8*row+6] = mass change / dt (SorPipeLine.seq.hpp:48-60) */
void og_sor_rhs(const og_grid *g, double dt, const double *u1, const double *v1,
                const double *w1, double *cf)
{
    const double rdt = 1.0 / dt;
    const long long sx = (long long)g->ny * g->nz, sy = g->nz;
#pragma omp parallel for schedule(static)
    for (int i = GC; i < g->nx - GC; ++i)
        for (int j = GC; j < g->ny - GC; ++j)
            for (int k = GC; k < g->nz - GC; ++k) {
                long long ic = icel(g, i, j, k), ii8 = icelcal(g, i, j, k) * 8;
                double mChange = (u1[ic] - u1[ic - sx]) * g->Dy[j] * g->Dz[k]
                               + (v1[ic] - v1[ic - sy]) * g->Dx[i] * g->Dz[k]
                               + (w1[ic] - w1[ic - 1]) * g->Dx[i] * g->Dy[j];
                cf[ii8 + 6] = mChange * rdt;
            }
}

static inline double sor_cell(const og_grid *g, const double *cf, const double *p, int i,
                              int j, int k, long long *icp)
{
    const long long sx = (long long)g->ny * g->nz, sy = g->nz;
    long long ic = icel(g, i, j, k), ii8 = icelcal(g, i, j, k) * 8;
    *icp = ic;
    return (-p[ic + sx] * cf[ii8] - p[ic - sx] * cf[ii8 + 1] - p[ic + sy] * cf[ii8 + 2]
            - p[ic - sy] * cf[ii8 + 3] - p[ic + 1] * cf[ii8 + 4] - p[ic - 1] * cf[ii8 + 5]
            + cf[ii8 + 6])
         * cf[ii8 + 7];
}

/* SorPipeLine_seq sweep loop (SorPipeLine.seq.hpp:68-117): lexicographic
 * Gauss-Seidel with over-relaxation, stop on the max-norm of the change
 * (SOR_ERROR_MAXVAL, SorPipeLine.top.hpp:7); ghost pressures stay fixed
 * during the solve.  Reported iterations = sweeps - 1 as in the reference. */
void og_sor_seq(const og_grid *g, double omega, double tol, int itmax, const double *cf,
                double *p, int *iters, double *err)
{
    int it = 0;
    double residual;
    do {
        residual = 0.0;
        for (int i = GC; i < g->nx - GC; ++i)
            for (int j = GC; j < g->ny - GC; ++j)
                for (int k = GC; k < g->nz - GC; ++k) {
                    long long ic;
                    double pNEW = sor_cell(g, cf, p, i, j, k, &ic);
                    double pChange = fabs(pNEW - p[ic]);
                    p[ic] += omega * (pNEW - p[ic]);
                    if (pChange > residual) residual = pChange;
                }
        ++it;
    } while (residual > tol && it < itmax);
    *err = residual;
    *iters = it - 1;
}

/* Red-black reordering of the same sweep (new: the GPU-parallel ordering).
 * One sweep = all cells with (i+j+k) even, then all with (i+j+k) odd, same
 * update formula, same max-norm stop rule and iteration report. */
void og_sor_redblack(const og_grid *g, double omega, double tol, int itmax,
                     const double *cf, double *p, int *iters, double *err)
{
    int it = 0;
    double residual;
    do {
        residual = 0.0;
        for (int color = 0; color < 2; ++color) {
            double cres = 0.0;
#pragma omp parallel for schedule(static) reduction(max : cres)
            for (int i = GC; i < g->nx - GC; ++i)
                for (int j = GC; j < g->ny - GC; ++j) {
                    int k0 = GC + ((i + j + GC + color) & 1);
                    for (int k = k0; k < g->nz - GC; k += 2) {
                        long long ic;
                        double pNEW = sor_cell(g, cf, p, i, j, k, &ic);
                        double pChange = fabs(pNEW - p[ic]);
                        p[ic] += omega * (pNEW - p[ic]);
                        if (pChange > cres) cres = pChange;
                    }
                }
            if (cres > residual) residual = cres;
        }
        ++it;
    } while (residual > tol && it < itmax);
    *err = residual;
    *iters = it - 1;
}

/* ------------------------------------------------------------------------ */
/* Pressure_transform_X_result (inc/pressure/Transform.hpp:8-24) */
void og_pressure_transform(const og_grid *g, const double *x, double *p)
{
#pragma omp parallel for schedule(static)
    for (int i = GC; i < g->nx - GC; ++i)
        for (int j = GC; j < g->ny - GC; ++j)
            for (int k = GC; k < g->nz - GC; ++k) p[icel(g, i, j, k)] = x[icelcal(g, i, j, k)];
}

/* update_UandF_omp (inc/dfib/updateUandF.hpp:95-190): projection
 * T2 = u* - dt grad p, direct forcing u = eta*uS + (1 - eta_face)*T2 with a
 * resting body (uS = 0), forcing f = (u - T2)/dt.  Last normal face skipped. */
void og_update_uf(const og_grid *g, double dt, const double *p, const double *eta,
                  const double *u1, const double *v1, const double *w1,
                  double *u3, double *v3, double *w3, double *f)
{
    const long long N = n_cal(g);
    const long long sx = (long long)g->ny * g->nz, sy = g->nz;
    const double uS = 0.0, vS = 0.0, wS = 0.0;
#pragma omp parallel for schedule(static)
    for (int i = GC; i < g->nx - GC - 1; ++i)
        for (int j = GC; j < g->ny - GC; ++j)
            for (int k = GC; k < g->nz - GC; ++k) {
                long long ic = icel(g, i, j, k), icP = ic + sx;
                double T2u = u1[ic] - dt * (p[icP] - p[ic]) / g->Dxs[i];
                double et = eta[ic] + (eta[icP] - eta[ic]) * ((g->Dxs[i] * 0.5) / g->Dx[i]);
                u3[ic] = eta[ic] * uS + (1.0 - et) * T2u;
                f[icelcal(g, i, j, k)] = (u3[ic] - T2u) / dt;
            }
#pragma omp parallel for schedule(static)
    for (int i = GC; i < g->nx - GC; ++i)
        for (int j = GC; j < g->ny - GC - 1; ++j)
            for (int k = GC; k < g->nz - GC; ++k) {
                long long ic = icel(g, i, j, k), icP = ic + sy;
                double T2v = v1[ic] - dt * (p[icP] - p[ic]) / g->Dys[j];
                double et = eta[ic] + (eta[icP] - eta[ic]) * ((g->Dys[j] * 0.5) / g->Dy[j]);
                v3[ic] = eta[ic] * vS + (1.0 - et) * T2v;
                f[icelcal(g, i, j, k) + N] = (v3[ic] - T2v) / dt;
            }
    const int wkend = g->nz - GC - (g->periodic_z ? 0 : 1);
#pragma omp parallel for schedule(static)
    for (int i = GC; i < g->nx - GC; ++i)
        for (int j = GC; j < g->ny - GC; ++j)
            for (int k = GC; k < wkend; ++k) {
                long long ic = icel(g, i, j, k), icP = ic + 1;
                double T2w = w1[ic] - dt * (p[icP] - p[ic]) / g->Dzs[k];
                double et = eta[ic] + (eta[icP] - eta[ic]) * ((g->Dzs[k] * 0.5) / g->Dz[k]);
                w3[ic] = eta[ic] * wS + (1.0 - et) * T2w;
                f[icelcal(g, i, j, k) + 2 * N] = (w3[ic] - T2w) / dt;
            }
}

/* virtualF_Int + Delay_IO_CD_CL (inc/dfib/virtualForceIntergrator.hpp:5-37,
 * 120-127): Cd = -2 sum(f_x dV) / lz, Cl = -2 sum(f_y dV) / lz, with
 * dV = Dx*Dy*Dz (grid/Generator.hpp:47-53). */
void og_cdcl(const og_grid *g, const double *f, double *cd, double *cl)
{
    const long long N = n_cal(g);
    double *dv = (double *)malloc((size_t)N * sizeof(double));
#pragma omp parallel for schedule(static)
    for (int i = GC; i < g->nx - GC; ++i)
        for (int j = GC; j < g->ny - GC; ++j)
            for (int k = GC; k < g->nz - GC; ++k)
                dv[icelcal(g, i, j, k)] = g->Dx[i] * g->Dy[j] * g->Dz[k];
    double sx = og_dot(f, dv, N), sy = og_dot(f + N, dv, N);
    free(dv);
    *cd = -2.0 * sx / g->lz;
    *cl = -2.0 * sy / g->lz;
}

/* ------------------------------------------------------------------------ */
/* BC_staggered_main (inc/BoundaryCondition/Boundary_Condition.hpp:37-175).
 * dir/num are 6x3 row-major tables [face][component].  Normal components:
 * ghost = Dir + Num*interior; tangential: ghost = 2 Dir + (2 Num - 1)*interior.
 * The outflow/top/back faces also overwrite the last interior normal face.
 * Faces run in the order 0..5 (the reference's single-thread order; its
 * OpenMP `nowait` loops let faces 2..5 race with faces 1 and 3). */
void og_bc_main(const og_grid *g, const double *dir, const double *num,
                double *u, double *v, double *w, double *p)
{
    og_bc_main_ex(g, dir, num, u, v, w, p, 0);
}

void og_periodic_z(const og_grid *g, double *a)
{
    const int nz = g->nz, nzc = g->nzc;
    for (int i = 0; i < g->nx; ++i)
        for (int j = 0; j < g->ny; ++j) {
            a[icel(g, i, j, 0)] = a[icel(g, i, j, nzc)];
            a[icel(g, i, j, 1)] = a[icel(g, i, j, 1 + nzc)];
            a[icel(g, i, j, nz - 2)] = a[icel(g, i, j, nz - 2 - nzc)];
            a[icel(g, i, j, nz - 1)] = a[icel(g, i, j, nz - 1 - nzc)];
        }
}

void og_bc_main_ex(const og_grid *g, const double *dir, const double *num, double *u, double *v,
                   double *w, double *p, int skip_outflow)
{
    const int nx = g->nx, ny = g->ny, nz = g->nz;
#define DIR(b, c) dir[(b) * 3 + (c)]
#define NUM(b, c) num[(b) * 3 + (c)]
    for (int j = GC; j < ny - GC; ++j)
        for (int k = GC; k < nz - GC; ++k) { /* BC_0 */
            u[icel(g, 1, j, k)] = u[icel(g, 0, j, k)] = DIR(0, 0) + NUM(0, 0) * u[icel(g, 2, j, k)];
            v[icel(g, 1, j, k)] = v[icel(g, 0, j, k)] =
                DIR(0, 1) * 2. + (2.0 * NUM(0, 1) - 1.0) * v[icel(g, 2, j, k)];
            w[icel(g, 1, j, k)] = w[icel(g, 0, j, k)] =
                DIR(0, 2) * 2. + (2.0 * NUM(0, 2) - 1.0) * w[icel(g, 2, j, k)];
        }
    for (int j = GC; j < ny - GC && !skip_outflow; ++j)
        for (int k = GC; k < nz - GC; ++k) { /* BC_1 */
            u[icel(g, nx - 1, j, k)] = u[icel(g, nx - 2, j, k)] = u[icel(g, nx - 3, j, k)] =
                DIR(1, 0) + NUM(1, 0) * u[icel(g, nx - 4, j, k)];
            v[icel(g, nx - 1, j, k)] = v[icel(g, nx - 2, j, k)] =
                DIR(1, 1) * 2. + (2.0 * NUM(1, 1) - 1.0) * v[icel(g, nx - 3, j, k)];
            w[icel(g, nx - 1, j, k)] = w[icel(g, nx - 2, j, k)] =
                DIR(1, 2) * 2. + (2.0 * NUM(1, 2) - 1.0) * w[icel(g, nx - 3, j, k)];
        }
    for (int i = GC; i < nx - GC; ++i)
        for (int k = GC; k < nz - GC; ++k) { /* BC_2 */
            u[icel(g, i, 1, k)] = u[icel(g, i, 0, k)] =
                DIR(2, 0) * 2. + (2.0 * NUM(2, 0) - 1.0) * u[icel(g, i, 2, k)];
            v[icel(g, i, 1, k)] = v[icel(g, i, 0, k)] = DIR(2, 1) + NUM(2, 1) * v[icel(g, i, 2, k)];
            w[icel(g, i, 1, k)] = w[icel(g, i, 0, k)] =
                DIR(2, 2) * 2. + (2.0 * NUM(2, 2) - 1.0) * w[icel(g, i, 2, k)];
        }
    for (int i = GC; i < nx - GC; ++i)
        for (int k = GC; k < nz - GC; ++k) { /* BC_3 */
            v[icel(g, i, ny - 1, k)] = v[icel(g, i, ny - 2, k)] = v[icel(g, i, ny - 3, k)] =
                DIR(3, 1) + NUM(3, 1) * v[icel(g, i, ny - 4, k)];
            u[icel(g, i, ny - 1, k)] = u[icel(g, i, ny - 2, k)] =
                DIR(3, 0) * 2. + (2.0 * NUM(3, 0) - 1.0) * u[icel(g, i, ny - 3, k)];
            w[icel(g, i, ny - 1, k)] = w[icel(g, i, ny - 2, k)] =
                DIR(3, 2) * 2. + (2.0 * NUM(3, 2) - 1.0) * w[icel(g, i, ny - 3, k)];
        }
    for (int i = GC; i < nx - GC && !g->periodic_z; ++i)
        for (int j = GC; j < ny - GC; ++j) { /* BC_4 */
            u[icel(g, i, j, 1)] = u[icel(g, i, j, 0)] =
                DIR(4, 0) * 2. + (2.0 * NUM(4, 0) - 1.0) * u[icel(g, i, j, 2)];
            v[icel(g, i, j, 1)] = v[icel(g, i, j, 0)] =
                DIR(4, 1) * 2. + (2.0 * NUM(4, 1) - 1.0) * v[icel(g, i, j, 2)];
            w[icel(g, i, j, 1)] = w[icel(g, i, j, 0)] = DIR(4, 2) + NUM(4, 2) * w[icel(g, i, j, 2)];
        }
    for (int i = GC; i < nx - GC && !g->periodic_z; ++i)
        for (int j = GC; j < ny - GC; ++j) { /* BC_5 */
            w[icel(g, i, j, nz - 1)] = w[icel(g, i, j, nz - 2)] = w[icel(g, i, j, nz - 3)] =
                DIR(5, 2) + NUM(5, 2) * w[icel(g, i, j, nz - 4)];
            u[icel(g, i, j, nz - 1)] = u[icel(g, i, j, nz - 2)] =
                DIR(5, 0) * 2. + (2.0 * NUM(5, 0) - 1.0) * u[icel(g, i, j, nz - 3)];
            v[icel(g, i, j, nz - 1)] = v[icel(g, i, j, nz - 2)] =
                DIR(5, 1) * 2. + (2.0 * NUM(5, 1) - 1.0) * v[icel(g, i, j, nz - 3)];
        }
#undef DIR
#undef NUM
    if (g->periodic_z) { /* z faces periodic instead of BC_4 / BC_5 (extension) */
        og_periodic_z(g, u);
        og_periodic_z(g, v);
        og_periodic_z(g, w);
    }
    /* pressure ghosts: zero normal gradient (lines 145-171) */
    for (int j = GC; j < ny - GC; ++j)
        for (int k = GC; k < nz - GC; ++k) {
            p[icel(g, 1, j, k)] = p[icel(g, 0, j, k)] = p[icel(g, 2, j, k)];
            p[icel(g, nx - 2, j, k)] = p[icel(g, nx - 1, j, k)] = p[icel(g, nx - 3, j, k)];
        }
    for (int i = GC; i < nx - GC; ++i)
        for (int k = GC; k < nz - GC; ++k) {
            p[icel(g, i, 1, k)] = p[icel(g, i, 0, k)] = p[icel(g, i, 2, k)];
            p[icel(g, i, ny - 2, k)] = p[icel(g, i, ny - 1, k)] = p[icel(g, i, ny - 3, k)];
        }
    if (g->periodic_z) {
        og_periodic_z(g, p);
        return;
    }
    for (int i = GC; i < nx - GC; ++i)
        for (int j = GC; j < ny - GC; ++j) {
            p[icel(g, i, j, 1)] = p[icel(g, i, j, 0)] = p[icel(g, i, j, 2)];
            p[icel(g, i, j, nz - 2)] = p[icel(g, i, j, nz - 1)] = p[icel(g, i, j, nz - 3)];
        }
}

void og_bc_convective(const og_grid *g, double dt, double uc, const double *u0, const double *v0,
                      const double *w0, double *u3, double *v3, double *w3)
{
    const int nx = g->nx, ny = g->ny, nz = g->nz;
    const double C = uc * dt / g->Dx[nx - 3], Ct = uc * dt / g->Dxs[nx - 3];
    double qin = 0.0, qout = 0.0;
    for (int j = GC; j < ny - GC; ++j)
        for (int k = GC; k < nz - GC; ++k) {
            const long long b = icel(g, nx - 3, j, k), gc = icel(g, nx - 2, j, k);
            const double ub = u0[b] - C * (u0[b] - u0[icel(g, nx - 4, j, k)]);
            const double vg = v0[gc] - Ct * (v0[gc] - v0[b]);
            const double wg = w0[gc] - Ct * (w0[gc] - w0[b]);
            u3[b] = ub;
            v3[gc] = v3[icel(g, nx - 1, j, k)] = vg;
            w3[gc] = w3[icel(g, nx - 1, j, k)] = wg;
            const double area = g->Dy[j] * g->Dz[k];
            qin += u0[icel(g, 1, j, k)] * area;
            qout += ub * area;
        }
    const double scale = qout != 0.0 ? qin / qout : 1.0;
    for (int j = GC; j < ny - GC; ++j)
        for (int k = GC; k < nz - GC; ++k) {
            const long long b = icel(g, nx - 3, j, k);
            const double x = u3[b] * scale;
            u3[b] = u3[icel(g, nx - 2, j, k)] = u3[icel(g, nx - 1, j, k)] = x;
        }
}

/* BC_staggered_copy (inc/BoundaryCondition/updateBC.hpp:6-111): copy the
 * boundary values of the old field into the new one. */
void og_bc_copy(const og_grid *g, const double *uo, const double *vo, const double *wo,
                double *u, double *v, double *w)
{
    const int nx = g->nx, ny = g->ny, nz = g->nz;
#define CP(a, b, i, j, k) a[icel(g, i, j, k)] = b[icel(g, i, j, k)]
    for (int j = GC; j < ny - GC; ++j)
        for (int k = GC; k < nz - GC; ++k) {
            CP(u, uo, 1, j, k); CP(u, uo, 0, j, k);
            CP(v, vo, 1, j, k); CP(v, vo, 0, j, k);
            CP(w, wo, 1, j, k); CP(w, wo, 0, j, k);
            CP(u, uo, nx - 1, j, k); CP(u, uo, nx - 3, j, k); CP(u, uo, nx - 2, j, k);
            CP(v, vo, nx - 2, j, k); CP(v, vo, nx - 1, j, k);
            CP(w, wo, nx - 2, j, k); CP(w, wo, nx - 1, j, k);
        }
    for (int i = GC; i < nx - GC; ++i)
        for (int k = GC; k < nz - GC; ++k) {
            CP(u, uo, i, 1, k); CP(u, uo, i, 0, k);
            CP(v, vo, i, 1, k); CP(v, vo, i, 0, k);
            CP(w, wo, i, 1, k); CP(w, wo, i, 0, k);
            CP(u, uo, i, ny - 2, k); CP(u, uo, i, ny - 1, k);
            CP(v, vo, i, ny - 3, k); CP(v, vo, i, ny - 2, k); CP(v, vo, i, ny - 1, k);
            CP(w, wo, i, ny - 2, k); CP(w, wo, i, ny - 1, k);
        }
    for (int i = GC; i < nx - GC; ++i)
        for (int j = GC; j < ny - GC; ++j) {
            CP(u, uo, i, j, 1); CP(u, uo, i, j, 0);
            CP(v, vo, i, j, 1); CP(v, vo, i, j, 0);
            CP(w, wo, i, j, 1); CP(w, wo, i, j, 0);
            CP(u, uo, i, j, nz - 2); CP(u, uo, i, j, nz - 1);
            CP(v, vo, i, j, nz - 2); CP(v, vo, i, j, nz - 1);
            CP(w, wo, i, j, nz - 3); CP(w, wo, i, j, nz - 2); CP(w, wo, i, j, nz - 1);
        }
#undef CP
}

/* ------------------------------------------------------------------------ */
/* DFIB_CylinderZ (inc/dfib/setEta.hpp:136-204): volume fraction of a
 * z-aligned cylinder; cut cells are sampled on nsub x nsub sub-cell centres.
 * eta must be zero on entry (the driver fills it with 0, RUN_CPU_PC_METHOD.hpp:258).
 * Centre and radius are parameters here (hard-coded at setEta.hpp:145-147). */
/* Exact-area option of the cut-cell fraction (an extension: the reference
 * sub-samples nsub x nsub points).  Area of the disc of radius r centred at
 * the origin inside [x0, x1] x [y0, y1]: the integral over t of
 * (min(y1, s) - max(y0, -s))+ with s(t) = sqrt(r^2 - t^2), split where s
 * crosses |y0| or |y1|; on each piece the bounds are constants or +-s, and
 * the integral of s is S(t) = (t s(t) + r^2 asin(t / r)) / 2. */
static double disc_prim(double t, double r)
{
    const double u = fmax(-1.0, fmin(1.0, t / r));
    return 0.5 * (t * sqrt(fmax(r * r - t * t, 0.0)) + r * r * asin(u));
}

double og_disc_rect_area(double x0, double x1, double y0, double y1, double r)
{
    const double a = fmax(x0, -r), b = fmin(x1, r);
    if (!(a < b)) return 0.0;
    double t[6];
    int n = 0;
    t[n++] = a;
    t[n++] = b;
    const double ys[2] = {y0, y1};
    for (int q = 0; q < 2; ++q) {
        const double y = fabs(ys[q]);
        if (y < r) {
            const double c = sqrt(r * r - y * y);
            if (c > a && c < b) t[n++] = c;
            if (-c > a && -c < b) t[n++] = -c;
        }
    }
    for (int q = 1; q < n; ++q) /* insertion sort of at most 6 */
        for (int m = q; m > 0 && t[m - 1] > t[m]; --m) {
            const double tmp = t[m - 1];
            t[m - 1] = t[m];
            t[m] = tmp;
        }
    double area = 0.0;
    for (int q = 0; q + 1 < n; ++q) {
        const double lo = t[q], hi = t[q + 1];
        if (!(hi > lo)) continue;
        const double mid = 0.5 * (lo + hi), sm = sqrt(fmax(r * r - mid * mid, 0.0));
        const int top_s = sm < y1, bot_s = -sm > y0;
        const double top = top_s ? sm : y1, bot = bot_s ? -sm : y0;
        if (!(top > bot)) continue;
        const double is = disc_prim(hi, r) - disc_prim(lo, r);
        area += (top_s ? is : y1 * (hi - lo)) - (bot_s ? -is : y0 * (hi - lo));
    }
    return area;
}

void og_eta_cylinder_z(const og_grid *g, double cx, double cy, double radius, int nsub,
                       double *eta)
{
    if (nsub == 0) { /* exact areas, same cells and z copy as the sub-sampled form */
        const int nx = g->nx, ny = g->ny, nz = g->nz;
        for (int i = GC; i < nx - GC; ++i)
            for (int j = GC; j < ny - GC; ++j) {
                const long long ic = icel(g, i, j, 0);
                const double diagonal = sqrt(g->Dx[i] * g->Dx[i] + g->Dy[j] * g->Dy[j]) * 0.5;
                const double ex = ((g->X[i] + g->X[i + 1]) * 0.5) - cx, ey = ((g->Y[j] + g->Y[j + 1]) * 0.5) - cy;
                const double distance = sqrt(ex * ex + ey * ey);
                if (fabs(distance - radius) < diagonal) {
                    const double x0 = g->X[i] - cx, y0 = g->Y[j] - cy;
                    eta[ic] = og_disc_rect_area(x0, x0 + g->Dx[i], y0, y0 + g->Dy[j], radius) / (g->Dx[i] * g->Dy[j]);
                } else {
                    eta[ic] = distance > radius ? 0.0 : 1.0;
                }
            }
        for (int i = 0; i < nx - 1; ++i)
            for (int j = 0; j < ny - 1; ++j)
                for (int k = 1; k < nz - 1; ++k) eta[icel(g, i, j, k)] = eta[icel(g, i, j, 0)];
        return;
    }
    const int nx = g->nx, ny = g->ny, nz = g->nz;
    const double *X = g->X, *Y = g->Y, *Dx = g->Dx, *Dy = g->Dy;
    const double scale = pow((double)nsub, -2.0);
#pragma omp parallel for schedule(dynamic)
    for (int i = GC; i < nx - GC; ++i) {
        double *sdx = (double *)malloc((size_t)(nsub + 1) * sizeof(double));
        double *sdy = (double *)malloc((size_t)(nsub + 1) * sizeof(double));
        for (int j = GC; j < ny - GC; ++j) {
            long long ic = icel(g, i, j, 0);
            double diagonal = sqrt(Dx[i] * Dx[i] + Dy[j] * Dy[j]) * 0.5;
            double ex = ((X[i] + X[i + 1]) * 0.5) - cx, ey = ((Y[j] + Y[j + 1]) * 0.5) - cy;
            double distance = sqrt(ex * ex + ey * ey);
            if (fabs(distance - radius) < diagonal) {
                long long xi = 0;
                double dyg = Dy[j] / (double)nsub, dxg = Dx[i] / (double)nsub;
                for (int q = 0; q < nsub + 1; ++q) {
                    sdy[q] = Y[j] + (double)q * dyg;
                    sdx[q] = X[i] + (double)q * dxg;
                }
                for (int ii = 0; ii < nsub; ++ii)
                    for (int jj = 0; jj < nsub; ++jj) {
                        double a = (sdx[ii] + sdx[ii + 1]) * 0.5 - cx;
                        double b = (sdy[jj] + sdy[jj + 1]) * 0.5 - cy;
                        if (sqrt(a * a + b * b) <= radius) ++xi;
                    }
                eta[ic] = (double)xi * scale;
            } else if (distance > radius) {
                eta[ic] = 0.;
            } else {
                eta[ic] = 1.;
            }
        }
        free(sdx);
        free(sdy);
    }
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < ny - 1; ++j)
            for (int k = 1; k < nz - 1; ++k) eta[icel(g, i, j, k)] = eta[icel(g, i, j, 0)];
}

/* ------------------------------------------------------------------------ */
/* max over interior cells of |div u| (finite-volume divergence per unit
 * volume, the quantity createBMatrix_omp differentiates). */
double og_div_inf(const og_grid *g, const double *u, const double *v, const double *w)
{
    const long long sx = (long long)g->ny * g->nz, sy = g->nz;
    double m = 0.0;
#pragma omp parallel for schedule(static) reduction(max : m)
    for (int i = GC; i < g->nx - GC; ++i)
        for (int j = GC; j < g->ny - GC; ++j)
            for (int k = GC; k < g->nz - GC; ++k) {
                long long ic = icel(g, i, j, k);
                double d = (u[ic] - u[ic - sx]) / g->Dx[i] + (v[ic] - v[ic - sy]) / g->Dy[j]
                         + (w[ic] - w[ic - 1]) / g->Dz[k];
                d = fabs(d);
                if (d > m) m = d;
            }
    return m;
}

/* get_Cfl (analyses/cfl.hpp:3-80).  The per-cell sum starts at 0 and takes
   u/Dxs (i < nx-gC-1), v/Dys (j < ny-gC-1), w/Dzs (k < nz-gC-1) in that order. */
double og_cfl(const og_grid *g, double dt, const double *u, const double *v, const double *w,
              double *umax, double *umin, double *cfl_max)
{
    const long long n = (long long)g->nxc * g->nyc * g->nzc;
    double *c = (double *)calloc((size_t)n, sizeof(double));
    for (int i = GC; i < g->nx - GC - 1; ++i)
        for (int j = GC; j < g->ny - GC; ++j)
            for (int k = GC; k < g->nz - GC; ++k) {
                const long long ic = icel(g, i, j, k);
                c[icelcal(g, i, j, k)] += u[ic] / g->Dxs[i];
                if (u[ic] > umax[0]) umax[0] = u[ic];
                if (u[ic] < umin[0]) umin[0] = u[ic];
            }
    for (int i = GC; i < g->nx - GC; ++i)
        for (int j = GC; j < g->ny - GC - 1; ++j)
            for (int k = GC; k < g->nz - GC; ++k) {
                const long long ic = icel(g, i, j, k);
                c[icelcal(g, i, j, k)] += v[ic] / g->Dys[j];
                if (v[ic] > umax[1]) umax[1] = v[ic];
                if (v[ic] < umin[1]) umin[1] = v[ic];
            }
    for (int i = GC; i < g->nx - GC; ++i)
        for (int j = GC; j < g->ny - GC; ++j)
            for (int k = GC; k < g->nz - GC - 1; ++k) {
                const long long ic = icel(g, i, j, k);
                c[icelcal(g, i, j, k)] += w[ic] / g->Dzs[k];
                if (w[ic] > umax[2]) umax[2] = w[ic];
                if (w[ic] < umin[2]) umin[2] = w[ic];
            }
    double m = c[0];
    for (long long t = 1; t < n; ++t)
        if (c[t] > m) m = c[t];
    free(c);
    const double cfl = m * dt;
    if (cfl > *cfl_max) *cfl_max = cfl;
    return cfl;
}

/* simuClass::timestepper (simuClass.hpp:185-199) */
double og_timestepper(double re, const double *umax, const double *umin, double cfl_factor,
                      double grid_fo_factor, double dt_min)
{
    double dt = 1e10;
    for (int q = 0; q < 3; ++q) {
        const double a = cfl_factor / (re * umax[q] * umax[q]);
        if (a < dt) dt = a;
    }
    for (int q = 0; q < 3; ++q) {
        const double b = grid_fo_factor * 0.5 * re * umin[q] * umin[q];
        if (b < dt) dt = b;
    }
    if (dt < dt_min) dt = dt_min;
    return dt;
}

/* CheckSteadyStatebyMaxVal_omp (analyses/CheckSteadystate.hpp:166-215) */
void og_steady_max(const og_grid *g, const double *u0, const double *v0, const double *w0,
                   const double *u3, const double *v3, const double *w3, double *out3)
{
    const double *a[3] = {u0, v0, w0}, *b[3] = {u3, v3, w3};
    for (int q = 0; q < 3; ++q) {
        double m = 0.0;
        for (int i = GC; i < g->nx - GC; ++i)
            for (int j = GC; j < g->ny - GC; ++j)
                for (int k = GC; k < g->nz - GC; ++k) {
                    const long long ic = icel(g, i, j, k);
                    const double d = a[q][ic] - b[q][ic];
                    if (d > m) m = d;
                }
        out3[q] = m;
    }
}

/* SmagorinskyModel (source/smagorinskyModel.hpp:31-78) with GradientGauss
   (:6-27): central differences 0.5/D (phi[-] - phi[+]) with the staggered
   width along the component's own axis; temp = |2 ux^2 + vy^2 + wz^2 +
   (uy + vx)^2 + (uz + wx)^2 + (vz + wy)^2| (the factor 2 on the first term
   only, as written); vis = (Cs delta)^2 sqrt(temp), delta = (Dx Dy Dz)^(1/3),
   Cs = 0.18; vis compact (icelCal). */
void og_smagorinsky(const og_grid *g, const double *u, const double *v, const double *w, double *vis)
{
    const long long sx = (long long)g->ny * g->nz, sy = g->nz;
    const double CS = 0.18;
    for (int i = GC; i < g->nx - GC; ++i)
        for (int j = GC; j < g->ny - GC; ++j)
            for (int k = GC; k < g->nz - GC; ++k) {
                const long long ic = icel(g, i, j, k);
                const double ux = 0.5 / g->Dxs[i] * (u[ic - sx] - u[ic + sx]);
                const double uy = 0.5 / g->Dy[j] * (u[ic - sy] - u[ic + sy]);
                const double uz = 0.5 / g->Dz[k] * (u[ic - 1] - u[ic + 1]);
                const double vx = 0.5 / g->Dx[i] * (v[ic - sx] - v[ic + sx]);
                const double vy = 0.5 / g->Dys[j] * (v[ic - sy] - v[ic + sy]);
                const double vz = 0.5 / g->Dz[k] * (v[ic - 1] - v[ic + 1]);
                const double wx = 0.5 / g->Dx[i] * (w[ic - sx] - w[ic + sx]);
                const double wy = 0.5 / g->Dy[j] * (w[ic - sy] - w[ic + sy]);
                const double wz = 0.5 / g->Dzs[k] * (w[ic - 1] - w[ic + 1]);
                const double temp = fabs(2.0 * (ux * ux) + vy * vy + wz * wz + (uy + vx) * (uy + vx)
                                         + (uz + wx) * (uz + wx) + (vz + wy) * (vz + wy));
                const double delta = pow(g->Dx[i] * g->Dy[j] * g->Dz[k], 1.0 / 3.0);
                const double cd = CS * delta;
                vis[icelcal(g, i, j, k)] = cd * cd * sqrt(temp);
            }
}

/* ------------------------------------------------------------------------ */
/* Whole time step. */
struct og_sim {
    og_grid g;
    og_step_cfg cfg;
    double dir[18], num[18];
    long long ng, n;
    long long loop;
    double *fld[16];
    double *xm, *xp, *ym, *yp, *zm, *zp, *val;
    int *cols;
    double *vals, *cf;
    og_bicg *bicg;
};

og_sim *og_sim_create(const og_grid *g, const og_step_cfg *cfg, const double *dir,
                      const double *num, const double *eta)
{
    if (g->periodic_z && cfg->solver >= 2) return NULL; /* periodic z: the Krylov solvers only */
    og_sim *s = (og_sim *)calloc(1, sizeof(og_sim));
    s->g = *g;
    s->cfg = *cfg;
    memcpy(s->dir, dir, sizeof(s->dir));
    memcpy(s->num, num, sizeof(s->num));
    s->ng = (long long)g->nx * g->ny * g->nz;
    s->n = n_cal(g);
    s->loop = 1;
    for (int q = 0; q < 11; ++q) s->fld[q] = (double *)calloc((size_t)s->ng, sizeof(double));
    s->fld[11] = (double *)calloc((size_t)(3 * s->n), sizeof(double));
    s->fld[12] = (double *)calloc((size_t)(3 * s->n), sizeof(double));
    for (int q = 13; q < 16; ++q) s->fld[q] = (double *)calloc((size_t)s->n, sizeof(double));
    if (eta) memcpy(s->fld[10], eta, (size_t)s->ng * sizeof(double));
    s->xm = (double *)calloc((size_t)g->nxc, sizeof(double));
    s->xp = (double *)calloc((size_t)g->nxc, sizeof(double));
    s->ym = (double *)calloc((size_t)g->nyc, sizeof(double));
    s->yp = (double *)calloc((size_t)g->nyc, sizeof(double));
    s->zm = (double *)calloc((size_t)g->nzc, sizeof(double));
    s->zp = (double *)calloc((size_t)g->nzc, sizeof(double));
    s->val = (double *)calloc((size_t)s->n, sizeof(double));
    s->bicg = og_bicg_create(s->n, cfg->tol, cfg->maxit);
    og_bicg_set_periodic_z(s->bicg, g->periodic_z);
    if (cfg->solver == 1) {
        s->cols = (int *)calloc((size_t)(7 * s->n), sizeof(int));
        s->vals = (double *)calloc((size_t)(7 * s->n), sizeof(double));
        og_ell_assemble(&s->g, s->cols, s->vals, s->fld[15]);
        og_bicg_set_ell(s->bicg, s->cols, s->vals);
    } else {
        og_spe_setup(&s->g, s->xm, s->xp, s->ym, s->yp, s->zm, s->zp, s->val, s->fld[15]);
        og_bicg_set_spe(s->bicg, g->nxc, g->nyc, g->nzc, s->xm, s->xp, s->ym, s->yp, s->zm,
                        s->zp, s->fld[15]);
    }
    if (cfg->solver >= 2) {
        s->cf = (double *)calloc((size_t)(8 * s->n), sizeof(double));
        og_sor_coef(&s->g, s->cf);
    }
    return s;
}

void og_sim_destroy(og_sim *s)
{
    if (!s) return;
    for (int q = 0; q < 16; ++q) free(s->fld[q]);
    free(s->xm); free(s->xp); free(s->ym); free(s->yp); free(s->zm); free(s->zp);
    free(s->val); free(s->cols); free(s->vals); free(s->cf);
    og_bicg_destroy(s->bicg);
    free(s);
}

double *og_sim_field(og_sim *s, int which) { return s->fld[which]; }
long long og_sim_loop(const og_sim *s) { return s->loop; }
/* restart from fields set through og_sim_field: simuClass::loop of the next step */
void og_sim_set_loop(og_sim *s, long long loop) { s->loop = loop; }

/* Initial state (RUN_CPU_PC_METHOD.hpp:77-119): T0=T1=T3=(ui,vi,wi), p=0,
 * then the first boundary update of T0 and the copy of its boundary into T1.
 * A caller that perturbs T0 does it between og_sim_init and og_sim_start. */
void og_sim_init(og_sim *s, double ui, double vi, double wi)
{
    for (long long m = 0; m < s->ng; ++m) {
        s->fld[0][m] = ui; s->fld[1][m] = vi; s->fld[2][m] = wi;
        s->fld[9][m] = 0.0;
    }
}

void og_sim_start(og_sim *s)
{
    size_t bytes = (size_t)s->ng * sizeof(double);
    for (int c = 0; c < 3; ++c) {
        memcpy(s->fld[3 + c], s->fld[c], bytes);
        memcpy(s->fld[6 + c], s->fld[c], bytes);
    }
    og_bc_main(&s->g, s->dir, s->num, s->fld[0], s->fld[1], s->fld[2], s->fld[9]);
    og_bc_copy(&s->g, s->fld[0], s->fld[1], s->fld[2], s->fld[3], s->fld[4], s->fld[5]);
}

static void sim_pressure(og_sim *s, int *iters, double *err)
{
    const og_grid *g = &s->g;
    double **F = s->fld;
    if (s->cfg.solver <= 1) {
        if (s->cfg.compat)
            og_rhs_compat(g, s->cfg.dt, F[15], F[3], F[4], F[5], F[14]);
        else
            og_rhs(g, s->cfg.dt, F[15], F[3], F[4], F[5], F[14]);
        og_bicg_solve(s->bicg, F[14], F[13], iters, err);
        og_pressure_transform(g, F[13], F[9]);
    } else {
        og_sor_rhs(g, s->cfg.dt, F[3], F[4], F[5], s->cf);
        if (s->cfg.solver == 2)
            og_sor_seq(g, s->cfg.omega, s->cfg.tol, s->cfg.sor_maxit, s->cf, F[9], iters, err);
        else
            og_sor_redblack(g, s->cfg.omega, s->cfg.tol, s->cfg.sor_maxit, s->cf, F[9], iters,
                            err);
    }
}

/* One iteration of the main loop.  method 0 follows
 * runSeqOmp_predictionMethod (RUN_CPU_PC_METHOD.hpp:287-627): three
 * predictor passes that accumulate the forcing into a source term, then the
 * final pass; method 1 follows runSeqOmp (RUN_CPU.hpp:290-462).  The
 * pressure is not solved in the first step (pLoopIni = 1). */
int og_sim_step(og_sim *s, int *iters4, double *err4, double *cd, double *cl)
{
    const og_grid *g = &s->g;
    double **F = s->fld;
    const double dt = s->cfg.dt;
    int npass = s->cfg.method == 0 ? 4 : 1;
    if (s->cfg.method == 0) memset(F[12], 0, (size_t)(3 * s->n) * sizeof(double));
    for (int pass = 0; pass < npass; ++pass) {
        int it = 0;
        double er = 0.0;
        og_convdiff(g, dt, s->cfg.nu, F[0], F[1], F[2], F[3], F[4], F[5]);
        if (s->cfg.method == 0) og_src_add(g, s->cfg.aligned_src, F[3], F[4], F[5], F[12]);
        if (g->periodic_z) /* the divergence at the first cell reads w on face 1 = face nz-3 */
            for (int c = 3; c < 6; ++c) og_periodic_z(g, F[c]);
        if (s->loop > 1) sim_pressure(s, &it, &er);
        if (g->periodic_z) og_periodic_z(g, F[9]); /* the top w face's gradient reads p above it */
        og_update_uf(g, dt, F[9], F[10], F[3], F[4], F[5], F[6], F[7], F[8], F[11]);
        if (s->cfg.method == 0 && pass < 3) og_src_accumulate(g, dt, F[12], F[11]);
        if (iters4) iters4[pass] = it;
        if (err4) err4[pass] = er;
    }
    size_t bytes = (size_t)s->ng * sizeof(double);
    const int conv = s->cfg.conv_uc > 0.0;
    if (conv) og_bc_convective(g, dt, s->cfg.conv_uc, F[0], F[1], F[2], F[6], F[7], F[8]);
    for (int c = 0; c < 3; ++c) memcpy(F[c], F[6 + c], bytes);
    og_bc_main_ex(g, s->dir, s->num, F[0], F[1], F[2], F[9], conv);
    og_bc_copy(g, F[0], F[1], F[2], F[3], F[4], F[5]);
    og_cdcl(g, F[11], cd, cl);
    s->loop++;
    return 0;
}
