// poisson.cu -- pressure Poisson solve on the device: operator assembly
// (matrix-free SPE_matrix1 and device-resident ELL), SpMV, the BiCGSTAB of
// bicgstabRe2 split into fused kernels with device-resident scalars, the
// red-black SOR of SorPipeLine, and the FP64 residual / correction kernels of
// the mixed-precision defect correction.
//
// Every reducing kernel uses the deterministic last-block reduction of
// cfd_internal.cuh and a fixed launch shape, so a solve is bitwise
// reproducible run to run.  Kernels of an iteration return at once when the
// solve has finished (BicgScal::done), so the host may queue iterations
// ahead of the convergence test.
#include <cstdlib>

#include "cfd_internal.cuh"
#include "kernels.h"

namespace cfd {

// ---------------------------------------------------------------------------
// operator application
template <class V>
__device__ __forceinline__ void decompose(const SpeOp<V> &A, long long row, int &i, int &j, int &k)
{
    const unsigned int r = (unsigned int)row;
    const unsigned int ii = A.fsxc.div(r);
    const unsigned int rem = r - ii * (unsigned int)A.sxc;
    const unsigned int jj = A.fnzc.div(rem);
    i = (int)ii;
    j = (int)jj;
    k = (int)(rem - jj * (unsigned int)A.nzc);
}

template <class V>
__device__ __forceinline__ V apply_row(const SpeOp<V> &A, const V *__restrict__ x, long long row)
{
    int i, j, k;
    decompose(A, row, i, j, k);
    const long long xw = i > 0 ? row - A.sxc : row;
    const long long xe = i < A.nxc - 1 ? row + A.sxc : row;
    const long long ys = j > 0 ? row - A.nzc : row;
    const long long yn = j < A.nyc - 1 ? row + A.nzc : row;
    const long long zb = k > 0 ? row - 1 : (A.pz ? row + (A.nzc - 1) : row);
    const long long zt = k < A.nzc - 1 ? row + 1 : (A.pz ? row - (A.nzc - 1) : row);
    V s = __ldg(A.cxm + i) * x[xw];
    s = fma(__ldg(A.cym + j), x[ys], s);
    s = fma(__ldg(A.czm + k), x[zb], s);
    s = fma(__ldg(A.czp + k), x[zt], s);
    s = fma(__ldg(A.cyp + j), x[yn], s);
    s = fma(__ldg(A.cxp + i), x[xe], s);
    return fma(-A.jp[row], s, x[row]);
}

template <class V>
__device__ __forceinline__ V apply_row(const EllOp<V> &A, const V *__restrict__ x, long long row)
{
    V s = V(0);
#pragma unroll
    for (int q = 0; q < 7; ++q) {
        const long long o = (long long)q * A.n + row;
        s = fma(__ldg(A.vals + o), x[__ldg(A.cols + o)], s);
    }
    return s;
}

// Same operator with the x values supplied by a functor (used by the fused
// kernels that form their input vector on the fly) and, when A.jp is null,
// the Jacobi scale recomputed as 1 / (sum of the present coefficients): the
// diagonal of SPE_matrix1 (SPE_sparseMatrix1.hpp:86-96).
template <class V, class F>
__device__ __forceinline__ V apply_row_f(const SpeOp<V> &A, long long row, F &&xat)
{
    int i, j, k;
    decompose(A, row, i, j, k);
    const long long xw = i > 0 ? row - A.sxc : row;
    const long long xe = i < A.nxc - 1 ? row + A.sxc : row;
    const long long ys = j > 0 ? row - A.nzc : row;
    const long long yn = j < A.nyc - 1 ? row + A.nzc : row;
    const long long zb = k > 0 ? row - 1 : (A.pz ? row + (A.nzc - 1) : row);
    const long long zt = k < A.nzc - 1 ? row + 1 : (A.pz ? row - (A.nzc - 1) : row);
    const V cxm = __ldg(A.cxm + i), cxp = __ldg(A.cxp + i), cym = __ldg(A.cym + j), cyp = __ldg(A.cyp + j);
    const V czm = __ldg(A.czm + k), czp = __ldg(A.czp + k);
    V s = cxm * xat(xw);
    s = fma(cym, xat(ys), s);
    s = fma(czm, xat(zb), s);
    s = fma(czp, xat(zt), s);
    s = fma(cyp, xat(yn), s);
    s = fma(cxp, xat(xe), s);
    const V jp = A.jp ? A.jp[row] : V(1) / (((((cxm + cxp) + cym) + cyp) + czm) + czp);
    return fma(-jp, s, xat(row));
}

template <class Op>
__global__ void __launch_bounds__(kBlock) k_apply(Op A, const double *__restrict__ x, double *__restrict__ r)
{
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < A.n;
         row += (long long)gridDim.x * blockDim.x)
        r[row] = apply_row(A, x, row);
}

// ---------------------------------------------------------------------------
// SPE_matrix1::setupPressure + set_Jp_pc (SPE_sparseMatrix1.hpp:40-121).
// c{x,y,z} hold [minus-face | plus-face] coefficients of interior length,
// zeroed where the neighbour does not exist; jp = 1/diag with the
// reference's summation order, so it is bitwise the reference's jp.
__device__ __forceinline__ double inv2(double a, double b) { return __ddiv_rn(__ddiv_rn(1.0, a), b); }

// periodic (z of a periodic context): the first cell's minus face and the
// last cell's plus face couple across the period
__global__ void k_spe_axes(int n, const double *__restrict__ D, const double *__restrict__ Ds,
                           double *__restrict__ c, int periodic)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    c[i] = (i == 0 && !periodic) ? 0.0 : inv2(D[i + GC], Ds[i + GC - 1]);
    c[n + i] = (i == n - 1 && !periodic) ? 0.0 : inv2(D[i + GC], Ds[i + GC]);
}

__global__ void k_spe_jp(Geo g, const double *__restrict__ Dx, const double *__restrict__ Dy,
                         const double *__restrict__ Dz, const double *__restrict__ Dxs,
                         const double *__restrict__ Dys, const double *__restrict__ Dzs,
                         double *__restrict__ jp)
{
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < g.n;
         row += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(row / g.sxc);
        const long long rem = row - (long long)i * g.sxc;
        const int j = (int)(rem / g.nzc), k = (int)(rem - (long long)j * g.nzc);
        const double xm = inv2(Dx[i + GC], Dxs[i + GC - 1]), xp = inv2(Dx[i + GC], Dxs[i + GC]);
        const double ym = inv2(Dy[j + GC], Dys[j + GC - 1]), yp = inv2(Dy[j + GC], Dys[j + GC]);
        const double zm = inv2(Dz[k + GC], Dzs[k + GC - 1]), zp = inv2(Dz[k + GC], Dzs[k + GC]);
        double v = __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(xm, ym), zm), xp), yp), zp);
        if (i == 0) v = __dsub_rn(v, xm);
        if (i == g.nxc - 1) v = __dsub_rn(v, xp);
        if (j == 0) v = __dsub_rn(v, ym);
        if (j == g.nyc - 1) v = __dsub_rn(v, yp);
        if (k == 0 && !g.pz) v = __dsub_rn(v, zm);
        if (k == g.nzc - 1 && !g.pz) v = __dsub_rn(v, zp);
        jp[row] = __ddiv_rn(1.0, v);
    }
}

void launch_spe_setup(cudaStream_t s, const Geo &g, const double *Dx, const double *Dy,
                      const double *Dz, const double *Dxs, const double *Dys, const double *Dzs,
                      double *cx, double *cy, double *cz, double *jp)
{
    k_spe_axes<<<(g.nxc + 127) / 128, 128, 0, s>>>(g.nxc, Dx, Dxs, cx, 0);
    k_spe_axes<<<(g.nyc + 127) / 128, 128, 0, s>>>(g.nyc, Dy, Dys, cy, 0);
    k_spe_axes<<<(g.nzc + 127) / 128, 128, 0, s>>>(g.nzc, Dz, Dzs, cz, g.pz);
    k_spe_jp<<<blocks_for(g.n, 65536), kBlock, 0, s>>>(g, Dx, Dy, Dz, Dxs, Dys, Dzs, jp);
}

// createPressureMatrix (PressureMatrix.hpp:5-117) + ELL_matrix::set
// (ELL_sparseMatrix.hpp:246-320) assembled on the device, one row per
// thread: slot 0 = diagonal val*jp, then the -x,+x,-y,+y,-z,+z neighbours
// that exist, then padding (col = N-1, val = 0).  Stored slot-major.
__global__ void k_ell_assemble(Geo g, const double *__restrict__ Dx, const double *__restrict__ Dy,
                               const double *__restrict__ Dz, const double *__restrict__ Dxs,
                               const double *__restrict__ Dys, const double *__restrict__ Dzs,
                               int *__restrict__ cols, double *__restrict__ vals, double *__restrict__ jp)
{
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < g.n;
         row += (long long)gridDim.x * blockDim.x) {
        const int ic = (int)(row / g.sxc);
        const long long rem = row - (long long)ic * g.sxc;
        const int jc = (int)(rem / g.nzc), kc = (int)(rem - (long long)jc * g.nzc);
        const int i = ic + GC, j = jc + GC, k = kc + GC;
        const double xp = inv2(Dx[i], Dxs[i]), yp = inv2(Dy[j], Dys[j]), zp = inv2(Dz[k], Dzs[k]);
        const double xm = inv2(Dx[i], Dxs[i - 1]), ym = inv2(Dy[j], Dys[j - 1]), zm = inv2(Dz[k], Dzs[k - 1]);
        double aa = 0.0, bb = 0.0, cc = 0.0;
        if (ic == 0) aa = -xm;
        if (ic == g.nxc - 1) aa = -xp;
        if (jc == 0) bb = -ym;
        if (jc == g.nyc - 1) bb = -yp;
        if (kc == 0 && !g.pz) cc = -zm;
        if (kc == g.nzc - 1 && !g.pz) cc = -zp;
        double v = __dadd_rn(xm, xp);
        v = __dadd_rn(v, ym); v = __dadd_rn(v, yp); v = __dadd_rn(v, zm); v = __dadd_rn(v, zp);
        v = __dadd_rn(v, aa); v = __dadd_rn(v, bb); v = __dadd_rn(v, cc);
        const double jr = __ddiv_rn(1., v);
        jp[row] = jr;
        int c[7];
        double w[7];
        int s = 0;
        c[s] = (int)row; w[s++] = __dmul_rn(v, jr);
        if (ic != 0) { c[s] = (int)(row - g.sxc); w[s++] = __dmul_rn(-xm, jr); }
        if (ic != g.nxc - 1) { c[s] = (int)(row + g.sxc); w[s++] = __dmul_rn(-xp, jr); }
        if (jc != 0) { c[s] = (int)(row - g.nzc); w[s++] = __dmul_rn(-ym, jr); }
        if (jc != g.nyc - 1) { c[s] = (int)(row + g.nzc); w[s++] = __dmul_rn(-yp, jr); }
        if (kc != 0) { c[s] = (int)(row - 1); w[s++] = __dmul_rn(-zm, jr); }
        else if (g.pz) { c[s] = (int)(row + g.nzc - 1); w[s++] = __dmul_rn(-zm, jr); }
        if (kc != g.nzc - 1) { c[s] = (int)(row + 1); w[s++] = __dmul_rn(-zp, jr); }
        else if (g.pz) { c[s] = (int)(row - (g.nzc - 1)); w[s++] = __dmul_rn(-zp, jr); }
        for (; s < 7; ++s) { c[s] = (int)(g.n - 1); w[s] = 0.0; }
#pragma unroll
        for (int q = 0; q < 7; ++q) {
            cols[(long long)q * g.n + row] = c[q];
            vals[(long long)q * g.n + row] = w[q];
        }
    }
}

void launch_ell_assemble(cudaStream_t s, const Geo &g, const double *Dx, const double *Dy,
                         const double *Dz, const double *Dxs, const double *Dys, const double *Dzs,
                         int *cols, double *vals, double *jp)
{
    k_ell_assemble<<<blocks_for(g.n, 65536), kBlock, 0, s>>>(g, Dx, Dy, Dz, Dxs, Dys, Dzs, cols, vals, jp);
}

template <class Op>
void launch_apply(cfd_launch_ctx &c, const Op &A, const double *x, double *r)
{
    k_apply<Op><<<blocks_for(A.n, c.grid_cap), kBlock, 0, c.s>>>(A, x, r);
}
template void launch_apply<SpeOp<double>>(cfd_launch_ctx &, const SpeOp<double> &, const double *, double *);
template void launch_apply<EllOp<double>>(cfd_launch_ctx &, const EllOp<double> &, const double *, double *);

// ---------------------------------------------------------------------------
// BiCGSTAB (bicgstabRe2.hpp:93-189).
//
// init      r0 = b - A x; px2 = px1; px1 = x; r1 = p1 = r0;
//           norm0 = |b|, rho = r1.r0                              (lines 98-115)
// per iteration
//   ap      ap = A p1; alpha = rho / (ap.r0)                      (120-121)
//   s       s = r1 - alpha ap                                     (122-124)
//   as      as = A s;  omega = (as.s)/(as.as)                     (126-128)
//   xr      x += alpha p1 + omega s; r1 = s - omega as;
//           stop if |r1|/norm0 < tol; cap at maxit;
//           rho' = r1.r0; beta = (alpha/omega)(rho'/rho);
//           restart decision                                      (130-171)
//   p       p1 = r1 + beta (p1 - omega ap)  or restart r0=p1=r1   (172-182)
template <class Op, class V>
__global__ void __launch_bounds__(kBlock)
k_bicg_init(Op A, const V *__restrict__ b, V *__restrict__ x, V *__restrict__ r0, V *__restrict__ r1,
            V *__restrict__ p1, V *__restrict__ px1, V *__restrict__ px2, BicgScal *sc,
            double *partials, unsigned int *counter)
{
    double acc[2] = {0.0, 0.0};
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < A.n;
         row += (long long)gridDim.x * blockDim.x) {
        const V bb = b[row];
        const V r = bb - apply_row(A, x, row);
        r0[row] = r;
        r1[row] = r;
        p1[row] = r;
        if (px1) {
            px2[row] = px1[row];
            px1[row] = x[row];
        }
        acc[0] += (double)bb * (double)bb;
        acc[1] += (double)r * (double)r;
    }
    double tot[2];
    if (grid_reduce<2>(acc, partials, counter, tot) && threadIdx.x == 0) {
        sc->norm0 = sqrt(tot[0]);
        sc->rho = tot[1];
        sc->r0n2 = tot[1];
        sc->iter = 0;
        sc->restart = 0;
        sc->nonfinite = 0;
        sc->timestep += 1;
        sc->done = tot[0] == 0.0 ? BICG_ZERO_RHS : BICG_RUNNING;
        sc->relres = tot[0] == 0.0 ? 0.0 : sqrt(tot[1]) / sc->norm0;
    }
}

template <class Op, class V>
__global__ void __launch_bounds__(kBlock)
k_bicg_ap(Op A, const V *__restrict__ p1, const V *__restrict__ r0, V *__restrict__ ap, BicgScal *sc,
          double *partials, unsigned int *counter)
{
    if (sc->done) return;
    V pa = V(0);
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < A.n;
         row += (long long)gridDim.x * blockDim.x) {
        const V a = apply_row(A, p1, row);
        ap[row] = a;
        pa = fma(a, r0[row], pa);
    }
    double acc[1] = {(double)pa}, tot[1];
    if (grid_reduce<1>(acc, partials, counter, tot) && threadIdx.x == 0) sc->alpha = sc->rho / tot[0];
}

template <class V>
__global__ void __launch_bounds__(kBlock)
k_bicg_s(long long n, const V *__restrict__ r1, const V *__restrict__ ap, V *__restrict__ s1,
         const BicgScal *sc)
{
    if (sc->done) return;
    const V alpha = (V)sc->alpha;
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < n;
         row += (long long)gridDim.x * blockDim.x)
        s1[row] = fma(-alpha, ap[row], r1[row]);
}

template <class Op, class V>
__global__ void __launch_bounds__(kBlock)
k_bicg_as(Op A, const V *__restrict__ s1, V *__restrict__ as, BicgScal *sc, double *partials,
          unsigned int *counter)
{
    if (sc->done) return;
    V pa0 = V(0), pa1 = V(0);
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < A.n;
         row += (long long)gridDim.x * blockDim.x) {
        const V a = apply_row(A, s1, row);
        as[row] = a;
        pa0 = fma(a, s1[row], pa0);
        pa1 = fma(a, a, pa1);
    }
    double acc[2] = {(double)pa0, (double)pa1}, tot[2];
    if (grid_reduce<2>(acc, partials, counter, tot) && threadIdx.x == 0) sc->omega = tot[0] / tot[1];
}

template <class V>
__global__ void __launch_bounds__(kBlock)
k_bicg_xr(long long n, V *__restrict__ x, const V *__restrict__ p1, const V *__restrict__ s1,
          const V *__restrict__ as, const V *__restrict__ r0, V *__restrict__ r1, BicgScal *sc,
          double *partials, unsigned int *counter)
{
    if (sc->done) return;
    const V alpha = (V)sc->alpha, omega = (V)sc->omega;
    V pa0 = V(0), pa1 = V(0);
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < n;
         row += (long long)gridDim.x * blockDim.x) {
        const V s = s1[row];
        x[row] = fma(omega, s, fma(alpha, p1[row], x[row]));  // x + alpha p + omega s, 2 FMA
        const V r = fma(-omega, as[row], s);
        r1[row] = r;
        pa0 = fma(r, r, pa0);
        pa1 = fma(r, r0[row], pa1);
    }
    double acc[2] = {(double)pa0, (double)pa1}, tot[2];
    if (grid_reduce<2>(acc, partials, counter, tot) && threadIdx.x == 0) {
        const double rel = sqrt(tot[0]) / sc->norm0;
        sc->relres = rel;
        if (rel < sc->tol) {
            sc->done = BICG_CONVERGED;
        } else if (sc->iter >= sc->maxit) {
            sc->done = BICG_CAPPED;
        } else {
            const double pre = sc->rho;
            int restart;
            if (sc->restart_rel > 0.0) {
                restart = !(fabs(tot[1]) >= sc->restart_rel * sqrt(tot[0] * sc->r0n2));
                sc->rho = restart ? tot[0] : tot[1];
                if (restart) sc->r0n2 = tot[0];
            } else {
                // bicgstabRe2.hpp:166-182 (rho keeps r1.r0 of the old shadow)
                restart = !(sc->timestep < 10 || fabs(pre) > sc->restart_tol);
                sc->rho = tot[1];
            }
            sc->beta = (sc->alpha / sc->omega) * (tot[1] / pre);
            sc->restart = restart;
            sc->restarts += restart;
            sc->iter += 1;
            sc->total_iters += 1;
        }
    }
}

template <class V>
__global__ void __launch_bounds__(kBlock)
k_bicg_p(long long n, V *__restrict__ r0, const V *__restrict__ r1, V *__restrict__ p1,
         const V *__restrict__ ap, const BicgScal *sc)
{
    if (sc->done) return;
    if (sc->restart) {
        for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < n;
             row += (long long)gridDim.x * blockDim.x) {
            const V r = r1[row];
            r0[row] = r;
            p1[row] = r;
        }
        return;
    }
    const V beta = (V)sc->beta, omega = (V)sc->omega;
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < n;
         row += (long long)gridDim.x * blockDim.x)
        p1[row] = fma(beta, fma(-omega, ap[row], p1[row]), r1[row]);
}

// ---------------------------------------------------------------------------
// Fused kernels of the FP32 inner solves (memory-bound, so forming an input
// vector at the seven stencil points costs FP32 issue slots, not bytes).
//
// k_bicg_pap: the p update of iteration k-1 fused with the SpMV of iteration
// k: pn = r1 + beta (p - omega ap) (or r1 after a restart, which also sets
// r0 = r1), apn = A pn, alpha = rho / (apn . r0).  p/ap are read from one
// buffer pair and written to the other.
template <class V>
__global__ void __launch_bounds__(kBlock)
k_bicg_pap(SpeOp<V> A, const V *__restrict__ r1, const V *__restrict__ p, const V *__restrict__ ap,
           V *__restrict__ pn, V *__restrict__ apn, V *__restrict__ r0, BicgScal *sc, double *partials,
           unsigned int *counter)
{
    if (sc->done) return;
    const bool restart = sc->restart != 0;
    const V beta = restart ? V(0) : (V)sc->beta, omega = restart ? V(0) : (V)sc->omega;
    auto pat = [&](long long q) { return fma(beta, fma(-omega, ap[q], p[q]), r1[q]); };
    V pa = V(0);
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < A.n;
         row += (long long)gridDim.x * blockDim.x) {
        const V a = apply_row_f(A, row, pat);
        const V pr = pat(row);
        pn[row] = pr;
        apn[row] = a;
        V rr0;
        if (restart) {
            rr0 = r1[row];
            r0[row] = rr0;
        } else {
            rr0 = r0[row];
        }
        pa = fma(a, rr0, pa);
    }
    double acc[1] = {(double)pa}, tot[1];
    if (grid_reduce<1>(acc, partials, counter, tot) && threadIdx.x == 0) sc->alpha = sc->rho / tot[0];
}

// k_bicg_sas: s = r1 - alpha ap fused with as = A s and the two dots.
template <class V>
__global__ void __launch_bounds__(kBlock)
k_bicg_sas(SpeOp<V> A, const V *__restrict__ r1, const V *__restrict__ ap, V *__restrict__ s1,
           V *__restrict__ as, BicgScal *sc, double *partials, unsigned int *counter)
{
    if (sc->done) return;
    const V alpha = (V)sc->alpha;
    auto sat = [&](long long q) { return fma(-alpha, ap[q], r1[q]); };
    V pa0 = V(0), pa1 = V(0);
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < A.n;
         row += (long long)gridDim.x * blockDim.x) {
        const V a = apply_row_f(A, row, sat);
        const V sv = sat(row);
        s1[row] = sv;
        as[row] = a;
        pa0 = fma(a, sv, pa0);
        pa1 = fma(a, a, pa1);
    }
    double acc[2] = {(double)pa0, (double)pa1}, tot[2];
    if (grid_reduce<2>(acc, partials, counter, tot) && threadIdx.x == 0) sc->omega = tot[0] / tot[1];
}

// k_bicg_ap1: the first SpMV of a solve (p1 = r0 after init), jp on the fly.
template <class V>
__global__ void __launch_bounds__(kBlock)
k_bicg_ap1(SpeOp<V> A, const V *__restrict__ p1, const V *__restrict__ r0, V *__restrict__ ap, BicgScal *sc,
           double *partials, unsigned int *counter)
{
    if (sc->done) return;
    auto pat = [&](long long q) { return p1[q]; };
    V pa = V(0);
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < A.n;
         row += (long long)gridDim.x * blockDim.x) {
        const V a = apply_row_f(A, row, pat);
        ap[row] = a;
        pa = fma(a, r0[row], pa);
    }
    double acc[1] = {(double)pa}, tot[1];
    if (grid_reduce<1>(acc, partials, counter, tot) && threadIdx.x == 0) sc->alpha = sc->rho / tot[0];
}

// One fused iteration reading p/ap from buffer pair `from` and writing the
// other pair (first == true: the solve's first iteration, p1 = r0).
template <class V>
void launch_bicg_fused_iteration(cfd_launch_ctx &c, const SpeOp<V> &A, V *x, const BicgVecs<V> &w,
                                 V *p_alt, V *ap_alt, BicgScal *sc, int from, bool first)
{
    const int G = c.red_blocks;
    V *P[2] = {w.p1, p_alt}, *AP[2] = {w.ap, ap_alt};
    const int to = first ? from : 1 - from;
    if (first)
        k_bicg_ap1<V><<<G, kBlock, 0, c.s>>>(A, P[from], w.r0, AP[from], sc, c.partials, c.counter);
    else
        k_bicg_pap<V><<<G, kBlock, 0, c.s>>>(A, w.r1, P[from], AP[from], P[to], AP[to], w.r0, sc, c.partials,
                                             c.counter);
    k_bicg_sas<V><<<G, kBlock, 0, c.s>>>(A, w.r1, AP[to], w.s1, w.as, sc, c.partials, c.counter);
    k_bicg_xr<V><<<G, kBlock, 0, c.s>>>(A.n, x, P[to], w.s1, w.as, w.r0, w.r1, sc, c.partials, c.counter);
}
template void launch_bicg_fused_iteration<float>(cfd_launch_ctx &, const SpeOp<float> &, float *,
                                                 const BicgVecs<float> &, float *, float *, BicgScal *, int, bool);

// ---------------------------------------------------------------------------
// FP32 Jacobi-preconditioned CG of the mixed-precision inner solves.
//
// A e = r with A = J L (J = diag(jp)) is the same system as M e = P r with
// M = D_V L symmetric positive semi-definite (D_V = cell volumes; the face
// coefficients dV c_nb = face area / distance are symmetric) and P = D_V
// diag(L) = diag(M).  CG needs one SpMV per iteration and, unlike BiCGSTAB,
// no bi-orthogonality that FP32 rounding erodes.
//
// P at row (i,j,k): dV (sx_i + sy_j + sz_k) with sx = cxm + cxp (present
// neighbours only), dV = wx_i wy_j wz_k.
// P = dV (sx + sy + sz): the Jacobi preconditioner of M, in one association
// that every CG kernel shares (the stencil kernels form z = h / P on the fly
// and the update kernel forms h . z with the same rounding)
__device__ __forceinline__ float cg_P(float wx, float sx, float wyz, float syz) { return (wx * wyz) * (sx + syz); }

__device__ __forceinline__ float fv_P(const FvOp<float> &F, int i, int j, int k)
{
    return cg_P(__ldg(F.wx + i), __ldg(F.sx + i), __ldg(F.wy + j) * __ldg(F.wz + k), __ldg(F.sy + j) + __ldg(F.sz + k));
}

// q = M x at `row` with x values from a functor
template <class Fn>
__device__ __forceinline__ float fv_apply(const FvOp<float> &F, long long row, int i, int j, int k, Fn &&xat)
{
    const SpeOp<float> &A = F.A;
    const long long xw = i > 0 ? row - A.sxc : row;
    const long long xe = i < A.nxc - 1 ? row + A.sxc : row;
    const long long ys = j > 0 ? row - A.nzc : row;
    const long long yn = j < A.nyc - 1 ? row + A.nzc : row;
    const long long zb = k > 0 ? row - 1 : (A.pz ? row + (A.nzc - 1) : row);
    const long long zt = k < A.nzc - 1 ? row + 1 : (A.pz ? row - (A.nzc - 1) : row);
    float s = __ldg(A.cxm + i) * xat(xw);
    s = fmaf(__ldg(A.cym + j), xat(ys), s);
    s = fmaf(__ldg(A.czm + k), xat(zb), s);
    s = fmaf(__ldg(A.czp + k), xat(zt), s);
    s = fmaf(__ldg(A.cyp + j), xat(yn), s);
    s = fmaf(__ldg(A.cxp + i), xat(xe), s);
    const float diag = __ldg(F.sx + i) + __ldg(F.sy + j) + __ldg(F.sz + k);
    const float dv = __ldg(F.wx + i) * __ldg(F.wy + j) * __ldg(F.wz + k);
    return dv * fmaf(diag, xat(row), -s);
}

// init: h = P r (in place), p = z = P^-1 h = r, rho = h.z
__global__ void __launch_bounds__(kBlock)
k_cg_init(FvOp<float> F, float *__restrict__ h, float *__restrict__ p, BicgScal *sc, double *partials,
          unsigned int *counter)
{
    float pa = 0.f;
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < F.A.n;
         row += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decompose(F.A, row, i, j, k);
        const float r = h[row];
        const float hv = fv_P(F, i, j, k) * r;
        h[row] = hv;
        p[row] = r;
        pa = fmaf(hv, r, pa);
    }
    float acc[1] = {pa};
    double tot[1];
    if (grid_reduce_f<1>(acc, partials, counter, tot) && threadIdx.x == 0) {
        sc->rho = tot[0];
        sc->r0n2 = tot[0];
        sc->norm0 = sqrt(tot[0]);
        sc->iter = 0;
        sc->restart = 0;
        sc->timestep += 1;
        sc->done = tot[0] > 0.0 ? BICG_RUNNING : BICG_ZERO_RHS;
        sc->relres = tot[0] > 0.0 ? 1.0 : 0.0;
        sc->wait_timeout = 0;
    }
}

// shared plane of the tiled kernel: (kBlock / TK + 2) x (TK + 2) floats,
// largest for TK = 8
constexpr int kCgTileSmem = (kBlock / 8 + 2) * (8 + 2);

// pn = z + beta p (z = P^-1 h), q = M pn, alpha = rho / (pn . q).
//
// 2.5D tiling: a block owns a (TJ x TK) tile of the (j, k) plane and marches
// along i over a chunk of planes.  Each thread keeps pn at i-1, i, i+1 in
// registers and stages plane i in a double-buffered shared plane with a
// one-cell halo in j and k (the 2 TK + 2 TJ halo cells are spread over the
// first threads), so one barrier per plane suffices.  The raw z and p loads
// run two planes ahead of their use to keep enough bytes in flight.  Values
// outside the domain are 0; their coefficients are 0 as well.
// first: the solve's first iteration, pn = z (beta = 0, p not read, pn not
// written: the caller passes pn = z).
// dyn: p and pn are the two buffers of the run-time alternation (p is read
// from buffer sc->pp, pn written to the other; see k_cg_pq_tma)
template <bool first>
__global__ void __launch_bounds__(kBlock, 5)
k_cg_pq(FvOp<float> F, const float *__restrict__ z, const float *p_, float *pn_, float *__restrict__ q,
        BicgScal *sc, double *partials, unsigned int *counter, int TK, int ichunk, int dyn = 0)
{
    pdl_wait();
    pdl_allow();
    if (sc->done) return;
    const int sel = dyn ? sc->pp : 0;
    const float *__restrict__ p = dyn ? (sel ? pn_ : p_) : p_;
    float *__restrict__ pn = dyn ? (sel ? const_cast<float *>(p_) : pn_) : pn_;
    const SpeOp<float> &A = F.A;
    const int TJ = kBlock / TK, SW = TK + 2;
    const int t = threadIdx.x, tk = t % TK, tj = t / TK;
    const int nxc = A.nxc, nyc = A.nyc, nzc = A.nzc;
    const long long sxc = A.sxc;
    const int tiles_k = (nzc + TK - 1) / TK, tiles_j = (nyc + TJ - 1) / TJ;
    const int tiles = tiles_k * tiles_j, items = tiles * ((nxc + ichunk - 1) / ichunk);
    const float beta = first ? 0.f : (float)sc->beta;
    // halo cell of this thread in tile coordinates (-1..TJ, -1..TK)
    int hj = 0, hk = 0;
    const bool hv = t < 2 * TK + 2 * TJ;
    if (t < TK) {
        hj = -1; hk = t;
    } else if (t < 2 * TK) {
        hj = TJ; hk = t - TK;
    } else if (t < 2 * TK + TJ) {
        hj = t - 2 * TK; hk = -1;
    } else if (hv) {
        hj = t - 2 * TK - TJ; hk = TK;
    }
    const int cslot = (tj + 1) * SW + tk + 1, hslot = (hj + 1) * SW + hk + 1;
    // raw (z, p) at (i, jj, kk), zeros outside the domain (p not read when first)
    auto ld = [&](int i, int jj, int kk, float &zv, float &pv) {
        zv = 0.f;
        pv = 0.f;
        if (A.pz) kk = kk < 0 ? kk + nzc : (kk >= nzc ? kk - nzc : kk);  // periodic z: wrap the halo
        if (i >= 0 && i < nxc && jj >= 0 && jj < nyc && kk >= 0 && kk < nzc) {
            const long long r = (long long)i * sxc + (jj * nzc + kk);
            zv = z[r];
            if (!first) pv = p[r];
        }
    };
    __shared__ float sm[2][kCgTileSmem];
    float pa = 0.f, pz = 0.f;
    for (int item = blockIdx.x; item < items; item += gridDim.x) {
        const int tile = item % tiles, chunk = item / tiles;
        const int k0 = (tile % tiles_k) * TK, j0 = (tile / tiles_k) * TJ;
        const int k = k0 + tk, j = j0 + tj, hjj = j0 + hj, hkk = k0 + hk;
        const int ib = chunk * ichunk, ie = min(nxc, ib + ichunk);
        const bool in = j < nyc && k < nzc;
        const float cym = in ? __ldg(A.cym + j) : 0.f, cyp = in ? __ldg(A.cyp + j) : 0.f;
        const float czm = in ? __ldg(A.czm + k) : 0.f, czp = in ? __ldg(A.czp + k) : 0.f;
        const float syz = in ? __ldg(F.sy + j) + __ldg(F.sz + k) : 0.f;
        const float wyz = in ? __ldg(F.wy + j) * __ldg(F.wz + k) : 0.f;
        float zm, pm, z0, p0, z1, p1, z2, p2;
        float hz0 = 0.f, hp0 = 0.f, hz1 = 0.f, hp1 = 0.f;
        ld(ib - 1, j, k, zm, pm);
        ld(ib, j, k, z0, p0);
        ld(ib + 1, j, k, z1, p1);
        ld(ib + 2, j, k, z2, p2);
        if (hv) {
            ld(ib, hjj, hkk, hz0, hp0);
            ld(ib + 1, hjj, hkk, hz1, hp1);
        }
        float vm = fmaf(beta, pm, zm), vc = fmaf(beta, p0, z0), zc = z0;
        for (int i = ib; i < ie; ++i) {
            float z3, p3, hz2 = 0.f, hp2 = 0.f;
            ld(i + 3, j, k, z3, p3);
            if (hv) ld(i + 2, hjj, hkk, hz2, hp2);
            const float vp = fmaf(beta, p1, z1);
            float *buf = sm[i & 1];
            buf[cslot] = vc;
            if (hv) buf[hslot] = fmaf(beta, hp0, hz0);
            __syncthreads();
            if (in) {
                const float vs = buf[cslot - SW], vn = buf[cslot + SW];
                const float vb = buf[cslot - 1], vt = buf[cslot + 1];
                float sum = __ldg(A.cxm + i) * vm;
                sum = fmaf(cym, vs, sum);
                sum = fmaf(czm, vb, sum);
                sum = fmaf(czp, vt, sum);
                sum = fmaf(cyp, vn, sum);
                sum = fmaf(__ldg(A.cxp + i), vp, sum);
                const float diag = __ldg(F.sx + i) + syz;
                const float qv = (__ldg(F.wx + i) * wyz) * fmaf(diag, vc, -sum);
                const long long r = (long long)i * sxc + (j * nzc + k);
                if (!first) pn[r] = vc;
                q[r] = qv;
                pa = fmaf(vc, qv, pa);
                pz = fmaf(zc, qv, pz);
            }
            vm = vc;
            vc = vp;
            zc = z1;
            z1 = z2; p1 = p2; z2 = z3; p2 = p3;
            hz0 = hz1; hp0 = hp1; hz1 = hz2; hp1 = hp2;
        }
        __syncthreads();  // the next item rewrites both planes
    }
    float acc[2] = {pa, pz};
    double tot[2];
    if (grid_reduce_f<2>(acc, partials, counter, tot) && threadIdx.x == 0) {
        sc->alpha = sc->rho / tot[0];
        sc->qz = tot[1];
    }
}

// ---- TMA-fed CG stencil ------------------------------------------------------
// The same operation as k_cg_pq, with the z and p planes streamed into
// shared memory by the tensor-memory accelerator.  A block owns a TK x TJ
// tile of the (k, j) plane; each of its 256 threads handles one float4 of k.
// One elected thread keeps kCgStages planes of z (and p) in flight: each TMA
// box is one plane of the tile plus a halo of one row in j and four cells in
// k (so the box starts on a 16-byte boundary), and the TMA fills the parts
// outside the domain with zeros, which is the value the stencil needs there.
// Per plane the block forms pn = z + beta p over the tile and its halo in a
// shared plane (three rotating buffers), then applies M at the previous plane
// with its x neighbours held in registers.  The mbarrier waits are bounded:
// when a wait gives up (wait_limit try-waits), the block records
// sc->wait_timeout, issues no further copies, waits out the copies it has in
// flight and skips its remaining work, so a lost copy can neither hang the
// GPU nor land in shared memory after the block has exited; the host turns
// the flag into an error.
constexpr int kCgStages = 4;
constexpr long long kCgWaitLimit = 1LL << 24;   // default try-waits of a pipeline wait
constexpr long long kCgDrainLimit = 1LL << 24;  // try-waits per copy when draining after a timeout

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait: false if the phase did not complete within `limit` try-waits
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, long long limit)
{
    for (long long it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void tma_load_3d(unsigned dst, const CUtensorMap *map, int c0, int c1, int c2,
                                            unsigned bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
        : "memory");
}

template <int TK>
struct CgTile {
    static constexpr int TKQ = TK / 4;           // threads along k
    static constexpr int TJ = kBlock / TKQ;      // rows along j
    static constexpr int BX = TK + 8;            // box width (floats): 4-cell halo each side
    static constexpr int BY = TJ + 2;            // box height: 1-row halo each side
    static constexpr int BOXB = BX * BY * 4;     // bytes of one box
    static constexpr int STRIDE = (BOXB + 127) / 128 * 128;
    static constexpr int NHALO = 2 * TKQ + 2 * TJ;  // halo float4 items per plane
    static constexpr size_t smem(int nv) { return 128 + (size_t)(kCgStages * nv + 3) * STRIDE + 128; }
};

// dyn: the two p buffers alternate at run time (sc->pp holds p; mp / pn_out
// are buffer 0, mp2 / pn_out2 buffer 1): p is read from buffer pp and pn
// written to the other, so a loop body of one iteration replays correctly
template <bool first, int TK, bool FZ>
__global__ void __launch_bounds__(kBlock)
k_cg_pq_tma(FvOp<float> F, const __grid_constant__ CUtensorMap mh, const __grid_constant__ CUtensorMap mp,
            const __grid_constant__ CUtensorMap mp2, float *pn_out0, float *pn_out2, int dyn, float *__restrict__ q,
            BicgScal *sc, double *partials, unsigned int *counter, int ichunk, long long wait_limit)
{
    using G = CgTile<TK>;
    constexpr int NV = first ? 1 : 2;
    constexpr int MAXH = (G::NHALO + kBlock - 1) / kBlock;  // halo items per thread
    pdl_wait();
    pdl_allow();
    if (sc->done) return;
    const int sel = dyn ? sc->pp : 0;
    const CUtensorMap *mpp = sel ? &mp2 : &mp;
    float *__restrict__ pn_out = dyn ? (sel ? pn_out0 : pn_out2) : pn_out0;
    extern __shared__ unsigned char dsm[];
    const unsigned base = (smem_u32(dsm) + 127u) & ~127u;
    unsigned char *gbase = dsm + (base - smem_u32(dsm));
    const unsigned bars = base;                       // kCgStages mbarriers (8 B each)
    const unsigned stage0 = base + 128;               // stages: [stage][vector] boxes
    float *stg = reinterpret_cast<float *>(gbase + 128);
    float *pnb = reinterpret_cast<float *>(gbase + 128 + (size_t)kCgStages * NV * G::STRIDE);
    constexpr int SF = G::STRIDE / 4;                 // floats per box slot
    __shared__ int bad;

    const SpeOp<float> &A = F.A;
    const int nxc = A.nxc, nyc = A.nyc, nzc = A.nzc;
    const long long sxc = A.sxc;
    const int t = threadIdx.x, tk4 = t % G::TKQ, tj = t / G::TKQ;
    const int tiles_k = (nzc + TK - 1) / TK, tiles_j = (nyc + G::TJ - 1) / G::TJ;
    const int tiles = tiles_k * tiles_j, items = tiles * ((nxc + ichunk - 1) / ichunk);
    const float beta = first ? 0.f : (float)sc->beta;
    if (t == 0) {
        bad = 0;
        for (int s = 0; s < kCgStages; ++s) mbar_init(bars + 8 * s, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    long long issued_hi = 0;  // thread 0: global plane counter of the last plane issued + 1
    // one plane's TMA boxes into the stage of global plane counter g
    auto issue = [&](long long g, int k0, int j0, int ip) {
        issued_hi = g + 1;
        const int st = (int)(g % kCgStages);
        const unsigned bar = bars + 8 * st;
        mbar_expect_tx(bar, NV * G::BOXB);
        tma_load_3d(stage0 + (unsigned)(st * NV) * G::STRIDE, &mh, k0 - 4, j0 - 1, ip, bar);
        if (!first) tma_load_3d(stage0 + (unsigned)(st * NV + 1) * G::STRIDE, mpp, k0 - 4, j0 - 1, ip, bar);
    };
    // box position (row, float4 column) of halo item h
    auto halo_pos = [&](int h, int &row, int &col) {
        if (h < G::TKQ) { row = 0; col = 1 + h; }
        else if (h < 2 * G::TKQ) { row = G::TJ + 1; col = 1 + h - G::TKQ; }
        else if (h < 2 * G::TKQ + G::TJ) { row = 1 + h - 2 * G::TKQ; col = 0; }
        else { row = 1 + h - 2 * G::TKQ - G::TJ; col = G::TKQ + 1; }
    };
    const int cslot = (tj + 1) * G::BX + 4 + 4 * tk4;  // this thread's float4 in a box / pn plane
    float pa = 0.f, pz = 0.f;
    long long g0 = 0;  // planes consumed by this block so far (mbarrier phases)
    long long g_stop = -1;  // the plane whose wait gave up (-1: none)
    for (int item = blockIdx.x; item < items && g_stop < 0; item += gridDim.x) {
        const int tile = item % tiles, chunk = item / tiles;
        const int k0 = (tile % tiles_k) * TK, j0 = (tile / tiles_k) * G::TJ;
        const int ib = chunk * ichunk, ie = min(nxc, ib + ichunk);
        const int np = ie - ib + 2;  // planes ib-1 .. ie
        const int j = j0 + tj, k = k0 + 4 * tk4;
        const bool in = j < nyc && k < nzc;
        if (t == 0)
            for (int s = 0; s < kCgStages && s < np; ++s) issue(g0 + s, k0, j0, ib - 1 + s);
        float4 czm = make_float4(0.f, 0.f, 0.f, 0.f), czp = czm, syz = czm, wyz = czm;
        float cym = 0.f, cyp = 0.f;
        if (in) {
            cym = __ldg(A.cym + j);
            cyp = __ldg(A.cyp + j);
            czm = __ldg(reinterpret_cast<const float4 *>(A.czm + k));
            czp = __ldg(reinterpret_cast<const float4 *>(A.czp + k));
            const float4 sz = __ldg(reinterpret_cast<const float4 *>(F.sz + k));
            const float4 wz = __ldg(reinterpret_cast<const float4 *>(F.wz + k));
            const float sy = __ldg(F.sy + j), wy = __ldg(F.wy + j);
            syz = make_float4(sy + sz.x, sy + sz.y, sy + sz.z, sy + sz.w);
            wyz = make_float4(wy * wz.x, wy * wz.y, wy * wz.z, wy * wz.w);
        }
        // (wy wz, sy + sz) of this thread's halo items, zero outside the domain
        float4 hwyz[MAXH], hsyz[MAXH];
        if (!first && FZ) {
#pragma unroll
            for (int m = 0; m < MAXH; ++m) {
                hwyz[m] = make_float4(0.f, 0.f, 0.f, 0.f);
                hsyz[m] = hwyz[m];
                const int h = t + m * kBlock;
                if (h >= G::NHALO) continue;
                int row, col;
                halo_pos(h, row, col);
                const int jj = j0 - 1 + row;
                if (jj < 0 || jj >= nyc) continue;
                const float wy = __ldg(F.wy + jj), sy = __ldg(F.sy + jj);
                float hw[4], hs[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int kk = k0 - 4 + 4 * col + e;
                    const bool ok = kk >= 0 && kk < nzc;
                    hw[e] = ok ? wy * __ldg(F.wz + kk) : 0.f;
                    hs[e] = ok ? sy + __ldg(F.sz + kk) : 0.f;
                }
                hwyz[m] = make_float4(hw[0], hw[1], hw[2], hw[3]);
                hsyz[m] = make_float4(hs[0], hs[1], hs[2], hs[3]);
            }
        }
        float4 p1 = make_float4(0.f, 0.f, 0.f, 0.f), p2 = p1;
        float4 z1 = p1;  // the loaded vector (z, or h when FZ) at this thread's cells of plane tt - 1
        for (int tt = 0; tt < np; ++tt) {
            const long long g = g0 + tt;
            const int st = (int)(g % kCgStages);
            const int ip = ib - 1 + tt;
            const bool iv = ip >= 0 && ip < nxc;
            const float wxi = iv ? __ldg(F.wx + ip) : 0.f, sxi = iv ? __ldg(F.sx + ip) : 0.f;
            const int timed_out = mbar_wait(bars + 8 * st, (unsigned)((g / kCgStages) & 1), wait_limit) ? 0 : 1;
            const float *hs_ = stg + (size_t)(st * NV) * SF;
            const float *ps = stg + (size_t)(st * NV + 1) * SF;
            float *pb = pnb + (size_t)(tt % 3) * SF;
            // pn = z + beta p with z = h / P (FZ) or z as loaded (first: pn = p0
            // as loaded); wq, sq = (wy wz, sy + sz)
            auto form = [&](int off, const float4 &wq, const float4 &sq) {
                float4 zv = *reinterpret_cast<const float4 *>(hs_ + off);
                if (!first && !FZ) {
                    const float4 pv = *reinterpret_cast<const float4 *>(ps + off);
                    zv.x = fmaf(beta, pv.x, zv.x);
                    zv.y = fmaf(beta, pv.y, zv.y);
                    zv.z = fmaf(beta, pv.z, zv.z);
                    zv.w = fmaf(beta, pv.w, zv.w);
                } else if (!first) {
                    const float4 pv = *reinterpret_cast<const float4 *>(ps + off);
                    auto zf = [&](float hv, float w, float sv, float pp) {
                        const float ipv = w != 0.f ? __frcp_rn(cg_P(wxi, sxi, w, sv)) : 0.f;
                        return fmaf(beta, pp, iv ? hv * ipv : 0.f);
                    };
                    zv = make_float4(zf(zv.x, wq.x, sq.x, pv.x), zf(zv.y, wq.y, sq.y, pv.y),
                                     zf(zv.z, wq.z, sq.z, pv.z), zf(zv.w, wq.w, sq.w, pv.w));
                }
                *reinterpret_cast<float4 *>(pb + off) = zv;
                return zv;
            };
            const float4 zraw = *reinterpret_cast<const float4 *>(hs_ + cslot);
            const float4 nxt = form(cslot, wyz, syz);
#pragma unroll
            for (int m = 0; m < MAXH; ++m) {
                const int h = t + m * kBlock;
                if (h < G::NHALO) {
                    int row, col;
                    halo_pos(h, row, col);
                    if (first || !FZ) form(row * G::BX + 4 * col, wyz, syz);
                    else form(row * G::BX + 4 * col, hwyz[m], hsyz[m]);
                }
            }
            // one barrier for the block, and the same verdict in every thread
            if (__syncthreads_or(timed_out)) {
                g_stop = g;
                break;
            }
            // the stage of plane tt is consumed: refill it with plane tt + kCgStages
            if (t == 0 && tt + kCgStages < np) issue(g + kCgStages, k0, j0, ib - 1 + tt + kCgStages);
            if (tt >= 2 && in) {
                const int c = ib + tt - 2;  // plane of the stencil (pn at c-1, c, c+1 = p2, p1, nxt)
                const float *pc = pnb + (size_t)((tt - 1) % 3) * SF;
                const float4 vs = *reinterpret_cast<const float4 *>(pc + cslot - G::BX);
                const float4 vn = *reinterpret_cast<const float4 *>(pc + cslot + G::BX);
                const float kb = pc[cslot - 1], kt = pc[cslot + 4];
                const float cxm = __ldg(A.cxm + c), cxp = __ldg(A.cxp + c);
                const float sxv = __ldg(F.sx + c), wxv = __ldg(F.wx + c);
                const float4 vc = p1;
                auto cell = [&](float vm_, float vs_, float vb_, float vt_, float vn_, float vp_, float vc_,
                                float czm_, float czp_, float syz_, float wyz_) {
                    float sum = cxm * vm_;
                    sum = fmaf(cym, vs_, sum);
                    sum = fmaf(czm_, vb_, sum);
                    sum = fmaf(czp_, vt_, sum);
                    sum = fmaf(cyp, vn_, sum);
                    sum = fmaf(cxp, vp_, sum);
                    return (wxv * wyz_) * fmaf(sxv + syz_, vc_, -sum);
                };
                float4 qv;
                qv.x = cell(p2.x, vs.x, kb, vc.y, vn.x, nxt.x, vc.x, czm.x, czp.x, syz.x, wyz.x);
                qv.y = cell(p2.y, vs.y, vc.x, vc.z, vn.y, nxt.y, vc.y, czm.y, czp.y, syz.y, wyz.y);
                qv.z = cell(p2.z, vs.z, vc.y, vc.w, vn.z, nxt.z, vc.z, czm.z, czp.z, syz.z, wyz.z);
                qv.w = cell(p2.w, vs.w, vc.z, kt, vn.w, nxt.w, vc.w, czm.w, czp.w, syz.w, wyz.w);
                const long long r = (long long)c * sxc + (long long)j * nzc + k;
                if (!first) *reinterpret_cast<float4 *>(pn_out + r) = vc;
                *reinterpret_cast<float4 *>(q + r) = qv;
                pa = fmaf(vc.x, qv.x, pa);
                pa = fmaf(vc.y, qv.y, pa);
                pa = fmaf(vc.z, qv.z, pa);
                pa = fmaf(vc.w, qv.w, pa);
                pz = fmaf(z1.x, qv.x, fmaf(z1.y, qv.y, fmaf(z1.z, qv.z, fmaf(z1.w, qv.w, pz))));
            }
            p2 = p1;
            p1 = nxt;
            z1 = zraw;
        }
        g0 += np;
        __syncthreads();  // the next item rewrites the pn planes
    }
    if (g_stop >= 0) {
        // a wait gave up: no copy was issued after it; wait out the ones in
        // flight (planes g_stop .. issued_hi - 1, at most one per stage) so
        // none lands in shared memory after the block has exited
        if (t == 0) {
            bad = 1;
            for (long long g = g_stop; g < issued_hi; ++g)
                mbar_wait(bars + 8 * (int)(g % kCgStages), (unsigned)((g / kCgStages) & 1), kCgDrainLimit);
        }
        __syncthreads();
    }
    if (t == 0 && bad) sc->wait_timeout = 1;
    // pn . q gives alpha; q . z (z as loaded) serves the flexible beta of
    // the multigrid-CG
    float acc[2] = {pa, pz};
    double tot[2];
    if (grid_reduce_f<2>(acc, partials, counter, tot) && threadIdx.x == 0) {
        sc->alpha = sc->rho / tot[0];
        sc->qz = tot[1];
    }
}

// Update of the TMA path: e += alpha p, h -= alpha q, rho' = h . (h / P) with
// 1/P formed from the per-axis tables (no z vector: the stencil kernel forms
// z itself), four rows per thread step (nz a multiple of 4)
__global__ void __launch_bounds__(kBlock, 4)
k_cg_upd_fv(FvOp<float> F, float *__restrict__ e, const float *__restrict__ p, float *__restrict__ h,
            const float *__restrict__ q, BicgScal *sc, double *partials, unsigned int *counter)
{
    if (sc->done) return;
    const SpeOp<float> &A = F.A;
    const float alpha = (float)sc->alpha;
    float pa = 0.f;
    const long long n4 = A.n >> 2;
    const unsigned sxc = (unsigned)A.sxc, nzc = (unsigned)A.nzc;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n4; v += stride) {
        const unsigned row = 4u * (unsigned)v;
        const unsigned i = A.fsxc.div(row), rem = row - i * sxc;
        const unsigned j = A.fnzc.div(rem), k = rem - j * nzc;
        const float wx = __ldg(F.wx + i), sx = __ldg(F.sx + i), wy = __ldg(F.wy + j), sy = __ldg(F.sy + j);
        const float4 wz = __ldg(reinterpret_cast<const float4 *>(F.wz + k));
        const float4 sz = __ldg(reinterpret_cast<const float4 *>(F.sz + k));
        float4 ev = reinterpret_cast<float4 *>(e)[v];
        const float4 pv = reinterpret_cast<const float4 *>(p)[v];
        float4 hv = reinterpret_cast<float4 *>(h)[v];
        const float4 qv = reinterpret_cast<const float4 *>(q)[v];
        ev.x = fmaf(alpha, pv.x, ev.x); ev.y = fmaf(alpha, pv.y, ev.y);
        ev.z = fmaf(alpha, pv.z, ev.z); ev.w = fmaf(alpha, pv.w, ev.w);
        hv.x = fmaf(-alpha, qv.x, hv.x); hv.y = fmaf(-alpha, qv.y, hv.y);
        hv.z = fmaf(-alpha, qv.z, hv.z); hv.w = fmaf(-alpha, qv.w, hv.w);
        reinterpret_cast<float4 *>(e)[v] = ev;
        reinterpret_cast<float4 *>(h)[v] = hv;
        pa = fmaf(hv.x, hv.x * __frcp_rn(cg_P(wx, sx, wy * wz.x, sy + sz.x)), pa);
        pa = fmaf(hv.y, hv.y * __frcp_rn(cg_P(wx, sx, wy * wz.y, sy + sz.y)), pa);
        pa = fmaf(hv.z, hv.z * __frcp_rn(cg_P(wx, sx, wy * wz.z, sy + sz.z)), pa);
        pa = fmaf(hv.w, hv.w * __frcp_rn(cg_P(wx, sx, wy * wz.w, sy + sz.w)), pa);
    }
    float acc[1] = {pa};
    double tot[1];
    if (grid_reduce_f<1>(acc, partials, counter, tot) && threadIdx.x == 0) {
        const double rel = sqrt(fabs(tot[0]) / sc->r0n2);
        sc->relres = rel;
        if (rel < sc->tol) {
            sc->done = BICG_CONVERGED;
        } else if (sc->iter >= sc->maxit) {
            sc->done = BICG_CAPPED;
        } else {
            sc->beta = tot[0] / sc->rho;
            sc->rho = tot[0];
            sc->iter += 1;
            sc->total_iters += 1;
        }
    }
}

// e += alpha p, h -= alpha q, z = iP h, rho' = h . z (pure streaming, four
// rows per thread step); convergence on sqrt(rho'/rho0)
__global__ void __launch_bounds__(kBlock, 6)
k_cg_upd(long long n, float *__restrict__ e, const float *__restrict__ p, float *__restrict__ h,
         const float *__restrict__ q, const float *__restrict__ iP, float *__restrict__ z, BicgScal *sc,
         double *partials, unsigned int *counter)
{
    if (sc->done) return;
    const float alpha = (float)sc->alpha;
    float pa = 0.f;
    const long long n4 = n >> 2;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n4; v += stride) {
        float4 ev = reinterpret_cast<float4 *>(e)[v];
        const float4 pv = reinterpret_cast<const float4 *>(p)[v];
        float4 hv = reinterpret_cast<float4 *>(h)[v];
        const float4 qv = reinterpret_cast<const float4 *>(q)[v];
        const float4 iv = reinterpret_cast<const float4 *>(iP)[v];
        ev.x = fmaf(alpha, pv.x, ev.x); ev.y = fmaf(alpha, pv.y, ev.y);
        ev.z = fmaf(alpha, pv.z, ev.z); ev.w = fmaf(alpha, pv.w, ev.w);
        hv.x = fmaf(-alpha, qv.x, hv.x); hv.y = fmaf(-alpha, qv.y, hv.y);
        hv.z = fmaf(-alpha, qv.z, hv.z); hv.w = fmaf(-alpha, qv.w, hv.w);
        const float4 zv = make_float4(hv.x * iv.x, hv.y * iv.y, hv.z * iv.z, hv.w * iv.w);
        reinterpret_cast<float4 *>(e)[v] = ev;
        reinterpret_cast<float4 *>(h)[v] = hv;
        reinterpret_cast<float4 *>(z)[v] = zv;
        pa = fmaf(hv.x, zv.x, pa); pa = fmaf(hv.y, zv.y, pa);
        pa = fmaf(hv.z, zv.z, pa); pa = fmaf(hv.w, zv.w, pa);
    }
    for (long long r = 4 * n4 + (long long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
        e[r] = fmaf(alpha, p[r], e[r]);
        const float hv = fmaf(-alpha, q[r], h[r]);
        h[r] = hv;
        const float zv = hv * iP[r];
        z[r] = zv;
        pa = fmaf(hv, zv, pa);
    }
    float acc[1] = {pa};
    double tot[1];
    if (grid_reduce_f<1>(acc, partials, counter, tot) && threadIdx.x == 0) {
        const double rel = sqrt(fabs(tot[0]) / sc->r0n2);
        sc->relres = rel;
        if (rel < sc->tol) {
            sc->done = BICG_CONVERGED;
        } else if (sc->iter >= sc->maxit) {
            sc->done = BICG_CAPPED;
        } else {
            sc->beta = tot[0] / sc->rho;
            sc->rho = tot[0];
            sc->iter += 1;
            sc->total_iters += 1;
        }
    }
}

// iP = 1 / P (FP32), once per context
__global__ void k_cg_ip(FvOp<float> F, float *__restrict__ iP)
{
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < F.A.n;
         row += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decompose(F.A, row, i, j, k);
        iP[row] = 1.0f / fv_P(F, i, j, k);
    }
}

// launch shape of the tiled kernel: a k tile of 32/16/8 cells, the i range
// cut into chunks so that tiles x chunks fills the reduction grid (blocks
// loop over tile-chunk items when there are more tiles than blocks)
struct CgShape {
    int TK, ichunk, grid;
};
static CgShape cg_shape(const cfd_launch_ctx &c, const FvOp<float> &F)
{
    const SpeOp<float> &A = F.A;
    CgShape s;
    s.TK = A.nzc >= 24 ? 32 : (A.nzc >= 12 ? 16 : 8);
    const int TJ = kBlock / s.TK;
    const int tiles = ((A.nzc + s.TK - 1) / s.TK) * ((A.nyc + TJ - 1) / TJ);
    int chunks = c.cg_grid / tiles;
    if (chunks < 1) chunks = 1;
    if (chunks > A.nxc) chunks = A.nxc;
    s.ichunk = (A.nxc + chunks - 1) / chunks;
    chunks = (A.nxc + s.ichunk - 1) / s.ichunk;
    s.grid = tiles * chunks < c.cg_grid ? tiles * chunks : c.cg_grid;
    return s;
}

void launch_cg_init(cfd_launch_ctx &c, const FvOp<float> &F, float *h, float *p, BicgScal *sc)
{
    k_cg_init<<<c.red_blocks, kBlock, 0, c.s>>>(F, h, p, sc, c.partials, c.counter);
}

// grid shape of the TMA kernel for one launch
static void cg_tma_launch_shape(const CgTma &t, const FvOp<float> &F, int &ichunk, int &grid)
{
    const SpeOp<float> &A = F.A;
    const int TJ = t.TJ;
    const int tiles = ((A.nzc + t.TK - 1) / t.TK) * ((A.nyc + TJ - 1) / TJ);
    int chunks = t.grid / tiles;
    if (chunks < 1) chunks = 1;
    if (chunks > A.nxc) chunks = A.nxc;
    ichunk = (A.nxc + chunks - 1) / chunks;
    chunks = (A.nxc + ichunk - 1) / ichunk;
    grid = tiles * chunks < t.grid ? tiles * chunks : t.grid;
}

template <bool first, int TK>
static void launch_tma_t(cfd_launch_ctx &c, const FvOp<float> &F, const CgTma &t, const CUtensorMap *mz,
                         const CUtensorMap *mp, float *pn, float *q, BicgScal *sc, bool form_z,
                         const CUtensorMap *mp2, float *pn2, int dyn)
{
    int ichunk, grid;
    cg_tma_launch_shape(t, F, ichunk, grid);
    const size_t sm = CgTile<TK>::smem(first ? 1 : 2);
    if (form_z)
        launch_pdl(k_cg_pq_tma<first, TK, true>, dim3(grid), dim3(kBlock), sm, c.s, F, *mz, *mp, *mp2, pn, pn2, dyn, q,
                   sc, c.partials, c.counter, ichunk, t.wait_limit);
    else
        launch_pdl(k_cg_pq_tma<first, TK, false>, dim3(grid), dim3(kBlock), sm, c.s, F, *mz, *mp, *mp2, pn, pn2, dyn, q,
                   sc, c.partials, c.counter, ichunk, t.wait_limit);
}

// z_map: the z vector (or p itself on the first iteration), p_map: p
// dyn: p_map / pn are buffer 0 and p_map2 / pn2 buffer 1 of the run-time
// alternation (k_cg_pq_tma)
static void launch_cg_pq_tma(cfd_launch_ctx &c, const FvOp<float> &F, const CgTma &t, bool first,
                             const CUtensorMap *z_map, const CUtensorMap *p_map, float *pn, float *q, BicgScal *sc,
                             bool form_z, const CUtensorMap *p_map2 = nullptr, float *pn2 = nullptr, int dyn = 0)
{
    if (!p_map2) {
        p_map2 = p_map;
        pn2 = pn;
    }
    if (t.TK == 32) {
        if (first) launch_tma_t<true, 32>(c, F, t, z_map, p_map, pn, q, sc, form_z, p_map2, pn2, dyn);
        else launch_tma_t<false, 32>(c, F, t, z_map, p_map, pn, q, sc, form_z, p_map2, pn2, dyn);
    } else if (t.TK == 16) {
        if (first) launch_tma_t<true, 16>(c, F, t, z_map, p_map, pn, q, sc, form_z, p_map2, pn2, dyn);
        else launch_tma_t<false, 16>(c, F, t, z_map, p_map, pn, q, sc, form_z, p_map2, pn2, dyn);
    } else {
        if (first) launch_tma_t<true, 8>(c, F, t, z_map, p_map, pn, q, sc, form_z, p_map2, pn2, dyn);
        else launch_tma_t<false, 8>(c, F, t, z_map, p_map, pn, q, sc, form_z, p_map2, pn2, dyn);
    }
}

void launch_cg_pq_mg(cfd_launch_ctx &c, const FvOp<float> &F, const CgTma *tma, float *z, float *p, float *p_alt,
                     float *q, BicgScal *sc, int from, bool first, bool dyn)
{
    float *P[2] = {p, p_alt};
    const int to = first ? from : 1 - from;
    if (tma && tma->ok) {
        if (dyn && !first) {
            launch_cg_pq_tma(c, F, *tma, false, &tma->zv, &tma->p, p, q, sc, false, &tma->palt, p_alt, 1);
            return;
        }
        const CUtensorMap *pmap = from == 0 ? &tma->p : &tma->palt;
        launch_cg_pq_tma(c, F, *tma, first, first ? pmap : &tma->zv, pmap, P[to], q, sc, false);
        return;
    }
    const CgShape cs = cg_shape(c, F);
    if (first)
        launch_pdl(k_cg_pq<true>, dim3(cs.grid), dim3(kBlock), 0, c.s, F, (const float *)P[from],
                   (const float *)P[from], P[from], q, sc, c.partials, c.counter, cs.TK, cs.ichunk, 0);
    else if (dyn)
        launch_pdl(k_cg_pq<false>, dim3(cs.grid), dim3(kBlock), 0, c.s, F, (const float *)z, (const float *)p, p_alt,
                   q, sc, c.partials, c.counter, cs.TK, cs.ichunk, 1);
    else
        launch_pdl(k_cg_pq<false>, dim3(cs.grid), dim3(kBlock), 0, c.s, F, (const float *)z, (const float *)P[from],
                   P[to], q, sc, c.partials, c.counter, cs.TK, cs.ichunk, 0);
}

void launch_cg_iteration(cfd_launch_ctx &c, const FvOp<float> &F, const float *iP, float *e, float *h, float *z,
                         float *p, float *p_alt, float *q, BicgScal *sc, int from, bool first, const CgTma *tma)
{
    float *P[2] = {p, p_alt};
    const int to = first ? from : 1 - from;
    if (tma && tma->ok) {
        const CUtensorMap *pmap = from == 0 ? &tma->p : &tma->palt;
        // first iteration: pn = p0, which k_cg_init wrote into P[from]
        launch_cg_pq_tma(c, F, *tma, first, first ? pmap : &tma->zh, pmap, P[to], q, sc, tma->form_z);
        if (tma->form_z)
            k_cg_upd_fv<<<c.cg_grid, kBlock, 0, c.s>>>(F, e, P[to], h, q, sc, c.partials, c.counter);
        else
            k_cg_upd<<<c.cg_grid, kBlock, 0, c.s>>>(F.A.n, e, P[to], h, q, iP, z, sc, c.partials, c.counter);
        return;
    }
    const CgShape cs = cg_shape(c, F);
    // first iteration: pn = p0 (written by k_cg_init into P[from]), read as z
    if (first)
        k_cg_pq<true><<<cs.grid, kBlock, 0, c.s>>>(F, P[from], P[from], P[from], q, sc, c.partials, c.counter,
                                                   cs.TK, cs.ichunk);
    else
        k_cg_pq<false><<<cs.grid, kBlock, 0, c.s>>>(F, z, P[from], P[to], q, sc, c.partials, c.counter, cs.TK,
                                                    cs.ichunk);
    k_cg_upd<<<c.cg_grid, kBlock, 0, c.s>>>(F.A.n, e, P[to], h, q, iP, z, sc, c.partials, c.counter);
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled()
{
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *ptr = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(ptr);
        else
            cudaGetLastError();
    }
    return fn;
}

// [nxc][nyc][nzc] FP32 vector, box {TK + 8, TJ + 2, 1} (k, j, i)
static bool make_map(CUtensorMap &m, const float *base, const SpeOp<float> &A, int TK, int TJ)
{
    EncodeTiledFn fn = encode_tiled();
    if (!fn || !base || (reinterpret_cast<unsigned long long>(base) & 15ull)) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)A.nzc, (cuuint64_t)A.nyc, (cuuint64_t)A.nxc};
    const cuuint64_t strides[2] = {(cuuint64_t)A.nzc * 4, (cuuint64_t)A.nyc * A.nzc * 4};
    const cuuint32_t box[3] = {(cuuint32_t)(TK + 8), (cuuint32_t)(TJ + 2), 1};
    const cuuint32_t es[3] = {1, 1, 1};
    return fn(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int TK, bool FZ>
static bool tma_attrs_v(size_t &smem, int &per_sm)
{
    smem = CgTile<TK>::smem(2);
    if (cudaFuncSetAttribute(k_cg_pq_tma<false, TK, FZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess ||
        cudaFuncSetAttribute(k_cg_pq_tma<true, TK, FZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)CgTile<TK>::smem(1)) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_pq_tma<false, TK, FZ>, kBlock, smem) !=
            cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return per_sm > 0;
}

template <int TK>
static bool tma_attrs(size_t &smem, int &per_sm)
{
    int a = 0, b = 0;
    if (!tma_attrs_v<TK, false>(smem, a) || !tma_attrs_v<TK, true>(smem, b)) return false;
    per_sm = a < b ? a : b;
    return true;
}

bool cg_tma_setup(CgTma &t, const FvOp<float> &F, const float *z, const float *h, const float *p,
                  const float *p_alt, int sms, int red_blocks)
{
    t.ok = false;
    const SpeOp<float> &A = F.A;
    if (A.nzc % 4 != 0) return false;
    if (A.pz) return false;  // the boxes' zero fill at the z ends is the Neumann halo, not a wrapped one
    if (const char *e = std::getenv("CFDGPU_NO_TMA"))
        if (e[0] == '1') return false;
    t.TK = A.nzc >= 24 ? 32 : (A.nzc >= 12 ? 16 : 8);
    t.TJ = kBlock / (t.TK / 4);
    int per_sm = 0;
    bool ok = t.TK == 32 ? tma_attrs<32>(t.smem, per_sm) : t.TK == 16 ? tma_attrs<16>(t.smem, per_sm)
                                                                      : tma_attrs<8>(t.smem, per_sm);
    if (!ok) return false;
    t.grid = per_sm * sms < red_blocks ? per_sm * sms : red_blocks;
    // z formed from h in the stencil kernel (default): 8 fewer bytes per row
    // and iteration for a few more operations; measured 6% (4.2 M cells) and
    // 12% (33.5 M cells) faster per step than reading a z vector
    t.form_z = true;
    if (const char *e = std::getenv("CFDGPU_CG_FORM_Z")) t.form_z = e[0] != '0';
    if (!make_map(t.zh, t.form_z ? h : z, A, t.TK, t.TJ) || !make_map(t.zv, z, A, t.TK, t.TJ) ||
        !make_map(t.p, p, A, t.TK, t.TJ) ||
        !make_map(t.palt, p_alt, A, t.TK, t.TJ))
        return false;
    t.ok = true;
    return true;
}

int cg_resident_grid(int sms, int red_blocks)
{
    int a = 0, b = 0, d = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_cg_pq<false>, kBlock, 0) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_cg_upd, kBlock, 0) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d, k_cg_upd_fv, kBlock, 0) != cudaSuccess) {
        cudaGetLastError();
        return red_blocks;
    }
    int per_sm = a < b ? a : b;
    per_sm = per_sm < d ? per_sm : d;
    const int g = per_sm > 0 ? per_sm * sms : red_blocks;
    return g < red_blocks ? g : red_blocks;
}

void launch_cg_ip(cfd_launch_ctx &c, const FvOp<float> &F, float *iP)
{
    k_cg_ip<<<blocks_for(F.A.n, c.grid_cap), kBlock, 0, c.s>>>(F, iP);
}

void launch_cg_part(cfd_launch_ctx &c, const FvOp<float> &F, const float *iP, float *e, float *h, float *z,
                    float *p, float *pn, float *q, BicgScal *sc, int part, const CgTma *tma)
{
    if (tma && tma->ok) {  // z (or h), p = the buffers of the maps
        if (part == 0) launch_cg_pq_tma(c, F, *tma, false, &tma->zh, &tma->p, pn, q, sc, tma->form_z);
        else if (tma->form_z) k_cg_upd_fv<<<c.cg_grid, kBlock, 0, c.s>>>(F, e, pn, h, q, sc, c.partials, c.counter);
        else k_cg_upd<<<c.cg_grid, kBlock, 0, c.s>>>(F.A.n, e, pn, h, q, iP, z, sc, c.partials, c.counter);
        return;
    }
    if (part == 0) {
        const CgShape cs = cg_shape(c, F);
        k_cg_pq<false><<<cs.grid, kBlock, 0, c.s>>>(F, z, p, pn, q, sc, c.partials, c.counter, cs.TK, cs.ichunk);
    } else {
        k_cg_upd<<<c.cg_grid, kBlock, 0, c.s>>>(F.A.n, e, pn, h, q, iP, z, sc, c.partials, c.counter);
    }
}

// per-axis tables of the finite-volume form: out[i] = cm + cp (the diagonal
// share of the axis), out[n + i] = the interior cell width (16-byte aligned
// when n is a multiple of 4, for float4 loads)
__global__ void k_fv_axes(int n, const float *__restrict__ c, const float *__restrict__ width, float *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        out[i] = c[i] + c[n + i];
        out[n + i] = width[i];
    }
}

void launch_fv_axes(cudaStream_t s, int n, const float *c, const float *width, float *out)
{
    k_fv_axes<<<(n + 127) / 128, 128, 0, s>>>(n, c, width, out);
}

// NaN/Inf reset at the iteration cap (bicgstabRe2.hpp:143-163): non-finite
// entries of x take the previous initial guess px1; if more than 10% were
// reset, x becomes the guess before that (px2).
template <class V>
__global__ void __launch_bounds__(kBlock)
k_bicg_nonfinite(long long n, V *__restrict__ x, const V *__restrict__ px1, BicgScal *sc,
                 double *partials, unsigned int *counter)
{
    double acc[1] = {0.0};
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < n;
         row += (long long)gridDim.x * blockDim.x) {
        const V v = x[row];
        if (!isfinite((double)v)) {
            x[row] = px1[row];
            acc[0] += 1.0;
        }
    }
    double tot[1];
    if (grid_reduce<1>(acc, partials, counter, tot) && threadIdx.x == 0) sc->nonfinite = (int)tot[0];
}

template <class V>
__global__ void k_bicg_px2(long long n, V *__restrict__ x, const V *__restrict__ px2, const BicgScal *sc)
{
    if (!((double)sc->nonfinite > (double)n * 0.1)) return;
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < n;
         row += (long long)gridDim.x * blockDim.x)
        x[row] = px2[row];
}

template <class Op, class V>
void launch_bicg_init(cfd_launch_ctx &c, const Op &A, const V *b, V *x, const BicgVecs<V> &w,
                      V *px1, V *px2, BicgScal *sc)
{
    k_bicg_init<Op, V><<<c.red_blocks, kBlock, 0, c.s>>>(A, b, x, w.r0, w.r1, w.p1, px1, px2, sc,
                                                         c.partials, c.counter);
}

template <class Op, class V>
void launch_bicg_iteration(cfd_launch_ctx &c, const Op &A, V *x, const BicgVecs<V> &w, BicgScal *sc)
{
    const int G = c.red_blocks;
    k_bicg_ap<Op, V><<<G, kBlock, 0, c.s>>>(A, w.p1, w.r0, w.ap, sc, c.partials, c.counter);
    k_bicg_s<V><<<G, kBlock, 0, c.s>>>(A.n, w.r1, w.ap, w.s1, sc);
    k_bicg_as<Op, V><<<G, kBlock, 0, c.s>>>(A, w.s1, w.as, sc, c.partials, c.counter);
    k_bicg_xr<V><<<G, kBlock, 0, c.s>>>(A.n, x, w.p1, w.s1, w.as, w.r0, w.r1, sc, c.partials, c.counter);
    k_bicg_p<V><<<G, kBlock, 0, c.s>>>(A.n, w.r0, w.r1, w.p1, w.ap, sc);
}

template <class Op, class V>
void launch_bicg_iteration_part(cfd_launch_ctx &c, const Op &A, V *x, const BicgVecs<V> &w, BicgScal *sc,
                                int part)
{
    const int G = c.red_blocks;
    switch (part) {
    case 0: k_bicg_ap<Op, V><<<G, kBlock, 0, c.s>>>(A, w.p1, w.r0, w.ap, sc, c.partials, c.counter); break;
    case 1: k_bicg_s<V><<<G, kBlock, 0, c.s>>>(A.n, w.r1, w.ap, w.s1, sc); break;
    case 2: k_bicg_as<Op, V><<<G, kBlock, 0, c.s>>>(A, w.s1, w.as, sc, c.partials, c.counter); break;
    case 3: k_bicg_xr<V><<<G, kBlock, 0, c.s>>>(A.n, x, w.p1, w.s1, w.as, w.r0, w.r1, sc, c.partials, c.counter); break;
    default: k_bicg_p<V><<<G, kBlock, 0, c.s>>>(A.n, w.r0, w.r1, w.p1, w.ap, sc); break;
    }
}
#define CFD_PART_INST(OP, V)                                                                        \
    template void launch_bicg_iteration_part<OP, V>(cfd_launch_ctx &, const OP &, V *, const BicgVecs<V> &, \
                                                    BicgScal *, int);
CFD_PART_INST(SpeOp<double>, double)
CFD_PART_INST(EllOp<double>, double)
CFD_PART_INST(SpeOp<float>, float)
CFD_PART_INST(EllOp<float>, float)

template <class V>
void launch_bicg_nan_reset(cfd_launch_ctx &c, long long n, V *x, const V *px1, const V *px2,
                           BicgScal *sc)
{
    k_bicg_nonfinite<V><<<c.red_blocks, kBlock, 0, c.s>>>(n, x, px1, sc, c.partials, c.counter);
    k_bicg_px2<V><<<blocks_for(n, c.grid_cap), kBlock, 0, c.s>>>(n, x, px2, sc);
}

template void launch_bicg_init<SpeOp<double>, double>(cfd_launch_ctx &, const SpeOp<double> &,
    const double *, double *, const BicgVecs<double> &, double *, double *, BicgScal *);
template void launch_bicg_init<EllOp<double>, double>(cfd_launch_ctx &, const EllOp<double> &,
    const double *, double *, const BicgVecs<double> &, double *, double *, BicgScal *);
template void launch_bicg_init<SpeOp<float>, float>(cfd_launch_ctx &, const SpeOp<float> &,
    const float *, float *, const BicgVecs<float> &, float *, float *, BicgScal *);
template void launch_bicg_init<EllOp<float>, float>(cfd_launch_ctx &, const EllOp<float> &,
    const float *, float *, const BicgVecs<float> &, float *, float *, BicgScal *);
template void launch_bicg_iteration<SpeOp<double>, double>(cfd_launch_ctx &, const SpeOp<double> &,
    double *, const BicgVecs<double> &, BicgScal *);
template void launch_bicg_iteration<EllOp<double>, double>(cfd_launch_ctx &, const EllOp<double> &,
    double *, const BicgVecs<double> &, BicgScal *);
template void launch_bicg_iteration<SpeOp<float>, float>(cfd_launch_ctx &, const SpeOp<float> &,
    float *, const BicgVecs<float> &, BicgScal *);
template void launch_bicg_iteration<EllOp<float>, float>(cfd_launch_ctx &, const EllOp<float> &,
    float *, const BicgVecs<float> &, BicgScal *);
template void launch_bicg_nan_reset<double>(cfd_launch_ctx &, long long, double *, const double *,
                                            const double *, BicgScal *);

// ---------------------------------------------------------------------------
// SOR (SorPipeLine.seq.hpp:30-117) in red-black order with colour-split
// coefficients (the layout is described with launch_sor_coef_rb in
// kernels.h).  Every value is formed with the reference's operations in its
// order, each rounded on its own (no contraction into FMAs), so the sweeps
// are bit-for-bit those of a sequential red-black loop: the cells of one
// colour do not read each other.

// slot -> cell of colour c; false for the unused last slot of a short row
__device__ __forceinline__ bool sor_cell_of(const Geo &g, FastDiv fpairs, int colour, int i0, unsigned t, int &i,
                                            int &j, int &k)
{
    const unsigned jj = fpairs.div(t);
    const int m = (int)(t - jj * fpairs.d);
    i = i0 + GC;
    j = (int)jj + GC;
    k = GC + ((i + j + GC + colour) & 1) + 2 * m;
    return k < g.nz - GC;
}

__global__ void k_sor_coef_rb(Geo g, FastDiv fpairs, const double *__restrict__ Dx, const double *__restrict__ Dy,
                              const double *__restrict__ Dz, const double *__restrict__ Dxs,
                              const double *__restrict__ Dys, const double *__restrict__ Dzs, double *__restrict__ cf)
{
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    const int colour = blockIdx.z;
    if (t >= (unsigned)g.nyc * fpairs.d) return;
    const long long nh = (long long)g.nxc * g.nyc * fpairs.d;
    const long long h = (long long)blockIdx.y * g.nyc * fpairs.d + t;
    double *o = cf + (long long)colour * 7 * nh + h;
    int i, j, k;
    if (!sor_cell_of(g, fpairs, colour, blockIdx.y, t, i, j, k)) {
        // unused slot: a zero row that changes nothing
        for (int q = 0; q < 7; ++q) o[q * nh] = 0.0;
        return;
    }
    // grid::coef products and SorPipeLine.seq.hpp:30-43 quotients, in order
    const double yz = __dmul_rn(Dy[j], Dz[k]), xz = __dmul_rn(Dx[i], Dz[k]), xy = __dmul_rn(Dx[i], Dy[j]);
    const double c0 = __ddiv_rn(yz, Dxs[i]), c1 = __ddiv_rn(yz, Dxs[i - 1]);
    const double c2 = __ddiv_rn(xz, Dys[j]), c3 = __ddiv_rn(xz, Dys[j - 1]);
    const double c4 = __ddiv_rn(xy, Dzs[k]), c5 = __ddiv_rn(xy, Dzs[k - 1]);
    double sum = __dadd_rn(c0, c1);
    sum = __dadd_rn(sum, c2);
    sum = __dadd_rn(sum, c3);
    sum = __dadd_rn(sum, c4);
    sum = __dadd_rn(sum, c5);
    o[0] = c0;
    o[nh] = c1;
    o[2 * nh] = c2;
    o[3 * nh] = c3;
    o[4 * nh] = c4;
    o[5 * nh] = c5;
    o[6 * nh] = __ddiv_rn(-1.0, sum);
}

void launch_sor_coef_rb(cudaStream_t s, const Geo &g, const double *Dx, const double *Dy, const double *Dz,
                        const double *Dxs, const double *Dys, const double *Dzs, double *cf)
{
    const FastDiv fp((unsigned)sor_pairs(g));
    const dim3 grid((unsigned)((g.nyc * sor_pairs(g) + kBlock - 1) / kBlock), (unsigned)g.nxc, 2);
    k_sor_coef_rb<<<grid, kBlock, 0, s>>>(g, fp, Dx, Dy, Dz, Dxs, Dys, Dzs, cf);
}

// mass change / dt (SorPipeLine.seq.hpp:48-60), the reference's operation order
template <class T>
__global__ void k_sor_rhs_rb(Geo g, FastDiv fpairs, Metrics<double> m, double rdt, const T *__restrict__ u1,
                             const T *__restrict__ v1, const T *__restrict__ w1, double *__restrict__ rhs,
                             BicgScal *sc, SorAcc *acc)
{
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    const int colour = blockIdx.z;
    if (t == 0 && blockIdx.y == 0 && colour == 0) {
        sc->done = BICG_RUNNING;
        sc->iter = 0;
        sc->relres = 0.0;
        acc->mx[0] = acc->mx[1] = 0ull;
        acc->ticket = 0u;
    }
    if (t >= (unsigned)g.nyc * fpairs.d) return;
    const long long nh = (long long)g.nxc * g.nyc * fpairs.d;
    const long long h = (long long)blockIdx.y * g.nyc * fpairs.d + t;
    int i, j, k;
    if (!sor_cell_of(g, fpairs, colour, blockIdx.y, t, i, j, k)) {
        rhs[colour * nh + h] = 0.0;
        return;
    }
    const long long ic = icel(g, i, j, k);
    const double Dx = m.x(AX_D, i), Dy = m.y(AX_D, j), Dz = m.z(AX_D, k);
    const double du = __dsub_rn((double)u1[ic], (double)u1[ic - g.sx]);
    const double dv = __dsub_rn((double)v1[ic], (double)v1[ic - g.sy]);
    const double dw = __dsub_rn((double)w1[ic], (double)w1[ic - 1]);
    double mc = __dmul_rn(__dmul_rn(du, Dy), Dz);
    mc = __dadd_rn(mc, __dmul_rn(__dmul_rn(dv, Dx), Dz));
    mc = __dadd_rn(mc, __dmul_rn(__dmul_rn(dw, Dx), Dy));
    rhs[colour * nh + h] = __dmul_rn(mc, rdt);
}

template <class T>
void launch_sor_rhs_rb(cudaStream_t s, const Geo &g, const Metrics<double> &m, double rdt, const T *u1,
                       const T *v1, const T *w1, double *rhs, BicgScal *sc, SorAcc *acc)
{
    const FastDiv fp((unsigned)sor_pairs(g));
    const dim3 grid((unsigned)((g.nyc * sor_pairs(g) + kBlock - 1) / kBlock), (unsigned)g.nxc, 2);
    k_sor_rhs_rb<T><<<grid, kBlock, 0, s>>>(g, fp, m, rdt, u1, v1, w1, rhs, sc, acc);
}
template void launch_sor_rhs_rb<double>(cudaStream_t, const Geo &, const Metrics<double> &, double, const double *,
                                        const double *, const double *, double *, BicgScal *, SorAcc *);
template void launch_sor_rhs_rb<float>(cudaStream_t, const Geo &, const Metrics<double> &, double, const float *,
                                       const float *, const float *, double *, BicgScal *, SorAcc *);

// One colour of a sweep.  The second colour's last block (by ticket) closes
// the sweep: the do-while test of SorPipeLine.seq.hpp:112 on the larger of
// the two colours' maxima.
__global__ void __launch_bounds__(kBlock)
k_sor_rb(Geo g, FastDiv fpairs, const double *__restrict__ cf, const double *__restrict__ rhs, double *p,
         double omega, double tol, int itmax, int colour, BicgScal *sc, SorAcc *acc)
{
    if (*(volatile int *)&sc->done != BICG_RUNNING) return;
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    const long long nh = (long long)g.nxc * g.nyc * fpairs.d;
    double mx = 0.0;
    int i, j, k;
    if (t < (unsigned)g.nyc * fpairs.d && sor_cell_of(g, fpairs, colour, blockIdx.y, t, i, j, k)) {
        const long long h = (long long)blockIdx.y * g.nyc * fpairs.d + t;
        const double *c = cf + (long long)colour * 7 * nh + h;
        const long long ic = icel(g, i, j, k);
        // (-p[+x] c0 - p[-x] c1 - p[+y] c2 - p[-y] c3 - p[+z] c4 - p[-z] c5 + rhs) c6
        double s = __dmul_rn(-p[ic + g.sx], __ldg(c));
        s = __dsub_rn(s, __dmul_rn(p[ic - g.sx], __ldg(c + nh)));
        s = __dsub_rn(s, __dmul_rn(p[ic + g.sy], __ldg(c + 2 * nh)));
        s = __dsub_rn(s, __dmul_rn(p[ic - g.sy], __ldg(c + 3 * nh)));
        s = __dsub_rn(s, __dmul_rn(p[ic + 1], __ldg(c + 4 * nh)));
        s = __dsub_rn(s, __dmul_rn(p[ic - 1], __ldg(c + 5 * nh)));
        s = __dadd_rn(s, __ldg(rhs + colour * nh + h));
        const double pnew = __dmul_rn(s, __ldg(c + 6 * nh));
        const double pc = p[ic];
        const double d = __dsub_rn(pnew, pc);
        p[ic] = __dadd_rn(pc, __dmul_rn(omega, d));
        mx = fabs(d);  // a NaN wins the maximum and ends the solve
    }
    grid_max_nonneg(mx, &acc->mx[colour]);
    if (colour == 0) return;
    __shared__ bool last;
    __threadfence();
    if (threadIdx.x == 0) {
        const unsigned nb = gridDim.x * gridDim.y;
        last = atomicAdd(&acc->ticket, 1u) == nb - 1;
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    const unsigned long long b0 = atomicAdd(&acc->mx[0], 0ull), b1 = atomicAdd(&acc->mx[1], 0ull);
    const double res = __longlong_as_double((long long)(b0 > b1 ? b0 : b1));
    const int it = sc->iter + 1;
    sc->iter = it;
    if (!(res > tol && it < itmax)) {
        sc->relres = res;
        sc->done = res > tol ? BICG_CAPPED : BICG_CONVERGED;
    }
    acc->mx[0] = acc->mx[1] = 0ull;
    acc->ticket = 0u;
}

void launch_sor_rb_colour(cudaStream_t s, const Geo &g, const double *cf, const double *rhs, double *p,
                          double omega, double tol, int itmax, int colour, BicgScal *sc, SorAcc *acc)
{
    const FastDiv fp((unsigned)sor_pairs(g));
    const dim3 grid((unsigned)((g.nyc * sor_pairs(g) + kBlock - 1) / kBlock), (unsigned)g.nxc);
    k_sor_rb<<<grid, kBlock, 0, s>>>(g, fp, cf, rhs, p, omega, tol, itmax, colour, sc, acc);
}

void launch_sor_rb_sweep(cudaStream_t s, const Geo &g, const double *cf, const double *rhs, double *p,
                         double omega, double tol, int itmax, BicgScal *sc, SorAcc *acc)
{
    launch_sor_rb_colour(s, g, cf, rhs, p, omega, tol, itmax, 0, sc, acc);
    launch_sor_rb_colour(s, g, cf, rhs, p, omega, tol, itmax, 1, sc, acc);
}

// ---- mixed-precision SOR (the FP32 sweeps of an FP64 defect correction) ----
// rho = sum_q c_q p_q - rhs - (sum c) p at every cell, FP64, stored in FP32
// in icelCal order: the right-hand side of the correction equation
// (sum c) e - sum_q c_q e_q = rho, whose solution added to p satisfies the
// SOR equations (a Jacobi step would change p by rho / sum c)
__global__ void __launch_bounds__(kBlock)
k_sor_residual(Geo g, FastDiv fpairs, const double *__restrict__ cf, const double *__restrict__ rhs,
               const double *__restrict__ p, float *__restrict__ rho, const BicgScal *sc)
{
    if (*(volatile const int *)&sc->done != BICG_RUNNING) return;
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    const int colour = blockIdx.z;
    if (t >= (unsigned)g.nyc * fpairs.d) return;
    const long long nh = (long long)g.nxc * g.nyc * fpairs.d;
    const long long h = (long long)blockIdx.y * g.nyc * fpairs.d + t;
    int i, j, k;
    if (!sor_cell_of(g, fpairs, colour, blockIdx.y, t, i, j, k)) return;
    const double *c = cf + (long long)colour * 7 * nh + h;
    const long long ic = icel(g, i, j, k);
    const double c0 = __ldg(c), c1 = __ldg(c + nh), c2 = __ldg(c + 2 * nh), c3 = __ldg(c + 3 * nh);
    const double c4 = __ldg(c + 4 * nh), c5 = __ldg(c + 5 * nh);
    double s = -__ldg(rhs + colour * nh + h);
    s = fma(p[ic + g.sx], c0, s);
    s = fma(p[ic - g.sx], c1, s);
    s = fma(p[ic + g.sy], c2, s);
    s = fma(p[ic - g.sy], c3, s);
    s = fma(p[ic + 1], c4, s);
    s = fma(p[ic - 1], c5, s);
    const double sum = ((c0 + c1) + (c2 + c3)) + (c4 + c5);
    rho[icelcal(g, i, j, k)] = (float)fma(-sum, p[ic], s);
}

void launch_sor_residual(cudaStream_t s, const Geo &g, const double *cf, const double *rhs, const double *p,
                         float *rho, const BicgScal *sc)
{
    const FastDiv fp((unsigned)sor_pairs(g));
    const dim3 grid((unsigned)((g.nyc * sor_pairs(g) + kBlock - 1) / kBlock), (unsigned)g.nxc, 2);
    k_sor_residual<<<grid, kBlock, 0, s>>>(g, fp, cf, rhs, p, rho, sc);
}

// p += e and e = 0 over the interior; the FP32 sweeps join the sweep count
__global__ void k_sor_correct(Geo g, double *__restrict__ p, float *__restrict__ e, int sweeps, BicgScal *sc)
{
    if (*(volatile int *)&sc->done != BICG_RUNNING) return;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0) sc->iter += sweeps;
    if (t >= g.n) return;
    const unsigned t32 = (unsigned)t;
    const unsigned ii = g.fsxc.div(t32), rem = t32 - ii * (unsigned)g.sxc, jj = g.fsyc.div(rem);
    const long long ic = icel(g, (int)ii + GC, (int)jj + GC, (int)(rem - jj * (unsigned)g.syc) + GC);
    p[ic] += (double)e[t];
    e[t] = 0.f;
}

void launch_sor_correct(cudaStream_t s, const Geo &g, double *p, float *e, int sweeps, BicgScal *sc)
{
    k_sor_correct<<<(unsigned)((g.n + kBlock - 1) / kBlock), kBlock, 0, s>>>(g, p, e, sweeps, sc);
}

// the inner tolerance of the next solve (stream-ordered)
__global__ void k_set_tol(BicgScal *sc, double tol) { sc->tol = tol; }

void launch_set_tol(cudaStream_t s, BicgScal *sc, double tol) { k_set_tol<<<1, 1, 0, s>>>(sc, tol); }

// ---------------------------------------------------------------------------
// Device-side solve loops: the condition of the graph's WHILE node
__global__ void k_loop_cond(cudaGraphConditionalHandle h, BicgScal *sc, int cap, int first)
{
    if (threadIdx.x != 0) return;
    const int trips = first ? 0 : sc->loop_trips + 1;
    sc->loop_trips = trips;
    cudaGraphSetConditional(h, (sc->done == BICG_RUNNING && !sc->wait_timeout && trips < cap) ? 1u : 0u);
}

void launch_loop_cond(cudaStream_t s, cudaGraphConditionalHandle h, BicgScal *sc, int cap, int first)
{
    k_loop_cond<<<1, 32, 0, s>>>(h, sc, cap, first);
}

// ---- the defect correction's outer loop on the device ------------------------
// The host loop of solve_mixed, step for step: stop when |r| / |b| < tol or
// the ratio is not finite, fail at the sweep cap; before each sweep the inner
// tolerance max(inner_tol, min(0.5, adapt tol / rel)).
__device__ void outer_decide(cudaGraphConditionalHandle h, OuterScal *os, BicgScal *sc_in, const OuterCfg &cfg)
{
    if (os->state == OUTER_RUNNING) {
        if (os->rel < cfg.tol) os->state = OUTER_CONVERGED;
        else if (!isfinite(os->rel)) os->state = OUTER_NONFINITE;
        else if (os->sweeps >= cfg.max_outer) os->state = OUTER_CAPPED;
    }
    const bool go = os->state == OUTER_RUNNING && os->loop_trips < cfg.cap;
    if (go) sc_in->tol = cfg.adapt > 0.0 ? fmax(cfg.inner_tol, fmin(0.5, cfg.adapt * cfg.tol / os->rel)) : cfg.inner_tol;
    cudaGraphSetConditional(h, go ? 1u : 0u);
}

__global__ void k_outer_start(cudaGraphConditionalHandle h, OuterScal *os, const double *norm2, BicgScal *sc_in,
                              OuterCfg cfg)
{
    if (threadIdx.x != 0) return;
    os->norm0 = sqrt(norm2[1]);
    os->rel = os->norm0 == 0.0 ? 0.0 : sqrt(norm2[0]) / os->norm0;  // NaN stays NaN
    os->sweeps = os->iters = os->inner_trips = os->loop_trips = 0;
    os->state = os->norm0 == 0.0 ? OUTER_ZERO_RHS : OUTER_RUNNING;
    outer_decide(h, os, sc_in, cfg);
}

__global__ void k_outer_inner_done(OuterScal *os, const BicgScal *sc_in)
{
    if (threadIdx.x != 0) return;
    os->iters += sc_in->iter;
    os->inner_trips += sc_in->loop_trips;
    if (sc_in->wait_timeout) os->state = OUTER_INNER_WAIT;
    else if (sc_in->done == BICG_RUNNING) os->state = OUTER_INNER_CAP;
    else if (!(sc_in->relres < 1.0)) os->state = OUTER_DIVERGED;  // the host loop counts this sweep too
    if (os->state != OUTER_RUNNING && os->state != OUTER_INNER_WAIT && os->state != OUTER_INNER_CAP) os->sweeps += 1;
}

__global__ void k_outer_next(cudaGraphConditionalHandle h, OuterScal *os, const double *norm2, BicgScal *sc_in,
                             OuterCfg cfg)
{
    if (threadIdx.x != 0) return;
    os->loop_trips += 1;
    if (os->state == OUTER_RUNNING) {
        os->sweeps += 1;
        os->rel = sqrt(norm2[0]) / os->norm0;
    }
    outer_decide(h, os, sc_in, cfg);
}

void launch_outer_start(cudaStream_t s, cudaGraphConditionalHandle h, OuterScal *os, const double *norm2,
                        BicgScal *sc_in, OuterCfg cfg)
{
    k_outer_start<<<1, 32, 0, s>>>(h, os, norm2, sc_in, cfg);
}
void launch_outer_inner_done(cudaStream_t s, OuterScal *os, const BicgScal *sc_in)
{
    k_outer_inner_done<<<1, 32, 0, s>>>(os, sc_in);
}
void launch_outer_next(cudaStream_t s, cudaGraphConditionalHandle h, OuterScal *os, const double *norm2,
                       BicgScal *sc_in, OuterCfg cfg)
{
    k_outer_next<<<1, 32, 0, s>>>(h, os, norm2, sc_in, cfg);
}

// ---------------------------------------------------------------------------
// Mixed precision: FP64 residual of the scaled system, written as the
// FP32 right-hand side of the next inner solve, and the FP64 correction.
// (BN: also |b|^2 in the same pass, the defect correction's reference
// norm).  The kernel is bound by the FP64 pipe, so |r|^2 is summed in FP32
// per thread from the FP32 residual it stores (a relative error near 1e-7
// in a stopping test), and only the stencil and b - A x run in FP64.
template <class Op, class V, bool BN>
__global__ void __launch_bounds__(kBlock)
k_residual64(Op A, const double *__restrict__ b, const double *__restrict__ x, V *__restrict__ r32,
             double *partials, unsigned int *counter, double *out, double *bout)
{
    float ra = 0.f;
    double bb = 0.0;
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < A.n;
         row += (long long)gridDim.x * blockDim.x) {
        const double bv = b[row];
        const V r = (V)(bv - apply_row(A, x, row));
        r32[row] = r;
        ra = fmaf((float)r, (float)r, ra);
        if constexpr (BN) bb = fma(bv, bv, bb);
    }
    if constexpr (BN) {
        double acc[2] = {(double)ra, bb}, tot[2];
        if (grid_reduce<2>(acc, partials, counter, tot) && threadIdx.x == 0) {
            *out = tot[0];
            *bout = tot[1];
        }
    } else {
        float acc[1] = {ra};
        double tot[1];
        if (grid_reduce_f<1>(acc, partials, counter, tot) && threadIdx.x == 0) *out = tot[0];
    }
}

template <class V>
void launch_residual64(cfd_launch_ctx &c, const SpeOp<double> &A, const double *b, const double *x,
                       V *r32, double *norm2_out, double *bnorm2_out)
{
    if (bnorm2_out)
        k_residual64<SpeOp<double>, V, true><<<c.red_blocks, kBlock, 0, c.s>>>(A, b, x, r32, c.partials, c.counter,
                                                                               norm2_out, bnorm2_out);
    else
        k_residual64<SpeOp<double>, V, false><<<c.red_blocks, kBlock, 0, c.s>>>(A, b, x, r32, c.partials, c.counter,
                                                                                norm2_out, nullptr);
}
template <class V>
void launch_residual64_ell(cfd_launch_ctx &c, const EllOp<double> &A, const double *b,
                           const double *x, V *r32, double *norm2_out, double *bnorm2_out)
{
    if (bnorm2_out)
        k_residual64<EllOp<double>, V, true><<<c.red_blocks, kBlock, 0, c.s>>>(A, b, x, r32, c.partials, c.counter,
                                                                               norm2_out, bnorm2_out);
    else
        k_residual64<EllOp<double>, V, false><<<c.red_blocks, kBlock, 0, c.s>>>(A, b, x, r32, c.partials, c.counter,
                                                                                norm2_out, nullptr);
}
template void launch_residual64<float>(cfd_launch_ctx &, const SpeOp<double> &, const double *,
                                       const double *, float *, double *, double *);
template void launch_residual64_ell<float>(cfd_launch_ctx &, const EllOp<double> &, const double *,
                                           const double *, float *, double *, double *);

// x += e (FP64 accumulation of an FP32 correction)
template <class V>
__global__ void k_correct(long long n, double *__restrict__ x, const V *__restrict__ e, const double *scale)
{
    const double sc = scale ? *scale : 1.0;
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < n;
         row += (long long)gridDim.x * blockDim.x)
        x[row] += sc * (double)e[row];
}

// x += scale e (scale: a device scalar, 1 when null)
template <class V>
void launch_correct(cfd_launch_ctx &c, long long n, double *x, const V *e, const double *scale)
{
    k_correct<V><<<blocks_for(n, c.grid_cap), kBlock, 0, c.s>>>(n, x, e, scale);
}
template void launch_correct<float>(cfd_launch_ctx &, long long, double *, const float *, const double *);

__global__ void k_extrapolate(long long n, double *__restrict__ x, const double *__restrict__ h0,
                              const double *__restrict__ h1, const double *__restrict__ h2)
{
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < n;
         row += (long long)gridDim.x * blockDim.x)
        x[row] = h2 ? 3.0 * (h2[row] - h1[row]) + h0[row] : 2.0 * h1[row] - h0[row];
}

void launch_extrapolate(cfd_launch_ctx &c, long long n, double *x, const double *h0, const double *h1,
                        const double *h2)
{
    k_extrapolate<<<blocks_for(n, c.grid_cap), kBlock, 0, c.s>>>(n, x, h0, h1, h2);
}

__global__ void k_correct_gated(long long n, double *__restrict__ x, const float *__restrict__ e, const double *scale,
                                const OuterScal *os)
{
    if (os->state != OUTER_RUNNING) return;
    const double sc = scale ? *scale : 1.0;
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < n;
         row += (long long)gridDim.x * blockDim.x)
        x[row] += sc * (double)e[row];
}

void launch_correct_gated(cfd_launch_ctx &c, long long n, double *x, const float *e, const double *scale,
                          const OuterScal *os)
{
    k_correct_gated<<<blocks_for(n, c.grid_cap), kBlock, 0, c.s>>>(n, x, e, scale, os);
}

}  // namespace cfd
