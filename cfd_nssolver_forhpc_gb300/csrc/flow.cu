// flow.cu -- velocity-side kernels of the time step: QUICK convection-
// diffusion, predictor-corrector source coupling, Poisson right-hand side,
// projection + direct forcing, drag/lift, boundary conditions, immersed-body
// volume fraction and the divergence check.  Templates on the velocity type
// T (double for the FP64 path, float for the mixed-precision path); the
// pressure, Poisson vectors and all reductions stay FP64.
#include "cfd_internal.cuh"
#include "kernels.h"

namespace cfd {

// ---------------------------------------------------------------------------
// QUICK face values.  quick_a follows QuickUnitA and quick_b QuickUnitB
// (inc/source/convection_and_difussion.hpp:20-84): the upwind choice picks
// the curvature factor and the two one-sided gradients, then one formula
// evaluates the face value.
template <class T>
__device__ __forceinline__ void quick_a(T Up, T Un, T pp, T p, T c, T n, T nn, const Axis<T> &a,
                                        int I, T &phiP, T &phiN)
{
    const T pc = p - c, cn = c - n;
    T cf, g1, r1, g2, r2;
    if (Up > T(0)) { cf = a(AX_CAPP, I); g1 = pc;     r1 = a(AX_RD, I + 1); g2 = cn; r2 = a(AX_RD, I); }
    else           { cf = a(AX_CAPN, I); g1 = pp - p; r1 = a(AX_RD, I + 2); g2 = pc; r2 = a(AX_RD, I + 1); }
    phiP = T(0.5) * (c + p) - cf * (g1 * r1 - g2 * r2);
    if (Un > T(0)) { cf = a(AX_CANP, I); g1 = cn; r1 = a(AX_RD, I);     g2 = n - nn; r2 = a(AX_RD, I - 1); }
    else           { cf = a(AX_CANN, I); g1 = pc; r1 = a(AX_RD, I + 1); g2 = cn;     r2 = a(AX_RD, I); }
    phiN = T(0.5) * (n + c) - cf * (g1 * r1 - g2 * r2);
}

template <class T>
__device__ __forceinline__ void quick_b(T Up, T Un, T pp, T p, T c, T n, T nn, const Axis<T> &a,
                                        int I, T &phiP, T &phiN)
{
    const T pc = p - c, cn = c - n;
    T cf, g1, r1, g2, r2;
    if (Up > T(0)) { cf = a(AX_CBPP, I); g1 = pc;     r1 = a(AX_RDS, I);     g2 = cn; r2 = a(AX_RDS, I - 1); }
    else           { cf = a(AX_CBPN, I); g1 = pp - p; r1 = a(AX_RDS, I + 1); g2 = pc; r2 = a(AX_RDS, I); }
    phiP = T(0.5) * (c + p) - cf * (g1 * r1 - g2 * r2);
    if (Un > T(0)) { cf = a(AX_CBNP, I); g1 = cn; r1 = a(AX_RDS, I - 1); g2 = n - nn; r2 = a(AX_RDS, I - 2); }
    else           { cf = a(AX_CBNN, I); g1 = pc; r1 = a(AX_RDS, I);     g2 = cn;     r2 = a(AX_RDS, I - 1); }
    phiN = T(0.5) * (n + c) - cf * (g1 * r1 - g2 * r2);
}

__device__ __forceinline__ void cell_of(const Geo &g, long long t, int &i, int &j, int &k)
{
    const unsigned int t32 = (unsigned int)t;
    const unsigned int ii = g.fsxc.div(t32);
    const unsigned int rem = t32 - ii * (unsigned int)g.sxc;
    const unsigned int jj = g.fsyc.div(rem);
    i = (int)ii + GC;
    j = (int)jj + GC;
    k = (int)(rem - jj * (unsigned int)g.syc) + GC;
}

// SmagorinskyModel (source/smagorinskyModel.hpp:31-78) with GradientGauss
// (:6-27): central differences 0.5/D (phi[-] - phi[+]) with the staggered
// width along the component's own axis; temp = |2 ux^2 + vy^2 + wz^2 +
// (uy + vx)^2 + (uz + wx)^2 + (vz + wy)^2| (the factor 2 on the first term
// only, as the reference writes it); nu_t = (0.18 delta)^2 sqrt(temp) with
// delta = (Dx Dy Dz)^(1/3).  One cell per thread, FP64.
template <class T>
__global__ void __launch_bounds__(kBlock)
k_smagorinsky(Geo g, Metrics<double> m, const T *__restrict__ u, const T *__restrict__ v, const T *__restrict__ w,
              T *__restrict__ vis)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.n) return;
    int i, j, k;
    cell_of(g, t, i, j, k);
    const long long ic = icel(g, i, j, k), sx = g.sx, sy = g.sy;
    auto D = [&](const T *f, long long s) { return (double)f[ic - s] - (double)f[ic + s]; };
    const double ux = 0.5 / m.x(AX_DS, i) * D(u, sx), uy = 0.5 / m.y(AX_D, j) * D(u, sy);
    const double uz = 0.5 / m.z(AX_D, k) * D(u, 1);
    const double vx = 0.5 / m.x(AX_D, i) * D(v, sx), vy = 0.5 / m.y(AX_DS, j) * D(v, sy);
    const double vz = 0.5 / m.z(AX_D, k) * D(v, 1);
    const double wx = 0.5 / m.x(AX_D, i) * D(w, sx), wy = 0.5 / m.y(AX_D, j) * D(w, sy);
    const double wz = 0.5 / m.z(AX_DS, k) * D(w, 1);
    const double temp = fabs(__dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(2.0, __dmul_rn(ux, ux)),
                                                                              __dmul_rn(vy, vy)),
                                                                    __dmul_rn(wz, wz)),
                                                          __dmul_rn(uy + vx, uy + vx)),
                                                __dmul_rn(uz + wx, uz + wx)),
                                      __dmul_rn(vz + wy, vz + wy)));
    const double delta = pow(m.x(AX_D, i) * m.y(AX_D, j) * m.z(AX_D, k), 1.0 / 3.0);
    const double cd = 0.18 * delta;
    vis[t] = (T)(__dmul_rn(cd, cd) * sqrt(temp));
}

// ConvectionDifussion (convection_and_difussion.hpp:168-446): explicit Euler
// u* = u + dt(-div(u u) + nu lap u) for the three staggered components of
// one cell per thread.  The normal component skips the domain's last face
// (d = 1, lines 193, 274, 357).  With src != nullptr the PC source is added
// at the same cell (aligned convention).
template <class T>
__global__ void __launch_bounds__(kBlock)
k_convdiff(Geo g, Metrics<T> m, T dt, T nudt, const T *__restrict__ u0, const T *__restrict__ v0,
           const T *__restrict__ w0, T *__restrict__ u1, T *__restrict__ v1, T *__restrict__ w1,
           const T *__restrict__ src, const T *__restrict__ vis, T nu)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.n) return;
    int i, j, k;
    cell_of(g, t, i, j, k);
    const long long sx = g.sx, sy = g.sy;
    const long long ic = icel(g, i, j, k);
    const Axis<T> &X = m.x, &Y = m.y, &Z = m.z;
    const T uc = __ldg(u0 + ic), vc = __ldg(v0 + ic), wc = __ldg(w0 + ic);
    // LES (TERBULENCE_SMAGORINSKY, convection_and_difussion.hpp:246-250):
    // the diffusion of this cell's faces uses nu + nu_t
    if (vis) nudt = (nu + vis[t]) * dt;
    const T u_xp = __ldg(u0 + ic + sx), u_xm = __ldg(u0 + ic - sx);
    const T v_yp = __ldg(v0 + ic + sy), v_ym = __ldg(v0 + ic - sy);
    const T w_zp = __ldg(w0 + ic + 1), w_zm = __ldg(w0 + ic - 1);

    if (i < g.nx - GC - 1) {  // ---- u, lines 196-269
        const T IT = X(AX_IT, i);
        const T Up = T(0.5) * (u_xp + uc), Un = T(0.5) * (u_xm + uc);
        const T Vp = vc + (__ldg(v0 + ic + sx) - vc) * IT;
        const T Vn = v_ym + (__ldg(v0 + ic - sy + sx) - v_ym) * IT;
        const T Wp = wc + (__ldg(w0 + ic + sx) - wc) * IT;
        const T Wn = w_zm + (__ldg(w0 + ic - 1 + sx) - w_zm) * IT;
        const T u_yp = __ldg(u0 + ic + sy), u_ym = __ldg(u0 + ic - sy);
        const T u_zp = __ldg(u0 + ic + 1), u_zm = __ldg(u0 + ic - 1);
        T uPx, uNx, uPy, uNy, uPz, uNz;
        quick_a(Up, Un, __ldg(u0 + ic + 2 * sx), u_xp, uc, u_xm, __ldg(u0 + ic - 2 * sx), X, i, uPx, uNx);
        quick_b(Vp, Vn, __ldg(u0 + ic + 2 * sy), u_yp, uc, u_ym, __ldg(u0 + ic - 2 * sy), Y, j, uPy, uNy);
        quick_b(Wp, Wn, __ldg(u0 + ic + 2), u_zp, uc, u_zm, __ldg(u0 + ic - 2), Z, k, uPz, uNz);
        const T conv = -dt * ((uPx * uPx - uNx * uNx) * X(AX_RDS, i) + (uPy * Vp - uNy * Vn) * Y(AX_RD, j)
                              + (uPz * Wp - uNz * Wn) * Z(AX_RD, k));
        const T diff = nudt * (((u_xp - uc) * X(AX_RD, i + 1) - (uc - u_xm) * X(AX_RD, i)) * X(AX_RDS, i)
                               + ((u_yp - uc) * Y(AX_RDS, j) - (uc - u_ym) * Y(AX_RDS, j - 1)) * Y(AX_RD, j)
                               + ((u_zp - uc) * Z(AX_RDS, k) - (uc - u_zm) * Z(AX_RDS, k - 1)) * Z(AX_RD, k));
        T r = uc + conv + diff;
        if (src) r += src[t];
        u1[ic] = r;
    }
    if (j < g.ny - GC - 1) {  // ---- v, lines 278-351
        const T IT = Y(AX_IT, j);
        const T Vp = T(0.5) * (v_yp + vc), Vn = T(0.5) * (v_ym + vc);
        const T Up = uc + (__ldg(u0 + ic + sy) - uc) * IT;
        const T Un = u_xm + (__ldg(u0 + ic - sx + sy) - u_xm) * IT;
        const T Wp = wc + (__ldg(w0 + ic + sy) - wc) * IT;
        const T Wn = w_zm + (__ldg(w0 + ic - 1 + sy) - w_zm) * IT;
        const T v_xp = __ldg(v0 + ic + sx), v_xm = __ldg(v0 + ic - sx);
        const T v_zp = __ldg(v0 + ic + 1), v_zm = __ldg(v0 + ic - 1);
        T vPx, vNx, vPy, vNy, vPz, vNz;
        quick_b(Up, Un, __ldg(v0 + ic + 2 * sx), v_xp, vc, v_xm, __ldg(v0 + ic - 2 * sx), X, i, vPx, vNx);
        quick_a(Vp, Vn, __ldg(v0 + ic + 2 * sy), v_yp, vc, v_ym, __ldg(v0 + ic - 2 * sy), Y, j, vPy, vNy);
        quick_b(Wp, Wn, __ldg(v0 + ic + 2), v_zp, vc, v_zm, __ldg(v0 + ic - 2), Z, k, vPz, vNz);
        const T conv = -dt * ((Up * vPx - Un * vNx) * X(AX_RD, i) + (vPy * vPy - vNy * vNy) * Y(AX_RDS, j)
                              + (Wp * vPz - Wn * vNz) * Z(AX_RD, k));
        const T diff = nudt * (((v_xp - vc) * X(AX_RDS, i) - (vc - v_xm) * X(AX_RDS, i - 1)) * X(AX_RD, i)
                               + ((v_yp - vc) * Y(AX_RD, j + 1) - (vc - v_ym) * Y(AX_RD, j)) * Y(AX_RDS, j)
                               + ((v_zp - vc) * Z(AX_RDS, k) - (vc - v_zm) * Z(AX_RDS, k - 1)) * Z(AX_RD, k));
        T r = vc + conv + diff;
        if (src) r += src[g.n + t];
        v1[ic] = r;
    }
    if (k < g.nz - GC - 1 + g.pz) {  // ---- w, lines 360-434 (periodic z: the top face too)
        const T IT = Z(AX_IT, k);
        const T Wp = T(0.5) * (w_zp + wc), Wn = T(0.5) * (w_zm + wc);
        const T Up = uc + (__ldg(u0 + ic + 1) - uc) * IT;
        const T Un = u_xm + (__ldg(u0 + ic - sx + 1) - u_xm) * IT;
        const T Vp = vc + (__ldg(v0 + ic + 1) - vc) * IT;
        const T Vn = v_ym + (__ldg(v0 + ic - sy + 1) - v_ym) * IT;
        const T w_xp = __ldg(w0 + ic + sx), w_xm = __ldg(w0 + ic - sx);
        const T w_yp = __ldg(w0 + ic + sy), w_ym = __ldg(w0 + ic - sy);
        T wPx, wNx, wPy, wNy, wPz, wNz;
        quick_b(Up, Un, __ldg(w0 + ic + 2 * sx), w_xp, wc, w_xm, __ldg(w0 + ic - 2 * sx), X, i, wPx, wNx);
        quick_b(Vp, Vn, __ldg(w0 + ic + 2 * sy), w_yp, wc, w_ym, __ldg(w0 + ic - 2 * sy), Y, j, wPy, wNy);
        quick_a(Wp, Wn, __ldg(w0 + ic + 2), w_zp, wc, w_zm, __ldg(w0 + ic - 2), Z, k, wPz, wNz);
        const T conv = -dt * ((Up * wPx - Un * wNx) * X(AX_RD, i) + (Vp * wPy - Vn * wNy) * Y(AX_RD, j)
                              + (wPz * wPz - wNz * wNz) * Z(AX_RDS, k));
        const T diff = nudt * (((w_xp - wc) * X(AX_RDS, i) - (wc - w_xm) * X(AX_RDS, i - 1)) * X(AX_RD, i)
                               + ((w_yp - wc) * Y(AX_RDS, j) - (wc - w_ym) * Y(AX_RDS, j - 1)) * Y(AX_RD, j)
                               + ((w_zp - wc) * Z(AX_RD, k + 1) - (wc - w_zm) * Z(AX_RD, k)) * Z(AX_RDS, k));
        T r = wc + conv + diff;
        if (src) r += src[2 * g.n + t];
        w1[ic] = r;
    }
}

// Source coupling with the reference's index convention
// (RUN_CPU_PC_METHOD.hpp:309-316): element m of the ghosted array gets
// src[m] for m < N.
template <class T>
__global__ void k_src_add_ref(long long n, T *__restrict__ u1, T *__restrict__ v1, T *__restrict__ w1,
                              const T *__restrict__ src)
{
    for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n;
         m += (long long)gridDim.x * blockDim.x) {
        u1[m] += src[m];
        v1[m] += src[n + m];
        w1[m] += src[2 * n + m];
    }
}

template <class T>
__global__ void k_src_add_aligned(Geo g, T *__restrict__ u1, T *__restrict__ v1, T *__restrict__ w1,
                                  const T *__restrict__ src)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.n) return;
    int i, j, k;
    cell_of(g, t, i, j, k);
    const long long ic = icel(g, i, j, k);
    u1[ic] += src[t];
    v1[ic] += src[g.n + t];
    w1[ic] += src[2 * g.n + t];
}

// source_termF += dt * f (RUN_CPU_PC_METHOD.hpp:393-401)
template <class T>
__global__ void k_src_accumulate(long long n3, T dt, T *__restrict__ src, const T *__restrict__ f)
{
    for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n3;
         m += (long long)gridDim.x * blockDim.x)
        src[m] += dt * f[m];
}

// createBMatrix_omp (b_matrix.hpp:76-79): b = -jp (1/dt) div u*.  With
// partials != nullptr it also reduces sum(dV * d) and sum(dV) with
// d = -(1/dt) div u* for the compatibility projection; the last block stores
// mean = sum(dV d)/sum(dV) in *mean.
template <class T>
__global__ void __launch_bounds__(kBlock)
k_rhs(Geo g, Metrics<double> m, double ddt, const double *__restrict__ jp, const T *__restrict__ u1,
      const T *__restrict__ v1, const T *__restrict__ w1, double *__restrict__ b, double *partials,
      unsigned int *counter, double *mean)
{
    double acc[2] = {0.0, 0.0};
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < g.n;
         t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_of(g, t, i, j, k);
        const long long ic = icel(g, i, j, k);
        const double div = ((double)u1[ic] - (double)u1[ic - g.sx]) * m.x(AX_RD, i)
                         + ((double)v1[ic] - (double)v1[ic - g.sy]) * m.y(AX_RD, j)
                         + ((double)w1[ic] - (double)w1[ic - 1]) * m.z(AX_RD, k);
        b[t] = -jp[t] * ddt * div;
        if (partials) {
            const double vol = m.x(AX_D, i) * m.y(AX_D, j) * m.z(AX_D, k);
            acc[0] += vol * (-ddt * div);
            acc[1] += vol;
        }
    }
    if (!partials) return;
    double tot[2];
    if (grid_reduce<2>(acc, partials, counter, tot) && threadIdx.x == 0) *mean = tot[0] / tot[1];
}

// b -= jp * mean
__global__ void k_rhs_compat(long long n, const double *__restrict__ jp, const double *__restrict__ mean,
                             double *__restrict__ b)
{
    const double mu = *mean;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x)
        b[t] = b[t] - jp[t] * mu;
}

// ---------------------------------------------------------------------------
// One predictor-corrector pass without re-evaluating the convection-
// diffusion.  Every pass of RUN_CPU_PC_METHOD.hpp:287-627 starts with
// ConvectionDifussion(T0 -> T1) of the same T0 (lines 304, 455), so the
// step evaluates it once into C and each pass forms
//   T1 = C + src     at the faces the convection-diffusion writes,
//   T1 = T1 + src    at the other elements m < N (reference index convention:
//                    element m of the ghosted array gets src[m], lines 309-316),
// which is bit for bit what ConvectionDifussion followed by the source
// coupling leaves in T1.  The same pass then evaluates createBMatrix_omp
// (b_matrix.hpp:76-79) from those T1 values and, for the compatibility
// projection, the volume-weighted sum of the unscaled right-hand side.

// the faces ConvectionDifussion writes: interior cells, the normal
// component's last face skipped (periodic z: the top w face included)
__device__ __forceinline__ bool cd_writes(const Geo &g, int c, int i, int j, int k)
{
    if (i < GC || j < GC || k < GC || i >= g.nx - GC || j >= g.ny - GC || k >= g.nz - GC) return false;
    if (c == 0) return i < g.nx - GC - 1;
    if (c == 1) return j < g.ny - GC - 1;
    return k < g.nz - GC - 1 + g.pz;
}

// T1 += src at the elements m < N the convection-diffusion does not write
// (reference index convention); runs before k_pass, which reads them
template <class T>
__global__ void __launch_bounds__(kBlock)
k_pass_ghosts(Geo g, T *__restrict__ u1, T *__restrict__ v1, T *__restrict__ w1, const T *__restrict__ src)
{
    for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < g.n;
         m += (long long)gridDim.x * blockDim.x) {
        const unsigned q = (unsigned)m;
        const unsigned i = g.fsx.div(q), r = q - i * (unsigned)g.sx, j = g.fsy.div(r);
        const int k = (int)(r - j * (unsigned)g.sy);
        if (!cd_writes(g, 0, (int)i, (int)j, k)) u1[m] += src[m];
        if (!cd_writes(g, 1, (int)i, (int)j, k)) v1[m] += src[g.n + m];
        if (!cd_writes(g, 2, (int)i, (int)j, k)) w1[m] += src[2 * g.n + m];
    }
}

// Pass arguments (PassArgs, kernels.h).  src_mode: 0 no source (the first
// pass), 1 the reference's index convention, 2 aligned (the source of the
// cell).  b == nullptr: no right-hand side (the first step, or the SOR
// solver, which forms its own).
template <class T>
__device__ __forceinline__ T pass_value(const Geo &g, const PassArgs<T> &A, int c, int i, int j, int k)
{
    if (g.pz && k < GC) k += g.nzc;  // the periodic image of a bottom ghost face
    const long long q = icel(g, i, j, k);
    if (!cd_writes(g, c, i, j, k)) return A.T1[c][q];  // as k_pass_ghosts left it
    T v = A.C[c][q];
    if (A.src_mode == 1) {
        if (q < g.n) v += A.src[c * g.n + q];
    } else if (A.src_mode == 2) {
        v += A.src[c * g.n + icelcal(g, i, j, k)];
    }
    return v;
}

// The face value of pass_value away from the boundary, where every face the
// pass reads is written by the convection-diffusion: q the ghosted index of
// the face, r the compact index of its cell.
template <class T>
__device__ __forceinline__ T pass_inner(const Geo &g, const PassArgs<T> &A, int c, long long q, long long r)
{
    T v = A.C[c][q];
    if (A.src_mode == 1) {
        if (q < g.n) v += A.src[c * g.n + q];
    } else if (A.src_mode == 2) {
        v += A.src[c * g.n + r];
    }
    return v;
}

// RHS: form b; PART: also the volume-weighted sum of the unscaled right-hand
// side, whose mean (over the total volume A.vol) the last block stores.
template <class T, bool RHS, bool PART>
__global__ void __launch_bounds__(kBlock, 5)
k_pass(Geo g, Metrics<double> m, Metrics<float> m32, PassArgs<T> A)
{
    double acc = 0.0;
    ff accf = {0.f, 0.f};
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < g.n;
         t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_of(g, t, i, j, k);
        const long long ic = icel(g, i, j, k);
        // away from the x and y boundaries the u and v faces of the cell and
        // below it are convection-diffusion faces; the w faces are too except
        // the top one of the column and the ghost one below it (selected per
        // cell: a warp holds a whole k row, so a k-boundary test here keeps
        // the warp on this path); periodic z leaves the k ends to the
        // general path
        const bool inner = i > GC && j > GC && i < g.nx - GC - 1 && j < g.ny - GC - 1 &&
                           (!g.pz || (k > GC && k < g.nz - GC - 1));
        T ue, vn, wt, uw = T(0), vs = T(0), wb = T(0);
        if (inner) {
            const bool wt_cd = k < g.nz - GC - 1 + g.pz, wb_cd = k > GC;
            ue = pass_inner(g, A, 0, ic, t);
            vn = pass_inner(g, A, 1, ic, t);
            wt = wt_cd ? pass_inner(g, A, 2, ic, t) : A.T1[2][ic];
            A.T1[0][ic] = ue;
            A.T1[1][ic] = vn;
            if (wt_cd) A.T1[2][ic] = wt;
            if (RHS) {
                uw = pass_inner(g, A, 0, ic - g.sx, t - g.sxc);
                vs = pass_inner(g, A, 1, ic - g.sy, t - g.syc);
                wb = wb_cd ? pass_inner(g, A, 2, ic - 1, t - 1) : A.T1[2][ic - 1];
            }
        } else {
            ue = pass_value(g, A, 0, i, j, k);
            vn = pass_value(g, A, 1, i, j, k);
            wt = pass_value(g, A, 2, i, j, k);
            if (cd_writes(g, 0, i, j, k)) A.T1[0][ic] = ue;
            if (cd_writes(g, 1, i, j, k)) A.T1[1][ic] = vn;
            if (cd_writes(g, 2, i, j, k)) A.T1[2][ic] = wt;
            if (RHS) {
                uw = pass_value(g, A, 0, i - 1, j, k);
                vs = pass_value(g, A, 1, i, j - 1, k);
                wb = pass_value(g, A, 2, i, j, k - 1);
            }
        }
        if constexpr (!RHS) continue;
        if constexpr (sizeof(T) == sizeof(double)) {
            // createBMatrix_omp in FP64, the arithmetic of k_rhs
            const double div = ((double)ue - (double)uw) * m.x(AX_RD, i) + ((double)vn - (double)vs) * m.y(AX_RD, j)
                             + ((double)wt - (double)wb) * m.z(AX_RD, k);
            A.b[t] = -A.jp[t] * A.ddt * div;
            if (PART) acc += m.x(AX_D, i) * m.y(AX_D, j) * m.z(AX_D, k) * (-A.ddt * div);
        } else {
            // FP32 velocities: their differences are exact as float pairs and the
            // rest runs in float-float, so b keeps the digits FP64 would
            auto rd = [](const Axis<float> &a, int x) { return ff{a(AX_RD, x), a(AX_RDL, x)}; };
            const ff div = ff_add(ff_add(ff_mul(ff_two_diff((float)ue, (float)uw), rd(m32.x, i)),
                                         ff_mul(ff_two_diff((float)vn, (float)vs), rd(m32.y, j))),
                                  ff_mul(ff_two_diff((float)wt, (float)wb), rd(m32.z, k)));
            const ff d = ff_mul(div, A.mddt);  // the unscaled right-hand side
            A.b[t] = ff_to_double(ff_mul(ff{__ldg(A.jph + t), __ldg(A.jpl + t)}, d));
            if (PART) {
                auto wd = [](const Axis<float> &a, int x) { return ff{a(AX_D, x), a(AX_DL, x)}; };
                const ff vol = ff_mul(ff_mul(wd(m32.x, i), wd(m32.y, j)), wd(m32.z, k));
                accf = ff_add(accf, ff_mul(vol, d));
            }
        }
    }
    if constexpr (!PART) return;
    if constexpr (sizeof(T) != sizeof(double)) acc = ff_to_double(accf);
    double v[1] = {acc}, tot[1];
    if (grid_reduce<1>(v, A.partials, A.counter, tot) && threadIdx.x == 0) *A.mean = tot[0] / A.vol;
}

// update_UandF_omp (updateUandF.hpp:95-190) of one pass with the step's
// other uses of f fused: src += dt f in the predictor passes
// (RUN_CPU_PC_METHOD.hpp:393-401; f itself is then not stored, nothing
// reads it), f stored and reduced to Cd and Cl in the final pass
// (virtualF_Int, virtualForceIntergrator.hpp:26-32, with k_cdcl's launch
// shape and summation order).  The faces update_UandF skips keep the f they
// had (it never writes them), which is what the source and the sums read.
template <class T>
__global__ void __launch_bounds__(kBlock, 6)
k_update_pass(Geo g, Metrics<T> m, Metrics<double> m64, double dt, T rdt, const double *__restrict__ p,
              const T *__restrict__ eta, const T *__restrict__ u1, const T *__restrict__ v1,
              const T *__restrict__ w1, T *__restrict__ u3, T *__restrict__ v3, T *__restrict__ w3,
              T *__restrict__ f, int store_f, T *__restrict__ src, T srcdt, double lz, double *partials,
              unsigned int *counter, double *cdcl)
{
    double acc[2] = {0.0, 0.0};
    const float dtf = (float)dt;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < g.n;
         t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_of(g, t, i, j, k);
        const long long ic = icel(g, i, j, k);
        const double pc = p[ic];
        const T ec = eta[ic];
        // dt (p_nb - p_c): FP64 fields keep update_uf's arithmetic; FP32
        // fields take the FP64 difference to FP32 and scale it there (the FP64
        // pipe is the scarce one, and the product is rounded to FP32 anyway)
        auto grad = [&](double pn) -> T {
            if constexpr (sizeof(T) == sizeof(double)) return (T)(dt * (pn - pc));
            else return (T)(pn - pc) * dtf;
        };
        T fv[3] = {T(0), T(0), T(0)};
        if (i < g.nx - GC - 1) {
            const T T2 = u1[ic] - grad(p[ic + g.sx]) * m.x(AX_RDS, i);
            const T ef = ec + (eta[ic + g.sx] - ec) * m.x(AX_IT, i);
            const T un = (T(1) - ef) * T2;
            u3[ic] = un;
            fv[0] = (un - T2) * rdt;
        }
        if (j < g.ny - GC - 1) {
            const T T2 = v1[ic] - grad(p[ic + g.sy]) * m.y(AX_RDS, j);
            const T ef = ec + (eta[ic + g.sy] - ec) * m.y(AX_IT, j);
            const T vn = (T(1) - ef) * T2;
            v3[ic] = vn;
            fv[1] = (vn - T2) * rdt;
        }
        if (k < g.nz - GC - 1 + g.pz) {
            const T T2 = w1[ic] - grad(p[ic + 1]) * m.z(AX_RDS, k);
            const T ef = ec + (eta[ic + 1] - ec) * m.z(AX_IT, k);
            const T wn = (T(1) - ef) * T2;
            w3[ic] = wn;
            fv[2] = (wn - T2) * rdt;
        }
        if (store_f) {
            if (i < g.nx - GC - 1) f[t] = fv[0];
            if (j < g.ny - GC - 1) f[g.n + t] = fv[1];
            if (k < g.nz - GC - 1 + g.pz) f[2 * g.n + t] = fv[2];
        }
        if (src) {
            const T f0 = i < g.nx - GC - 1 ? fv[0] : f[t];
            const T f1 = j < g.ny - GC - 1 ? fv[1] : f[g.n + t];
            const T f2 = k < g.nz - GC - 1 + g.pz ? fv[2] : f[2 * g.n + t];
            src[t] += srcdt * f0;
            src[g.n + t] += srcdt * f1;
            src[2 * g.n + t] += srcdt * f2;
        }
        if (cdcl) {
            const double vol = m64.x(AX_D, i) * m64.y(AX_D, j) * m64.z(AX_D, k);
            acc[0] += (double)(i < g.nx - GC - 1 ? fv[0] : f[t]) * vol;
            acc[1] += (double)(j < g.ny - GC - 1 ? fv[1] : f[g.n + t]) * vol;
        }
    }
    if (!cdcl) return;
    double tot[2];
    if (grid_reduce<2>(acc, partials, counter, tot) && threadIdx.x == 0) {
        cdcl[0] = -2.0 * tot[0] / lz;
        cdcl[1] = -2.0 * tot[1] / lz;
    }
}

__global__ void k_split_lo(long long n, const double *__restrict__ a, float *__restrict__ lo)
{
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x)
        lo[t] = ff_of(a[t]).lo;
}

// Pressure_transform_X_result (Transform.hpp:8-24)
__global__ void k_transform(Geo g, const double *__restrict__ x, double *__restrict__ p)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.n) return;
    int i, j, k;
    cell_of(g, t, i, j, k);
    p[icel(g, i, j, k)] = x[t];
}

// update_UandF_omp (updateUandF.hpp:95-190): T2 = u* - dt grad p;
// u = eta*uS + (1 - eta_face) T2 with uS = 0; f = (u - T2)/dt.  One cell per
// thread, all three components; the last normal face is skipped.
template <class T>
__global__ void __launch_bounds__(kBlock)
k_update_uf(Geo g, Metrics<T> m, double dt, T rdt, const double *__restrict__ p,
            const T *__restrict__ eta, const T *__restrict__ u1, const T *__restrict__ v1,
            const T *__restrict__ w1, T *__restrict__ u3, T *__restrict__ v3, T *__restrict__ w3,
            T *__restrict__ f)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.n) return;
    int i, j, k;
    cell_of(g, t, i, j, k);
    const long long ic = icel(g, i, j, k);
    const double pc = p[ic];
    const T ec = eta[ic];
    if (i < g.nx - GC - 1) {
        const T T2 = u1[ic] - (T)(dt * (p[ic + g.sx] - pc)) * m.x(AX_RDS, i);
        const T ef = ec + (eta[ic + g.sx] - ec) * m.x(AX_IT, i);
        const T un = (T(1) - ef) * T2;
        u3[ic] = un;
        f[t] = (un - T2) * rdt;
    }
    if (j < g.ny - GC - 1) {
        const T T2 = v1[ic] - (T)(dt * (p[ic + g.sy] - pc)) * m.y(AX_RDS, j);
        const T ef = ec + (eta[ic + g.sy] - ec) * m.y(AX_IT, j);
        const T vn = (T(1) - ef) * T2;
        v3[ic] = vn;
        f[g.n + t] = (vn - T2) * rdt;
    }
    if (k < g.nz - GC - 1 + g.pz) {  // periodic z: the top face is an unknown too
        const T T2 = w1[ic] - (T)(dt * (p[ic + 1] - pc)) * m.z(AX_RDS, k);
        const T ef = ec + (eta[ic + 1] - ec) * m.z(AX_IT, k);
        const T wn = (T(1) - ef) * T2;
        w3[ic] = wn;
        f[2 * g.n + t] = (wn - T2) * rdt;
    }
}

// virtualF_Int (virtualForceIntergrator.hpp:26-32) for x and y at once:
// out[0] = Cd = -2 sum(f_x dV)/lz, out[1] = Cl = -2 sum(f_y dV)/lz.
template <class T>
__global__ void __launch_bounds__(kBlock)
k_cdcl(Geo g, Metrics<double> m, double lz, const T *__restrict__ f, double *partials,
       unsigned int *counter, double *out)
{
    double acc[2] = {0.0, 0.0};
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < g.n;
         t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_of(g, t, i, j, k);
        const double vol = m.x(AX_D, i) * m.y(AX_D, j) * m.z(AX_D, k);
        acc[0] += (double)f[t] * vol;
        acc[1] += (double)f[g.n + t] * vol;
    }
    double tot[2];
    if (grid_reduce<2>(acc, partials, counter, tot) && threadIdx.x == 0) {
        out[0] = -2.0 * tot[0] / lz;
        out[1] = -2.0 * tot[1] / lz;
    }
}

// ---------------------------------------------------------------------------
// BC_staggered_main (Boundary_Condition.hpp:37-175).  The faces depend on
// each other through the interior faces that faces 1, 3 and 5 overwrite, so
// the update runs as three launches in the reference's single-thread order:
// phase 0 = faces 0/1, phase 1 = faces 2/3, phase 2 = faces 4/5.  Products
// and sums use explicit round-to-nearest intrinsics (no fused multiply-add),
// which makes the ghost values bitwise equal to the reference's.
template <class T> __device__ __forceinline__ T mul_rn(T a, T b);
template <class T> __device__ __forceinline__ T add_rn(T a, T b);
template <> __device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
template <> __device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
template <> __device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
template <> __device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }

template <class T>
__device__ __forceinline__ T bc_norm(const BcTab &bc, int b, int c, T x)
{   // normal component: Dir + Num * interior
    return add_rn((T)bc.dir[b * 3 + c], mul_rn((T)bc.num[b * 3 + c], x));
}
template <class T>
__device__ __forceinline__ T bc_tan(const BcTab &bc, int b, int c, T x)
{   // tangential component: 2 Dir + (2 Num - 1) * interior
    return add_rn((T)(bc.dir[b * 3 + c] * 2.), mul_rn((T)(2.0 * bc.num[b * 3 + c] - 1.0), x));
}

// Periodic z (an extension; the reference's table has no periodic face): the
// two ghost planes at each z end take the interior planes one period away,
// over the whole (i, j) range including the x and y ghosts.  The sources
// are interior planes, so the four copies of a column are independent.
template <class T>
__global__ void k_sync_z(Geo g, T *__restrict__ a0, T *__restrict__ a1, T *__restrict__ a2)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)g.nx * g.ny) return;
    const long long base = t * g.nz;  // icel(i, j, 0) of column t = i ny + j
    const int nzc = g.nzc, nz = g.nz;
    auto col = [&](T *f) {
        if (!f) return;
        f[base + 0] = f[base + nzc];
        f[base + 1] = f[base + 1 + nzc];
        f[base + nz - 2] = f[base + nz - 2 - nzc];
        f[base + nz - 1] = f[base + nz - 1 - nzc];
    };
    col(a0);
    col(a1);
    col(a2);
}

template <class T>
void launch_sync_z(cudaStream_t s, const Geo &g, T *a0, T *a1, T *a2)
{
    const long long cols = (long long)g.nx * g.ny;
    k_sync_z<T><<<(int)((cols + kBlock - 1) / kBlock), kBlock, 0, s>>>(g, a0, a1, a2);
}

template <class T>
__global__ void k_bc_main(Geo g, BcTab bc, int phase, T *__restrict__ u, T *__restrict__ v,
                          T *__restrict__ w, double *__restrict__ p)
{
    // phase 0: (a,b) = (j,k); phase 1: (i,k); phase 2: (i,j); all interior
    const int na = phase == 0 ? g.nyc : g.nxc;
    const int nb = phase == 2 ? g.nyc : g.nzc;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)na * nb) return;
    const int a = (int)(t / nb) + GC, b = (int)(t % nb) + GC;
    if (phase == 0) {
        const int j = a, k = b, nx = g.nx;
        auto I = [&](int i) { return icel(g, i, j, k); };
        T x = bc.inflow ? add_rn((T)bc.inflow[j - GC], mul_rn((T)bc.num[0], u[I(2)])) : bc_norm<T>(bc, 0, 0, u[I(2)]);
        u[I(1)] = x; u[I(0)] = x;
        x = bc_tan<T>(bc, 0, 1, v[I(2)]); v[I(1)] = x; v[I(0)] = x;
        x = bc_tan<T>(bc, 0, 2, w[I(2)]); w[I(1)] = x; w[I(0)] = x;
        if (!bc.skip_outflow) {
            x = bc_norm<T>(bc, 1, 0, u[I(nx - 4)]); u[I(nx - 3)] = x; u[I(nx - 2)] = x; u[I(nx - 1)] = x;
            x = bc_tan<T>(bc, 1, 1, v[I(nx - 3)]); v[I(nx - 2)] = x; v[I(nx - 1)] = x;
            x = bc_tan<T>(bc, 1, 2, w[I(nx - 3)]); w[I(nx - 2)] = x; w[I(nx - 1)] = x;
        }
        double q = p[I(2)]; p[I(1)] = q; p[I(0)] = q;
        q = p[I(nx - 3)]; p[I(nx - 2)] = q; p[I(nx - 1)] = q;
    } else if (phase == 1) {
        const int i = a, k = b, ny = g.ny;
        auto J = [&](int j) { return icel(g, i, j, k); };
        T x = bc_tan<T>(bc, 2, 0, u[J(2)]); u[J(1)] = x; u[J(0)] = x;
        x = bc_norm<T>(bc, 2, 1, v[J(2)]); v[J(1)] = x; v[J(0)] = x;
        x = bc_tan<T>(bc, 2, 2, w[J(2)]); w[J(1)] = x; w[J(0)] = x;
        x = bc_norm<T>(bc, 3, 1, v[J(ny - 4)]); v[J(ny - 3)] = x; v[J(ny - 2)] = x; v[J(ny - 1)] = x;
        x = bc_tan<T>(bc, 3, 0, u[J(ny - 3)]); u[J(ny - 2)] = x; u[J(ny - 1)] = x;
        x = bc_tan<T>(bc, 3, 2, w[J(ny - 3)]); w[J(ny - 2)] = x; w[J(ny - 1)] = x;
        double q = p[J(2)]; p[J(1)] = q; p[J(0)] = q;
        q = p[J(ny - 3)]; p[J(ny - 2)] = q; p[J(ny - 1)] = q;
    } else {
        const int i = a, j = b, nz = g.nz;
        auto K = [&](int k) { return icel(g, i, j, k); };
        T x = bc_tan<T>(bc, 4, 0, u[K(2)]); u[K(1)] = x; u[K(0)] = x;
        x = bc_tan<T>(bc, 4, 1, v[K(2)]); v[K(1)] = x; v[K(0)] = x;
        x = bc_norm<T>(bc, 4, 2, w[K(2)]); w[K(1)] = x; w[K(0)] = x;
        x = bc_norm<T>(bc, 5, 2, w[K(nz - 4)]); w[K(nz - 3)] = x; w[K(nz - 2)] = x; w[K(nz - 1)] = x;
        x = bc_tan<T>(bc, 5, 0, u[K(nz - 3)]); u[K(nz - 2)] = x; u[K(nz - 1)] = x;
        x = bc_tan<T>(bc, 5, 1, v[K(nz - 3)]); v[K(nz - 2)] = x; v[K(nz - 1)] = x;
        double q = p[K(2)]; p[K(1)] = q; p[K(0)] = q;
        q = p[K(nz - 3)]; p[K(nz - 2)] = q; p[K(nz - 1)] = q;
    }
}

// Convective outflow (extension): per interior (j, k) of the x-max face,
//   u_b = u0_b - C (u0_b - u0_{b-1}),  C = uc dt / Dx[nx-3]   (face nx-3)
//   v_g = v0_g - Ct (v0_g - v0_{g-1}), Ct = uc dt / Dxs[nx-3] (ghost nx-2)
// (w as v), written into the new field; the flux sums of the inflow face
// (u0 at face 1) and of the new outflow face give the scale of the second
// kernel, which also fills the outer ghosts.
template <class T>
__global__ void __launch_bounds__(kBlock)
k_bc_conv(Geo g, Metrics<double> m, double dt, double uc, const T *__restrict__ u0, const T *__restrict__ v0,
          const T *__restrict__ w0, T *__restrict__ u3, T *__restrict__ v3, T *__restrict__ w3, double *partials,
          unsigned int *counter, double *scale_out)
{
    const int nx = g.nx;
    const double C = uc * dt / m.x(AX_D, nx - 3), Ct = uc * dt / m.x(AX_DS, nx - 3);
    double acc[2] = {0.0, 0.0};
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < (long long)g.nyc * g.nzc;
         t += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(t / g.nzc) + GC, k = (int)(t % g.nzc) + GC;
        auto I = [&](int i) { return icel(g, i, j, k); };
        const double ub = (double)u0[I(nx - 3)] - C * ((double)u0[I(nx - 3)] - (double)u0[I(nx - 4)]);
        const double vg = (double)v0[I(nx - 2)] - Ct * ((double)v0[I(nx - 2)] - (double)v0[I(nx - 3)]);
        const double wg = (double)w0[I(nx - 2)] - Ct * ((double)w0[I(nx - 2)] - (double)w0[I(nx - 3)]);
        u3[I(nx - 3)] = (T)ub;
        v3[I(nx - 2)] = (T)vg; v3[I(nx - 1)] = (T)vg;
        w3[I(nx - 2)] = (T)wg; w3[I(nx - 1)] = (T)wg;
        const double area = m.y(AX_D, j) * m.z(AX_D, k);
        acc[0] += (double)u0[I(1)] * area;
        acc[1] += (double)(T)ub * area;
    }
    double tot[2];
    if (grid_reduce<2>(acc, partials, counter, tot) && threadIdx.x == 0)
        *scale_out = tot[1] != 0.0 ? tot[0] / tot[1] : 1.0;
}

template <class T>
__global__ void k_bc_conv_scale(Geo g, const double *__restrict__ scale, T *__restrict__ u3)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)g.nyc * g.nzc) return;
    const int j = (int)(t / g.nzc) + GC, k = (int)(t % g.nzc) + GC, nx = g.nx;
    const long long b = icel(g, nx - 3, j, k);
    const T x = (T)((double)u3[b] * *scale);
    u3[b] = x;
    u3[b + g.sx] = x;
    u3[b + 2 * g.sx] = x;
}

template <class T>
void launch_bc_convective(cfd_launch_ctx &c, const Geo &g, const Metrics<double> &m, double dt, double uc,
                          const T *u0, const T *v0, const T *w0, T *u3, T *v3, T *w3, double *scale_out)
{
    k_bc_conv<T><<<c.red_blocks, kBlock, 0, c.s>>>(g, m, dt, uc, u0, v0, w0, u3, v3, w3, c.partials, c.counter,
                                                  scale_out);
    const int blocks = (int)(((long long)g.nyc * g.nzc + kBlock - 1) / kBlock);
    k_bc_conv_scale<T><<<blocks, kBlock, 0, c.s>>>(g, scale_out, u3);
}

// BC_staggered_copy (updateBC.hpp:6-111): the three face sets are disjoint,
// so one launch covers them (blockIdx.y = face pair).
template <class T>
__global__ void k_bc_copy(Geo g, const T *__restrict__ uo, const T *__restrict__ vo,
                          const T *__restrict__ wo, T *__restrict__ u, T *__restrict__ v,
                          T *__restrict__ w)
{
    const int phase = blockIdx.y;
    const int na = phase == 0 ? g.nyc : g.nxc;
    const int nb = phase == 2 ? g.nyc : g.nzc;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)na * nb) return;
    const int a = (int)(t / nb) + GC, b = (int)(t % nb) + GC;
    long long s[8];  // ghost / boundary positions along the face normal
    int e;           // last index along the normal axis (n - 1)
    long long stride, base;
    if (phase == 0) { e = g.nx - 1; stride = g.sx; base = icel(g, 0, a, b); }
    else if (phase == 1) { e = g.ny - 1; stride = g.sy; base = icel(g, a, 0, b); }
    else { e = g.nz - 1; stride = 1; base = icel(g, a, b, 0); }
    s[0] = base;
    s[1] = base + stride;
    s[2] = base + (long long)(e - 1) * stride;
    s[3] = base + (long long)e * stride;
    s[4] = base + (long long)(e - 2) * stride;  // last interior normal face
    for (int q = 0; q < 4; ++q) { u[s[q]] = uo[s[q]]; v[s[q]] = vo[s[q]]; w[s[q]] = wo[s[q]]; }
    if (phase == 0) u[s[4]] = uo[s[4]];
    else if (phase == 1) v[s[4]] = vo[s[4]];
    else w[s[4]] = wo[s[4]];
}

// ---------------------------------------------------------------------------
// DFIB_CylinderZ (setEta.hpp:136-204).  One block per (i, j) column of the
// k = 0 plane; the cut-cell sub-sampling is spread over the block and the
// inside count is an exact integer sum.  All arithmetic uses explicit
// round-to-nearest operations, so eta is bitwise the reference's.
__global__ void k_eta_plane(Geo g, const double *__restrict__ X, const double *__restrict__ Y,
                            const double *__restrict__ Dx, const double *__restrict__ Dy, double cx,
                            double cy, double radius, int nsub, double scale, double *__restrict__ eta)
{
    const int i = blockIdx.x + GC, j = blockIdx.y + GC;
    const long long ic = icel(g, i, j, 0);
    const double diag = __dmul_rn(__dsqrt_rn(__dadd_rn(__dmul_rn(Dx[i], Dx[i]), __dmul_rn(Dy[j], Dy[j]))), 0.5);
    const double ex = __dsub_rn(__dmul_rn(__dadd_rn(X[i], X[i + 1]), 0.5), cx);
    const double ey = __dsub_rn(__dmul_rn(__dadd_rn(Y[j], Y[j + 1]), 0.5), cy);
    const double dist = __dsqrt_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)));
    if (!(fabs(__dsub_rn(dist, radius)) < diag)) {
        if (threadIdx.x == 0) eta[ic] = dist > radius ? 0.0 : 1.0;
        return;
    }
    const double dxg = __ddiv_rn(Dx[i], (double)nsub), dyg = __ddiv_rn(Dy[j], (double)nsub);
    unsigned int cnt = 0;
    const int total = nsub * nsub;
    for (int s = threadIdx.x; s < total; s += blockDim.x) {
        const int ii = s / nsub, jj = s - ii * nsub;
        const double x0 = __dadd_rn(X[i], __dmul_rn((double)ii, dxg));
        const double x1 = __dadd_rn(X[i], __dmul_rn((double)(ii + 1), dxg));
        const double y0 = __dadd_rn(Y[j], __dmul_rn((double)jj, dyg));
        const double y1 = __dadd_rn(Y[j], __dmul_rn((double)(jj + 1), dyg));
        const double a = __dsub_rn(__dmul_rn(__dadd_rn(x0, x1), 0.5), cx);
        const double b = __dsub_rn(__dmul_rn(__dadd_rn(y0, y1), 0.5), cy);
        if (__dsqrt_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b))) <= radius) ++cnt;
    }
    __shared__ unsigned int sm[32];
    for (int off = 16; off > 0; off >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, off);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int c = 0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) c += sm[q];
        eta[ic] = __dmul_rn((double)c, scale);
    }
}

// Exact-area option (nsub == 0; an extension of the sub-sampling): area of
// the disc of radius r at the origin inside [x0, x1] x [y0, y1], the integral
// over t of (min(y1, s) - max(y0, -s))+ with s = sqrt(r^2 - t^2), split where
// s crosses |y0| or |y1|; S(t) = (t s + r^2 asin(t / r)) / 2 integrates s.
__device__ double disc_prim(double t, double r)
{
    const double u = fmax(-1.0, fmin(1.0, t / r));
    return 0.5 * (t * sqrt(fmax(r * r - t * t, 0.0)) + r * r * asin(u));
}

__device__ double disc_rect_area(double x0, double x1, double y0, double y1, double r)
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
    for (int q = 1; q < n; ++q)
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
        const bool top_s = sm < y1, bot_s = -sm > y0;
        const double top = top_s ? sm : y1, bot = bot_s ? -sm : y0;
        if (!(top > bot)) continue;
        const double is = disc_prim(hi, r) - disc_prim(lo, r);
        area += (top_s ? is : y1 * (hi - lo)) - (bot_s ? -is : y0 * (hi - lo));
    }
    return area;
}

// the k = 0 plane with exact areas: one thread per interior (i, j); the
// inside / outside classification of the sub-sampled form (which is exact)
__global__ void k_eta_plane_exact(Geo g, const double *__restrict__ X, const double *__restrict__ Y,
                                  const double *__restrict__ Dx, const double *__restrict__ Dy, double cx,
                                  double cy, double radius, double *__restrict__ eta)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)g.nxc * g.nyc) return;
    const int i = (int)(t / g.nyc) + GC, j = (int)(t % g.nyc) + GC;
    const long long ic = icel(g, i, j, 0);
    const double diag = sqrt(Dx[i] * Dx[i] + Dy[j] * Dy[j]) * 0.5;
    const double ex = (X[i] + X[i + 1]) * 0.5 - cx, ey = (Y[j] + Y[j + 1]) * 0.5 - cy;
    const double dist = sqrt(ex * ex + ey * ey);
    if (fabs(dist - radius) < diag) {
        const double x0 = X[i] - cx, y0 = Y[j] - cy;
        eta[ic] = disc_rect_area(x0, x0 + Dx[i], y0, y0 + Dy[j], radius) / (Dx[i] * Dy[j]);
    } else {
        eta[ic] = dist > radius ? 0.0 : 1.0;
    }
}

// eta(i,j,k) = eta(i,j,0) for i < nx-1, j < ny-1, 1 <= k < nz-1 (setEta.hpp:200-203)
__global__ void k_eta_extrude(Geo g, double *__restrict__ eta)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nij = (long long)(g.nx - 1) * (g.ny - 1);
    if (t >= nij * (g.nz - 2)) return;
    const int k = (int)(t / nij) + 1;
    const long long ij = t % nij;
    const int i = (int)(ij / (g.ny - 1)), j = (int)(ij % (g.ny - 1));
    eta[icel(g, i, j, k)] = eta[icel(g, i, j, 0)];
}

// max |div u| over interior cells in FP64
template <class T>
__global__ void __launch_bounds__(kBlock)
k_div_inf(Geo g, Metrics<double> m, const T *__restrict__ u, const T *__restrict__ v,
          const T *__restrict__ w, unsigned long long *slot)
{
    double mx = 0.0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < g.n;
         t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_of(g, t, i, j, k);
        const long long ic = icel(g, i, j, k);
        const double d = ((double)u[ic] - (double)u[ic - g.sx]) * m.x(AX_RD, i)
                       + ((double)v[ic] - (double)v[ic - g.sy]) * m.y(AX_RD, j)
                       + ((double)w[ic] - (double)w[ic - 1]) * m.z(AX_RD, k);
        const double a = fabs(d);
        mx = (a > mx || a != a) ? a : mx;
    }
    grid_max_nonneg(mx, slot);
}

// Divergence of the projected field T2 = u* - dt grad p (updateUandF.hpp:136,
// 158, 179) per interior cell, with the reference's face rules: faces between
// two interior cells are projected, the domain-boundary faces and the
// skipped last normal faces keep u*.  slot[0] <- max |div T2|, slot[1] <-
// max |div T2 - c| with c = -dt * (removed RHS mean), the value a converged
// solve of the compatible system leaves in every cell.
template <class T>
__global__ void __launch_bounds__(kBlock)
k_div_projected(Geo g, Metrics<double> m, double dt, const double *__restrict__ p,
                const T *__restrict__ u1, const T *__restrict__ v1, const T *__restrict__ w1,
                const double *__restrict__ mean, unsigned long long *slot, bool slot3)
{
    const double c = -dt * (mean ? *mean : 0.0);
    double mx = 0.0, md = 0.0, mu = 0.0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < g.n;
         t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_of(g, t, i, j, k);
        const long long ic = icel(g, i, j, k);
        const double pc = p[ic];
        double ue = (double)u1[ic], uw = (double)u1[ic - g.sx];
        if (i < g.nx - GC - 1) ue -= dt * (p[ic + g.sx] - pc) * m.x(AX_RDS, i);
        if (i > GC) uw -= dt * (pc - p[ic - g.sx]) * m.x(AX_RDS, i - 1);
        double vn = (double)v1[ic], vs = (double)v1[ic - g.sy];
        if (j < g.ny - GC - 1) vn -= dt * (p[ic + g.sy] - pc) * m.y(AX_RDS, j);
        if (j > GC) vs -= dt * (pc - p[ic - g.sy]) * m.y(AX_RDS, j - 1);
        double wt = (double)w1[ic], wb = (double)w1[ic - 1];
        if (k < g.nz - GC - 1 + g.pz) wt -= dt * (p[ic + 1] - pc) * m.z(AX_RDS, k);
        if (k > GC || g.pz) wb -= dt * (pc - p[ic - 1]) * m.z(AX_RDS, k - 1);
        const double d = (ue - uw) * m.x(AX_RD, i) + (vn - vs) * m.y(AX_RD, j) + (wt - wb) * m.z(AX_RD, k);
        const double a = fabs(d), b = fabs(d - c);
        mx = (a > mx || a != a) ? a : mx;
        md = (b > md || b != b) ? b : md;
        if (slot3) {  // the divergence of u* itself
            const double du = ((double)u1[ic] - (double)u1[ic - g.sx]) * m.x(AX_RD, i)
                            + ((double)v1[ic] - (double)v1[ic - g.sy]) * m.y(AX_RD, j)
                            + ((double)w1[ic] - (double)w1[ic - 1]) * m.z(AX_RD, k);
            const double e = fabs(du);
            mu = (e > mu || e != e) ? e : mu;
        }
    }
    grid_max_nonneg(mx, slot);
    __syncthreads();
    grid_max_nonneg(md, slot + 1);
    if (slot3) {
        __syncthreads();
        grid_max_nonneg(mu, slot + 2);
    }
}

template <class T>
__global__ void k_fill(long long n, T *__restrict__ a, T val)
{
    for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n;
         m += (long long)gridDim.x * blockDim.x)
        a[m] = val;
}

template <class A, class B>
__global__ void k_convert(long long n, const A *__restrict__ a, B *__restrict__ b)
{
    for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n;
         m += (long long)gridDim.x * blockDim.x)
        b[m] = (B)a[m];
}

// ---------------------------------------------------------------------------
// Monitors.  get_Cfl (analyses/cfl.hpp:3-80): per cell the signed sum
// u/Dxs + v/Dys + w/Dzs over the faces the convection-diffusion writes (the
// last normal face skipped), true FP64 divisions in the reference's order;
// out = {max c, max u, -min u, max v, -min v, max w, -min w}.
template <class T>
__global__ void __launch_bounds__(kBlock)
k_cfl(Geo g, Metrics<double> m, const T *__restrict__ u, const T *__restrict__ v, const T *__restrict__ w,
      double *partials, unsigned int *counter, double *out)
{
    double acc[7] = {-INFINITY, -INFINITY, -INFINITY, -INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < g.n;
         t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_of(g, t, i, j, k);
        const long long ic = icel(g, i, j, k);
        double c = 0.0;
        if (i < g.nx - GC - 1) {
            const double a = (double)u[ic];
            c += a / m.x(AX_DS, i);
            acc[1] = fmax(acc[1], a);
            acc[2] = fmax(acc[2], -a);
        }
        if (j < g.ny - GC - 1) {
            const double a = (double)v[ic];
            c += a / m.y(AX_DS, j);
            acc[3] = fmax(acc[3], a);
            acc[4] = fmax(acc[4], -a);
        }
        if (k < g.nz - GC - 1) {
            const double a = (double)w[ic];
            c += a / m.z(AX_DS, k);
            acc[5] = fmax(acc[5], a);
            acc[6] = fmax(acc[6], -a);
        }
        acc[0] = fmax(acc[0], c);
    }
    double tot[7];
    if (grid_reduce_max<7>(acc, partials, counter, tot) && threadIdx.x == 0)
        for (int q = 0; q < 7; ++q) out[q] = tot[q];
}

// CheckSteadyStatebyMaxVal_omp (analyses/CheckSteadystate.hpp:166-215):
// max(0, max over interior cells of (a - b)) per component
template <class T>
__global__ void __launch_bounds__(kBlock)
k_steady_max(Geo g, const T *__restrict__ ua, const T *__restrict__ va, const T *__restrict__ wa,
             const T *__restrict__ ub, const T *__restrict__ vb, const T *__restrict__ wb, double *partials,
             unsigned int *counter, double *out)
{
    double acc[3] = {0.0, 0.0, 0.0};
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < g.n;
         t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_of(g, t, i, j, k);
        const long long ic = icel(g, i, j, k);
        acc[0] = fmax(acc[0], (double)ua[ic] - (double)ub[ic]);
        acc[1] = fmax(acc[1], (double)va[ic] - (double)vb[ic]);
        acc[2] = fmax(acc[2], (double)wa[ic] - (double)wb[ic]);
    }
    double tot[3];
    if (grid_reduce_max<3>(acc, partials, counter, tot) && threadIdx.x == 0)
        for (int q = 0; q < 3; ++q) out[q] = tot[q];
}

// ---------------------------------------------------------------------------
// host launchers
static inline int nblk(long long n) { return (int)((n + kBlock - 1) / kBlock); }

template <class T>
void launch_convdiff(cudaStream_t s, const Geo &g, const Metrics<T> &m, T dt, T nudt, const T *u0,
                     const T *v0, const T *w0, T *u1, T *v1, T *w1, const T *src_aligned, const T *vis, T nu)
{
    k_convdiff<T><<<nblk(g.n), kBlock, 0, s>>>(g, m, dt, nudt, u0, v0, w0, u1, v1, w1, src_aligned, vis, nu);
}

template <class T>
void launch_smagorinsky(cudaStream_t s, const Geo &g, const Metrics<double> &m, const T *u, const T *v,
                        const T *w, T *vis)
{
    k_smagorinsky<T><<<nblk(g.n), kBlock, 0, s>>>(g, m, u, v, w, vis);
}

template <class T>
void launch_src_add(cfd_launch_ctx &c, const Geo &g, int aligned, T *u1, T *v1, T *w1, const T *src)
{
    if (aligned)
        k_src_add_aligned<T><<<nblk(g.n), kBlock, 0, c.s>>>(g, u1, v1, w1, src);
    else
        k_src_add_ref<T><<<blocks_for(g.n, c.grid_cap), kBlock, 0, c.s>>>(g.n, u1, v1, w1, src);
}

template <class T>
void launch_src_accumulate(cfd_launch_ctx &c, long long n3, T dt, T *src, const T *f)
{
    k_src_accumulate<T><<<blocks_for(n3, c.grid_cap), kBlock, 0, c.s>>>(n3, dt, src, f);
}

template <class T>
void launch_rhs(cfd_launch_ctx &c, const Geo &g, const Metrics<double> &m, double ddt,
                const double *jp, const T *u1, const T *v1, const T *w1, double *b, bool compat,
                double *mean)
{
    if (compat) {
        k_rhs<T><<<c.red_blocks, kBlock, 0, c.s>>>(g, m, ddt, jp, u1, v1, w1, b, c.partials,
                                                     c.counter, mean);
        k_rhs_compat<<<blocks_for(g.n, c.grid_cap), kBlock, 0, c.s>>>(g.n, jp, mean, b);
    } else {
        k_rhs<T><<<blocks_for(g.n, c.grid_cap), kBlock, 0, c.s>>>(g, m, ddt, jp, u1, v1, w1, b, nullptr,
                                                                   nullptr, nullptr);
    }
}

template <class T>
void launch_pass(cfd_launch_ctx &c, const Geo &g, const Metrics<double> &m, const Metrics<float> &m32,
                 const PassArgs<T> &A, bool ghosts)
{
    if (ghosts) k_pass_ghosts<T><<<blocks_for(g.n, c.grid_cap), kBlock, 0, c.s>>>(g, A.T1[0], A.T1[1], A.T1[2], A.src);
    PassArgs<T> B = A;
    B.mddt = ff_of(-A.ddt);
    if (!A.b) {
        k_pass<T, false, false><<<nblk(g.n), kBlock, 0, c.s>>>(g, m, m32, B);
    } else if (!A.partials) {
        k_pass<T, true, false><<<nblk(g.n), kBlock, 0, c.s>>>(g, m, m32, B);
    } else {
        // one sum per block: the partials buffer holds kMaxReduce per block
        // of the reduction grid
        const int grid = (int)std::min<long long>(nblk(g.n), (long long)kMaxReduce * c.red_blocks);
        k_pass<T, true, true><<<grid, kBlock, 0, c.s>>>(g, m, m32, B);
    }
    if (A.partials) {
        const double *jp = A.jp;
        if (jp) k_rhs_compat<<<blocks_for(g.n, c.grid_cap), kBlock, 0, c.s>>>(g.n, jp, A.mean, A.b);
    }
}

template <class T>
void launch_update_pass(cfd_launch_ctx &c, const Geo &g, const Metrics<T> &m, const Metrics<double> &m64, double dt,
                        const double *p, const T *eta, const T *u1, const T *v1, const T *w1, T *u3, T *v3, T *w3,
                        T *f, bool store_f, T *src, double lz, double *cdcl)
{
    // the drag/lift sums need k_cdcl's launch shape (the same sums, bit for bit)
    const int grid = cdcl ? c.red_blocks : (int)((g.n + kBlock - 1) / kBlock);
    k_update_pass<T><<<grid, kBlock, 0, c.s>>>(g, m, m64, dt, (T)(1.0 / dt), p, eta, u1, v1, w1, u3, v3, w3, f,
                                               store_f ? 1 : 0, src, (T)dt, lz, c.partials, c.counter, cdcl);
}

void launch_split_lo(cfd_launch_ctx &c, long long n, const double *a, float *lo)
{
    k_split_lo<<<blocks_for(n, c.grid_cap), kBlock, 0, c.s>>>(n, a, lo);
}

void launch_transform(cudaStream_t s, const Geo &g, const double *x, double *p)
{
    k_transform<<<nblk(g.n), kBlock, 0, s>>>(g, x, p);
}

template <class T>
void launch_update_uf(cudaStream_t s, const Geo &g, const Metrics<T> &m, double dt, T rdt,
                      const double *p, const T *eta, const T *u1, const T *v1, const T *w1, T *u3,
                      T *v3, T *w3, T *f)
{
    k_update_uf<T><<<nblk(g.n), kBlock, 0, s>>>(g, m, dt, rdt, p, eta, u1, v1, w1, u3, v3, w3, f);
}

template <class T>
void launch_cdcl(cfd_launch_ctx &c, const Geo &g, const Metrics<double> &m, double lz, const T *f,
                 double *out2)
{
    k_cdcl<T><<<c.red_blocks, kBlock, 0, c.s>>>(g, m, lz, f, c.partials, c.counter, out2);
}

template <class T>
void launch_bc_main(cudaStream_t s, const Geo &g, const BcTab &bc, T *u, T *v, T *w, double *p)
{
    k_bc_main<T><<<nblk((long long)g.nyc * g.nzc), kBlock, 0, s>>>(g, bc, 0, u, v, w, p);
    k_bc_main<T><<<nblk((long long)g.nxc * g.nzc), kBlock, 0, s>>>(g, bc, 1, u, v, w, p);
    if (g.pz) {  // periodic z replaces faces 4 and 5, after the x and y faces
        launch_sync_z<T>(s, g, u, v, w);
        launch_sync_z<double>(s, g, p, nullptr, nullptr);
        return;
    }
    k_bc_main<T><<<nblk((long long)g.nxc * g.nyc), kBlock, 0, s>>>(g, bc, 2, u, v, w, p);
}

template <class T>
void launch_bc_copy(cudaStream_t s, const Geo &g, const T *uo, const T *vo, const T *wo, T *u, T *v,
                    T *w)
{
    long long mx = (long long)g.nyc * g.nzc;
    if ((long long)g.nxc * g.nzc > mx) mx = (long long)g.nxc * g.nzc;
    if ((long long)g.nxc * g.nyc > mx) mx = (long long)g.nxc * g.nyc;
    dim3 grid(nblk(mx), 3);
    k_bc_copy<T><<<grid, kBlock, 0, s>>>(g, uo, vo, wo, u, v, w);
}

void launch_eta_cylinder_z(cudaStream_t s, const Geo &g, const double *X, const double *Y,
                           const double *Dx, const double *Dy, double cx, double cy, double radius,
                           int nsub, double scale, double *eta)
{
    if (nsub == 0) {
        k_eta_plane_exact<<<nblk((long long)g.nxc * g.nyc), kBlock, 0, s>>>(g, X, Y, Dx, Dy, cx, cy, radius, eta);
    } else {
        dim3 grid(g.nxc, g.nyc);
        k_eta_plane<<<grid, kBlock, 0, s>>>(g, X, Y, Dx, Dy, cx, cy, radius, nsub, scale, eta);
    }
    const long long n = (long long)(g.nx - 1) * (g.ny - 1) * (g.nz - 2);
    k_eta_extrude<<<nblk(n), kBlock, 0, s>>>(g, eta);
}

template <class T>
void launch_div_inf(cfd_launch_ctx &c, const Geo &g, const Metrics<double> &m, const T *u,
                    const T *v, const T *w, unsigned long long *slot)
{
    k_div_inf<T><<<c.red_blocks, kBlock, 0, c.s>>>(g, m, u, v, w, slot);
}

template <class T>
void launch_div_projected(cfd_launch_ctx &c, const Geo &g, const Metrics<double> &m, double dt,
                          const double *p, const T *u1, const T *v1, const T *w1, const double *mean,
                          unsigned long long *slot2, bool with_ustar)
{
    k_div_projected<T><<<c.red_blocks, kBlock, 0, c.s>>>(g, m, dt, p, u1, v1, w1, mean, slot2, with_ustar);
}

template <class T>
void launch_cfl(cfd_launch_ctx &c, const Geo &g, const Metrics<double> &m, const T *u, const T *v, const T *w,
                double *out)
{
    k_cfl<T><<<c.red_blocks, kBlock, 0, c.s>>>(g, m, u, v, w, c.partials, c.counter, out);
}

template <class T>
void launch_steady_max(cfd_launch_ctx &c, const Geo &g, const T *ua, const T *va, const T *wa, const T *ub,
                       const T *vb, const T *wb, double *out)
{
    k_steady_max<T><<<c.red_blocks, kBlock, 0, c.s>>>(g, ua, va, wa, ub, vb, wb, c.partials, c.counter, out);
}

template <class T>
void launch_fill(cfd_launch_ctx &c, long long n, T *a, T val)
{
    k_fill<T><<<blocks_for(n, c.grid_cap), kBlock, 0, c.s>>>(n, a, val);
}

template <class A, class B>
void launch_convert(cfd_launch_ctx &c, long long n, const A *a, B *b)
{
    k_convert<A, B><<<blocks_for(n, c.grid_cap), kBlock, 0, c.s>>>(n, a, b);
}

// Copy with conversion where one side is a registered host buffer reached
// through its device mapping (NVLink-C2C on Grace systems): 16-byte vector
// accesses, four elements per thread step, so many link transactions are in
// flight; a scalar tail covers n % 4.  Both pointers are 16-byte aligned
// (checked by the caller).
template <class A, class B>
__device__ __forceinline__ void ld4(const A *p, A (&v)[4])
{
    if constexpr (sizeof(A) == 8) {
        const double2 a = reinterpret_cast<const double2 *>(p)[0], b = reinterpret_cast<const double2 *>(p)[1];
        v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
    } else {
        const float4 a = *reinterpret_cast<const float4 *>(p);
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    }
}
template <class B>
__device__ __forceinline__ void st4(B *p, const B (&v)[4])
{
    if constexpr (sizeof(B) == 8) {
        reinterpret_cast<double2 *>(p)[0] = make_double2(v[0], v[1]);
        reinterpret_cast<double2 *>(p)[1] = make_double2(v[2], v[3]);
    } else {
        *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
    }
}

template <class A, class B>
__global__ void __launch_bounds__(kBlock) k_link_copy(long long n, const A *__restrict__ a, B *__restrict__ b)
{
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x, st = (long long)gridDim.x * blockDim.x;
    const long long n4 = n >> 2;
    for (long long q = t0; q < n4; q += st) {
        A v[4];
        ld4<A, B>(a + 4 * q, v);
        B w[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) w[e] = (B)v[e];
        st4<B>(b + 4 * q, w);
    }
    for (long long m = 4 * n4 + t0; m < n; m += st) b[m] = (B)a[m];
}

template <class A, class B>
void launch_link_copy(cfd_launch_ctx &c, long long n, const A *a, B *b)
{
    k_link_copy<A, B><<<blocks_for((n + 3) / 4, c.grid_cap), kBlock, 0, c.s>>>(n, a, b);
}

#define CFD_FLOW_INSTANTIATE(T)                                                                   \
    template void launch_convdiff<T>(cudaStream_t, const Geo &, const Metrics<T> &, T, T,        \
                                     const T *, const T *, const T *, T *, T *, T *, const T *,  \
                                     const T *, T);                                              \
    template void launch_smagorinsky<T>(cudaStream_t, const Geo &, const Metrics<double> &,      \
                                        const T *, const T *, const T *, T *); \
    template void launch_src_add<T>(cfd_launch_ctx &, const Geo &, int, T *, T *, T *, const T *); \
    template void launch_src_accumulate<T>(cfd_launch_ctx &, long long, T, T *, const T *);      \
    template void launch_rhs<T>(cfd_launch_ctx &, const Geo &, const Metrics<double> &, double,  \
                                const double *, const T *, const T *, const T *, double *, bool, \
                                double *);                                                       \
    template void launch_update_uf<T>(cudaStream_t, const Geo &, const Metrics<T> &, double, T,  \
                                      const double *, const T *, const T *, const T *, const T *, \
                                      T *, T *, T *, T *);                                       \
    template void launch_cdcl<T>(cfd_launch_ctx &, const Geo &, const Metrics<double> &, double, \
                                 const T *, double *);                                           \
    template void launch_sync_z<T>(cudaStream_t, const Geo &, T *, T *, T *);                    \
    template void launch_pass<T>(cfd_launch_ctx &, const Geo &, const Metrics<double> &,          \
                                 const Metrics<float> &, const PassArgs<T> &, bool);             \
    template void launch_update_pass<T>(cfd_launch_ctx &, const Geo &, const Metrics<T> &,        \
                                        const Metrics<double> &, double, const double *, const T *, \
                                        const T *, const T *, const T *, T *, T *, T *, T *, bool, \
                                        T *, double, double *);                                   \
    template void launch_bc_main<T>(cudaStream_t, const Geo &, const BcTab &, T *, T *, T *,     \
                                    double *);                                                   \
    template void launch_bc_convective<T>(cfd_launch_ctx &, const Geo &, const Metrics<double> &, double,  \
                                          double, const T *, const T *, const T *, T *, T *, T *,  \
                                          double *);                                               \
    template void launch_bc_copy<T>(cudaStream_t, const Geo &, const T *, const T *, const T *,  \
                                    T *, T *, T *);                                              \
    template void launch_div_inf<T>(cfd_launch_ctx &, const Geo &, const Metrics<double> &,      \
                                    const T *, const T *, const T *, unsigned long long *);      \
    template void launch_fill<T>(cfd_launch_ctx &, long long, T *, T);                           \
    template void launch_cfl<T>(cfd_launch_ctx &, const Geo &, const Metrics<double> &, const T *,   \
                                const T *, const T *, double *);                                   \
    template void launch_steady_max<T>(cfd_launch_ctx &, const Geo &, const T *, const T *, const T *, \
                                       const T *, const T *, const T *, double *);                \
    template void launch_div_projected<T>(cfd_launch_ctx &, const Geo &, const Metrics<double> &,  \
                                          double, const double *, const T *, const T *, const T *, \
                                          const double *, unsigned long long *, bool);

CFD_FLOW_INSTANTIATE(double)
CFD_FLOW_INSTANTIATE(float)
template void launch_convert<double, float>(cfd_launch_ctx &, long long, const double *, float *);
template void launch_convert<float, double>(cfd_launch_ctx &, long long, const float *, double *);
template void launch_link_copy<double, float>(cfd_launch_ctx &, long long, const double *, float *);
template void launch_link_copy<float, double>(cfd_launch_ctx &, long long, const float *, double *);
template void launch_link_copy<double, double>(cfd_launch_ctx &, long long, const double *, double *);

}  // namespace cfd
