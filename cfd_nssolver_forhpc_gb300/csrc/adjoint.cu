// adjoint.cu -- discrete-adjoint (reverse-mode) kernels of the time step.
//
// Each kernel is the transpose of the linearisation of one forward kernel of
// flow.cu, taken at the forward state the tape holds.  Adjoint variables are
// FP64 in every context; forward data are read in the context's velocity
// type T and widened.  Kernels that gather (projection, right-hand side,
// boundary copy) write every adjoint element from one thread and are
// deterministic; the convection-diffusion transpose scatters its stencil
// with FP64 atomics, so its sums depend on the arrival order in the last
// bits only.
#include "cfd_internal.cuh"
#include "kernels.h"

namespace cfd {

namespace {

inline int nblk(long long n) { return (int)((n + kBlock - 1) / kBlock); }

__device__ __forceinline__ void cell_idx(const Geo &g, long long t, int &i, int &j, int &k)
{
    const unsigned int t32 = (unsigned int)t;
    const unsigned int ii = g.fsxc.div(t32);
    const unsigned int rem = t32 - ii * (unsigned int)g.sxc;
    const unsigned int jj = g.fsyc.div(rem);
    i = (int)ii + GC;
    j = (int)jj + GC;
    k = (int)(rem - jj * (unsigned int)g.syc) + GC;
}

__device__ __forceinline__ double vol(const Metrics<double> &m, int i, int j, int k)
{
    return m.x(AX_D, i) * m.y(AX_D, j) * m.z(AX_D, k);
}

}  // namespace

// ---------------------------------------------------------------------------
// Convection-diffusion (k_convdiff, convection_and_difussion.hpp:168-446).
//
// Output component d at face ic is
//   r = phi_c + sum_a [ -dt w_a F_a + nudt D_a ]
// with, along each axis a, the QUICK face pair (phiP, phiN) of phi = vel[d]
// from the five values phi[ic + q s_a], q = -2..2, and
//   a == d: F = phiP^2 - phiN^2                  (QuickUnitA, w = 1/Ds)
//   a != d: F = phiP Vp - phiN Vn,  Vp/Vn = vel[a] interpolated to the
//           d-face at the + and - side of axis a   (QuickUnitB, w = 1/D)
// The upwind switches are piecewise constants of the linearisation; they are
// evaluated in T exactly as the forward kernel does.

// Derivatives of a QUICK face pair with respect to (pp, p, c, n, nn) for
// adjoints gP, gN of phiP, phiN.  A form (own axis): curvature rows
// CAP*/CAN* with 1/D; B form: CBP*/CBN* with 1/Ds (index offset o = 1 / 0).
template <bool A>
__device__ __forceinline__ void quick_rev(bool up, bool un, const Axis<double> &ax, int I, double c_,
                                          double p_, double pp_, double n_, double nn_, double gP, double gN,
                                          double &phiP, double &phiN, double (&d)[5])
{
    // d[0] = pp, d[1] = p, d[2] = c, d[3] = n, d[4] = nn
    const int R = A ? AX_RD : AX_RDS, o = A ? 1 : 0;
    double cf, r1, r2;
    if (up) {
        cf = ax(A ? AX_CAPP : AX_CBPP, I); r1 = ax(R, I + o); r2 = ax(R, I + o - 1);
        phiP = 0.5 * (c_ + p_) - cf * ((p_ - c_) * r1 - (c_ - n_) * r2);
        d[1] += gP * (0.5 - cf * r1);
        d[2] += gP * (0.5 + cf * r1 + cf * r2);
        d[3] += gP * (-cf * r2);
    } else {
        cf = ax(A ? AX_CAPN : AX_CBPN, I); r1 = ax(R, I + o + 1); r2 = ax(R, I + o);
        phiP = 0.5 * (c_ + p_) - cf * ((pp_ - p_) * r1 - (p_ - c_) * r2);
        d[0] += gP * (-cf * r1);
        d[1] += gP * (0.5 + cf * r1 + cf * r2);
        d[2] += gP * (0.5 - cf * r2);
    }
    if (un) {
        cf = ax(A ? AX_CANP : AX_CBNP, I); r1 = ax(R, I + o - 1); r2 = ax(R, I + o - 2);
        phiN = 0.5 * (n_ + c_) - cf * ((c_ - n_) * r1 - (n_ - nn_) * r2);
        d[2] += gN * (0.5 - cf * r1);
        d[3] += gN * (0.5 + cf * r1 + cf * r2);
        d[4] += gN * (-cf * r2);
    } else {
        cf = ax(A ? AX_CANN : AX_CBNN, I); r1 = ax(R, I + o); r2 = ax(R, I + o - 1);
        phiN = 0.5 * (n_ + c_) - cf * ((p_ - c_) * r1 - (c_ - n_) * r2);
        d[1] += gN * (-cf * r1);
        d[2] += gN * (0.5 + cf * r1 + cf * r2);
        d[3] += gN * (0.5 - cf * r2);
    }
}

// QUICK face pair values only (the forward value phiP/phiN multiplies the
// adjoint of the advecting velocity)
template <bool A>
__device__ __forceinline__ void quick_val(bool up, bool un, const Axis<double> &ax, int I, double c_,
                                          double p_, double pp_, double n_, double nn_, double &phiP,
                                          double &phiN)
{
    double d[5] = {0, 0, 0, 0, 0};
    quick_rev<A>(up, un, ax, I, c_, p_, pp_, n_, nn_, 0.0, 0.0, phiP, phiN, d);
}

template <class T, int D>
__device__ __forceinline__ void cd_adjoint_component(const Geo &g, const Metrics<double> &m, double dt,
                                                     double nudt, const T *const (&vel)[3],
                                                     double *const (&adj)[3], long long ic,
                                                     const int (&I)[3], double lam)
{
    const long long s[3] = {g.sx, (long long)g.sy, 1};
    const Axis<double> *axp[3] = {&m.x, &m.y, &m.z};
    const T *phi = vel[D];
    const T pcT = phi[ic];
    const double pc = (double)pcT;
    double gc = lam;  // r = phi_c + ...
    const Axis<double> &AD = *axp[D];
    const double ITd = AD(AX_IT, I[D]);
    const T ITT = (T)ITd;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const Axis<double> &ax = *axp[a];
        const int Ia = I[a];
        const long long sa = s[a];
        const T ppT = phi[ic + 2 * sa], pT = phi[ic + sa], nT = phi[ic - sa], nnT = phi[ic - 2 * sa];
        const double pp = ppT, p = pT, n = nT, nn = nnT;
        double d[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        // diffusion
        {
            double c1, c2, w;
            if (a == D) { c1 = ax(AX_RD, Ia + 1); c2 = ax(AX_RD, Ia); w = ax(AX_RDS, Ia); }
            else        { c1 = ax(AX_RDS, Ia);    c2 = ax(AX_RDS, Ia - 1); w = ax(AX_RD, Ia); }
            const double gd = nudt * lam * w;
            d[1] += gd * c1;
            d[2] -= gd * (c1 + c2);
            d[3] += gd * c2;
        }
        // convection
        if (a == D) {
            const T Up = T(0.5) * (pT + pcT), Un = T(0.5) * (nT + pcT);
            const double cx = -dt * ax(AX_RDS, Ia) * lam;
            double phiP, phiN;
            quick_val<true>(Up > T(0), Un > T(0), ax, Ia, pc, p, pp, n, nn, phiP, phiN);
            quick_rev<true>(Up > T(0), Un > T(0), ax, Ia, pc, p, pp, n, nn, 2.0 * phiP * cx, -2.0 * phiN * cx,
                            phiP, phiN, d);
        } else {
            const T *va = vel[a];
            const long long sd = s[D];
            const T vpcT = va[ic], vpdT = va[ic + sd], vncT = va[ic - sa], vndT = va[ic - sa + sd];
            const T Vp = vpcT + (vpdT - vpcT) * ITT;
            const T Vn = vncT + (vndT - vncT) * ITT;
            const double cy = -dt * ax(AX_RD, Ia) * lam;
            double phiP, phiN;
            quick_val<false>(Vp > T(0), Vn > T(0), ax, Ia, pc, p, pp, n, nn, phiP, phiN);
            quick_rev<false>(Vp > T(0), Vn > T(0), ax, Ia, pc, p, pp, n, nn, (double)Vp * cy, -(double)Vn * cy,
                             phiP, phiN, d);
            const double gVp = phiP * cy, gVn = -phiN * cy;
            atomicAdd(adj[a] + ic, gVp * (1.0 - ITd));
            atomicAdd(adj[a] + ic + sd, gVp * ITd);
            atomicAdd(adj[a] + ic - sa, gVn * (1.0 - ITd));
            atomicAdd(adj[a] + ic - sa + sd, gVn * ITd);
        }
        atomicAdd(adj[D] + ic + 2 * sa, d[0]);
        atomicAdd(adj[D] + ic + sa, d[1]);
        atomicAdd(adj[D] + ic - sa, d[3]);
        atomicAdd(adj[D] + ic - 2 * sa, d[4]);
        gc += d[2];
    }
    atomicAdd(adj[D] + ic, gc);
}

// a{u,v,w} += (dCD/dT0)^T l{u,v,w}; l read at the faces the forward kernel
// writes (the domain's last normal face is skipped, d = 1)
template <class T>
__global__ void __launch_bounds__(kBlock)
k_adj_convdiff(Geo g, Metrics<double> m, double dt, double nudt, const T *__restrict__ u0,
               const T *__restrict__ v0, const T *__restrict__ w0, const double *__restrict__ lu,
               const double *__restrict__ lv, const double *__restrict__ lw, double *au, double *av, double *aw)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.n) return;
    int i, j, k;
    cell_idx(g, t, i, j, k);
    const long long ic = icel(g, i, j, k);
    const T *const vel[3] = {u0, v0, w0};
    double *const adj[3] = {au, av, aw};
    const int I[3] = {i, j, k};
    if (i < g.nx - GC - 1) {
        const double l = lu[ic];
        if (l != 0.0) cd_adjoint_component<T, 0>(g, m, dt, nudt, vel, adj, ic, I, l);
    }
    if (j < g.ny - GC - 1) {
        const double l = lv[ic];
        if (l != 0.0) cd_adjoint_component<T, 1>(g, m, dt, nudt, vel, adj, ic, I, l);
    }
    if (k < g.nz - GC - 1) {
        const double l = lw[ic];
        if (l != 0.0) cd_adjoint_component<T, 2>(g, m, dt, nudt, vel, adj, ic, I, l);
    }
}

// ---------------------------------------------------------------------------
// Projection + direct forcing (k_update_uf, updateUandF.hpp:95-190).  Per
// face of component d (computed when i_d < n_d - GC - 1):
//   T2 = u1 - dt (p[+] - p[c]) / Ds,  ef = eta_c + (eta[+] - eta_c) IT,
//   u3 = (1 - ef) T2,  f = (u3 - T2) / dt.
// With adjoints a3 (of u3) and af (of f):
//   lun = a3 + af/dt,  lT2 = (1 - ef) lun - af/dt,  lef = -T2 lun.
// af = af_in + dt * asrc (the source accumulation src += dt f of the passes
// before the last) + the drag/lift weights -2 dV wcd/lz (x), -2 dV wcl/lz (y).
// Each thread gathers its cell's p and eta adjoints from its own three faces
// and the three faces of its minus neighbours, so no two threads write the
// same element.  a3 is read only (the caller clears it).
template <class T>
__device__ __forceinline__ void uf_face_adj(const Geo &g, const Metrics<double> &m, double dt,
                                            const UfAdjArgs &A, const T *const (&u1)[3], const T *eta, int d,
                                            long long t, int i, int j, int k, double &lT2, double &lef)
{
    const long long s[3] = {g.sx, (long long)g.sy, 1};
    const long long sc[3] = {g.sxc, (long long)g.syc, 1};
    const Axis<double> *axp[3] = {&m.x, &m.y, &m.z};
    const int I[3] = {i, j, k};
    const long long ic = icel(g, i, j, k);
    const double rds = (*axp[d])(AX_RDS, I[d]), it = (*axp[d])(AX_IT, I[d]);
    const double T2 = (double)u1[d][ic] - dt * (A.x[t + sc[d]] - A.x[t]) * rds;
    const double ec = (double)eta[ic];
    const double ef = ec + ((double)eta[ic + s[d]] - ec) * it;
    double af = A.af ? A.af[d * g.n + t] : 0.0;
    if (A.asrc) af += A.src_dt * A.asrc[d * g.n + t];
    if (d < 2) {
        const double w = d == 0 ? A.wcd : A.wcl;
        if (w != 0.0) af += -2.0 * vol(m, i, j, k) * w / A.lz;
    }
    const double a3 = A.a3[d] ? A.a3[d][ic] : 0.0;
    const double rdt = 1.0 / dt;
    const double lun = a3 + af * rdt;
    lT2 = (1.0 - ef) * lun - af * rdt;
    lef = -T2 * lun;
}

template <class T>
__global__ void __launch_bounds__(kBlock)
k_adj_update_uf(Geo g, Metrics<double> m, double dt, UfAdjArgs A, const T *__restrict__ u1,
                const T *__restrict__ v1, const T *__restrict__ w1, const T *__restrict__ eta)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.n) return;
    int i, j, k;
    cell_idx(g, t, i, j, k);
    const T *const u[3] = {u1, v1, w1};
    const int I[3] = {i, j, k};
    const int nlim[3] = {g.nx - GC - 1, g.ny - GC - 1, g.nz - GC - 1};
    const long long sc[3] = {g.sxc, (long long)g.syc, 1};
    const Axis<double> *axp[3] = {&m.x, &m.y, &m.z};
    const long long ic = icel(g, i, j, k);
    double lx = 0.0, le = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const Axis<double> &ax = *axp[d];
        if (I[d] < nlim[d]) {  // own face
            double lT2, lef;
            uf_face_adj<T>(g, m, dt, A, u, eta, d, t, i, j, k, lT2, lef);
            A.a1[d][ic] += lT2;
            lx += dt * ax(AX_RDS, I[d]) * lT2;
            le += lef * (1.0 - ax(AX_IT, I[d]));
        }
        if (I[d] - 1 >= GC) {  // face of the minus neighbour (always computed)
            int ii = i, jj = j, kk = k;
            if (d == 0) --ii; else if (d == 1) --jj; else --kk;
            double lT2, lef;
            uf_face_adj<T>(g, m, dt, A, u, eta, d, t - sc[d], ii, jj, kk, lT2, lef);
            lx -= dt * ax(AX_RDS, I[d] - 1) * lT2;
            le += lef * ax(AX_IT, I[d] - 1);
        }
    }
    A.ax[t] += lx;
    A.aeta[ic] += le;
}

// ---------------------------------------------------------------------------
// Right-hand side (k_rhs + k_rhs_compat, b_matrix.hpp:76-79):
//   b_t = jp_t (d_t - mean),  d_t = -(1/dt) div_t,  mean = sum(dV d)/sum(dV)
// (mean = 0 without the compatibility projection).  Transpose with g = lb:
//   ld_t = jp_t g_t - dV_t G / V,  G = sum(jp g),  V = sum(dV)
//   ldiv_t = -(1/dt) ld_t;  lu[face i] = ldiv_i / Dx_i - ldiv_{i+1} / Dx_{i+1}
// The reduction gives G and V; the gather writes each face once (the ghost
// face below the first interior cell included).
__global__ void __launch_bounds__(kBlock)
k_adj_rhs_reduce(Geo g, Metrics<double> m, const double *__restrict__ jp, const double *__restrict__ lb,
                 double *partials, unsigned int *counter, double *out)
{
    double acc[2] = {0.0, 0.0};
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < g.n;
         t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_idx(g, t, i, j, k);
        acc[0] += jp[t] * lb[t];
        acc[1] += vol(m, i, j, k);
    }
    double tot[2];
    if (grid_reduce<2>(acc, partials, counter, tot) && threadIdx.x == 0) {
        out[0] = tot[0];
        out[1] = tot[1];
    }
}

__global__ void __launch_bounds__(kBlock)
k_adj_rhs(Geo g, Metrics<double> m, double ddt, const double *__restrict__ jp, const double *__restrict__ lb,
          const double *__restrict__ red, double *au, double *av, double *aw)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.n) return;
    int i, j, k;
    cell_idx(g, t, i, j, k);
    const double Gv = red ? red[0] / red[1] : 0.0;
    auto ldiv = [&](long long r, int ii, int jj, int kk) {
        return -ddt * (jp[r] * lb[r] - (red ? vol(m, ii, jj, kk) * Gv : 0.0));
    };
    const double lc = ldiv(t, i, j, k);
    const long long ic = icel(g, i, j, k);
    double *const a[3] = {au, av, aw};
    const Axis<double> *axp[3] = {&m.x, &m.y, &m.z};
    const int I[3] = {i, j, k};
    const int last[3] = {g.nx - GC - 1, g.ny - GC - 1, g.nz - GC - 1};
    const long long s[3] = {g.sx, (long long)g.sy, 1};
    const long long sc[3] = {g.sxc, (long long)g.syc, 1};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const Axis<double> &ax = *axp[d];
        double v = lc * ax(AX_RD, I[d]);
        if (I[d] < last[d]) {
            int ii = i, jj = j, kk = k;
            if (d == 0) ++ii; else if (d == 1) ++jj; else ++kk;
            v -= ldiv(t + sc[d], ii, jj, kk) * ax(AX_RD, I[d] + 1);
        }
        a[d][ic] += v;
        if (I[d] == GC) a[d][ic - s[d]] -= lc * ax(AX_RD, I[d]);
    }
}

// ---------------------------------------------------------------------------
// Poisson solve.  x = A^+ b with A = jp L (the Jacobi-scaled operator) and
// L = D_V^-1 M, M symmetric (the finite-volume form).  A^T y = lx is
// M (D_V^-1 jp y) = lx: w solves A w = jp lx / dV, and y = dV w / jp.  The
// compatibility projection of the right-hand side removes the null space:
// lb = (dV/jp)(w - wbar), wbar = sum(dV w)/sum(dV).
// k_adj_vsum: out = {sum a, sum dV a, sum dV}
__global__ void __launch_bounds__(kBlock)
k_adj_vsum(Geo g, Metrics<double> m, const double *__restrict__ a, double *partials, unsigned int *counter,
           double *out)
{
    double acc[3] = {0.0, 0.0, 0.0};
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < g.n;
         t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_idx(g, t, i, j, k);
        const double v = vol(m, i, j, k);
        acc[0] += a[t];
        acc[1] += v * a[t];
        acc[2] += v;
    }
    double tot[3];
    if (grid_reduce<3>(acc, partials, counter, tot) && threadIdx.x == 0) {
        out[0] = tot[0];
        out[1] = tot[1];
        out[2] = tot[2];
    }
}

// b' = jp (lx / dV - sum(lx) / sum(dV))
__global__ void k_adj_solve_in(Geo g, Metrics<double> m, const double *__restrict__ jp,
                               const double *__restrict__ lx, const double *__restrict__ red,
                               double *__restrict__ bp)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.n) return;
    int i, j, k;
    cell_idx(g, t, i, j, k);
    bp[t] = jp[t] * (lx[t] / vol(m, i, j, k) - red[0] / red[2]);
}

// lb = (dV / jp)(w - sum(dV w) / sum(dV))
__global__ void k_adj_solve_out(Geo g, Metrics<double> m, const double *__restrict__ jp,
                                const double *__restrict__ w, const double *__restrict__ red,
                                double *__restrict__ lb)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.n) return;
    int i, j, k;
    cell_idx(g, t, i, j, k);
    lb[t] = vol(m, i, j, k) / jp[t] * (w[t] - red[1] / red[2]);
}

// ---------------------------------------------------------------------------
// Boundary conditions (k_bc_main, Boundary_Condition.hpp:37-175).  The
// forward writes ghost = Dir + Num * interior (normal components) and
// 2 Dir + (2 Num - 1) * interior (tangential); the transpose moves the
// adjoints of the written elements onto the interior element they read and
// clears them.  Phases run in reverse order (2, 1, 0).  The adjoint of the
// x-min u value goes to the inflow profile (one entry per interior j).
__global__ void k_adj_bc_main(Geo g, BcTab bc, int phase, double *au, double *av, double *aw, double *ainflow)
{
    const int na = phase == 0 ? g.nyc : g.nxc;
    const int nb = phase == 2 ? g.nyc : g.nzc;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)na * nb) return;
    const int a = (int)(t / nb) + GC, b = (int)(t % nb) + GC;
    auto num = [&](int f, int c) { return bc.num[f * 3 + c]; };
    auto tg = [&](int f, int c) { return 2.0 * bc.num[f * 3 + c] - 1.0; };
    // move the adjoints at positions q[0..cnt) onto `to` with factor fac
    auto fold = [&](double *arr, const long long *q, int cnt, long long to, double fac) {
        double s = 0.0;
        for (int r = 0; r < cnt; ++r) { s += arr[q[r]]; arr[q[r]] = 0.0; }
        arr[to] += fac * s;
        return s;
    };
    long long st, base;
    int e;
    if (phase == 0) { st = g.sx; base = icel(g, 0, a, b); e = g.nx - 1; }
    else if (phase == 1) { st = g.sy; base = icel(g, a, 0, b); e = g.ny - 1; }
    else { st = 1; base = icel(g, a, b, 0); e = g.nz - 1; }
    auto P = [&](int q) { return base + (long long)q * st; };
    const long long lo[2] = {P(1), P(0)};
    const long long hi3[3] = {P(e - 2), P(e - 1), P(e)};
    const long long hi2[2] = {P(e - 1), P(e)};
    double *const arr[3] = {au, av, aw};
    const int fm = 2 * phase, fp = 2 * phase + 1;  // minus / plus face of this phase
    for (int c = 0; c < 3; ++c) {
        if (c == phase) {  // normal component
            fold(arr[c], hi3, 3, P(e - 3), num(fp, c));
            const double s = fold(arr[c], lo, 2, P(2), num(fm, c));
            if (phase == 0 && bc.inflow && ainflow) atomicAdd(ainflow + (a - GC), s);
        } else {
            fold(arr[c], hi2, 2, P(e - 2), tg(fp, c));
            fold(arr[c], lo, 2, P(2), tg(fm, c));
        }
    }
}

// BC_staggered_copy (k_bc_copy): a0[q] += a1[q], a1[q] = 0 on the copied set
__global__ void k_adj_bc_copy(Geo g, double *a0u, double *a0v, double *a0w, double *a1u, double *a1v,
                              double *a1w)
{
    const int phase = blockIdx.y;
    const int na = phase == 0 ? g.nyc : g.nxc;
    const int nb = phase == 2 ? g.nyc : g.nzc;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)na * nb) return;
    const int a = (int)(t / nb) + GC, b = (int)(t % nb) + GC;
    long long stride, base;
    int e;
    if (phase == 0) { e = g.nx - 1; stride = g.sx; base = icel(g, 0, a, b); }
    else if (phase == 1) { e = g.ny - 1; stride = g.sy; base = icel(g, a, 0, b); }
    else { e = g.nz - 1; stride = 1; base = icel(g, a, b, 0); }
    const long long s[5] = {base, base + stride, base + (long long)(e - 1) * stride, base + (long long)e * stride,
                            base + (long long)(e - 2) * stride};
    double *const a0[3] = {a0u, a0v, a0w};
    double *const a1[3] = {a1u, a1v, a1w};
    for (int c = 0; c < 3; ++c)
        for (int q = 0; q < (c == phase ? 5 : 4); ++q) {
            a0[c][s[q]] += a1[c][s[q]];
            a1[c][s[q]] = 0.0;
        }
}

// ---------------------------------------------------------------------------
// Source coupling and the convection-diffusion output.
// Reference convention (k_src_add_ref): T1[m] += src[m] for m < N, so
// asrc[m] += a1[m].
__global__ void k_adj_src_add_ref(long long n, const double *__restrict__ a1u, const double *__restrict__ a1v,
                                  const double *__restrict__ a1w, double *__restrict__ asrc)
{
    for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n;
         m += (long long)gridDim.x * blockDim.x) {
        asrc[m] += a1u[m];
        asrc[n + m] += a1v[m];
        asrc[2 * n + m] += a1w[m];
    }
}

// Aligned convention (k_src_add_aligned): T1[icel(t)] += src[t] at every
// interior cell, so asrc[t] += a1[icel(t)]
__global__ void k_adj_src_add_aligned(Geo g, const double *__restrict__ a1u, const double *__restrict__ a1v,
                                      const double *__restrict__ a1w, double *__restrict__ asrc)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.n) return;
    int i, j, k;
    cell_idx(g, t, i, j, k);
    const long long ic = icel(g, i, j, k);
    asrc[t] += a1u[ic];
    asrc[g.n + t] += a1v[ic];
    asrc[2 * g.n + t] += a1w[ic];
}

// The faces the convection-diffusion kernel writes: acd += a1, a1 = 0 there
// (with asrc != null the aligned source added inside that kernel: asrc += a1)
__global__ void k_adj_cd_gather(Geo g, double *a1u, double *a1v, double *a1w, double *cu, double *cv,
                                double *cw, double *asrc)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.n) return;
    int i, j, k;
    cell_idx(g, t, i, j, k);
    const long long ic = icel(g, i, j, k);
    double *const a1[3] = {a1u, a1v, a1w};
    double *const cd[3] = {cu, cv, cw};
    const int I[3] = {i, j, k};
    const int nlim[3] = {g.nx - GC - 1, g.ny - GC - 1, g.nz - GC - 1};
    for (int d = 0; d < 3; ++d) {
        if (I[d] >= nlim[d]) continue;
        const double v = a1[d][ic];
        cd[d][ic] += v;
        if (asrc) asrc[d * g.n + t] += v;
        a1[d][ic] = 0.0;
    }
}

// x[t] = p[icel(t)]: the pressure at interior cells in compact order
__global__ void k_gather_interior(Geo g, const double *__restrict__ p, double *__restrict__ x)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.n) return;
    int i, j, k;
    cell_idx(g, t, i, j, k);
    x[t] = p[icel(g, i, j, k)];
}

// a += b (n elements)
__global__ void k_adj_add(long long n, double *__restrict__ a, const double *__restrict__ b)
{
    for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n;
         m += (long long)gridDim.x * blockDim.x)
        a[m] += b[m];
}

// ---- launchers --------------------------------------------------------------
template <class T>
void launch_adj_convdiff(cudaStream_t s, const Geo &g, const Metrics<double> &m, double dt, double nudt,
                         const T *u0, const T *v0, const T *w0, const double *lu, const double *lv,
                         const double *lw, double *au, double *av, double *aw)
{
    k_adj_convdiff<T><<<nblk(g.n), kBlock, 0, s>>>(g, m, dt, nudt, u0, v0, w0, lu, lv, lw, au, av, aw);
}

template <class T>
void launch_adj_update_uf(cudaStream_t s, const Geo &g, const Metrics<double> &m, double dt,
                          const UfAdjArgs &A, const T *u1, const T *v1, const T *w1, const T *eta)
{
    k_adj_update_uf<T><<<nblk(g.n), kBlock, 0, s>>>(g, m, dt, A, u1, v1, w1, eta);
}

void launch_adj_rhs(cfd_launch_ctx &c, const Geo &g, const Metrics<double> &m, double ddt, const double *jp,
                    const double *lb, bool compat, double *red, double *au, double *av, double *aw)
{
    if (compat) k_adj_rhs_reduce<<<c.red_blocks, kBlock, 0, c.s>>>(g, m, jp, lb, c.partials, c.counter, red);
    k_adj_rhs<<<nblk(g.n), kBlock, 0, c.s>>>(g, m, ddt, jp, lb, compat ? red : nullptr, au, av, aw);
}

void launch_adj_solve_in(cfd_launch_ctx &c, const Geo &g, const Metrics<double> &m, const double *jp,
                         const double *lx, double *red, double *bp)
{
    k_adj_vsum<<<c.red_blocks, kBlock, 0, c.s>>>(g, m, lx, c.partials, c.counter, red);
    k_adj_solve_in<<<nblk(g.n), kBlock, 0, c.s>>>(g, m, jp, lx, red, bp);
}

void launch_adj_solve_out(cfd_launch_ctx &c, const Geo &g, const Metrics<double> &m, const double *jp,
                          const double *w, double *red, double *lb)
{
    k_adj_vsum<<<c.red_blocks, kBlock, 0, c.s>>>(g, m, w, c.partials, c.counter, red);
    k_adj_solve_out<<<nblk(g.n), kBlock, 0, c.s>>>(g, m, jp, w, red, lb);
}

void launch_adj_bc_main(cudaStream_t s, const Geo &g, const BcTab &bc, double *au, double *av, double *aw,
                        double *ainflow)
{
    const long long n[3] = {(long long)g.nyc * g.nzc, (long long)g.nxc * g.nzc, (long long)g.nxc * g.nyc};
    for (int ph = 2; ph >= 0; --ph) k_adj_bc_main<<<nblk(n[ph]), kBlock, 0, s>>>(g, bc, ph, au, av, aw, ainflow);
}

void launch_adj_bc_copy(cudaStream_t s, const Geo &g, double *a0u, double *a0v, double *a0w, double *a1u,
                        double *a1v, double *a1w)
{
    long long mx = (long long)g.nyc * g.nzc;
    if ((long long)g.nxc * g.nzc > mx) mx = (long long)g.nxc * g.nzc;
    if ((long long)g.nxc * g.nyc > mx) mx = (long long)g.nxc * g.nyc;
    k_adj_bc_copy<<<dim3(nblk(mx), 3), kBlock, 0, s>>>(g, a0u, a0v, a0w, a1u, a1v, a1w);
}

void launch_adj_src_add_ref(cfd_launch_ctx &c, long long n, const double *a1u, const double *a1v,
                            const double *a1w, double *asrc)
{
    k_adj_src_add_ref<<<blocks_for(n, c.grid_cap), kBlock, 0, c.s>>>(n, a1u, a1v, a1w, asrc);
}

void launch_adj_src_add_aligned(cudaStream_t s, const Geo &g, const double *a1u, const double *a1v,
                                const double *a1w, double *asrc)
{
    k_adj_src_add_aligned<<<nblk(g.n), kBlock, 0, s>>>(g, a1u, a1v, a1w, asrc);
}

void launch_adj_cd_gather(cudaStream_t s, const Geo &g, double *a1u, double *a1v, double *a1w, double *cu,
                          double *cv, double *cw, double *asrc)
{
    k_adj_cd_gather<<<nblk(g.n), kBlock, 0, s>>>(g, a1u, a1v, a1w, cu, cv, cw, asrc);
}

void launch_gather_interior(cudaStream_t s, const Geo &g, const double *p, double *x)
{
    k_gather_interior<<<nblk(g.n), kBlock, 0, s>>>(g, p, x);
}

void launch_adj_add(cfd_launch_ctx &c, long long n, double *a, const double *b)
{
    k_adj_add<<<blocks_for(n, c.grid_cap), kBlock, 0, c.s>>>(n, a, b);
}

#define CFD_ADJ_INSTANTIATE(T)                                                                         \
    template void launch_adj_convdiff<T>(cudaStream_t, const Geo &, const Metrics<double> &, double,   \
                                         double, const T *, const T *, const T *, const double *,      \
                                         const double *, const double *, double *, double *, double *); \
    template void launch_adj_update_uf<T>(cudaStream_t, const Geo &, const Metrics<double> &, double,  \
                                          const UfAdjArgs &, const T *, const T *, const T *, const T *);
CFD_ADJ_INSTANTIATE(double)
CFD_ADJ_INSTANTIATE(float)
#undef CFD_ADJ_INSTANTIATE

}  // namespace cfd
