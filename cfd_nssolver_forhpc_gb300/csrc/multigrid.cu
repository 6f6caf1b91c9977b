// multigrid.cu -- geometric multigrid V-cycle as the preconditioner of the
// FP32 inner CG of the mixed-precision Poisson solve (no counterpart in the
// reference, whose solvers are BiCGSTAB and SOR).
//
// The inner system is M e = h with M = dV L, the symmetric finite-volume form
// of the Poisson operator (M x)_c = dV_c (sum_a (cm_a + cp_a) x_c - cm_a x_-a
// - cp_a x_+a), Neumann faces having zero coefficients.  Levels are cell-
// centred: each axis is halved while its length is even and at least 4
// (semi-coarsening otherwise); coarse cell widths are the sums of their
// children's, centre distances (W[I] + W[I+1]) / 2, and the coarse operator
// is the same finite-volume form on that grid (rediscretisation).  Transfer:
// the residual, an integrated quantity, is summed over the children
// (restriction); the coarse correction is added to every child (prolongation,
// the transpose of the restriction).  Smoother: red-black Gauss-Seidel
// x_c = (b_c / dV_c + sum cm x_- + cp x_+) / (sum cm + cp), red then black
// before the coarse correction and black then red after it.  The coarsest
// level (at most kMgCoarsest cells) is solved exactly in the range of M: its
// right-hand side loses its mean (constants are M's null space) and is
// multiplied by the dense inverse of M + a 1 1^T, a > 0, built on the host.
// Every piece is a fixed symmetric linear map, so the V-cycle is a symmetric
// operator and CG keeps its short recurrences.
//
// Levels above kMgSmall cells run as grid-wide kernels (the smoother works
// on cell pairs along k, one thread per pair updating the cell of the
// requested colour); the small levels run inside one single-block kernel
// that performs their whole sub-cycle with block barriers.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <vector>

#include "context.h"

#include <cooperative_groups.h>

using namespace cfd;

namespace {

constexpr int kSmallThreads = 1024;
constexpr int kMgCoarsest = 256;     // cells of the coarsest level at most (dense inverse)
constexpr int kMgCoarseTarget = 64;  // coarsening goes on while a level has more cells and an axis halves
constexpr int kSweepSmemMax = 96 * 1024;  // shared memory of a fused-sweep block at most

// shared memory of a fused-sweep block: rings of 4 x planes (TJ + 4 rows),
// 4 b planes and 3 colour planes (TJ + 2 rows each), nz floats a row
inline size_t sweep_smem(int tj, int nz) { return (size_t)(4 * (tj + 4) + 7 * (tj + 2)) * nz * sizeof(float); }

inline int nblk(long long n) { return (int)((n + kBlock - 1) / kBlock); }

// smoothing sweeps of level l before and after the coarse correction
inline int level_sweeps(const Mg &G, int l) { return l == 0 ? G.sweeps0 : G.sweeps; }

__device__ __forceinline__ void decomp(const MgLevel &L, long long t, int &i, int &j, int &k)
{
    const unsigned u = (unsigned)t;
    const unsigned ii = L.fyz.div(u), r = u - ii * (unsigned)(L.ny * L.nz), jj = L.fz.div(r);
    i = (int)ii;
    j = (int)jj;
    k = (int)(r - jj * (unsigned)L.nz);
}

// table loads: read-only global loads for the grid-wide kernels, plain
// loads where the small-level kernel has staged the tables in shared memory
template <bool SM>
__device__ __forceinline__ float tl(const float *p)
{
    if constexpr (SM) return *p;
    else return __ldg(p);
}
template <bool SM>
__device__ __forceinline__ float4 tl4(const float *p)
{
    if constexpr (SM) return *reinterpret_cast<const float4 *>(p);
    else return __ldg(reinterpret_cast<const float4 *>(p));
}

// index type: 32-bit inside the small-level kernel's shared memory
template <bool SM>
using Ix = std::conditional_t<SM, int, long long>;

// 1 / diag of the smoother: the approximate reciprocal (2 ulp, one
// special-function instruction); every smoothing path and the small levels'
// per-cell tables use this same function, so the V-cycle stays one fixed
// symmetric operator
__device__ __forceinline__ float smooth_rcp(float d) { return __fdividef(1.0f, d); }

// the neighbour sum of L at (i, j, k), cell t.  PZ: the level is periodic in
// z (its end cells couple across the period).  A compile-time switch: the
// wrap costs the non-periodic smoother registers and occupancy.
template <bool SM = false, bool PZ = false>
__device__ __forceinline__ float mg_nb(const MgLevel &L, const float *__restrict__ x, int i, int j, int k, Ix<SM> t)
{
    const Ix<SM> sx = (Ix<SM>)L.ny * L.nz, sy = L.nz;
    float s = 0.f;
    if (i > 0) s = fmaf(tl<SM>(L.cm[0] + i), x[t - sx], s);
    if (i < L.nx - 1) s = fmaf(tl<SM>(L.cp[0] + i), x[t + sx], s);
    if (j > 0) s = fmaf(tl<SM>(L.cm[1] + j), x[t - sy], s);
    if (j < L.ny - 1) s = fmaf(tl<SM>(L.cp[1] + j), x[t + sy], s);
    if (k > 0) s = fmaf(tl<SM>(L.cm[2] + k), x[t - 1], s);
    else if (PZ) s = fmaf(tl<SM>(L.cm[2] + k), x[t + (L.nz - 1)], s);
    if (k < L.nz - 1) s = fmaf(tl<SM>(L.cp[2] + k), x[t + 1], s);
    else if (PZ) s = fmaf(tl<SM>(L.cp[2] + k), x[t - (L.nz - 1)], s);
    return s;
}

template <bool SM = false>
__device__ __forceinline__ float mg_diag(const MgLevel &L, int i, int j, int k)
{
    return tl<SM>(L.sum[0] + i) + tl<SM>(L.sum[1] + j) + tl<SM>(L.sum[2] + k);
}

template <bool SM = false>
__device__ __forceinline__ float mg_rdv(const MgLevel &L, int i, int j, int k)
{
    return tl<SM>(L.rw[0] + i) * tl<SM>(L.rw[1] + j) * tl<SM>(L.rw[2] + k);
}

// Gauss-Seidel update of one cell: x = (b / dV + neighbours) / diag; the
// small-level kernel reads 1 / dV and 1 / diag from its per-cell tables
// (the same values, computed once by k_mg_cell_tables)
template <bool SM = false, bool PZ = false>
__device__ __forceinline__ void gs_cell(const MgLevel &L, const float *__restrict__ b, float *__restrict__ x, int i,
                                        int j, int k, Ix<SM> t, bool zero_init)
{
    const float nb = zero_init ? 0.f : mg_nb<SM, PZ>(L, x, i, j, k, t);
    float v;
    if constexpr (SM) v = fmaf(b[t], L.rv[t], nb) * L.rg[t];
    else v = fmaf(b[t], mg_rdv<SM>(L, i, j, k), nb) * smooth_rcp(mg_diag<SM>(L, i, j, k));
    if (L.om != 1.f) v = zero_init ? L.om * v : fmaf(L.om, v - x[t], x[t]);
    x[t] = v;
}

// one colour over a level with nz % 4 == 0: one thread per quad of cells
// k = 4m..4m+3 (float4 rows), updating the two cells of that colour
// RHO: also accumulate b . x of the quads after the update into *rho
template <bool SM = false, class I = Ix<SM>, bool PZ = false, bool RHO = false>
__device__ __forceinline__ void smooth_quads(const MgLevel &L, const float *__restrict__ b, float *__restrict__ x,
                                             int color, bool zero_init, I t0, I stride, float *rho = nullptr)
{
    const I nq = (I)(L.n >> 2);
    const int n4 = L.nz >> 2;
    const I sx = (I)L.ny * L.nz, sy = L.nz;
    for (I q = t0; q < nq; q += stride) {
        const unsigned u = (unsigned)q;
        const unsigned i = L.fyq.div(u), r = u - i * (unsigned)(L.ny * n4), j = L.fq.div(r);
        const int k0 = 4 * (int)(r - j * (unsigned)n4);
        const I t = ((I)i * L.ny + j) * L.nz + k0;
        const int e0 = (int)((color + i + j) & 1u);  // first updated cell of the quad: e0, then e0 + 2
        const bool odd = e0 != 0;
        // the two cells of the colour sit at quad offsets e0 and e0 + 2:
        // pick their per-cell values with selects (no local arrays)
        auto pick = [odd](float a0, float a1) { return odd ? a1 : a0; };
        const float4 bv = *reinterpret_cast<const float4 *>(b + t);
        const float bA = pick(bv.x, bv.y), bB = pick(bv.z, bv.w);
        float rA, rB, dA, dB;
        if constexpr (SM) {
            const float4 rv = *reinterpret_cast<const float4 *>(L.rv + t);
            const float4 rg = *reinterpret_cast<const float4 *>(L.rg + t);
            rA = pick(rv.x, rv.y);
            rB = pick(rv.z, rv.w);
            dA = pick(rg.x, rg.y);
            dB = pick(rg.z, rg.w);
        } else {
            const float rxy = tl<SM>(L.rw[0] + i) * tl<SM>(L.rw[1] + j);
            const float sxy = tl<SM>(L.sum[0] + i) + tl<SM>(L.sum[1] + j);
            const float4 rz = tl4<SM>(L.rw[2] + k0);
            const float4 sz = tl4<SM>(L.sum[2] + k0);
            rA = rxy * pick(rz.x, rz.y);
            rB = rxy * pick(rz.z, rz.w);
            dA = smooth_rcp(sxy + pick(sz.x, sz.y));
            dB = smooth_rcp(sxy + pick(sz.z, sz.w));
        }
        float4 xc = make_float4(0.f, 0.f, 0.f, 0.f);
        float nA = 0.f, nB = 0.f;
        if (!zero_init) {
            xc = *reinterpret_cast<const float4 *>(x + t);
            float4 xm = make_float4(0.f, 0.f, 0.f, 0.f), xp = xm, ym = xm, yp = xm;
            if (i > 0) xm = *reinterpret_cast<const float4 *>(x + t - sx);
            if ((int)i < L.nx - 1) xp = *reinterpret_cast<const float4 *>(x + t + sx);
            if (j > 0) ym = *reinterpret_cast<const float4 *>(x + t - sy);
            if ((int)j < L.ny - 1) yp = *reinterpret_cast<const float4 *>(x + t + sy);
            const float zlo = k0 > 0 ? x[t - 1] : (PZ ? x[t + (L.nz - 1)] : 0.f);
            const float zhi = k0 + 4 < L.nz ? x[t + 4] : (PZ ? x[t + 4 - L.nz] : 0.f);
            const float cxm = tl<SM>(L.cm[0] + i), cxp = tl<SM>(L.cp[0] + i);
            const float cym = tl<SM>(L.cm[1] + j), cyp = tl<SM>(L.cp[1] + j);
            const float4 czm = tl4<SM>(L.cm[2] + k0);
            const float4 czp = tl4<SM>(L.cp[2] + k0);
            // cell A = e0: k-neighbours (zlo | x0, x1 | x2); cell B = e0 + 2: (x1 | x2, x3 | zhi)
            nA = cxm * pick(xm.x, xm.y);
            nA = fmaf(cxp, pick(xp.x, xp.y), nA);
            nA = fmaf(cym, pick(ym.x, ym.y), nA);
            nA = fmaf(cyp, pick(yp.x, yp.y), nA);
            nA = fmaf(pick(czm.x, czm.y), pick(zlo, xc.x), nA);
            nA = fmaf(pick(czp.x, czp.y), pick(xc.y, xc.z), nA);
            nB = cxm * pick(xm.z, xm.w);
            nB = fmaf(cxp, pick(xp.z, xp.w), nB);
            nB = fmaf(cym, pick(ym.z, ym.w), nB);
            nB = fmaf(cyp, pick(yp.z, yp.w), nB);
            nB = fmaf(pick(czm.z, czm.w), pick(xc.y, xc.z), nB);
            nB = fmaf(pick(czp.z, czp.w), pick(xc.w, zhi), nB);
        }
        float vA = fmaf(bA, rA, nA) * dA, vB = fmaf(bB, rB, nB) * dB;
        if (L.om != 1.f) {  // over-relaxation (xc is 0 from a zero start)
            const float oA = pick(xc.x, xc.y), oB = pick(xc.z, xc.w);
            vA = fmaf(L.om, vA - oA, oA);
            vB = fmaf(L.om, vB - oB, oB);
        }
        float xo[4];
        xo[0] = odd ? xc.x : vA;
        xo[1] = odd ? vA : xc.y;
        xo[2] = odd ? xc.z : vB;
        xo[3] = odd ? vB : xc.w;
        *reinterpret_cast<float4 *>(x + t) = make_float4(xo[0], xo[1], xo[2], xo[3]);
        if constexpr (RHO) *rho = fmaf(bv.x, xo[0], fmaf(bv.y, xo[1], fmaf(bv.z, xo[2], fmaf(bv.w, xo[3], *rho))));
    }
}

// quad decomposition of smooth_quads: thread index q -> (i, j, k0), cell t
template <class I>
__device__ __forceinline__ void quad_of(const MgLevel &L, I q, unsigned &i, unsigned &j, int &k0, I &t)
{
    const int n4 = L.nz >> 2;
    const unsigned u = (unsigned)q;
    i = L.fyq.div(u);
    const unsigned r = u - i * (unsigned)(L.ny * n4);
    j = L.fq.div(r);
    k0 = 4 * (int)(r - j * (unsigned)n4);
    t = ((I)i * L.ny + j) * L.nz + k0;
}

// the axis-table values a quad update reads: x- and x-faces, 1 / width and
// the coefficient sum of its column (i, j) and of its k quad
struct QuadTab {
    float cxm, cxp, cym, cyp, rwx, rwy, sx, sy;
    float4 czm, czp, rz, sz;
};

// the colour-`color` update of the two cells of a quad (offsets e0, e0 + 2)
// from the quad's and its neighbours' values and its table values:
// smooth_quads' arithmetic, term for term
__device__ __forceinline__ void quad_update_t(const QuadTab &T, unsigned i, unsigned j, const float4 &bv,
                                              const float4 &xc, const float4 &xm, const float4 &xp, const float4 &ym,
                                              const float4 &yp, float zlo, float zhi, int color, float4 &out)
{
    const int e0 = (int)((color + i + j) & 1u);
    const bool odd = e0 != 0;
    auto pick = [odd](float a0, float a1) { return odd ? a1 : a0; };
    const float bA = pick(bv.x, bv.y), bB = pick(bv.z, bv.w);
    const float rxy = T.rwx * T.rwy;
    const float sxy = T.sx + T.sy;
    const float rA = rxy * pick(T.rz.x, T.rz.y), rB = rxy * pick(T.rz.z, T.rz.w);
    const float dA = smooth_rcp(sxy + pick(T.sz.x, T.sz.y)), dB = smooth_rcp(sxy + pick(T.sz.z, T.sz.w));
    float nA = T.cxm * pick(xm.x, xm.y);
    nA = fmaf(T.cxp, pick(xp.x, xp.y), nA);
    nA = fmaf(T.cym, pick(ym.x, ym.y), nA);
    nA = fmaf(T.cyp, pick(yp.x, yp.y), nA);
    nA = fmaf(pick(T.czm.x, T.czm.y), pick(zlo, xc.x), nA);
    nA = fmaf(pick(T.czp.x, T.czp.y), pick(xc.y, xc.z), nA);
    float nB = T.cxm * pick(xm.z, xm.w);
    nB = fmaf(T.cxp, pick(xp.z, xp.w), nB);
    nB = fmaf(T.cym, pick(ym.z, ym.w), nB);
    nB = fmaf(T.cyp, pick(yp.z, yp.w), nB);
    nB = fmaf(pick(T.czm.z, T.czm.w), pick(xc.y, xc.z), nB);
    nB = fmaf(pick(T.czp.z, T.czp.w), pick(xc.w, zhi), nB);
    const float vA = fmaf(bA, rA, nA) * dA, vB = fmaf(bB, rB, nB) * dB;
    out = make_float4(odd ? xc.x : vA, odd ? vA : xc.y, odd ? xc.z : vB, odd ? vB : xc.w);
}

// the same with the tables read from the level as they are needed (the
// grid-wide kernels: loading them all first costs the two-row kernel
// registers)
__device__ __forceinline__ void quad_update(const MgLevel &L, unsigned i, unsigned j, int k0, const float4 &bv,
                                            const float4 &xc, const float4 &xm, const float4 &xp, const float4 &ym,
                                            const float4 &yp, float zlo, float zhi, int color, float4 &out)
{
    const int e0 = (int)((color + i + j) & 1u);
    const bool odd = e0 != 0;
    auto pick = [odd](float a0, float a1) { return odd ? a1 : a0; };
    const float bA = pick(bv.x, bv.y), bB = pick(bv.z, bv.w);
    const float rxy = __ldg(L.rw[0] + i) * __ldg(L.rw[1] + j);
    const float sxy = __ldg(L.sum[0] + i) + __ldg(L.sum[1] + j);
    const float4 rz = __ldg(reinterpret_cast<const float4 *>(L.rw[2] + k0));
    const float4 sz = __ldg(reinterpret_cast<const float4 *>(L.sum[2] + k0));
    const float rA = rxy * pick(rz.x, rz.y), rB = rxy * pick(rz.z, rz.w);
    const float dA = smooth_rcp(sxy + pick(sz.x, sz.y)), dB = smooth_rcp(sxy + pick(sz.z, sz.w));
    const float cxm = __ldg(L.cm[0] + i), cxp = __ldg(L.cp[0] + i);
    const float cym = __ldg(L.cm[1] + j), cyp = __ldg(L.cp[1] + j);
    const float4 czm = __ldg(reinterpret_cast<const float4 *>(L.cm[2] + k0));
    const float4 czp = __ldg(reinterpret_cast<const float4 *>(L.cp[2] + k0));
    float nA = cxm * pick(xm.x, xm.y);
    nA = fmaf(cxp, pick(xp.x, xp.y), nA);
    nA = fmaf(cym, pick(ym.x, ym.y), nA);
    nA = fmaf(cyp, pick(yp.x, yp.y), nA);
    nA = fmaf(pick(czm.x, czm.y), pick(zlo, xc.x), nA);
    nA = fmaf(pick(czp.x, czp.y), pick(xc.y, xc.z), nA);
    float nB = cxm * pick(xm.z, xm.w);
    nB = fmaf(cxp, pick(xp.z, xp.w), nB);
    nB = fmaf(cym, pick(ym.z, ym.w), nB);
    nB = fmaf(cyp, pick(yp.z, yp.w), nB);
    nB = fmaf(pick(czm.z, czm.w), pick(xc.y, xc.z), nB);
    nB = fmaf(pick(czp.z, czp.w), pick(xc.w, zhi), nB);
    const float vA = fmaf(bA, rA, nA) * dA, vB = fmaf(bB, rB, nB) * dB;
    out = make_float4(odd ? xc.x : vA, odd ? vA : xc.y, odd ? xc.z : vB, odd ? vB : xc.w);
}

// The first pre-smoothing sweep from x = 0 in one pass.  Colour 0 from zero
// gives x = (b / dV) / diag at the colour-0 cells and 0 at the others;
// colour 1 then reads colour-0 neighbours only, and each thread forms those
// values from b itself.  The result equals the two colour launches bit for
// bit (k_mg_smooth4 with zero_init, then colour 1).
template <class I>
__global__ void __launch_bounds__(kBlock) k_mg_first4(MgLevel L, const float *__restrict__ b, float *__restrict__ x,
                                                         const int *done)
{
    pdl_wait();
    pdl_allow();
    if (*done) return;
    const I nq = (I)(L.n >> 2);
    const I sx = (I)L.ny * L.nz, sy = L.nz;
    // the zero-start colour-0 values of the quad at (ii, jj, k0), index tt;
    // cells of colour 1 read as 0 (as the colour-0 launch leaves them)
    auto zero_start = [&](int ii, int jj, int k0, I tt) -> float4 {
        const float4 bv = *reinterpret_cast<const float4 *>(b + tt);
        const int e0 = (int)((ii + jj) & 1);
        const bool odd = e0 != 0;
        auto pick = [odd](float a0, float a1) { return odd ? a1 : a0; };
        const float rxy = __ldg(L.rw[0] + ii) * __ldg(L.rw[1] + jj);
        const float sxy = __ldg(L.sum[0] + ii) + __ldg(L.sum[1] + jj);
        const float4 rz = __ldg(reinterpret_cast<const float4 *>(L.rw[2] + k0));
        const float4 sz = __ldg(reinterpret_cast<const float4 *>(L.sum[2] + k0));
        const float vA = fmaf(pick(bv.x, bv.y), rxy * pick(rz.x, rz.y), 0.f) * smooth_rcp(sxy + pick(sz.x, sz.y));
        const float vB = fmaf(pick(bv.z, bv.w), rxy * pick(rz.z, rz.w), 0.f) * smooth_rcp(sxy + pick(sz.z, sz.w));
        return make_float4(odd ? 0.f : vA, odd ? vA : 0.f, odd ? 0.f : vB, odd ? vB : 0.f);
    };
    // one cell's zero-start value (for the z neighbours across the quad ends)
    auto zero_cell = [&](int ii, int jj, int kk, I tt) -> float {
        if (((ii + jj + kk) & 1) != 0) return 0.f;
        const float r = (__ldg(L.rw[0] + ii) * __ldg(L.rw[1] + jj)) * __ldg(L.rw[2] + kk);
        const float d = smooth_rcp((__ldg(L.sum[0] + ii) + __ldg(L.sum[1] + jj)) + __ldg(L.sum[2] + kk));
        return fmaf(b[tt], r, 0.f) * d;
    };
    for (I q = (I)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += (I)gridDim.x * blockDim.x) {
        unsigned i, j;
        int k0;
        I t;
        quad_of<I>(L, q, i, j, k0, t);
        const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 xc = zero_start((int)i, (int)j, k0, t);
        const float4 xm = i > 0 ? zero_start((int)i - 1, (int)j, k0, t - sx) : zero;
        const float4 xp = (int)i < L.nx - 1 ? zero_start((int)i + 1, (int)j, k0, t + sx) : zero;
        const float4 ym = j > 0 ? zero_start((int)i, (int)j - 1, k0, t - sy) : zero;
        const float4 yp = (int)j < L.ny - 1 ? zero_start((int)i, (int)j + 1, k0, t + sy) : zero;
        const float zlo = k0 > 0 ? zero_cell((int)i, (int)j, k0 - 1, t - 1)
                                 : (L.pz ? zero_cell((int)i, (int)j, L.nz - 1, t + (L.nz - 1)) : 0.f);
        const float zhi = k0 + 4 < L.nz ? zero_cell((int)i, (int)j, k0 + 4, t + 4)
                                        : (L.pz ? zero_cell((int)i, (int)j, 0, t + 4 - L.nz) : 0.f);
        const float4 bv = *reinterpret_cast<const float4 *>(b + t);
        float4 out;
        quad_update(L, i, j, k0, bv, xc, xm, xp, ym, yp, zlo, zhi, 1, out);
        *reinterpret_cast<float4 *>(x + t) = out;
    }
}

// The prolongation and the first post-smoothing colour (colour 1) in one
// pass: the colour-0 cells around each colour-1 cell are read as x + the
// coarse correction of their parent (the value k_mg_prolong would store) and
// the colour-1 cells get their Gauss-Seidel update.  Only colour-1 cells are
// stored: the colour-0 cells, which other threads read here, keep x, and the
// colour-0 pass that follows overwrites them without reading them (their
// update depends on their colour-1 neighbours only).  So after that pass the
// level equals k_mg_prolong, colour 1, colour 0 bit for bit.
template <class I>
__global__ void __launch_bounds__(kBlock) k_mg_prolong_first4(MgLevel L, MgLevel C, const float *__restrict__ b,
                                                                 float *__restrict__ x, const float *__restrict__ xc_,
                                                                 const int *done)
{
    pdl_wait();
    pdl_allow();
    if (*done) return;
    const I nq = (I)(L.n >> 2);
    const I sx = (I)L.ny * L.nz, sy = L.nz;
    const int fx = L.nx / C.nx, fy = L.ny / C.ny, fz = L.nz / C.nz;
    auto corr = [&](int ii, int jj, int kk) -> float {
        return __ldg(xc_ + ((long long)(ii / fx) * C.ny + jj / fy) * C.nz + kk / fz);
    };
    auto quad = [&](int ii, int jj, int k0, I tt) -> float4 {
        const float4 v = *reinterpret_cast<const float4 *>(x + tt);
        return make_float4(v.x + corr(ii, jj, k0), v.y + corr(ii, jj, k0 + 1), v.z + corr(ii, jj, k0 + 2),
                           v.w + corr(ii, jj, k0 + 3));
    };
    for (I q = (I)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += (I)gridDim.x * blockDim.x) {
        unsigned i, j;
        int k0;
        I t;
        quad_of<I>(L, q, i, j, k0, t);
        const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 raw = *reinterpret_cast<const float4 *>(x + t);
        const float4 xc = quad((int)i, (int)j, k0, t);
        const float4 xm = i > 0 ? quad((int)i - 1, (int)j, k0, t - sx) : zero;
        const float4 xp = (int)i < L.nx - 1 ? quad((int)i + 1, (int)j, k0, t + sx) : zero;
        const float4 ym = j > 0 ? quad((int)i, (int)j - 1, k0, t - sy) : zero;
        const float4 yp = (int)j < L.ny - 1 ? quad((int)i, (int)j + 1, k0, t + sy) : zero;
        const float zlo = k0 > 0 ? x[t - 1] + corr((int)i, (int)j, k0 - 1)
                                 : (L.pz ? x[t + (L.nz - 1)] + corr((int)i, (int)j, L.nz - 1) : 0.f);
        const float zhi = k0 + 4 < L.nz ? x[t + 4] + corr((int)i, (int)j, k0 + 4)
                                        : (L.pz ? x[t + 4 - L.nz] + corr((int)i, (int)j, 0) : 0.f);
        const float4 bv = *reinterpret_cast<const float4 *>(b + t);
        float4 out;
        quad_update(L, i, j, k0, bv, xc, xm, xp, ym, yp, zlo, zhi, 1, out);
        // colour 1 at offsets e0, e0 + 2; the colour-0 cells keep x
        if (((1u + i + j) & 1u) != 0) {
            out.x = raw.x;
            out.z = raw.z;
        } else {
            out.y = raw.y;
            out.w = raw.w;
        }
        *reinterpret_cast<float4 *>(x + t) = out;
    }
}

// one colour over the level: pairs (k = 2m, 2m + 1) when nz is even (one
// thread per pair updates the cell of that colour), single cells otherwise;
// zero_init starts from x = 0 (the other colour written as 0)
template <bool SM = false, bool PZ = false>
__device__ __forceinline__ void smooth_level(const MgLevel &L, const float *__restrict__ b, float *__restrict__ x,
                                             int color, bool zero_init, Ix<SM> t0, Ix<SM> stride)
{
    if ((L.nz & 1) == 0) {
        const Ix<SM> np = L.n >> 1;
        const int nh = L.nz >> 1;
        for (Ix<SM> q = t0; q < np; q += stride) {
            const unsigned u = (unsigned)q;
            const unsigned i = L.fyh.div(u), r = u - i * (unsigned)(L.ny * nh), j = L.fh.div(r);
            const int m = (int)(r - j * (unsigned)nh);
            const int k = 2 * m + (int)((color + i + j) & 1u);
            const Ix<SM> t = ((Ix<SM>)i * L.ny + j) * L.nz + k;
            gs_cell<SM, PZ>(L, b, x, (int)i, (int)j, k, t, zero_init);
            if (zero_init) x[t + ((k & 1) ? -1 : 1)] = 0.f;
        }
        return;
    }
    for (Ix<SM> t = t0; t < L.n; t += stride) {
        int i, j, k;
        decomp(L, t, i, j, k);
        if (((i + j + k) & 1) != color) {
            if (zero_init) x[t] = 0.f;
            continue;
        }
        gs_cell<SM, PZ>(L, b, x, i, j, k, t, zero_init);
    }
}

// coarse b = sum over the children of (b - M x) on the fine level.  The
// restriction follows a pre-smoothing that ends with colour 1, after which
// the residual of every colour-1 cell is zero (its Gauss-Seidel equation
// holds exactly for the colour-0 values around it, none of which changed
// since), so only the colour-0 children are summed.
template <bool SM = false, bool PZ = false>
__device__ __forceinline__ void restrict_level(const MgLevel &F, const MgLevel &C, const float *__restrict__ bf,
                                               const float *__restrict__ xf, float *__restrict__ bc, Ix<SM> t0,
                                               Ix<SM> stride)
{
    const int fx = F.nx / C.nx, fy = F.ny / C.ny, fz = F.nz / C.nz;
    for (Ix<SM> T = t0; T < C.n; T += stride) {
        int I, J, K;
        decomp(C, T, I, J, K);
        float s = 0.f;
        for (int a = 0; a < fx; ++a)
            for (int b2 = 0; b2 < fy; ++b2)
                for (int c = 0; c < fz; ++c) {
                    const int i = fx * I + a, j = fy * J + b2, k = fz * K + c;
                    if ((i + j + k) & 1) continue;
                    const Ix<SM> t = ((Ix<SM>)i * F.ny + j) * F.nz + k;
                    // one rounding per operation (no contraction), so the float4
                    // form (k_mg_restrict4) can match it bit for bit
                    const float dv = __fmul_rn(__fmul_rn(tl<SM>(F.w[0] + i), tl<SM>(F.w[1] + j)), tl<SM>(F.w[2] + k));
                    const float res = __fsub_rn(__fmul_rn(mg_diag<SM>(F, i, j, k), xf[t]), mg_nb<SM, PZ>(F, xf, i, j, k, t));
                    s = __fadd_rn(s, __fsub_rn(bf[t], __fmul_rn(dv, res)));
                }
        bc[T] = s;
    }
}

// fine x += coarse x: one thread per coarse cell writes its children
template <bool SM = false>
__device__ __forceinline__ void prolong_level(const MgLevel &F, const MgLevel &C, const float *__restrict__ xc,
                                              float *__restrict__ xf, Ix<SM> t0, Ix<SM> stride)
{
    const int fx = F.nx / C.nx, fy = F.ny / C.ny, fz = F.nz / C.nz;
    for (Ix<SM> T = t0; T < C.n; T += stride) {
        int I, J, K;
        decomp(C, T, I, J, K);
        const float v = xc[T];
        for (int a = 0; a < fx; ++a)
            for (int b2 = 0; b2 < fy; ++b2) {
                const Ix<SM> base = ((Ix<SM>)(fx * I + a) * F.ny + fy * J + b2) * F.nz + fz * K;
                for (int c = 0; c < fz; ++c) xf[base + c] += v;
            }
    }
}

// per-cell 1 / dV and 1 / diag of a level (for the small-level kernel)
__global__ void k_mg_cell_tables(MgLevel L, float *__restrict__ rv, float *__restrict__ rg)
{
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < L.n; t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decomp(L, t, i, j, k);
        rv[t] = mg_rdv(L, i, j, k);
        rg[t] = smooth_rcp(mg_diag(L, i, j, k));
    }
}

template <bool PZ>
__global__ void __launch_bounds__(kBlock) k_mg_smooth(MgLevel L, const float *b, float *x, int color, int zero_init,
                                                      const int *done)
{
    pdl_wait();
    pdl_allow();
    if (*done) return;
    smooth_level<false, PZ>(L, b, x, color, zero_init != 0, (long long)blockIdx.x * blockDim.x + threadIdx.x,
                 (long long)gridDim.x * blockDim.x);
}

// the float4 form (nz % 4 == 0) as its own kernel; I = int where every
// index of the level fits (fewer instructions per quad)
template <class I, bool PZ>
__global__ void __launch_bounds__(kBlock) k_mg_smooth4(MgLevel L, const float *b, float *x, int color,
                                                          int zero_init, const int *done)
{
    pdl_wait();
    pdl_allow();
    if (*done) return;
    smooth_quads<false, I, PZ>(L, b, x, color, zero_init != 0, (I)blockIdx.x * blockDim.x + threadIdx.x,
                           (I)gridDim.x * blockDim.x);
}

// One colour over a float4 level with even ny, two j rows (j0, j0 + 1) of one
// quad each per thread: the two rows are each other's y neighbours (whose
// cells of the other colour this pass does not change), so a thread loads
// four x rows, two y rows and the two b rows instead of two quads' worth of
// six.  quad_update is smooth_quads' arithmetic term for term, so the pass
// equals k_mg_smooth4 bit for bit.  Gauss-Seidel only (om == 1).
template <class I, bool PZ>
__global__ void __launch_bounds__(kBlock, 4) k_mg_smooth4x2(MgLevel L, const float *b, float *x, int color,
                                                            int zero_init, const int *done)
{
    pdl_wait();
    pdl_allow();
    if (*done) return;
    const int n4 = L.nz >> 2;
    const I nq2 = (I)(L.n >> 3);
    const I sx = (I)L.ny * L.nz, sy = L.nz;
    for (I q = (I)blockIdx.x * blockDim.x + threadIdx.x; q < nq2; q += (I)gridDim.x * blockDim.x) {
        const unsigned u = (unsigned)q;
        const unsigned i = L.fy2q.div(u), r = u - i * (unsigned)((L.ny >> 1) * n4), jp = L.fq.div(r);
        const int k0 = 4 * (int)(r - jp * (unsigned)n4);
        const unsigned j0 = 2 * jp;
        const I t0 = ((I)i * L.ny + j0) * L.nz + k0, t1 = t0 + sy;
        const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 b0 = *reinterpret_cast<const float4 *>(b + t0), b1 = *reinterpret_cast<const float4 *>(b + t1);
        float4 c0 = zero, c1 = zero, xm0 = zero, xm1 = zero, xp0 = zero, xp1 = zero, ym = zero, yp = zero;
        float zl0 = 0.f, zh0 = 0.f, zl1 = 0.f, zh1 = 0.f;
        if (!zero_init) {
            c0 = *reinterpret_cast<const float4 *>(x + t0);
            c1 = *reinterpret_cast<const float4 *>(x + t1);
            if (i > 0) {
                xm0 = *reinterpret_cast<const float4 *>(x + t0 - sx);
                xm1 = *reinterpret_cast<const float4 *>(x + t1 - sx);
            }
            if ((int)i < L.nx - 1) {
                xp0 = *reinterpret_cast<const float4 *>(x + t0 + sx);
                xp1 = *reinterpret_cast<const float4 *>(x + t1 + sx);
            }
            if (j0 > 0) ym = *reinterpret_cast<const float4 *>(x + t0 - sy);
            if ((int)j0 + 2 < L.ny) yp = *reinterpret_cast<const float4 *>(x + t1 + sy);
            if (k0 > 0) {
                zl0 = x[t0 - 1];
                zl1 = x[t1 - 1];
            } else if (PZ) {
                zl0 = x[t0 + (L.nz - 1)];
                zl1 = x[t1 + (L.nz - 1)];
            }
            if (k0 + 4 < L.nz) {
                zh0 = x[t0 + 4];
                zh1 = x[t1 + 4];
            } else if (PZ) {
                zh0 = x[t0 + 4 - L.nz];
                zh1 = x[t1 + 4 - L.nz];
            }
        }
        float4 o0, o1;
        quad_update(L, i, j0, k0, b0, c0, xm0, xp0, ym, c1, zl0, zh0, color, o0);
        quad_update(L, i, j0 + 1, k0, b1, c1, xm1, xp1, c0, yp, zl1, zh1, color, o1);
        *reinterpret_cast<float4 *>(x + t0) = o0;
        *reinterpret_cast<float4 *>(x + t1) = o1;
    }
}

template <bool PZ>
__global__ void __launch_bounds__(kBlock) k_mg_restrict(MgLevel F, MgLevel C, const float *bf, const float *xf,
                                                        float *bc, const int *done)
{
    pdl_wait();
    pdl_allow();
    if (*done) return;
    restrict_level<false, PZ>(F, C, bf, xf, bc, (long long)blockIdx.x * blockDim.x + threadIdx.x,
                   (long long)gridDim.x * blockDim.x);
}

__global__ void __launch_bounds__(kBlock) k_mg_prolong(MgLevel F, MgLevel C, const float *xc, float *xf,
                                                       const int *done)
{
    pdl_wait();
    pdl_allow();
    if (*done) return;
    prolong_level(F, C, xc, xf, (long long)blockIdx.x * blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
}

// ---- transfers on float4 rows (2x2x2 coarsening, nz % 4 == 0) -------------
// The restriction with one thread per pair of coarse cells along k: their
// colour-0 children are one cell in each quad k0 = 4 kp .. 4 kp + 3 of the
// four fine rows (2I + a, 2J + b), so the thread reads those four quads and
// their neighbour quads as float4 (the smoother's pattern) instead of one
// scalar per neighbour per child.  The sum runs over the rows in the order
// of restrict_level and each term is formed with its operations, so the
// result is the same bit for bit.
template <bool PZ>
__global__ void __launch_bounds__(kBlock)
k_mg_restrict4(MgLevel F, MgLevel C, const float *__restrict__ bf, const float *__restrict__ xf, float *__restrict__ bc,
               const int *done)
{
    pdl_wait();
    pdl_allow();
    if (*done) return;
    const int ncp = C.nz >> 1;
    const long long total = C.n >> 1;
    const long long sx = (long long)F.ny * F.nz, sy = F.nz;
    for (long long u = (long long)blockIdx.x * blockDim.x + threadIdx.x; u < total;
         u += (long long)gridDim.x * blockDim.x) {
        const long long line = u / ncp;
        const int kp = (int)(u - line * ncp);
        const int I = (int)(line / C.ny), J = (int)(line - (long long)I * C.ny);
        const int k0 = 4 * kp;
        const float4 czm = __ldg(reinterpret_cast<const float4 *>(F.cm[2] + k0));
        const float4 czp = __ldg(reinterpret_cast<const float4 *>(F.cp[2] + k0));
        const float4 sz = __ldg(reinterpret_cast<const float4 *>(F.sum[2] + k0));
        const float4 wz = __ldg(reinterpret_cast<const float4 *>(F.w[2] + k0));
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b2 = 0; b2 < 2; ++b2) {
                const int i = 2 * I + a, j = 2 * J + b2;
                const long long t = ((long long)i * F.ny + j) * F.nz + k0;
                const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
                const float4 xc = *reinterpret_cast<const float4 *>(xf + t);
                const float4 xm = i > 0 ? *reinterpret_cast<const float4 *>(xf + t - sx) : zero;
                const float4 xp = i < F.nx - 1 ? *reinterpret_cast<const float4 *>(xf + t + sx) : zero;
                const float4 ym = j > 0 ? *reinterpret_cast<const float4 *>(xf + t - sy) : zero;
                const float4 yp = j < F.ny - 1 ? *reinterpret_cast<const float4 *>(xf + t + sy) : zero;
                const float zlo = k0 > 0 ? xf[t - 1] : (PZ ? xf[t + (F.nz - 1)] : 0.f);
                const float zhi = k0 + 4 < F.nz ? xf[t + 4] : (PZ ? xf[t + 4 - F.nz] : 0.f);
                const float4 bv = *reinterpret_cast<const float4 *>(bf + t);
                const bool odd = ((i + j) & 1) != 0;  // the colour-0 cells: k0 + odd, k0 + odd + 2
                auto pick = [odd](float a0, float a1) { return odd ? a1 : a0; };
                const float cxm = __ldg(F.cm[0] + i), cxp = __ldg(F.cp[0] + i);
                const float cym = __ldg(F.cm[1] + j), cyp = __ldg(F.cp[1] + j);
                const float sxy = __fadd_rn(__ldg(F.sum[0] + i), __ldg(F.sum[1] + j));
                const float wxy = __fmul_rn(__ldg(F.w[0] + i), __ldg(F.w[1] + j));
                // mg_nb's terms in its order: x-, x+, y-, y+, z-, z+ (fmaf from 0)
                float nA = fmaf(cxm, pick(xm.x, xm.y), 0.f);
                nA = fmaf(cxp, pick(xp.x, xp.y), nA);
                nA = fmaf(cym, pick(ym.x, ym.y), nA);
                nA = fmaf(cyp, pick(yp.x, yp.y), nA);
                nA = fmaf(pick(czm.x, czm.y), pick(zlo, xc.x), nA);
                nA = fmaf(pick(czp.x, czp.y), pick(xc.y, xc.z), nA);
                float nB = fmaf(cxm, pick(xm.z, xm.w), 0.f);
                nB = fmaf(cxp, pick(xp.z, xp.w), nB);
                nB = fmaf(cym, pick(ym.z, ym.w), nB);
                nB = fmaf(cyp, pick(yp.z, yp.w), nB);
                nB = fmaf(pick(czm.z, czm.w), pick(xc.y, xc.z), nB);
                nB = fmaf(pick(czp.z, czp.w), pick(xc.w, zhi), nB);
                const float dA = __fmul_rn(wxy, pick(wz.x, wz.y)), dB = __fmul_rn(wxy, pick(wz.z, wz.w));
                const float rA = __fsub_rn(__fmul_rn(__fadd_rn(sxy, pick(sz.x, sz.y)), pick(xc.x, xc.y)), nA);
                const float rB = __fsub_rn(__fmul_rn(__fadd_rn(sxy, pick(sz.z, sz.w)), pick(xc.z, xc.w)), nB);
                s0 = __fadd_rn(s0, __fsub_rn(pick(bv.x, bv.y), __fmul_rn(dA, rA)));
                s1 = __fadd_rn(s1, __fsub_rn(pick(bv.z, bv.w), __fmul_rn(dB, rB)));
            }
        *reinterpret_cast<float2 *>(bc + ((long long)I * C.ny + J) * C.nz + 2 * kp) = make_float2(s0, s1);
    }
}

// The prolongation with one thread per fine quad: its four cells take the
// values of their two parents along k, one float4 read-add-write.
__global__ void __launch_bounds__(kBlock)
k_mg_prolong4(MgLevel F, MgLevel C, const float *__restrict__ xc, float *__restrict__ xf, const int *done)
{
    pdl_wait();
    pdl_allow();
    if (*done) return;
    const int n4 = F.nz >> 2;
    const long long nq = F.n >> 2;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nq;
         q += (long long)gridDim.x * blockDim.x) {
        const long long line = q / n4;
        const int k0 = 4 * (int)(q - line * n4);
        const int i = (int)(line / F.ny), j = (int)(line - (long long)i * F.ny);
        const float2 v = __ldg(reinterpret_cast<const float2 *>(xc + ((long long)(i >> 1) * C.ny + (j >> 1)) * C.nz +
                                                                (k0 >> 1)));
        float4 x = reinterpret_cast<float4 *>(xf)[q];
        x.x += v.x;
        x.y += v.x;
        x.z += v.y;
        x.w += v.y;
        reinterpret_cast<float4 *>(xf)[q] = x;
    }
}

// The two-row colour pass marching along x: a thread owns the quad pair
// (j0, j0 + 1; k0) on planes i0 .. i0 + ci - 1 and keeps planes i - 1, i and
// i + 1 of its two rows in registers, so a plane costs the loads of plane
// i + 2's rows (issued before the plane's update), b, the two y rows and the
// k neighbours, against ten quads and the k neighbours in k_mg_smooth4x2.  A
// colour pass reads only the other colour, which it does not change, so the
// window's values from before this thread's updates serve the next plane.
// quad_update's arithmetic: the pass equals k_mg_smooth4x2 bit for bit.
// Blocks: (quad pairs of a plane / kBlock, planes / ci); 32-bit indices.
template <bool PZ>
__global__ void __launch_bounds__(kBlock, 3) k_mg_smooth4m(MgLevel L, const float *__restrict__ b, float *x, int color,
                                                           int zero_init, int ci, const int *done)
{
    pdl_wait();
    pdl_allow();
    if (*done) return;
    const int n4 = L.nz >> 2, np = (L.ny >> 1) * n4;
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= np) return;
    const int jp = (int)L.fq.div((unsigned)w), k0 = 4 * (w - jp * n4), j0 = 2 * jp;
    const int i0 = blockIdx.y * ci, i1 = min(i0 + ci, L.nx);
    const int sx = L.ny * L.nz, sy = L.nz;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    auto ld = [&](int t) { return *reinterpret_cast<const float4 *>(x + t); };
    const int tb = (i0 * L.ny + j0) * L.nz + k0;  // row j0 of plane i0
    float4 m0 = zero, m1 = zero, c0 = zero, c1 = zero, p0 = zero, p1 = zero;
    if (!zero_init) {
        if (i0 > 0) {
            m0 = ld(tb - sx);
            m1 = ld(tb - sx + sy);
        }
        c0 = ld(tb);
        c1 = ld(tb + sy);
        if (i0 + 1 < L.nx) {
            p0 = ld(tb + sx);
            p1 = ld(tb + sx + sy);
        }
    }
    for (int i = i0; i < i1; ++i) {
        const int t0 = tb + (i - i0) * sx, t1 = t0 + sy;
        float4 n0 = zero, n1 = zero;
        if (!zero_init && i + 1 < i1 && i + 2 < L.nx) {
            n0 = ld(t0 + 2 * sx);
            n1 = ld(t1 + 2 * sx);
        }
        const float4 b0 = *reinterpret_cast<const float4 *>(b + t0), b1 = *reinterpret_cast<const float4 *>(b + t1);
        float4 ym = zero, yp = zero;
        float zl0 = 0.f, zh0 = 0.f, zl1 = 0.f, zh1 = 0.f;
        if (!zero_init) {
            if (j0 > 0) ym = ld(t0 - sy);
            if (j0 + 2 < L.ny) yp = ld(t1 + sy);
            if (k0 > 0) {
                zl0 = x[t0 - 1];
                zl1 = x[t1 - 1];
            } else if (PZ) {
                zl0 = x[t0 + (L.nz - 1)];
                zl1 = x[t1 + (L.nz - 1)];
            }
            if (k0 + 4 < L.nz) {
                zh0 = x[t0 + 4];
                zh1 = x[t1 + 4];
            } else if (PZ) {
                zh0 = x[t0 + 4 - L.nz];
                zh1 = x[t1 + 4 - L.nz];
            }
        }
        float4 o0, o1;
        quad_update(L, (unsigned)i, (unsigned)j0, k0, b0, c0, m0, p0, ym, c1, zl0, zh0, color, o0);
        quad_update(L, (unsigned)i, (unsigned)(j0 + 1), k0, b1, c1, m1, p1, c0, yp, zl1, zh1, color, o1);
        *reinterpret_cast<float4 *>(x + t0) = o0;
        *reinterpret_cast<float4 *>(x + t1) = o1;
        m0 = c0;
        m1 = c1;
        c0 = p0;
        c1 = p1;
        p0 = n0;
        p1 = n1;
    }
}

// ---- tiled smoothing phases (grid-wide float4 levels) -----------------------
// One block owns an interior tile of tx x ty columns (all of k) and holds it
// with a halo of h = 2 s columns on each side (s sweeps) in shared memory, x
// and b as float4 quads.  All 2 s colour passes of the phase run inside the
// block over the tile: a pass needs the other colour at the four column
// neighbours, so a value stays exact only one column further in from the
// tile edge per pass, and after 2 s passes the interior holds what the
// grid-wide colour launches produce.  The arithmetic is quad_update's (that
// of k_mg_smooth4), and the transfers are those of k_mg_restrict4 and
// k_mg_prolong4, term for term, so the level ends bit for bit as with the
// separate launches.  Columns outside the level hold 0 and are never updated,
// which is how the grid-wide launches read them.
//   PRE: from x = 0 (the first colour-0 pass reads no neighbours), the
//   pre-smoothing, then the restriction of the interior's children into the
//   coarse b; the interior's x is stored.
//   POST: x of the tile plus the coarse correction (the prolongation), the
//   post-smoothing (colour 1 first); the interior's x is stored to a second
//   buffer (xout = L.xalt), since other blocks still read the halo columns
//   of this one from L.x; the prolongation into the finer level reads it.
// One launch replaces the 2 s + 1 launches of the phase, each of which waits
// for the whole level; the price is the halo recomputation.  A phase can also
// run one sweep a launch (two passes, halo 2, or 3 where the restriction
// follows), halving the halo's share on larger levels:
//   ZERO: from x = 0, no transfer;  READ_R: from xin, then the restriction;
//   READ: from xin (post-smoothing colours).
enum { kTilePre = 0, kTilePost = 1, kTileZero = 2, kTileReadR = 3, kTileRead = 4 };
constexpr int kTileThreads = 512;
constexpr long long kTileCells = 1 << 17;  // levels up to this size run their phases as tiles
constexpr long long kTileSplitCells = 1 << 20;  // CFDGPU_MG_TILE_SPLIT=1: larger ones up to this, one sweep a launch
constexpr long long kFdCells = 4096;       // the separable solve takes the first level at most this size
constexpr size_t kFdSmemMax = 160 * 1024;  // ... whose shared-memory layout fits this
constexpr int kTileSmemMax = 160 * 1024;  // shared memory of a tile block at most

// x and b of the tile, then its k tables (cm, cp, 1 / w, sum, w as float4
// quads) and its column tables (the same five along x, then along y)
__host__ inline size_t tile_smem(const MgTile &T)
{
    return (2ull * T.wx * T.wy * T.n4 + 5ull * T.n4) * sizeof(float4) + 5ull * (T.wx + T.wy) * sizeof(float);
}

template <bool PZ, int MODE>
__global__ void __launch_bounds__(kTileThreads, 2)
k_mg_tile(MgLevel L, MgLevel C, MgTile T, const float *xin, float *__restrict__ xout, const int *done)
{
    constexpr bool ZERO_START = MODE == kTilePre || MODE == kTileZero;
    constexpr bool RESTRICT = MODE == kTilePre || MODE == kTileReadR;
    constexpr bool PRE = MODE == kTilePre || MODE == kTileZero || MODE == kTileReadR;  // colours 0, 1, ...
    pdl_wait();
    pdl_allow();
    if (*done) return;
    extern __shared__ float4 tile_sm4[];
    const int nq = T.wx * T.wy * T.n4;
    float4 *xs = tile_sm4, *bs = tile_sm4 + nq;
    const int ti = blockIdx.x / T.tiles_y, tj = blockIdx.x - ti * T.tiles_y;
    const int i0 = ti * T.tx - T.h, j0 = tj * T.ty - T.h;  // global column of tile column 0
    const int sq = T.wy * T.n4;                             // quad stride of a tile column along x
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    // the tables of the tile (0 outside the level, where nothing is updated)
    float4 *tz = bs + nq;                                  // czm, czp, rz, sz, wz: n4 quads each
    float *tx = reinterpret_cast<float *>(tz + 5 * T.n4);  // cm, cp, rw, sum, w: wx columns each
    float *ty = tx + 5 * T.wx;                             // the same along y: wy each
    for (int u = threadIdx.x; u < 5 * T.n4; u += blockDim.x) {
        const int f = u / T.n4, kq = u - f * T.n4;
        const float *src = f == 0 ? L.cm[2] : f == 1 ? L.cp[2] : f == 2 ? L.rw[2] : f == 3 ? L.sum[2] : L.w[2];
        tz[u] = __ldg(reinterpret_cast<const float4 *>(src) + kq);
    }
    for (int u = threadIdx.x; u < 5 * (T.wx + T.wy); u += blockDim.x) {
        const bool ax = u < 5 * T.wx;
        const int v = ax ? u : u - 5 * T.wx, w = ax ? T.wx : T.wy;
        const int f = v / w, c = v - f * w, g = (ax ? i0 : j0) + c, a = ax ? 0 : 1;
        const float *src = f == 0 ? L.cm[a] : f == 1 ? L.cp[a] : f == 2 ? L.rw[a] : f == 3 ? L.sum[a] : L.w[a];
        const bool in = g >= 0 && g < (ax ? L.nx : L.ny);
        (ax ? tx : ty)[v] = in ? __ldg(src + g) : 0.f;
    }
    auto tab = [&](int a, int bb, int kq) {
        QuadTab Q;
        Q.cxm = tx[a];
        Q.cxp = tx[T.wx + a];
        Q.rwx = tx[2 * T.wx + a];
        Q.sx = tx[3 * T.wx + a];
        Q.cym = ty[bb];
        Q.cyp = ty[T.wy + bb];
        Q.rwy = ty[2 * T.wy + bb];
        Q.sy = ty[3 * T.wy + bb];
        Q.czm = tz[kq];
        Q.czp = tz[T.n4 + kq];
        Q.rz = tz[2 * T.n4 + kq];
        Q.sz = tz[3 * T.n4 + kq];
        return Q;
    };
    // tile quad q -> tile column (a, bb), quad kq along k
    auto split = [&](int q, int &a, int &bb, int &kq) {
        const unsigned c = T.fn4.div((unsigned)q);
        kq = q - (int)c * T.n4;
        a = (int)T.fwy.div(c);
        bb = (int)c - a * T.wy;
    };
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
        int a, bb, kq;
        split(q, a, bb, kq);
        const int i = i0 + a, j = j0 + bb;
        float4 xv = zero, bv = zero;
        if (i >= 0 && i < L.nx && j >= 0 && j < L.ny) {
            const long long t = ((long long)i * L.ny + j) * L.nz + 4 * kq;
            bv = __ldg(reinterpret_cast<const float4 *>(L.b + t));
            if (!ZERO_START) xv = *reinterpret_cast<const float4 *>(xin + t);
            if (MODE == kTilePost) {
                const float2 v = __ldg(reinterpret_cast<const float2 *>(
                    C.x + ((long long)(i >> 1) * C.ny + (j >> 1)) * C.nz + 2 * kq));
                xv.x += v.x;
                xv.y += v.x;
                xv.z += v.y;
                xv.w += v.y;
            }
        }
        xs[q] = xv;
        bs[q] = bv;
    }
    __syncthreads();
    const int passes = 2 * T.sweeps;
    for (int p = 0; p < passes; ++p) {
        // pre-smoothing colours 0, 1, 0, 1 ..., post-smoothing 1, 0, 1, 0 ...
        // From zero, pass p updates the columns at least p from the tile edge
        // (pass 0 reads no neighbour), so after 2 s passes columns from
        // 2 s - 1 = h - 1 in are exact, as the restriction of the interior
        // needs.  From x, pass p updates the columns at least p + 1 from the
        // edge (the restriction then needs h = 2 s + 1).  Every updated column
        // has its four neighbours inside the tile.
        const int color = PRE ? (p & 1) : 1 - (p & 1);
        const int dmin = ZERO_START ? p : p + 1;
        const bool zero_pass = ZERO_START && p == 0;
        for (int q = threadIdx.x; q < nq; q += blockDim.x) {
            int a, bb, kq;
            split(q, a, bb, kq);
            const int d = min(min(a, T.wx - 1 - a), min(bb, T.wy - 1 - bb));
            const int i = i0 + a, j = j0 + bb;
            if (d < dmin || i < 0 || i >= L.nx || j < 0 || j >= L.ny) continue;
            float4 out;
            const QuadTab Q = tab(a, bb, kq);
            if (zero_pass) {
                quad_update_t(Q, (unsigned)i, (unsigned)j, bs[q], zero, zero, zero, zero, zero, 0.f, 0.f, color, out);
            } else {
                const float zlo = kq > 0 ? xs[q - 1].w : (PZ ? xs[q + T.n4 - 1].w : 0.f);
                const float zhi = kq < T.n4 - 1 ? xs[q + 1].x : (PZ ? xs[q - (T.n4 - 1)].x : 0.f);
                quad_update_t(Q, (unsigned)i, (unsigned)j, bs[q], xs[q], xs[q - sq], xs[q + sq], xs[q - T.n4],
                              xs[q + T.n4], zlo, zhi, color, out);
            }
            xs[q] = out;
        }
        __syncthreads();
    }
    if (RESTRICT) {
        // k_mg_restrict4 over the interior's coarse cells: one thread per
        // pair of coarse cells along k (the children's quad kq of the four
        // fine columns)
        const int cx = T.tx >> 1, cy = T.ty >> 1, nr = cx * cy * T.n4;
        for (int u = threadIdx.x; u < nr; u += blockDim.x) {
            const int col = u / T.n4, kq = u - col * T.n4;
            const int ca = col / cy, cb = col - ca * cy;
            const int I = (ti * T.tx >> 1) + ca, J = (tj * T.ty >> 1) + cb;
            if (I >= C.nx || J >= C.ny) continue;
            const float4 czm = tz[kq], czp = tz[T.n4 + kq], sz = tz[3 * T.n4 + kq], wz = tz[4 * T.n4 + kq];
            float s0 = 0.f, s1 = 0.f;
#pragma unroll
            for (int a2 = 0; a2 < 2; ++a2)
#pragma unroll
                for (int b2 = 0; b2 < 2; ++b2) {
                    const int i = 2 * I + a2, j = 2 * J + b2;
                    const int q = ((i - i0) * T.wy + (j - j0)) * T.n4 + kq;
                    const float4 xc = xs[q];
                    const float4 xm = xs[q - sq], xp = xs[q + sq], ym = xs[q - T.n4], yp = xs[q + T.n4];
                    const float zlo = kq > 0 ? xs[q - 1].w : (PZ ? xs[q + T.n4 - 1].w : 0.f);
                    const float zhi = kq < T.n4 - 1 ? xs[q + 1].x : (PZ ? xs[q - (T.n4 - 1)].x : 0.f);
                    const float4 bv = bs[q];
                    const bool odd = ((i + j) & 1) != 0;
                    auto pick = [odd](float v0, float v1) { return odd ? v1 : v0; };
                    const int a = i - i0, bb = j - j0;
                    const float cxm = tx[a], cxp = tx[T.wx + a];
                    const float cym = ty[bb], cyp = ty[T.wy + bb];
                    const float sxy = __fadd_rn(tx[3 * T.wx + a], ty[3 * T.wy + bb]);
                    const float wxy = __fmul_rn(tx[4 * T.wx + a], ty[4 * T.wy + bb]);
                    float nA = fmaf(cxm, pick(xm.x, xm.y), 0.f);
                    nA = fmaf(cxp, pick(xp.x, xp.y), nA);
                    nA = fmaf(cym, pick(ym.x, ym.y), nA);
                    nA = fmaf(cyp, pick(yp.x, yp.y), nA);
                    nA = fmaf(pick(czm.x, czm.y), pick(zlo, xc.x), nA);
                    nA = fmaf(pick(czp.x, czp.y), pick(xc.y, xc.z), nA);
                    float nB = fmaf(cxm, pick(xm.z, xm.w), 0.f);
                    nB = fmaf(cxp, pick(xp.z, xp.w), nB);
                    nB = fmaf(cym, pick(ym.z, ym.w), nB);
                    nB = fmaf(cyp, pick(yp.z, yp.w), nB);
                    nB = fmaf(pick(czm.z, czm.w), pick(xc.y, xc.z), nB);
                    nB = fmaf(pick(czp.z, czp.w), pick(xc.w, zhi), nB);
                    const float dA = __fmul_rn(wxy, pick(wz.x, wz.y)), dB = __fmul_rn(wxy, pick(wz.z, wz.w));
                    const float rA = __fsub_rn(__fmul_rn(__fadd_rn(sxy, pick(sz.x, sz.y)), pick(xc.x, xc.y)), nA);
                    const float rB = __fsub_rn(__fmul_rn(__fadd_rn(sxy, pick(sz.z, sz.w)), pick(xc.z, xc.w)), nB);
                    s0 = __fadd_rn(s0, __fsub_rn(pick(bv.x, bv.y), __fmul_rn(dA, rA)));
                    s1 = __fadd_rn(s1, __fsub_rn(pick(bv.z, bv.w), __fmul_rn(dB, rB)));
                }
            *reinterpret_cast<float2 *>(C.b + ((long long)I * C.ny + J) * C.nz + 2 * kq) = make_float2(s0, s1);
        }
    }
    // the interior's x
    const int nin = T.tx * T.ty * T.n4;
    for (int u = threadIdx.x; u < nin; u += blockDim.x) {
        const int col = u / T.n4, kq = u - col * T.n4;
        const int a = col / T.ty, bb = col - a * T.ty;
        const int i = ti * T.tx + a, j = tj * T.ty + bb;
        if (i >= L.nx || j >= L.ny) continue;
        const int q = ((a + T.h) * T.wy + (bb + T.h)) * T.n4 + kq;
        *reinterpret_cast<float4 *>(xout + ((long long)i * L.ny + j) * L.nz + 4 * kq) = xs[q];
    }
}

// ---- exact separable solve of the coarsest level ---------------------------
// The level operator is a sum of Kronecker products, M = Kx (x) Wy (x) Wz +
// Wx (x) Ky (x) Wz + Wx (x) Wy (x) Kz, with W_a = diag(cell widths) and K_a
// the symmetric tridiagonal (cyclic for periodic z) face-coefficient
// operator of axis a.  With K_a v = lambda W_a v solved per axis (V_a^T W_a
// V_a = I), M = W V L V^T W for V = Vx (x) Vy (x) Vz and L the sums
// lambda_x + lambda_y + lambda_z, so M^+ = V L^+ V^T: three mode products
// with the transposed eigenvector matrices, a division by the eigenvalue
// sums (the all-constant mode, M's null space, dropped), three mode products
// back (fast diagonalisation; Lynch, Rice and Thomas, 1964).  A fixed
// symmetric positive semi-definite map, so the V-cycle stays one.
struct FdDesc {
    int n[3];             // nx, ny, nz
    const float *v[3];    // eigenvectors, row-major n x n (row i, column = mode)
    const float *lam[3];  // eigenvalues
    int null_mode;        // drop the mode (0, 0, 0)
};

// One block solves the level in shared memory (the level's cells, two
// copies, and the three eigenvector matrices with the eigenvalues), six
// mode products separated by block barriers.  fd_mode forms out[.., p, ..] =
// sum_q A[p][q] in[.., q, ..] along AX with A = V^T (TR) or V; SCALE divides
// by the eigenvalue sums (the forward pass's last product, AX = 0, when
// every axis is in mode space).
constexpr int kFdThreads = 1024;

template <int AX, bool TR, bool SCALE>
__device__ __forceinline__ void fd_mode(const FdDesc &D, const float *V, const float *const *lam, const float *in,
                                        float *out, bool null_mode)
{
    const int nx = D.n[0], ny = D.n[1], nz = D.n[2], na = D.n[AX];
    const int n = nx * ny * nz, stride = AX == 0 ? ny * nz : AX == 1 ? nz : 1;
    for (int o = threadIdx.x; o < n; o += blockDim.x) {
        const int k = o % nz, j = (o / nz) % ny, i = o / (ny * nz);
        const int p = AX == 0 ? i : AX == 1 ? j : k;
        const float *col = in + (o - p * stride);
        float acc = 0.f;
        for (int q = 0; q < na; ++q) acc = fmaf(TR ? V[q * na + p] : V[p * na + q], col[q * stride], acc);
        if (SCALE) acc = (null_mode && o == 0) ? 0.f : acc / (lam[0][i] + lam[1][j] + lam[2][k]);
        out[o] = acc;
    }
}

__global__ void __launch_bounds__(kFdThreads) k_fd_block(FdDesc D, const float *__restrict__ b, float *__restrict__ x,
                                                         const int *done)
{
    pdl_wait();
    pdl_allow();
    if (*done) return;
    extern __shared__ float fd_sm[];
    const int nx = D.n[0], ny = D.n[1], nz = D.n[2], n = nx * ny * nz;
    float *s0 = fd_sm, *s1 = s0 + n, *v[3], *lam[3];
    v[0] = s1 + n;
    v[1] = v[0] + nx * nx;
    v[2] = v[1] + ny * ny;
    lam[0] = v[2] + nz * nz;
    lam[1] = lam[0] + nx;
    lam[2] = lam[1] + ny;
    for (int a = 0; a < 3; ++a) {
        const int na = D.n[a];
        for (int q = threadIdx.x; q < na * na; q += blockDim.x) v[a][q] = __ldg(D.v[a] + q);
        for (int q = threadIdx.x; q < na; q += blockDim.x) lam[a][q] = __ldg(D.lam[a] + q);
    }
    for (int q = threadIdx.x; q < n; q += blockDim.x) s0[q] = b[q];
    __syncthreads();
    const bool nm = D.null_mode != 0;
    fd_mode<2, true, false>(D, v[2], lam, s0, s1, nm);
    __syncthreads();
    fd_mode<1, true, false>(D, v[1], lam, s1, s0, nm);
    __syncthreads();
    fd_mode<0, true, true>(D, v[0], lam, s0, s1, nm);
    __syncthreads();
    fd_mode<0, false, false>(D, v[0], lam, s1, s0, nm);
    __syncthreads();
    fd_mode<1, false, false>(D, v[1], lam, s0, s1, nm);
    __syncthreads();
    fd_mode<2, false, false>(D, v[2], lam, s1, x, nm);
}

// its shared memory: two copies of the level, the eigenvector matrices and
// the eigenvalues
__host__ inline size_t fd_smem(int nx, int ny, int nz)
{
    return sizeof(float) * (2ull * nx * ny * nz + (size_t)nx * nx + (size_t)ny * ny + (size_t)nz * nz + nx + ny + nz);
}

// ---- fused red-black sweep (grid-wide levels, nz % 4 == 0) ------------------
// One symmetric-order sweep in one pass: xn = colour c1 applied after colour
// c0 to xo (c1 = 1 - c0), written to a second buffer so that no block reads a
// value another block has already replaced.  A block owns TJ rows of j (all
// of k) over a chunk of CI planes of i and marches along i: colour c0 at
// plane q over its rows and one halo row each side (from xo), then colour c1
// at plane q - 1 over its own rows (from the c0 values of planes q - 2 .. q).
// xo planes arrive two planes ahead and b planes one plane ahead through
// cp.async rings; c0 values live in a ring of three planes.  The arithmetic
// is that of smooth_quads term for term, so the result equals the two
// colour launches bit for bit.  zero_init: xo is 0 (not read).
constexpr int kSweepRing = 4;

__device__ __forceinline__ int mod_ring(int p, int m) { return ((p % m) + m) % m; }

__device__ __forceinline__ void cp16(unsigned dst, const void *src, bool valid)
{
    // 16-byte asynchronous copy; an invalid source fills zeros and reads nothing
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0)
                 : "memory");
}

__global__ void __launch_bounds__(1024)
k_mg_sweep(MgLevel L, const float *__restrict__ b, const float *__restrict__ xo, float *__restrict__ xn, int c0,
           int zero_init, const int *done)
{
    pdl_wait();
    pdl_allow();
    if (*done) return;
    extern __shared__ float4 sweep_sm4[];
    float *sm = reinterpret_cast<float *>(sweep_sm4);
    const int nx = L.nx, ny = L.ny, nz = L.nz, n4 = nz >> 2, TJ = L.sweep_tj, CI = L.sweep_ci;
    const int XR = TJ + 4, RR = TJ + 2;  // rows of an x plane (j0-2 .. j0+TJ+1) and of a b / c0 plane (j0-1 .. j0+TJ)
    float *xs = sm;                                  // [kSweepRing][XR * nz]
    float *bs = xs + kSweepRing * XR * nz;           // [kSweepRing][RR * nz]
    float *rs = bs + kSweepRing * RR * nz;           // [3][RR * nz]
    const int tiles_j = (ny + TJ - 1) / TJ;
    const int j0 = (blockIdx.x % tiles_j) * TJ, ib = (blockIdx.x / tiles_j) * CI, ie = min(nx, ib + CI);
    const int t = threadIdx.x, nt = blockDim.x;
    const long long sx = (long long)ny * nz;

    auto issue_x = [&](int p) {
        const unsigned base = (unsigned)__cvta_generic_to_shared(xs + mod_ring(p, kSweepRing) * XR * nz);
        for (int u = t; u < XR * n4; u += nt) {
            const int row = u / n4, m = u - row * n4, j = j0 - 2 + row;
            const bool ok = p >= 0 && p < nx && j >= 0 && j < ny;
            cp16(base + 16u * (unsigned)(row * n4 + m), ok ? (const void *)(xo + p * sx + (long long)j * nz + 4 * m) : xo, ok);
        }
    };
    auto issue_b = [&](int p) {
        const unsigned base = (unsigned)__cvta_generic_to_shared(bs + mod_ring(p, kSweepRing) * RR * nz);
        for (int u = t; u < RR * n4; u += nt) {
            const int row = u / n4, m = u - row * n4, j = j0 - 1 + row;
            const bool ok = p >= 0 && p < nx && j >= 0 && j < ny;
            cp16(base + 16u * (unsigned)(row * n4 + m), ok ? (const void *)(b + p * sx + (long long)j * nz + 4 * m) : b, ok);
        }
    };
    if (zero_init)
        for (int u = t; u < kSweepRing * XR * n4; u += nt) reinterpret_cast<float4 *>(xs)[u] = make_float4(0.f, 0.f, 0.f, 0.f);
    else {
        issue_x(ib - 2);
        issue_x(ib - 1);
        issue_x(ib);
    }
    issue_b(ib - 1);
    asm volatile("cp.async.commit_group;\n" ::: "memory");

    for (int q = ib - 1; q <= ie; ++q) {
        if (!zero_init) issue_x(q + 2);
        issue_b(q + 1);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        __syncthreads();
        // colour c0 at plane q, rows j0-1 .. j0+TJ
        {
            const float *xm = xs + mod_ring(q - 1, kSweepRing) * XR * nz;
            const float *xc = xs + mod_ring(q, kSweepRing) * XR * nz;
            const float *xp = xs + mod_ring(q + 1, kSweepRing) * XR * nz;
            const float *bq = bs + mod_ring(q, kSweepRing) * RR * nz;
            float *dst = rs + mod_ring(q, 3) * RR * nz;
            const bool qv = q >= 0 && q < nx;
            float cxm = 0.f, cxp = 0.f, rwx = 0.f, sux = 0.f;
            if (qv) {
                cxm = __ldg(L.cm[0] + q); cxp = __ldg(L.cp[0] + q);
                rwx = __ldg(L.rw[0] + q); sux = __ldg(L.sum[0] + q);
            }
            for (int u = t; u < RR * n4; u += nt) {
                const int rr = u / n4, m = u - rr * n4, j = j0 - 1 + rr, k0 = 4 * m;
                float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
                if (qv && j >= 0 && j < ny) {
                    const int xr = rr + 1;
                    const float4 c = *reinterpret_cast<const float4 *>(xc + xr * nz + k0);
                    const float4 vxm = *reinterpret_cast<const float4 *>(xm + xr * nz + k0);
                    const float4 vxp = *reinterpret_cast<const float4 *>(xp + xr * nz + k0);
                    const float4 vym = *reinterpret_cast<const float4 *>(xc + (xr - 1) * nz + k0);
                    const float4 vyp = *reinterpret_cast<const float4 *>(xc + (xr + 1) * nz + k0);
                    const float zlo = k0 > 0 ? xc[xr * nz + k0 - 1] : 0.f;
                    const float zhi = k0 + 4 < nz ? xc[xr * nz + k0 + 4] : 0.f;
                    const float4 bv = *reinterpret_cast<const float4 *>(bq + rr * nz + k0);
                    const float cym = __ldg(L.cm[1] + j), cyp = __ldg(L.cp[1] + j);
                    const float rxy = rwx * __ldg(L.rw[1] + j), sxy = sux + __ldg(L.sum[1] + j);
                    const float4 czm = __ldg(reinterpret_cast<const float4 *>(L.cm[2] + k0));
                    const float4 czp = __ldg(reinterpret_cast<const float4 *>(L.cp[2] + k0));
                    const float4 rz = __ldg(reinterpret_cast<const float4 *>(L.rw[2] + k0));
                    const float4 sz = __ldg(reinterpret_cast<const float4 *>(L.sum[2] + k0));
                    const int e0 = (c0 + q + j) & 1;
                    const bool odd = e0 != 0;
                    auto pick = [odd](float a0, float a1) { return odd ? a1 : a0; };
                    float nA = cxm * pick(vxm.x, vxm.y);
                    nA = fmaf(cxp, pick(vxp.x, vxp.y), nA);
                    nA = fmaf(cym, pick(vym.x, vym.y), nA);
                    nA = fmaf(cyp, pick(vyp.x, vyp.y), nA);
                    nA = fmaf(pick(czm.x, czm.y), pick(zlo, c.x), nA);
                    nA = fmaf(pick(czp.x, czp.y), pick(c.y, c.z), nA);
                    float nB = cxm * pick(vxm.z, vxm.w);
                    nB = fmaf(cxp, pick(vxp.z, vxp.w), nB);
                    nB = fmaf(cym, pick(vym.z, vym.w), nB);
                    nB = fmaf(cyp, pick(vyp.z, vyp.w), nB);
                    nB = fmaf(pick(czm.z, czm.w), pick(c.y, c.z), nB);
                    nB = fmaf(pick(czp.z, czp.w), pick(c.w, zhi), nB);
                    if (zero_init) nA = nB = 0.f;
                    const float vA = fmaf(pick(bv.x, bv.y), rxy * pick(rz.x, rz.y), nA) * smooth_rcp(sxy + pick(sz.x, sz.y));
                    const float vB = fmaf(pick(bv.z, bv.w), rxy * pick(rz.z, rz.w), nB) * smooth_rcp(sxy + pick(sz.z, sz.w));
                    out = make_float4(odd ? 0.f : vA, odd ? vA : 0.f, odd ? 0.f : vB, odd ? vB : 0.f);
                }
                *reinterpret_cast<float4 *>(dst + rr * nz + k0) = out;
            }
        }
        __syncthreads();
        // colour c1 at plane q - 1, rows j0 .. j0+TJ-1, from the c0 values
        const int qo = q - 1;
        if (qo >= ib) {
            const float *rm = rs + mod_ring(qo - 1, 3) * RR * nz;
            const float *rc = rs + mod_ring(qo, 3) * RR * nz;
            const float *rp = rs + mod_ring(qo + 1, 3) * RR * nz;
            const float *bq = bs + mod_ring(qo, kSweepRing) * RR * nz;
            const float cxm = __ldg(L.cm[0] + qo), cxp = __ldg(L.cp[0] + qo);
            const float rwx = __ldg(L.rw[0] + qo), sux = __ldg(L.sum[0] + qo);
            for (int u = t; u < TJ * n4; u += nt) {
                const int r = u / n4, m = u - r * n4, j = j0 + r, k0 = 4 * m;
                if (j >= ny) continue;
                const int cr = r + 1;
                const float4 c = *reinterpret_cast<const float4 *>(rc + cr * nz + k0);
                const float4 vxm = *reinterpret_cast<const float4 *>(rm + cr * nz + k0);
                const float4 vxp = *reinterpret_cast<const float4 *>(rp + cr * nz + k0);
                const float4 vym = *reinterpret_cast<const float4 *>(rc + (cr - 1) * nz + k0);
                const float4 vyp = *reinterpret_cast<const float4 *>(rc + (cr + 1) * nz + k0);
                const float zlo = k0 > 0 ? rc[cr * nz + k0 - 1] : 0.f;
                const float zhi = k0 + 4 < nz ? rc[cr * nz + k0 + 4] : 0.f;
                const float4 bv = *reinterpret_cast<const float4 *>(bq + cr * nz + k0);
                const float cym = __ldg(L.cm[1] + j), cyp = __ldg(L.cp[1] + j);
                const float rxy = rwx * __ldg(L.rw[1] + j), sxy = sux + __ldg(L.sum[1] + j);
                const float4 czm = __ldg(reinterpret_cast<const float4 *>(L.cm[2] + k0));
                const float4 czp = __ldg(reinterpret_cast<const float4 *>(L.cp[2] + k0));
                const float4 rz = __ldg(reinterpret_cast<const float4 *>(L.rw[2] + k0));
                const float4 sz = __ldg(reinterpret_cast<const float4 *>(L.sum[2] + k0));
                const int e0 = (1 - c0 + qo + j) & 1;  // first c1 cell of the quad
                const bool odd = e0 != 0;
                auto pick = [odd](float a0, float a1) { return odd ? a1 : a0; };
                float nA = cxm * pick(vxm.x, vxm.y);
                nA = fmaf(cxp, pick(vxp.x, vxp.y), nA);
                nA = fmaf(cym, pick(vym.x, vym.y), nA);
                nA = fmaf(cyp, pick(vyp.x, vyp.y), nA);
                nA = fmaf(pick(czm.x, czm.y), pick(zlo, c.x), nA);
                nA = fmaf(pick(czp.x, czp.y), pick(c.y, c.z), nA);
                float nB = cxm * pick(vxm.z, vxm.w);
                nB = fmaf(cxp, pick(vxp.z, vxp.w), nB);
                nB = fmaf(cym, pick(vym.z, vym.w), nB);
                nB = fmaf(cyp, pick(vyp.z, vyp.w), nB);
                nB = fmaf(pick(czm.z, czm.w), pick(c.y, c.z), nB);
                nB = fmaf(pick(czp.z, czp.w), pick(c.w, zhi), nB);
                const float vA = fmaf(pick(bv.x, bv.y), rxy * pick(rz.x, rz.y), nA) * smooth_rcp(sxy + pick(sz.x, sz.y));
                const float vB = fmaf(pick(bv.z, bv.w), rxy * pick(rz.z, rz.w), nB) * smooth_rcp(sxy + pick(sz.z, sz.w));
                // c0 cells keep the values of the first half of the sweep
                const float4 o = make_float4(odd ? c.x : vA, odd ? vA : c.y, odd ? c.z : vB, odd ? vB : c.w);
                *reinterpret_cast<float4 *>(xn + qo * sx + (long long)j * nz + k0) = o;
            }
        }
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// a small level's x and b in shared memory, each rounded up to 4 floats so
// the float4 smoother's rows stay 16-byte aligned
__host__ __device__ inline long long small_pad(long long n) { return (n + 3) & ~3LL; }

static_assert(kSmallThreads == 4 * kMgCoarsest, "coarsest product: 4 threads per row");

// level l of the small sub-cycle as seen in shared memory: x, b, the
// per-cell and the axis tables redirected to their staged copies
__device__ __forceinline__ MgLevel small_view(const MgSmall &S, float *sm, int l)
{
    MgLevel L = S.lev[l];
    float *p = sm + S.tab_off[l];
    const int dims[3] = {L.nx, L.ny, L.nz};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int m = (int)small_pad(dims[a]);
        L.cm[a] = p;
        L.cp[a] = p + m;
        L.sum[a] = p + 2 * m;
        L.w[a] = p + 3 * m;
        L.rw[a] = p + 4 * m;
        p += 5 * m;
    }
    L.rv = sm + S.rv_off[l];
    L.rg = L.rv + small_pad(L.n);
    L.x = sm + S.off[l];
    L.b = L.x + small_pad(L.n);
    return L;
}

// the whole sub-cycle of levels first..nlev-1 (nlev-1 the coarsest) in one
// block, in shared memory: copy in the static image (dense inverse, per-cell
// and axis tables; asynchronous 16-byte copies) and the first small level's
// b; pre-smooth and restrict down, solve the coarsest, prolong and
// post-smooth up; store the first small level's x.  Block barriers separate
// the phases.
template <bool PZ>
__global__ void __launch_bounds__(kSmallThreads) k_mg_small(MgSmall S)
{
    pdl_wait();
    pdl_allow();
    if (*S.done) return;
    extern __shared__ float4 small_sm4[];
    float *sm = reinterpret_cast<float *>(small_sm4);
    __shared__ float red[kSmallThreads / 32];
    __shared__ float part[4][kMgCoarsest];
    const int t0 = threadIdx.x, st = blockDim.x;
    const int first = S.first, last = S.nlev;
    const int nc = (int)S.lev[last - 1].n;
    {
        const unsigned base = (unsigned)__cvta_generic_to_shared(sm);
        for (int q = t0; q < (S.image_floats >> 2); q += st)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(base + 16u * q), "l"(S.image + 4 * q)
                         : "memory");
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        const MgLevel &G = S.lev[first];
        float *b = sm + S.off[first] + small_pad(G.n);
        for (int t = t0; t < (int)G.n; t += st) b[t] = G.b[t];
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        __syncthreads();
    }
    for (int l = first; l < last - 1; ++l) {
        const MgLevel L = small_view(S, sm, l);
        for (int s = 0; s < S.pre; ++s) {
            if (L.quads) smooth_quads<true, int, PZ>(L, L.b, L.x, 0, s == 0, t0, st);
            else smooth_level<true, PZ>(L, L.b, L.x, 0, s == 0, t0, st);
            __syncthreads();
            if (L.quads) smooth_quads<true, int, PZ>(L, L.b, L.x, 1, false, t0, st);
            else smooth_level<true, PZ>(L, L.b, L.x, 1, false, t0, st);
            __syncthreads();
        }
        const MgLevel C = small_view(S, sm, l + 1);
        restrict_level<true, PZ>(L, C, L.b, L.x, C.b, t0, st);
        __syncthreads();
    }
    {
        // coarsest: x = C (b - mean b), C = (M + a 1 1^T)^-1 symmetric, so
        // thread r sums column r over a quarter of the rows
        const MgLevel L = small_view(S, sm, last - 1);
        float s = 0.f;
        for (int t = t0; t < nc; t += st) s += L.b[t];
        for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
        __syncthreads();
        float tot = 0.f;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) tot += red[q];
        const float mean = tot / (float)nc;
        const int r = threadIdx.x % kMgCoarsest, q4 = threadIdx.x / kMgCoarsest;
        float acc = 0.f;
        if (r < nc) {
            if (S.cinv_off >= 0) {
                const float *cs = sm + S.cinv_off;
                for (int cidx = q4; cidx < nc; cidx += 4) acc = fmaf(cs[cidx * nc + r], L.b[cidx] - mean, acc);
            } else {
                for (int cidx = q4; cidx < nc; cidx += 4)
                    acc = fmaf(__ldg(S.cinv + (long long)cidx * nc + r), L.b[cidx] - mean, acc);
            }
        }
        part[q4][r] = acc;
        __syncthreads();
        if (threadIdx.x < nc)
            L.x[threadIdx.x] = (part[0][threadIdx.x] + part[1][threadIdx.x]) + (part[2][threadIdx.x] + part[3][threadIdx.x]);
        __syncthreads();
    }
    for (int l = last - 2; l >= first; --l) {
        const MgLevel L = small_view(S, sm, l);
        prolong_level<true>(L, S.lev[l + 1], small_view(S, sm, l + 1).x, L.x, t0, st);
        __syncthreads();
        for (int s = 0; s < S.post; ++s) {
            if (L.quads) smooth_quads<true, int, PZ>(L, L.b, L.x, 1, false, t0, st);
            else smooth_level<true, PZ>(L, L.b, L.x, 1, false, t0, st);
            __syncthreads();
            if (L.quads) smooth_quads<true, int, PZ>(L, L.b, L.x, 0, false, t0, st);
            else smooth_level<true, PZ>(L, L.b, L.x, 0, false, t0, st);
            __syncthreads();
        }
    }
    {
        const MgLevel &G = S.lev[first];
        const float *x = sm + S.off[first];
        for (int t = t0; t < (int)G.n; t += st) G.x[t] = x[t];
    }
}

// ---- the coarse levels in one thread-block cluster ---------------------------
namespace cgx = cooperative_groups;

// The slab of level L that CTA `rank` of the cluster owns: planes
// [rank P, (rank + 1) P) with P = nx / kClusterCtas, x then b in shared
// memory at `base`; x of a plane outside the slab is read from the CTA that
// owns it (distributed shared memory).
struct ClusterSlab {
    MgLevel L;
    int P, i0;
    float *x, *b;
    __device__ __forceinline__ long long loc(int i, int j, int k) const
    {
        return ((long long)(i - i0) * L.ny + j) * L.nz + k;
    }
    __device__ __forceinline__ float xat(cgx::cluster_group &cl, int i, int j, int k) const
    {
        if (i >= i0 && i < i0 + P) return x[loc(i, j, k)];
        const int r = i / P;
        const float *rx = cl.map_shared_rank(x, r);
        return rx[((long long)(i - r * P) * L.ny + j) * L.nz + k];
    }
};

__device__ __forceinline__ ClusterSlab cluster_slab(const MgCluster &S, float *sm, int l, int rank)
{
    ClusterSlab c;
    c.L = S.lev[l];
    c.P = c.L.nx / kClusterCtas;
    c.i0 = rank * c.P;
    c.x = sm + S.off[l];
    c.b = c.x + (long long)c.P * c.L.ny * c.L.nz;
    return c;
}

// mg_nb with the slab accessor (the same terms in the same order)
template <bool PZ>
__device__ __forceinline__ float cluster_nb(const ClusterSlab &c, cgx::cluster_group &cl, int i, int j, int k)
{
    const MgLevel &L = c.L;
    float s = 0.f;
    if (i > 0) s = fmaf(__ldg(L.cm[0] + i), c.xat(cl, i - 1, j, k), s);
    if (i < L.nx - 1) s = fmaf(__ldg(L.cp[0] + i), c.xat(cl, i + 1, j, k), s);
    if (j > 0) s = fmaf(__ldg(L.cm[1] + j), c.x[c.loc(i, j - 1, k)], s);
    if (j < L.ny - 1) s = fmaf(__ldg(L.cp[1] + j), c.x[c.loc(i, j + 1, k)], s);
    if (k > 0) s = fmaf(__ldg(L.cm[2] + k), c.x[c.loc(i, j, k - 1)], s);
    else if (PZ) s = fmaf(__ldg(L.cm[2] + k), c.x[c.loc(i, j, L.nz - 1)], s);
    if (k < L.nz - 1) s = fmaf(__ldg(L.cp[2] + k), c.x[c.loc(i, j, k + 1)], s);
    else if (PZ) s = fmaf(__ldg(L.cp[2] + k), c.x[c.loc(i, j, 0)], s);
    return s;
}

// x of the slab's neighbour plane i (i0 - 1 or i0 + P) as float4 rows
__device__ __forceinline__ const float *cluster_plane(const ClusterSlab &c, cgx::cluster_group &cl, int i)
{
    if (i >= c.i0 && i < c.i0 + c.P) return c.x + (long long)(i - c.i0) * c.L.ny * c.L.nz;
    const int r = i / c.P;
    return cl.map_shared_rank(c.x, r) + (long long)(i - r * c.P) * c.L.ny * c.L.nz;
}

// one colour over the slab; zero_init: from x = 0, the other colour written
// as 0.  Float4 levels: one thread a quad, quad_update's arithmetic (that of
// smooth_quads); others: gs_cell's arithmetic cell by cell.
template <bool PZ>
__device__ __forceinline__ void cluster_smooth(const ClusterSlab &c, cgx::cluster_group &cl, int color, bool zero_init)
{
    const MgLevel &L = c.L;
    const int ny = L.ny, nz = L.nz;
    if (L.quads) {
        const int n4 = nz >> 2;
        const int quads = c.P * ny * n4;
        const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int q = threadIdx.x; q < quads; q += blockDim.x) {
            const unsigned u = (unsigned)q;
            const unsigned li = L.fyq.div(u), r = u - li * (unsigned)(ny * n4), j = L.fq.div(r);
            const int k0 = 4 * (int)(r - j * (unsigned)n4);
            const int i = c.i0 + (int)li;
            const int t = ((int)li * ny + (int)j) * nz + k0;
            const float4 bv = *reinterpret_cast<const float4 *>(c.b + t);
            float4 xc = zero, xm = zero, xp = zero, ym = zero, yp = zero;
            float zlo = 0.f, zhi = 0.f;
            if (!zero_init) {
                xc = *reinterpret_cast<const float4 *>(c.x + t);
                const int rowoff = (int)j * nz + k0;
                if (i > 0) xm = *reinterpret_cast<const float4 *>(cluster_plane(c, cl, i - 1) + rowoff);
                if (i < L.nx - 1) xp = *reinterpret_cast<const float4 *>(cluster_plane(c, cl, i + 1) + rowoff);
                if (j > 0) ym = *reinterpret_cast<const float4 *>(c.x + t - nz);
                if ((int)j < ny - 1) yp = *reinterpret_cast<const float4 *>(c.x + t + nz);
                zlo = k0 > 0 ? c.x[t - 1] : (PZ ? c.x[t + nz - 1] : 0.f);
                zhi = k0 + 4 < nz ? c.x[t + 4] : (PZ ? c.x[t + 4 - nz] : 0.f);
            }
            float4 out;
            quad_update(L, (unsigned)i, j, k0, bv, xc, xm, xp, ym, yp, zlo, zhi, color, out);
            *reinterpret_cast<float4 *>(c.x + t) = out;
        }
        return;
    }
    const int cells = c.P * ny * nz;
    for (int t = threadIdx.x; t < cells; t += blockDim.x) {
        const unsigned u = (unsigned)t;
        const unsigned li = L.fyz.div(u), r = u - li * (unsigned)(ny * nz), jj = L.fz.div(r);
        const int j = (int)jj, k = (int)(r - jj * (unsigned)nz);
        const int i = c.i0 + (int)li;
        if (((i + j + k) & 1) != color) {
            if (zero_init) c.x[t] = 0.f;
            continue;
        }
        const float nb = zero_init ? 0.f : cluster_nb<PZ>(c, cl, i, j, k);
        const float rv = __ldg(L.rw[0] + i) * __ldg(L.rw[1] + j) * __ldg(L.rw[2] + k);
        const float dg = __ldg(L.sum[0] + i) + __ldg(L.sum[1] + j) + __ldg(L.sum[2] + k);
        c.x[t] = fmaf(c.b[t], rv, nb) * smooth_rcp(dg);
    }
}

// coarse b = sum over the colour-0 children of (b - M x) (restrict_level's
// arithmetic, one rounding per operation), coarse slab from the fine one
template <bool PZ>
__device__ __forceinline__ void cluster_restrict(const ClusterSlab &f, const ClusterSlab &c, cgx::cluster_group &cl)
{
    const MgLevel &F = f.L, &C = c.L;
    const int fx = F.nx / C.nx, fy = F.ny / C.ny, fz = F.nz / C.nz;
    const int cells = c.P * C.ny * C.nz;
    for (int T = threadIdx.x; T < cells; T += blockDim.x) {
        const unsigned u = (unsigned)T;
        const unsigned lI = C.fyz.div(u), r = u - lI * (unsigned)(C.ny * C.nz), JJ = C.fz.div(r);
        const int J = (int)JJ, K = (int)(r - JJ * (unsigned)C.nz);
        const int I = c.i0 + (int)lI;
        float s = 0.f;
        for (int a = 0; a < fx; ++a)
            for (int b2 = 0; b2 < fy; ++b2)
                for (int cc = 0; cc < fz; ++cc) {
                    const int i = fx * I + a, j = fy * J + b2, k = fz * K + cc;
                    if ((i + j + k) & 1) continue;
                    const long long t = f.loc(i, j, k);
                    const float dv = __fmul_rn(__fmul_rn(__ldg(F.w[0] + i), __ldg(F.w[1] + j)), __ldg(F.w[2] + k));
                    const float dg = __ldg(F.sum[0] + i) + __ldg(F.sum[1] + j) + __ldg(F.sum[2] + k);
                    const float res = __fsub_rn(__fmul_rn(dg, f.x[t]), cluster_nb<PZ>(f, cl, i, j, k));
                    s = __fadd_rn(s, __fsub_rn(f.b[t], __fmul_rn(dv, res)));
                }
        c.b[T] = s;
    }
}

// fine x += coarse x (the parent is in the same CTA: the slabs nest)
__device__ __forceinline__ void cluster_prolong(const ClusterSlab &f, const ClusterSlab &c)
{
    const MgLevel &F = f.L, &C = c.L;
    const int fx = F.nx / C.nx, fy = F.ny / C.ny, fz = F.nz / C.nz;
    const int cells = f.P * F.ny * F.nz;
    for (int t = threadIdx.x; t < cells; t += blockDim.x) {
        const unsigned u = (unsigned)t;
        const unsigned li = F.fyz.div(u), r = u - li * (unsigned)(F.ny * F.nz), jj = F.fz.div(r);
        const int j = (int)jj, k = (int)(r - jj * (unsigned)F.nz);
        const int i = f.i0 + (int)li;
        f.x[t] += c.x[c.loc(i / fx, j / fy, k / fz)];
    }
}

template <bool PZ>
__global__ void __cluster_dims__(kClusterCtas, 1, 1) __launch_bounds__(kClusterThreads, 1) k_mg_cluster(MgCluster S)
{
    pdl_wait();
    pdl_allow();
    if (*S.done) return;  // the same decision in every CTA of the cluster
    cgx::cluster_group cl = cgx::this_cluster();
    const int rank = (int)cl.block_rank();
    extern __shared__ float4 cluster_sm4[];
    float *sm = reinterpret_cast<float *>(cluster_sm4);
    const int first = S.first, last = S.nlev;
    {
        const ClusterSlab c = cluster_slab(S, sm, first, rank);
        const int cells = c.P * c.L.ny * c.L.nz;
        const float *gb = c.L.b + (long long)c.i0 * c.L.ny * c.L.nz;
        for (int t = threadIdx.x; t < cells; t += blockDim.x) c.b[t] = gb[t];
    }
    __syncthreads();
    for (int l = first; l < last - 1; ++l) {
        const ClusterSlab c = cluster_slab(S, sm, l, rank);
        for (int s = 0; s < S.pre; ++s) {
            cluster_smooth<PZ>(c, cl, 0, s == 0);
            cl.sync();
            cluster_smooth<PZ>(c, cl, 1, false);
            cl.sync();
        }
        cluster_restrict<PZ>(c, cluster_slab(S, sm, l + 1, rank), cl);
        cl.sync();
    }
    {
        // coarsest: x = C (b - mean b), C the regularised dense inverse; the
        // mean from the CTAs' partial sums in rank order
        const ClusterSlab c = cluster_slab(S, sm, last - 1, rank);
        const int cells = c.P * c.L.ny * c.L.nz;
        const int nc = (int)c.L.n;
        __shared__ float red[kClusterThreads / 32];
        float s = 0.f;
        for (int t = threadIdx.x; t < cells; t += blockDim.x) s += c.b[t];
        for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            float tot = 0.f;
            for (int q = 0; q < (int)(blockDim.x >> 5); ++q) tot += red[q];
            sm[S.part_off] = tot;
        }
        cl.sync();
        float tot = 0.f;
        for (int r = 0; r < kClusterCtas; ++r) tot += *cl.map_shared_rank(sm + S.part_off, r);
        const float mean = tot / (float)nc;
        const int row0 = c.i0 * c.L.ny * c.L.nz;
        for (int t = threadIdx.x; t < cells; t += blockDim.x) {
            const float *crow = S.cinv + (long long)(row0 + t) * nc;
            float acc = 0.f;
            for (int r = 0; r < kClusterCtas; ++r) {
                const float *rb = cl.map_shared_rank(c.b, r);
                for (int q = 0; q < cells; ++q) acc = fmaf(__ldg(crow + r * cells + q), rb[q] - mean, acc);
            }
            c.x[t] = acc;
        }
        cl.sync();
    }
    for (int l = last - 2; l >= first; --l) {
        const ClusterSlab c = cluster_slab(S, sm, l, rank);
        cluster_prolong(c, cluster_slab(S, sm, l + 1, rank));
        cl.sync();
        for (int s = 0; s < S.post; ++s) {
            cluster_smooth<PZ>(c, cl, 1, false);
            cl.sync();
            cluster_smooth<PZ>(c, cl, 0, false);
            cl.sync();
        }
    }
    {
        const ClusterSlab c = cluster_slab(S, sm, first, rank);
        const int cells = c.P * c.L.ny * c.L.nz;
        float *gx = c.L.x + (long long)c.i0 * c.L.ny * c.L.nz;
        for (int t = threadIdx.x; t < cells; t += blockDim.x) gx[t] = c.x[t];
    }
}

// ---- CG with the V-cycle preconditioner -------------------------------------
// h = P r / |r| (in place): the Jacobi-scaled residual in the finite-volume
// form, normalised by the FP64 residual norm (rn2 = |r|^2) so the FP32 solve
// works at unit scale whatever the outer tolerance; sc->rhs_scale = |r| for
// the correction, sc->r0n2 = |h - mean h|^2 for the stopping test.  M's null
// space is the constants, so the mean of h (FP32 rounding leaves one of about
// eps sqrt(n) |h|) is a part no iteration can reduce; the test measures the
// rest.
__global__ void __launch_bounds__(kBlock)
k_mg_h(FvOp<float> F, float *__restrict__ h, const double *rn2, BicgScal *sc, double *partials, unsigned int *counter)
{
    pdl_wait();
    pdl_allow();
    const double nr = (rn2 && *rn2 > 0.0) ? sqrt(*rn2) : 1.0;
    const float s = (float)(1.0 / nr);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        sc->rhs_scale = nr;
        sc->wait_timeout = 0;  // the solve's bounded waits (TMA pipeline) report here
    }
    float pa = 0.f, ps = 0.f;
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x, st = (long long)gridDim.x * blockDim.x;
    const int nz = F.A.nzc, ny = F.A.nyc;
    if ((nz & 3) == 0) {
        // float4 rows along k (nz % 4 == 0 keeps a quad inside one (i, j) line)
        const int n4 = nz >> 2;
        const long long nq = F.A.n >> 2;
        for (long long q = t0; q < nq; q += st) {
            const long long line = q / n4;
            const int k0 = 4 * (int)(q - line * n4), i = (int)(line / ny), j = (int)(line - (long long)i * ny);
            const float wxy = __ldg(F.wx + i), wy = __ldg(F.wy + j), sxy = __ldg(F.sx + i);
            const float sy = __ldg(F.sy + j);
            const float4 wz = __ldg(reinterpret_cast<const float4 *>(F.wz + k0));
            const float4 sz = __ldg(reinterpret_cast<const float4 *>(F.sz + k0));
            float4 hv = reinterpret_cast<float4 *>(h)[q];
            hv.x = wxy * (wy * wz.x) * (sxy + (sy + sz.x)) * (hv.x * s);
            hv.y = wxy * (wy * wz.y) * (sxy + (sy + sz.y)) * (hv.y * s);
            hv.z = wxy * (wy * wz.z) * (sxy + (sy + sz.z)) * (hv.z * s);
            hv.w = wxy * (wy * wz.w) * (sxy + (sy + sz.w)) * (hv.w * s);
            reinterpret_cast<float4 *>(h)[q] = hv;
            pa = fmaf(hv.x, hv.x, fmaf(hv.y, hv.y, fmaf(hv.z, hv.z, fmaf(hv.w, hv.w, pa))));
            ps += (hv.x + hv.y) + (hv.z + hv.w);
        }
    } else {
        for (long long row = t0; row < F.A.n; row += st) {
            const int nyz = ny * nz;
            const int i = (int)(row / nyz), r2 = (int)(row - (long long)i * nyz), j = r2 / nz, k = r2 - j * nz;
            const float dv = __ldg(F.wx + i) * (__ldg(F.wy + j) * __ldg(F.wz + k));
            const float v = dv * (__ldg(F.sx + i) + (__ldg(F.sy + j) + __ldg(F.sz + k))) * (h[row] * s);
            h[row] = v;
            pa = fmaf(v, v, pa);
            ps += v;
        }
    }
    float acc[2] = {pa, ps};
    double tot[2];
    if (grid_reduce_f<2>(acc, partials, counter, tot) && threadIdx.x == 0)
        sc->r0n2 = fmax(tot[0] - tot[1] * tot[1] / (double)F.A.n, 0.0);
}

// the CG scalars after rho' = h . z (not the first): the iteration cap, else
// the flexible beta and the iteration count
__device__ __forceinline__ void mg_rho_update(BicgScal *sc, double tot)
{
    if (sc->iter + 1 >= sc->maxit) {
        sc->done = BICG_CAPPED;
    } else {
        // flexible (Polak-Ribiere) beta = h.(z - z_old) / rho_old, with
        // h.z_old = rho_old - alpha q.z_old (q.z from the stencil launch):
        // keeps the recurrences sound with an FP32 V-cycle, symmetric only
        // to rounding
        sc->beta = (tot - (sc->rho - sc->alpha * sc->qz)) / sc->rho;
        sc->rho = tot;
        sc->iter += 1;
        sc->total_iters += 1;
    }
}

// rho = h . z; with p0 != null also p0 = z and the solve's initial scalars
// (sc->r0n2 was set by k_mg_h), else beta and the iteration count (the
// stopping test is in k_mg_upd, before the V-cycle)
__global__ void __launch_bounds__(kBlock)
k_mg_rho(long long n, const float *__restrict__ h, const float *__restrict__ z, float *__restrict__ p0, BicgScal *sc,
         double *partials, unsigned int *counter)
{
    pdl_wait();
    pdl_allow();
    if (!p0 && sc->done) return;
    float pa = 0.f;
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x, st = (long long)gridDim.x * blockDim.x;
    // float4 body (the vectors are cudaMalloc allocations: 16-byte aligned), scalar tail
    const long long nq = n >> 2;
    for (long long q = t0; q < nq; q += st) {
        const float4 zv = reinterpret_cast<const float4 *>(z)[q];
        const float4 hv = reinterpret_cast<const float4 *>(h)[q];
        if (p0) reinterpret_cast<float4 *>(p0)[q] = zv;
        pa = fmaf(hv.x, zv.x, fmaf(hv.y, zv.y, fmaf(hv.z, zv.z, fmaf(hv.w, zv.w, pa))));
    }
    for (long long r = 4 * nq + t0; r < n; r += st) {
        const float zv = z[r];
        if (p0) p0[r] = zv;
        pa = fmaf(h[r], zv, pa);
    }
    float acc[1] = {pa};
    double tot[1];
    if (!grid_reduce_f<1>(acc, partials, counter, tot) || threadIdx.x != 0) return;
    if (p0) {
        sc->pp = 0;
        sc->rho = tot[0];
        sc->norm0 = sqrt(sc->r0n2);
        sc->iter = 0;
        sc->restart = 0;
        sc->timestep += 1;
        sc->done = (tot[0] != 0.0 && sc->r0n2 != 0.0) ? BICG_RUNNING : BICG_ZERO_RHS;
        sc->relres = sc->done == BICG_RUNNING ? 1.0 : 0.0;
        return;
    }
    mg_rho_update(sc, tot[0]);
}

// The V-cycle's last launch, the colour-0 pass of the finest level's
// post-smoothing, with rho' = h . z of the CG reduced from the quads it
// writes (h = b and z = x of the finest level): k_mg_rho without its own
// pass over h and z.  A grid-stride launch of at most kMaxReduce x the
// reduction grid, one partial per block.
template <class I, bool PZ>
__global__ void __launch_bounds__(kBlock)
k_mg_smooth4_rho(MgLevel L, const float *b, float *x, BicgScal *sc, double *partials, unsigned int *counter)
{
    pdl_wait();
    pdl_allow();
    if (sc->done) return;
    float pa = 0.f;
    smooth_quads<false, I, PZ, true>(L, b, x, 0, false, (I)blockIdx.x * blockDim.x + threadIdx.x,
                                     (I)gridDim.x * blockDim.x, &pa);
    float acc[1] = {pa};
    double tot[1];
    if (!grid_reduce_f<1>(acc, partials, counter, tot) || threadIdx.x != 0) return;
    mg_rho_update(sc, tot[0]);
}

// e += alpha p, h -= alpha q and the stopping test on |h - mean h| /
// |h0 - mean h0| (the unpreconditioned residual without its null-space part):
// a converged solve skips the V-cycle after it
// p2 != null: p and p2 are the two buffers of the run-time alternation; pn
// is the one sc->pp does not name, and the last block flips sc->pp
__global__ void __launch_bounds__(kBlock)
k_mg_upd(long long n, float *__restrict__ e, const float *p_, float *__restrict__ h,
         const float *__restrict__ q, BicgScal *sc, double *partials, unsigned int *counter, const float *p2)
{
    pdl_wait();
    pdl_allow();
    if (sc->done) return;
    const float *__restrict__ p = p2 ? (sc->pp ? p_ : p2) : p_;
    const float alpha = (float)sc->alpha;
    float pa = 0.f, ps = 0.f;
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x, st = (long long)gridDim.x * blockDim.x;
    // float4 body (the vectors are cudaMalloc allocations: 16-byte aligned), scalar tail
    const long long nq = n >> 2;
    for (long long q4 = t0; q4 < nq; q4 += st) {
        float4 ev = reinterpret_cast<float4 *>(e)[q4];
        float4 hv = reinterpret_cast<float4 *>(h)[q4];
        const float4 pv = reinterpret_cast<const float4 *>(p)[q4];
        const float4 qv = reinterpret_cast<const float4 *>(q)[q4];
        ev.x = fmaf(alpha, pv.x, ev.x); ev.y = fmaf(alpha, pv.y, ev.y);
        ev.z = fmaf(alpha, pv.z, ev.z); ev.w = fmaf(alpha, pv.w, ev.w);
        hv.x = fmaf(-alpha, qv.x, hv.x); hv.y = fmaf(-alpha, qv.y, hv.y);
        hv.z = fmaf(-alpha, qv.z, hv.z); hv.w = fmaf(-alpha, qv.w, hv.w);
        reinterpret_cast<float4 *>(e)[q4] = ev;
        reinterpret_cast<float4 *>(h)[q4] = hv;
        pa = fmaf(hv.x, hv.x, fmaf(hv.y, hv.y, fmaf(hv.z, hv.z, fmaf(hv.w, hv.w, pa))));
        ps += (hv.x + hv.y) + (hv.z + hv.w);
    }
    for (long long r = 4 * nq + t0; r < n; r += st) {
        e[r] = fmaf(alpha, p[r], e[r]);
        const float hv = fmaf(-alpha, q[r], h[r]);
        h[r] = hv;
        pa = fmaf(hv, hv, pa);
        ps += hv;
    }
    float acc[2] = {pa, ps};
    double tot[2];
    if (!grid_reduce_f<2>(acc, partials, counter, tot) || threadIdx.x != 0) return;
    if (p2) sc->pp = 1 - sc->pp;
    const double rel = sqrt(fmax(tot[0] - tot[1] * tot[1] / (double)n, 0.0) / sc->r0n2);
    sc->relres = rel;
    if (rel < sc->tol) sc->done = BICG_CONVERGED;
    else if (!(rel == rel)) sc->done = BICG_CAPPED;
}

// per-axis device arrays {cm, cp, cm + cp, w, 1/w} of m entries; periodic:
// the end cells couple across the period (centre distance (W[m-1] + W[0]) / 2)
int upload_axis(cfd_ctx *c, const std::vector<double> &W, MgLevel &L, int a, bool periodic = false)
{
    const int m = (int)W.size();
    std::vector<float> all((size_t)5 * m, 0.f);
    for (int i = 0; i < m; ++i) {
        float cm = 0.f, cp = 0.f;
        if (i > 0) cm = (float)(1.0 / (W[i] * 0.5 * (W[i - 1] + W[i])));
        else if (periodic) cm = (float)(1.0 / (W[i] * 0.5 * (W[m - 1] + W[i])));
        if (i < m - 1) cp = (float)(1.0 / (W[i] * 0.5 * (W[i] + W[i + 1])));
        else if (periodic) cp = (float)(1.0 / (W[i] * 0.5 * (W[i] + W[0])));
        all[i] = cm;
        all[m + i] = cp;
        all[2 * m + i] = cm + cp;
        all[3 * m + i] = (float)W[i];
        all[4 * m + i] = (float)(1.0 / W[i]);
    }
    float *d = nullptr;
    CKS(dalloc_t(c, &d, all.size()));
    CK(cudaMemcpy(d, all.data(), all.size() * sizeof(float), cudaMemcpyHostToDevice));
    L.cm[a] = d;
    L.cp[a] = d + m;
    L.sum[a] = d + 2 * m;
    L.w[a] = d + 3 * m;
    L.rw[a] = d + 4 * m;
    return CFD_OK;
}

void set_divs(MgLevel &L)
{
    L.fyz = FastDiv((unsigned)(L.ny * L.nz));
    L.fz = FastDiv((unsigned)L.nz);
    const int nh = L.nz / 2 > 0 ? L.nz / 2 : 1;
    L.fyh = FastDiv((unsigned)(L.ny * nh));
    L.fh = FastDiv((unsigned)nh);
    const int nq = L.nz / 4 > 0 ? L.nz / 4 : 1;
    L.fyq = FastDiv((unsigned)(L.ny * nq));
    L.fy2q = FastDiv((unsigned)((L.ny / 2 > 0 ? L.ny / 2 : 1) * nq));
    L.fq = FastDiv((unsigned)nq);
    // float4 rows need nz % 4 == 0 and 16-byte aligned z-axis tables
    auto al = [](const void *p) { return (reinterpret_cast<unsigned long long>(p) & 15ull) == 0; };
    L.quads = L.nz % 4 == 0 && al(L.x) && al(L.b) && al(L.rw[2]) && al(L.sum[2]) && al(L.cm[2]) && al(L.cp[2]);
}

// dense (M + a 1 1^T)^-1 of a level given its per-axis widths (Gauss-Jordan
// in FP64; M symmetric positive semi-definite with constants as null space);
// pz: z neighbours wrap
int coarse_inverse(cfd_ctx *c, const std::vector<double> (&W)[3], float **out, bool pz = false)
{
    const int nx = (int)W[0].size(), ny = (int)W[1].size(), nz = (int)W[2].size(), n = nx * ny * nz;
    std::vector<double> A((size_t)n * n, 0.0), I((size_t)n * n, 0.0);
    auto id = [&](int i, int j, int k) { return (i * ny + j) * nz + k; };
    double dmax = 0.0;
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                const int r = id(i, j, k);
                const double dv = W[0][i] * W[1][j] * W[2][k];
                const int ax[3] = {i, j, k}, lim[3] = {nx, ny, nz};
                double diag = 0.0;
                for (int a = 0; a < 3; ++a)
                    for (int side = -1; side <= 1; side += 2) {
                        int o = ax[a] + side;
                        if (a == 2 && pz) o = (o + lim[a]) % lim[a];
                        if (o < 0 || o >= lim[a]) continue;
                        const double cf = dv / (W[a][ax[a]] * 0.5 * (W[a][ax[a]] + W[a][o]));
                        int ii = i, jj = j, kk = k;
                        (a == 0 ? ii : a == 1 ? jj : kk) = o;
                        A[(size_t)r * n + id(ii, jj, kk)] -= cf;
                        diag += cf;
                    }
                A[(size_t)r * n + r] += diag;
                dmax = std::max(dmax, diag);
            }
    const double alpha = dmax / n;
    for (size_t q = 0; q < A.size(); ++q) A[q] += alpha;
    for (int r = 0; r < n; ++r) I[(size_t)r * n + r] = 1.0;
    for (int col = 0; col < n; ++col) {
        int piv = col;
        for (int r = col + 1; r < n; ++r)
            if (std::fabs(A[(size_t)r * n + col]) > std::fabs(A[(size_t)piv * n + col])) piv = r;
        if (std::fabs(A[(size_t)piv * n + col]) == 0.0) return fail(CFD_ERR_STATE, "singular coarsest operator");
        if (piv != col)
            for (int q = 0; q < n; ++q) {
                std::swap(A[(size_t)piv * n + q], A[(size_t)col * n + q]);
                std::swap(I[(size_t)piv * n + q], I[(size_t)col * n + q]);
            }
        const double inv = 1.0 / A[(size_t)col * n + col];
        for (int q = 0; q < n; ++q) {
            A[(size_t)col * n + q] *= inv;
            I[(size_t)col * n + q] *= inv;
        }
        for (int r = 0; r < n; ++r) {
            if (r == col) continue;
            const double f = A[(size_t)r * n + col];
            if (f == 0.0) continue;
            for (int q = 0; q < n; ++q) {
                A[(size_t)r * n + q] -= f * A[(size_t)col * n + q];
                I[(size_t)r * n + q] -= f * I[(size_t)col * n + q];
            }
        }
    }
    // exact symmetry in float (the device product reads columns for rows)
    std::vector<float> f((size_t)small_pad((long long)n * n), 0.f);  // padded to whole 16-byte chunks
    for (int r = 0; r < n; ++r)
        for (int q = 0; q < n; ++q) f[(size_t)r * n + q] = (float)(0.5 * (I[(size_t)r * n + q] + I[(size_t)q * n + r]));
    CKS(dalloc_t(c, out, f.size()));
    CK(cudaMemcpy(*out, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice));
    return CFD_OK;
}

// eigenvalues (ascending) and eigenvectors (columns of v, row-major n x n)
// of the symmetric matrix a (destroyed) by cyclic Jacobi rotations, FP64
static void jacobi_eigen(std::vector<double> &a, int n, std::vector<double> &lam, std::vector<double> &v)
{
    v.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) v[(size_t)i * n + i] = 1.0;
    auto A = [&](int i, int j) -> double & { return a[(size_t)i * n + j]; };
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                tot += A(i, j) * A(i, j);
                if (i != j) off += A(i, j) * A(i, j);
            }
        if (off <= 1e-30 * tot) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = A(p, q);
                if (std::fabs(apq) <= 1e-300) continue;
                // the rotation that zeroes a_pq: t = tan(phi), the smaller root
                const double theta = (A(q, q) - A(p, p)) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
                for (int r = 0; r < n; ++r) {  // columns p, q
                    const double arp = A(r, p), arq = A(r, q);
                    A(r, p) = c * arp - sn * arq;
                    A(r, q) = sn * arp + c * arq;
                }
                for (int r = 0; r < n; ++r) {  // rows p, q
                    const double apr = A(p, r), aqr = A(q, r);
                    A(p, r) = c * apr - sn * aqr;
                    A(q, r) = sn * apr + c * aqr;
                }
                for (int r = 0; r < n; ++r) {
                    const double vrp = v[(size_t)r * n + p], vrq = v[(size_t)r * n + q];
                    v[(size_t)r * n + p] = c * vrp - sn * vrq;
                    v[(size_t)r * n + q] = sn * vrp + c * vrq;
                }
            }
    }
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::sort(order.begin(), order.end(), [&](int x, int y) { return A(x, x) < A(y, y); });
    lam.resize(n);
    std::vector<double> vs((size_t)n * n);
    for (int m = 0; m < n; ++m) {
        lam[m] = A(order[m], order[m]);
        for (int r = 0; r < n; ++r) vs[(size_t)r * n + m] = v[(size_t)r * n + order[m]];
    }
    v.swap(vs);
}

// the fast-diagonalisation tables of level G.fd_level from its cell widths:
// per axis K v = lambda W v through the symmetric S = W^-1/2 K W^-1/2, and
// V = W^-1/2 U; K has -1 / Ds off the diagonal (Ds the centre distance,
// both sides when a periodic axis has two cells) and the row sums on it
int fd_setup(cfd_ctx *c, Mg &G, const std::vector<double> (&W)[3], bool pz)
{
    double lam0[3], lmax[3];
    for (int a = 0; a < 3; ++a) {
        const int n = (int)W[a].size();
        std::vector<double> K((size_t)n * n, 0.0);
        for (int i = 0; i < n; ++i)
            for (int side = -1; side <= 1; side += 2) {
                int o = i + side;
                if (a == 2 && pz) o = (o + n) % n;
                if (o < 0 || o >= n || o == i) continue;
                const double cf = 1.0 / (0.5 * (W[a][i] + W[a][o]));
                K[(size_t)i * n + o] -= cf;
                K[(size_t)i * n + i] += cf;
            }
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) K[(size_t)i * n + j] /= std::sqrt(W[a][i] * W[a][j]);
        std::vector<double> lam, U;
        jacobi_eigen(K, n, lam, U);
        std::vector<float> vf((size_t)n * n), lf(n);
        for (int i = 0; i < n; ++i)
            for (int m = 0; m < n; ++m) vf[(size_t)i * n + m] = (float)(U[(size_t)i * n + m] / std::sqrt(W[a][i]));
        for (int m = 0; m < n; ++m) lf[m] = (float)lam[m];
        lam0[a] = lam[0];
        lmax[a] = lam[n - 1];
        CKS(dalloc_t(c, &G.fd_v[a], vf.size()));
        CKS(dalloc_t(c, &G.fd_l[a], lf.size()));
        CK(cudaMemcpy(G.fd_v[a], vf.data(), vf.size() * sizeof(float), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(G.fd_l[a], lf.data(), lf.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    // Neumann or periodic on every axis: constants are the null space
    G.fd_null = true;
    for (int a = 0; a < 3; ++a) G.fd_null = G.fd_null && std::fabs(lam0[a]) <= 1e-9 * std::max(lmax[a], 1e-300);
    CK(cudaFuncSetAttribute(k_fd_block, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFdSmemMax));
    return CFD_OK;
}

// shared-memory layout of the small kernel from level `first` on.  The
// static image first: the dense inverse (when staged), then per level the
// per-cell 1 / dV and 1 / diag and the axis tables; after it per level x and
// b.  Every piece is a multiple of 4 floats.  Returns the size in bytes.
long long small_layout(const Mg &G, int first, bool cinv, MgSmall *S)
{
    long long off = 0;
    const long long nc = G.lev[G.nlev - 1].n;
    if (S) S->cinv_off = cinv ? 0 : -1;
    if (cinv) off += small_pad(nc * nc);
    for (int l = first; l < G.nlev; ++l) {
        const MgLevel &L = G.lev[l];
        if (S) S->rv_off[l] = (int)off;
        off += 2 * small_pad(L.n);
        if (S) S->tab_off[l] = (int)off;
        off += 5 * (small_pad(L.nx) + small_pad(L.ny) + small_pad(L.nz));
    }
    if (S) S->image_floats = (int)off;
    for (int l = first; l < G.nlev; ++l) {
        if (S) S->off[l] = (int)off;
        off += 2 * small_pad(G.lev[l].n);
    }
    return off * (long long)sizeof(float);
}

// the static image of the small kernel's shared memory, in device memory
int small_image(cfd_ctx *c, Mg &G)
{
    MgSmall S{};
    small_layout(G, G.first_small, G.cinv_smem, &S);
    G.image_floats = S.image_floats;
    CKS(dalloc_t(c, &G.image, (size_t)S.image_floats));
    CK(cudaMemset(G.image, 0, (size_t)S.image_floats * sizeof(float)));
    const long long nc = G.lev[G.nlev - 1].n;
    if (G.cinv_smem)
        CK(cudaMemcpy(G.image + S.cinv_off, G.cinv, (size_t)(nc * nc) * sizeof(float), cudaMemcpyDeviceToDevice));
    for (int l = G.first_small; l < G.nlev; ++l) {
        const MgLevel &L = G.lev[l];
        float *rv = G.image + S.rv_off[l];
        k_mg_cell_tables<<<nblk(L.n), kBlock, 0, c->s>>>(L, rv, rv + small_pad(L.n));
        CK(cudaGetLastError());
        float *p = G.image + S.tab_off[l];
        const int dims[3] = {L.nx, L.ny, L.nz};
        for (int a = 0; a < 3; ++a) {
            const int m = (int)small_pad(dims[a]);
            const float *src[5] = {L.cm[a], L.cp[a], L.sum[a], L.w[a], L.rw[a]};
            for (int q = 0; q < 5; ++q)
                CK(cudaMemcpy(p + q * m, src[q], (size_t)dims[a] * sizeof(float), cudaMemcpyDeviceToDevice));
            p += 5 * m;
        }
    }
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

}  // namespace

namespace cfd {

static bool transfers4(const Mg &G, const MgLevel &F, const MgLevel &C);

// host set-up of the level hierarchy (level 0 is the CG's own operator)
int mg_setup(cfd_ctx *c)
{
    Mg &G = c->mg;
    if (G.nlev > 0) return CFD_OK;
    const Geo &g = c->g;
    if (const char *e = std::getenv("CFDGPU_MG_SWEEPS")) G.sweeps = std::atoi(e) > 0 ? std::atoi(e) : 2;
    G.sweeps0 = G.sweeps;
    if (const char *e = std::getenv("CFDGPU_MG_SWEEPS0")) G.sweeps0 = std::atoi(e) > 0 ? std::atoi(e) : G.sweeps;
    if (const char *e = std::getenv("CFDGPU_MG_PAIRS")) G.pairs = std::atoi(e) > 0 ? std::atoi(e) : 1;
    if (const char *e = std::getenv("CFDGPU_MG_FUSE_ENDS")) G.fuse_from = std::atoi(e) != 0 ? 0 : kMgMaxLevels;
    if (const char *e = std::getenv("CFDGPU_MG_FUSE_ENDS_FROM")) G.fuse_from = std::max(0, std::atoi(e));
    G.small_sweeps = G.sweeps;
    if (const char *e = std::getenv("CFDGPU_MG_TRANSFER4")) G.transfer4 = e[0] != '0';
    if (const char *e = std::getenv("CFDGPU_MG_ROWS2")) G.rows2 = e[0] != '0';
    if (const char *e = std::getenv("CFDGPU_MG_SMALL_SWEEPS")) G.small_sweeps = std::atoi(e) > 0 ? std::atoi(e) : G.sweeps;
    int march = 0;  // planes a thread of the marching colour pass covers (0: k_mg_smooth4x2)
    if (const char *e = std::getenv("CFDGPU_MG_MARCH")) march = std::max(0, std::atoi(e));
    long long small = kMgSmall;
    if (const char *e = std::getenv("CFDGPU_MG_SMALL")) small = std::atoll(e);
    float om = 1.f;  // smoother relaxation (1: Gauss-Seidel)
    if (const char *e = std::getenv("CFDGPU_MG_OMEGA")) om = std::max(0.5f, std::min(1.5f, (float)std::atof(e)));
    const FvOp<float> F = fv32(c);
    std::vector<double> W[3];
    std::vector<std::array<std::vector<double>, 3>> Wl(1);  // the widths of every level
    const int n0[3] = {g.nxc, g.nyc, g.nzc};
    for (int a = 0; a < 3; ++a) {
        W[a].resize(n0[a]);
        for (int i = 0; i < n0[a]; ++i) W[a][i] = c->hraw[3 + a][i + GC];
    }
    Wl[0] = {W[0], W[1], W[2]};
    MgLevel L0{};
    L0.nx = g.nxc; L0.ny = g.nyc; L0.nz = g.nzc; L0.n = g.n;
    L0.cm[0] = F.A.cxm; L0.cp[0] = F.A.cxp; L0.sum[0] = F.sx; L0.w[0] = F.wx;
    L0.cm[1] = F.A.cym; L0.cp[1] = F.A.cyp; L0.sum[1] = F.sy; L0.w[1] = F.wy;
    L0.cm[2] = F.A.czm; L0.cp[2] = F.A.czp; L0.sum[2] = F.sz; L0.w[2] = F.wz;
    for (int a = 0; a < 3; ++a) {  // 1 / width of level 0
        std::vector<float> rw(n0[a]);
        for (int i = 0; i < n0[a]; ++i) rw[i] = (float)(1.0 / W[a][i]);
        float *d = nullptr;
        CKS(dalloc_t(c, &d, rw.size()));
        CK(cudaMemcpy(d, rw.data(), rw.size() * sizeof(float), cudaMemcpyHostToDevice));
        L0.rw[a] = d;
    }
    L0.x = c->w32.r0;  // z
    L0.b = c->r32;     // h
    L0.pz = g.pz;
    L0.om = om;
    set_divs(L0);
    G.lev[0] = L0;
    int nl = 1;
    int n[3] = {g.nxc, g.nyc, g.nzc};
    long long target = kMgCoarseTarget;
    if (const char *e = std::getenv("CFDGPU_MG_COARSE")) target = std::max(8LL, std::min<long long>(kMgCoarsest, std::atoll(e)));
    while (nl < kMgMaxLevels && (long long)n[0] * n[1] * n[2] > target) {
        int f[3];
        bool any = false;
        for (int a = 0; a < 3; ++a) {
            f[a] = (n[a] % 2 == 0 && n[a] >= 4) ? 2 : 1;
            // periodic z halves only to an even length, so that red-black
            // stays a two-colouring across the wrap
            if (a == 2 && g.pz && n[a] % 4 != 0) f[a] = 1;
            any = any || f[a] == 2;
        }
        if (!any) break;
        MgLevel L{};
        for (int a = 0; a < 3; ++a) {
            std::vector<double> Wc(n[a] / f[a]);
            for (size_t I = 0; I < Wc.size(); ++I) Wc[I] = f[a] == 2 ? W[a][2 * I] + W[a][2 * I + 1] : W[a][I];
            W[a] = Wc;
            n[a] = (int)Wc.size();
            CKS(upload_axis(c, W[a], L, a, a == 2 && g.pz));
        }
        L.pz = g.pz;
        L.om = om;
        L.nx = n[0]; L.ny = n[1]; L.nz = n[2];
        L.n = (long long)n[0] * n[1] * n[2];
        CKS(dalloc_t(c, &L.x, (size_t)L.n));
        CKS(dalloc_t(c, &L.b, (size_t)L.n));
        set_divs(L);
        G.lev[nl++] = L;
        Wl.push_back({W[0], W[1], W[2]});
    }
    G.nlev = nl;
    for (int l = 0; l < nl; ++l) {
        MgLevel &L = G.lev[l];
        // two rows a thread only where a colour pass has work for many waves:
        // at a few hundred blocks the halved thread count costs more latency
        // than the shared row loads save
        L.rows2 = G.rows2 && L.quads && L.ny % 2 == 0 && L.om == 1.f && L.n >= (1LL << 21);
        L.march = L.rows2 ? march : 0;
    }
    // the exact separable solve replaces the first level below the finest
    // of at most kFdCells cells whose tables fit one block's shared memory,
    // and every coarser one (CFDGPU_MG_FD=0: the small levels in one block
    // with the dense coarsest solve)
    bool fd_on = true;
    long long fd_cells = kFdCells;
    if (const char *e = std::getenv("CFDGPU_MG_FD")) fd_on = e[0] != '0';
    if (const char *e = std::getenv("CFDGPU_MG_FD_CELLS")) fd_cells = std::max(1LL, std::atoll(e));
    G.fd_level = 0;
    if (const char *e = std::getenv("CFDGPU_MG_CLUSTER")) fd_on = fd_on && e[0] == '0';  // the cluster kernel instead
    if (fd_on)
        for (int l = 1; l < nl; ++l) {
            const MgLevel &L = G.lev[l];
            if (L.n <= fd_cells && fd_smem(L.nx, L.ny, L.nz) <= kFdSmemMax) {
                G.fd_level = l;
                break;
            }
        }
    if (G.fd_level > 0) {
        nl = G.fd_level + 1;
        G.nlev = nl;
        G.usable = true;
        G.first_small = G.fd_level;
        G.first_cluster = 0;
        CKS(fd_setup(c, G, {Wl[nl - 1][0], Wl[nl - 1][1], Wl[nl - 1][2]}, g.pz != 0));
    }
    const long long ncoarse = G.lev[nl - 1].n;
    if (G.fd_level == 0) G.usable = nl > 1 && ncoarse <= kMgCoarsest;
    if (!G.usable) return CFD_OK;
    if (G.fd_level == 0) {
    CKS(coarse_inverse(c, W, &G.cinv, g.pz != 0));
    // the first small level: at most `small` cells, and all levels from it
    // on fit the small kernel's shared memory; the dense inverse is staged
    // there too when it fits
    G.first_small = nl - 1;
    for (int l = 0; l < nl; ++l)
        if (G.lev[l].n <= small && small_layout(G, l, false, nullptr) <= kMgSmallSmem) {
            G.first_small = l;
            break;
        }
    G.cinv_smem = small_layout(G, G.first_small, true, nullptr) <= kMgSmallSmem;
    G.small_smem = (int)small_layout(G, G.first_small, G.cinv_smem, nullptr);
    if (G.small_smem > kMgSmallSmem) return fail(CFD_ERR_STATE, "multigrid: coarsest level too large for shared memory");
    CK(cudaFuncSetAttribute(k_mg_small<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMgSmallSmem));
    CK(cudaFuncSetAttribute(k_mg_small<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMgSmallSmem));
    CKS(small_image(c, G));
    // the coarse levels in one thread-block cluster, from the largest level
    // whose own and coarser levels all split into kClusterCtas nesting x slabs
    // that fit a CTA's shared memory (at most the small kernel's levels plus
    // the grid-wide ones above them that fit)
    G.first_cluster = 0;
    if (const char *e = std::getenv("CFDGPU_MG_CLUSTER")) G.cluster = e[0] != '0';
    if (G.cluster) {
        for (int l = 1; l <= G.first_small && l < nl; ++l) {
            long long floats = 0;
            bool ok = true;
            for (int q = l; q < nl && ok; ++q) {
                const MgLevel &L = G.lev[q];
                ok = L.nx % kClusterCtas == 0 && (q == l || G.lev[q - 1].nx % L.nx == 0);
                floats += (2LL * (L.nx / kClusterCtas) * L.ny * L.nz + 3) & ~3LL;
            }
            floats += 4;
            if (ok && floats * 4 <= kMgClusterSmem) {
                G.first_cluster = l;
                G.cluster_smem = (int)(floats * 4);
                break;
            }
        }
        if (G.first_cluster > 0) {
            auto k = g.pz ? k_mg_cluster<true> : k_mg_cluster<false>;
            CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, G.cluster_smem));
            cudaLaunchConfig_t cfg{};
            cfg.gridDim = dim3(kClusterCtas);
            cfg.blockDim = dim3(kClusterThreads);
            cfg.dynamicSmemBytes = (size_t)G.cluster_smem;
            int nclusters = 0;
            if (cudaOccupancyMaxActiveClusters(&nclusters, k, &cfg) != cudaSuccess || nclusters < 1) {
                cudaGetLastError();
                G.first_cluster = 0;  // not co-schedulable here: the small kernel instead
            }
        }
    }
    }  // the small levels (no separable solve)
    // fused sweeps on the grid-wide levels with float4 rows: about 128
    // threads a block (TJ rows x nz/4 quads), chunks of CI planes sized for
    // about six blocks per SM, a second x buffer each
    // off by default: at 512x256x32 a fused pass took 45 us against 2 x 12.4 us
    // for the two colour launches (the plane march is latency-bound)
    bool fused = false;
    if (const char *e = std::getenv("CFDGPU_MG_FUSED")) fused = std::atoi(e) != 0;
    int fused_from = 0;  // the first level that runs fused sweeps
    if (const char *e = std::getenv("CFDGPU_MG_FUSED_FROM")) {
        fused = true;
        fused_from = std::max(0, std::atoi(e));
    }
    int dev = 0, sms = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    for (int l = 0; l < mg_grid_levels(G); ++l) {
        MgLevel &L = G.lev[l];
        L.sweep_tj = L.sweep_ci = 0;
        if (!fused || l < fused_from || !L.quads || L.pz || L.om != 1.f || level_sweeps(G, l) % 2 != 0) continue;
        const int n4 = L.nz / 4;
        const int tj = std::max(1, std::min({128 / std::max(n4, 1), L.ny, 1024 / n4}));
        if (tj * n4 > 1024 || (long long)sweep_smem(tj, L.nz) > kSweepSmemMax) continue;
        const long long tiles = (L.ny + tj - 1) / tj;
        const int ci = (int)std::max(4LL, std::min(16LL, (long long)L.nx * tiles / (6LL * std::max(sms, 1))));
        CKS(dalloc_t(c, &L.xalt, (size_t)L.n));
        L.sweep_tj = tj;
        L.sweep_ci = ci;
    }
    CK(cudaFuncSetAttribute(k_mg_sweep, cudaFuncAttributeMaxDynamicSharedMemorySize, kSweepSmemMax));
    // tiled smoothing phases on the grid-wide levels of at most kTileCells
    // cells, whose colour launches are latency-bound (at 512x256x32 the
    // 65 536-cell level gains 11 us a V-cycle, the 524 288-cell level loses
    // 6: its tiles, 2.25 times the cells, are bound by the shared-memory and
    // L1 bandwidth of 128 SMs).  The finest level's post-smoothing always
    // stays launches: the CG's rho' is fused into its last colour and the
    // V-cycle's result is its x.  Tiles of 16 x 16 columns where they give a
    // wave of blocks, else 8 x 8; a second x buffer for the post-smoothing.
    long long tile_cells = kTileCells, split_cells = 0;
    int tile_from = kMgMaxLevels, tile_xy = 0;
    if (const char *e = std::getenv("CFDGPU_MG_TILE")) {
        tile_cells = e[0] != '0' ? tile_cells : 0;
        split_cells = e[0] != '0' ? split_cells : 0;
    }
    if (const char *e = std::getenv("CFDGPU_MG_TILE_SPLIT")) split_cells = e[0] != '0' ? kTileSplitCells : 0;
    if (const char *e = std::getenv("CFDGPU_MG_TILE_FROM")) tile_from = std::max(0, std::atoi(e));
    if (const char *e = std::getenv("CFDGPU_MG_TILE_XY")) tile_xy = std::max(0, std::atoi(e)) & ~1;
    for (int l = 0; l < mg_grid_levels(G); ++l) {
        MgLevel &L = G.lev[l];
        G.tile[l] = G.tile_r[l] = MgTile{};
        G.tile_split[l] = false;
        const int sw = level_sweeps(G, l);
        // one sweep a launch on the levels above tile_cells up to split_cells
        // (two sweeps a phase; off by default: at 512x256x32 the 524 288-cell
        // level took 10.82 ms a step so against 10.60 with colour launches)
        const bool split = l > 0 && l < tile_from && L.n > tile_cells && L.n <= split_cells && sw == 2;
        if (l < tile_from && (l == 0 || L.n > tile_cells) && !split) continue;
        if (!L.quads || L.om != 1.f || L.sweep_tj > 0 || !transfers4(G, L, G.lev[l + 1])) continue;
        const int n4 = L.nz / 4;
        auto make = [&](int t, int sweeps, int h) {
            MgTile T{};
            T.tx = T.ty = t;
            T.h = h;
            T.sweeps = sweeps;
            T.wx = t + 2 * h;
            T.wy = t + 2 * h;
            T.n4 = n4;
            T.tiles_y = (L.ny + t - 1) / t;
            T.fn4 = FastDiv((unsigned)n4);
            T.fwy = FastDiv((unsigned)T.wy);
            return T;
        };
        // a phase in one launch: s sweeps, halo 2 s; split: one sweep, halo 2,
        // and halo 3 for the launch that ends with the restriction
        const int ts = split ? 1 : sw, th = split ? 3 : 2 * sw;
        auto fits = [&](int t) { return tile_smem(make(t, ts, th)) <= (size_t)kTileSmemMax; };
        auto blocks = [&](int t) { return (long long)((L.nx + t - 1) / t) * ((L.ny + t - 1) / t); };
        int t = tile_xy;
        if (t == 0) t = fits(16) && blocks(16) >= sms ? 16 : 8;
        if (t < 2 || !fits(t)) continue;
        if (l > 0 && !L.xalt) CKS(dalloc_t(c, &L.xalt, (size_t)L.n));
        G.tile[l] = make(t, ts, 2 * ts);
        if (split) G.tile_r[l] = make(t, 1, 3);
        G.tile_split[l] = split;
    }
    for (auto k : {k_mg_tile<false, kTilePre>, k_mg_tile<false, kTilePost>, k_mg_tile<false, kTileZero>,
                   k_mg_tile<false, kTileReadR>, k_mg_tile<false, kTileRead>, k_mg_tile<true, kTilePre>,
                   k_mg_tile<true, kTilePost>, k_mg_tile<true, kTileZero>, k_mg_tile<true, kTileReadR>,
                   k_mg_tile<true, kTileRead>})
        CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kTileSmemMax));
    CKS(dalloc_t(c, &G.never, 1));
    CK(cudaMemset(G.never, 0, sizeof(int)));
    return CFD_OK;
}

static MgCluster cluster_desc(const Mg &G, const int *done)
{
    MgCluster S{};
    S.first = G.first_cluster;
    S.nlev = G.nlev;
    S.pre = G.sweeps;
    S.post = G.sweeps;
    S.done = done;
    S.cinv = G.cinv;
    int acc = 0;
    for (int l = 0; l < G.nlev; ++l) {
        S.lev[l] = G.lev[l];
        if (l < G.first_cluster) continue;
        const MgLevel &L = G.lev[l];
        S.off[l] = acc;
        acc += (int)((2LL * (L.nx / kClusterCtas) * L.ny * L.nz + 3) & ~3LL);
    }
    S.part_off = acc;
    return S;
}

static MgSmall small_desc(const Mg &G, const int *done)
{
    MgSmall S{};
    S.done = done;
    S.first = G.first_small;
    S.nlev = G.nlev;
    S.pre = G.small_sweeps;
    S.post = G.small_sweeps;
    S.cinv = G.cinv;
    S.image = G.image;
    for (int l = 0; l < G.nlev; ++l) S.lev[l] = G.lev[l];
    small_layout(G, G.first_small, G.cinv_smem, &S);
    return S;
}

static void smooth_launch(const MgLevel &L, int color, int zero_init, const int *done, cudaStream_t s);

// one fused sweep (colour c0 then 1 - c0) of a grid-wide level, xo -> xn
static void sweep_launch(const MgLevel &L, const float *xo, float *xn, int c0, int zero_init, const int *done,
                         cudaStream_t s)
{
    const int tiles = (L.ny + L.sweep_tj - 1) / L.sweep_tj, chunks = (L.nx + L.sweep_ci - 1) / L.sweep_ci;
    launch_pdl(k_mg_sweep, dim3(tiles * chunks), dim3(L.sweep_tj * (L.nz / 4)), sweep_smem(L.sweep_tj, L.nz), s, L,
               (const float *)L.b, xo, xn, c0, zero_init, done);
}

// the pre-smoothing (c0 = 0, from x = 0) or post-smoothing (c0 = 1, from x) of
// a grid-wide level: fused sweeps alternate between x and xalt and end in x
// (an even number of sweeps), else colour launches in place
// a level whose sweep ends run fused (k_mg_first4, k_mg_prolong_first4)
static bool fused_ends(const Mg &G, int l)
{
    const MgLevel &L = G.lev[l];
    return l >= G.fuse_from && L.quads && L.sweep_tj == 0 && L.om == 1.f;
}
static bool int_index(const MgLevel &L) { return L.n + (long long)L.ny * L.nz < (1LL << 31); }

// the CG's rho' fused into the V-cycle's last launch (k_mg_smooth4_rho)
struct RhoFuse {
    BicgScal *sc;
    double *partials;
    unsigned int *counter;
    long long grid_cap;  // kMaxReduce x the reduction grid: one partial per block
};

template <bool PZ>
static void rho_launch_t(const MgLevel &L, const RhoFuse &r, cudaStream_t s)
{
    const int grid = (int)std::min<long long>(nblk(L.n / 4), r.grid_cap);
    if (int_index(L))
        launch_pdl(k_mg_smooth4_rho<int, PZ>, dim3(grid), dim3(kBlock), 0, s, L, (const float *)L.b, L.x, r.sc,
                   r.partials, r.counter);
    else
        launch_pdl(k_mg_smooth4_rho<long long, PZ>, dim3(grid), dim3(kBlock), 0, s, L, (const float *)L.b, L.x, r.sc,
                   r.partials, r.counter);
}

// pre: the sweeps before the coarse correction; post_fused: the caller ran
// the first colour of the post-smoothing with the prolongation; rf: the
// last colour launch (colour 0 of the post-smoothing) also reduces rho'
static void smooth_phase(const Mg &G, int l, bool pre, const int *done, cudaStream_t s, bool post_fused = false,
                         const RhoFuse *rf = nullptr)
{
    const MgLevel &L = G.lev[l];
    const int sweeps = level_sweeps(G, l);
    auto last = [&](int q) {
        if (rf && q == sweeps - 1) {
            if (L.pz) rho_launch_t<true>(L, *rf, s);
            else rho_launch_t<false>(L, *rf, s);
        } else {
            smooth_launch(L, pre ? 1 : 0, 0, done, s);
        }
    };
    if (fused_ends(G, l)) {
        for (int q = 0; q < sweeps; ++q) {
            if (pre && q == 0) {
                if (int_index(L))
                    launch_pdl(k_mg_first4<int>, dim3(nblk(L.n / 4)), dim3(kBlock), 0, s, L, (const float *)L.b, L.x,
                               done);
                else
                    launch_pdl(k_mg_first4<long long>, dim3(nblk(L.n / 4)), dim3(kBlock), 0, s, L,
                               (const float *)L.b, L.x, done);
                continue;
            }
            if (!(post_fused && q == 0)) smooth_launch(L, pre ? 0 : 1, 0, done, s);
            last(q);
        }
        return;
    }
    if (L.sweep_tj > 0) {
        const float *src = L.x;
        for (int q = 0; q < sweeps; ++q) {
            float *dst = ((sweeps - 1 - q) % 2 == 0) ? L.x : L.xalt;
            sweep_launch(L, src, dst, pre ? 0 : 1, pre && q == 0, done, s);
            src = dst;
        }
        return;
    }
    for (int q = 0; q < sweeps; ++q) {
        smooth_launch(L, pre ? 0 : 1, pre && q == 0, done, s);
        last(q);
    }
}

// one colour of the smoother over a grid-wide level
template <bool PZ>
static void smooth_launch_t(const MgLevel &L, int color, int zero_init, const int *done, cudaStream_t s)
{
    if (L.rows2 && L.march > 0 && L.n + (long long)L.ny * L.nz < (1LL << 31)) {
        const int np = (L.ny / 2) * (L.nz / 4);
        const dim3 grid((unsigned)((np + kBlock - 1) / kBlock), (unsigned)((L.nx + L.march - 1) / L.march));
        launch_pdl(k_mg_smooth4m<PZ>, grid, dim3(kBlock), 0, s, L, (const float *)L.b, L.x, color, zero_init, L.march,
                   done);
        return;
    }
    if (L.rows2 && L.n + (long long)L.ny * L.nz < (1LL << 31)) {
        launch_pdl(k_mg_smooth4x2<int, PZ>, dim3(nblk(L.n / 8)), dim3(kBlock), 0, s, L, (const float *)L.b, L.x, color,
                   zero_init, done);
        return;
    }
    if (L.rows2) {
        launch_pdl(k_mg_smooth4x2<long long, PZ>, dim3(nblk(L.n / 8)), dim3(kBlock), 0, s, L, (const float *)L.b, L.x,
                   color, zero_init, done);
        return;
    }
    if (L.quads && L.n + (long long)L.ny * L.nz < (1LL << 31))
        launch_pdl(k_mg_smooth4<int, PZ>, dim3(nblk(L.n / 4)), dim3(kBlock), 0, s, L, (const float *)L.b, L.x, color,
                   zero_init, done);
    else if (L.quads)
        launch_pdl(k_mg_smooth4<long long, PZ>, dim3(nblk(L.n / 4)), dim3(kBlock), 0, s, L, (const float *)L.b, L.x,
                   color, zero_init, done);
    else
        launch_pdl(k_mg_smooth<PZ>, dim3(nblk((L.nz % 2 == 0) ? L.n / 2 : L.n)), dim3(kBlock), 0, s, L,
                   (const float *)L.b, L.x, color, zero_init, done);
}

static void smooth_launch(const MgLevel &L, int color, int zero_init, const int *done, cudaStream_t s)
{
    if (L.pz) smooth_launch_t<true>(L, color, zero_init, done, s);
    else smooth_launch_t<false>(L, color, zero_init, done, s);
}

// the float4-row transfers apply: 2x2x2 coarsening of a float4 level whose
// coarse level has an even nz (aligned float2 pairs), and the switch is on
static bool transfers4(const Mg &G, const MgLevel &F, const MgLevel &C)
{
    return G.transfer4 && F.quads && F.nx == 2 * C.nx && F.ny == 2 * C.ny && F.nz == 2 * C.nz && C.nz % 2 == 0 &&
           (reinterpret_cast<unsigned long long>(C.b) & 7ull) == 0 && (reinterpret_cast<unsigned long long>(C.x) & 7ull) == 0;
}

static void restrict_launch(const Mg &G, const MgLevel &F, const MgLevel &C, const int *done, cudaStream_t s,
                            bool pdl = true)
{
    if (transfers4(G, F, C)) {
        auto k4 = F.pz ? k_mg_restrict4<true> : k_mg_restrict4<false>;
        if (pdl) launch_pdl(k4, dim3(nblk(C.n / 2)), dim3(kBlock), 0, s, F, C, (const float *)F.b, (const float *)F.x, C.b, done);
        else k4<<<nblk(C.n / 2), kBlock, 0, s>>>(F, C, F.b, F.x, C.b, done);
        return;
    }
    auto k = F.pz ? k_mg_restrict<true> : k_mg_restrict<false>;
    if (pdl) launch_pdl(k, dim3(nblk(C.n)), dim3(kBlock), 0, s, F, C, (const float *)F.b, (const float *)F.x, C.b, done);
    else k<<<nblk(C.n), kBlock, 0, s>>>(F, C, F.b, F.x, C.b, done);
}

// the coarse levels: the cluster kernel where the hierarchy allows, else the
// single-block kernel of the small levels
static void coarse_launch(const Mg &G, const int *done, cudaStream_t s, bool pdl = true);

static void small_launch(const Mg &G, const int *done, cudaStream_t s, bool pdl = true)
{
    auto k = G.lev[0].pz ? k_mg_small<true> : k_mg_small<false>;
    if (pdl) launch_pdl(k, dim3(1), dim3(kSmallThreads), G.small_smem, s, small_desc(G, done));
    else k<<<1, kSmallThreads, G.small_smem, s>>>(small_desc(G, done));
}

// the separable solve of the coarsest level, b -> x, in one block
static void fd_launch(const Mg &G, const int *done, cudaStream_t s, bool pdl)
{
    const MgLevel &L = G.lev[G.fd_level];
    FdDesc D{};
    D.n[0] = L.nx;
    D.n[1] = L.ny;
    D.n[2] = L.nz;
    for (int a = 0; a < 3; ++a) {
        D.v[a] = G.fd_v[a];
        D.lam[a] = G.fd_l[a];
    }
    D.null_mode = G.fd_null ? 1 : 0;
    const size_t sm = fd_smem(L.nx, L.ny, L.nz);
    if (pdl) launch_pdl(k_fd_block, dim3(1), dim3(kFdThreads), sm, s, D, (const float *)L.b, L.x, done);
    else k_fd_block<<<1, kFdThreads, sm, s>>>(D, L.b, L.x, done);
}

static void coarse_launch(const Mg &G, const int *done, cudaStream_t s, bool pdl)
{
    if (G.fd_level > 0) {
        fd_launch(G, done, s, pdl);
        return;
    }
    if (G.first_cluster == 0) {
        small_launch(G, done, s, pdl);
        return;
    }
    auto k = G.lev[0].pz ? k_mg_cluster<true> : k_mg_cluster<false>;
    if (pdl) launch_pdl(k, dim3(kClusterCtas), dim3(kClusterThreads), G.cluster_smem, s, cluster_desc(G, done));
    else k<<<kClusterCtas, kClusterThreads, G.cluster_smem, s>>>(cluster_desc(G, done));
}

// the CG's rho' can run inside the V-cycle's last launch: the finest level
// is a grid-wide float4 level smoothed by colour launches
bool mg_fuses_rho(const Mg &G)
{
    return mg_grid_levels(G) > 0 && G.lev[0].quads && G.lev[0].sweep_tj == 0;
}

// the levels that run grid-wide launches (before the cluster or small kernel)
int mg_grid_levels(const Mg &G) { return G.first_cluster > 0 ? G.first_cluster : G.first_small; }

// the post-smoothing of level l runs as tiles (never on the finest level)
static bool tiled_post(const Mg &G, int l) { return l > 0 && G.tile[l].tx > 0; }

// where level l's x ends after its post-smoothing (what the prolongation
// into level l - 1 reads)
static const float *level_out(const Mg &G, int l) { return tiled_post(G, l) ? G.lev[l].xalt : G.lev[l].x; }

// one smoothing phase of level l as tiles (k_mg_tile): the pre-smoothing
// with the restriction, or the post-smoothing with the prolongation; in one
// launch, or one sweep a launch where the level splits its phases (two
// sweeps: ZERO to x, READ_R x to xalt; then the prolongation xalt to x and
// READ x to xalt, so the level ends in xalt either way)
template <bool PZ>
static void tile_launch_t(const Mg &G, int l, bool pre, const int *done, cudaStream_t s)
{
    const MgLevel &L = G.lev[l];
    MgLevel C = G.lev[l + 1];
    if (!pre) C.x = const_cast<float *>(level_out(G, l + 1));
    auto go = [&](auto k, const MgTile &T, const float *xin, float *xout) {
        const dim3 grid((unsigned)((L.nx + T.tx - 1) / T.tx * T.tiles_y));
        launch_pdl(k, grid, dim3(kTileThreads), tile_smem(T), s, L, C, T, xin, xout, done);
    };
    if (!G.tile_split[l]) {
        if (pre) go(k_mg_tile<PZ, kTilePre>, G.tile[l], (const float *)L.x, L.x);
        else go(k_mg_tile<PZ, kTilePost>, G.tile[l], (const float *)L.x, L.xalt);
        return;
    }
    if (pre) {
        go(k_mg_tile<PZ, kTileZero>, G.tile[l], (const float *)L.x, L.x);
        go(k_mg_tile<PZ, kTileReadR>, G.tile_r[l], (const float *)L.x, L.xalt);
    } else {
        go(k_mg_tile<PZ, kTilePost>, G.tile[l], (const float *)L.xalt, L.x);
        go(k_mg_tile<PZ, kTileRead>, G.tile[l], (const float *)L.x, L.xalt);
    }
}

static void tile_launch(const Mg &G, int l, bool pre, const int *done, cudaStream_t s)
{
    if (G.lev[l].pz) tile_launch_t<true>(G, l, pre, done, s);
    else tile_launch_t<false>(G, l, pre, done, s);
}

// z = V(h): one V-cycle; every kernel returns at once when *done.  With
// rho_sc (done == &rho_sc->done) the CG's rho' = h . z and its scalar update
// run inside the last launch where the finest level is a grid-wide float4
// level; returns whether they did (else the caller runs k_mg_rho).
bool mg_vcycle(cfd_ctx *c, const int *done, BicgScal *rho_sc)
{
    Mg &G = c->mg;
    const cudaStream_t s = c->s;
    const int fs = mg_grid_levels(G);
    const bool fuse_rho = rho_sc && mg_fuses_rho(G);
    const RhoFuse rf{rho_sc, c->lc.partials, c->lc.counter, (long long)kMaxReduce * c->lc.red_blocks};
    for (int l = 0; l < fs; ++l) {
        const MgLevel &L = G.lev[l];
        if (G.tile[l].tx > 0) {
            tile_launch(G, l, true, done, s);
            continue;
        }
        smooth_phase(G, l, true, done, s);
        restrict_launch(G, L, G.lev[l + 1], done, s);
    }
    coarse_launch(G, done, s);
    for (int l = fs - 1; l >= 0; --l) {
        const MgLevel &L = G.lev[l];
        const float *xc = level_out(G, l + 1);
        if (tiled_post(G, l)) {
            tile_launch(G, l, false, done, s);
            continue;
        }
        if (fused_ends(G, l)) {
            if (int_index(L))
                launch_pdl(k_mg_prolong_first4<int>, dim3(nblk(L.n / 4)), dim3(kBlock), 0, s, L, G.lev[l + 1],
                           (const float *)L.b, L.x, xc, done);
            else
                launch_pdl(k_mg_prolong_first4<long long>, dim3(nblk(L.n / 4)), dim3(kBlock), 0, s, L, G.lev[l + 1],
                           (const float *)L.b, L.x, xc, done);
            smooth_phase(G, l, false, done, s, true, l == 0 && fuse_rho ? &rf : nullptr);
            continue;
        }
        if (transfers4(G, L, G.lev[l + 1]))
            launch_pdl(k_mg_prolong4, dim3(nblk(L.n / 4)), dim3(kBlock), 0, s, L, G.lev[l + 1], xc, L.x, done);
        else
            launch_pdl(k_mg_prolong, dim3(nblk(G.lev[l + 1].n)), dim3(kBlock), 0, s, L, G.lev[l + 1], xc, L.x, done);
        smooth_phase(G, l, false, done, s, false, l == 0 && fuse_rho ? &rf : nullptr);
    }
    c->launches += mg_vcycle_launches(G);
    return fuse_rho;
}

// one piece of the V-cycle for timing: 0 finest smoothing colour, 1 finest
// restriction, 2 finest prolongation, 3 small-level kernel, 4 whole V-cycle
void mg_time_part(cfd_ctx *c, int part)
{
    Mg &G = c->mg;
    const cudaStream_t s = c->s;
    const MgLevel &L = G.lev[0];
    const int *done = G.never;
    if (part == 0) smooth_launch(L, 0, 0, done, s);
    else if (part == 1) restrict_launch(G, L, G.lev[1], done, s, false);
    else if (part == 2 && transfers4(G, L, G.lev[1]))
        k_mg_prolong4<<<nblk(L.n / 4), kBlock, 0, s>>>(L, G.lev[1], G.lev[1].x, L.x, done);
    else if (part == 2) k_mg_prolong<<<nblk(G.lev[1].n), kBlock, 0, s>>>(L, G.lev[1], G.lev[1].x, L.x, done);
    else if (part == 3) coarse_launch(G, done, s, false);
    else if (part == 5) {
        if (L.sweep_tj > 0) sweep_launch(L, L.x, L.xalt, 0, 0, done, s);
    }
    else if (part == 4) mg_vcycle(c, done);
}

// kernel launches of one V-cycle
long long mg_vcycle_launches(const Mg &G)
{
    long long n = 1;  // the coarse solve
    for (int l = 0; l < mg_grid_levels(G); ++l) {
        const MgLevel &L = G.lev[l];
        const long long sw = level_sweeps(G, l), per_sweep = L.sweep_tj > 0 ? 1 : 2;
        // pre-smoothing and restriction: one tile launch; or 2s - 1 colour
        // launches (the first sweep in one) and the restriction; or s fused
        // sweeps or 2s colours and the restriction
        if (G.tile[l].tx > 0) n += G.tile_split[l] ? 2 : 1;
        else if (fused_ends(G, l)) n += 2 * sw;
        else n += per_sweep * sw + 1;
        // prolongation and post-smoothing: one tile launch; or the
        // prolongation with the first colour and 2s - 1 colours; or the
        // prolongation and the sweeps
        if (tiled_post(G, l)) n += G.tile_split[l] ? 2 : 1;
        else if (fused_ends(G, l)) n += 2 * sw;
        else n += 1 + per_sweep * sw;
    }
    return n;
}

void mg_h(cfd_ctx *c, float *h, const double *rn2, BicgScal *sc)
{
    const FvOp<float> F = fv32(c);
    launch_pdl(k_mg_h, dim3(c->lc.red_blocks), dim3(kBlock), 0, c->s, F, h, rn2, sc, c->lc.partials, c->lc.counter);
}

void mg_rho(cfd_ctx *c, const float *h, const float *z, float *p0, BicgScal *sc)
{
    launch_pdl(k_mg_rho, dim3(c->lc.red_blocks), dim3(kBlock), 0, c->s, c->g.n, h, z, p0, sc, c->lc.partials,
               c->lc.counter);
}

void mg_upd(cfd_ctx *c, float *e, const float *p, float *h, const float *q, BicgScal *sc, const float *p2)
{
    launch_pdl(k_mg_upd, dim3(c->lc.red_blocks), dim3(kBlock), 0, c->s, c->g.n, e, p, h, q, sc, c->lc.partials,
               c->lc.counter, p2);
}

// ---- the FP32 sweeps of the mixed-precision SOR ---------------------------
// The correction equation of the FP64 defect correction around SOR is
// sum_c e - sum_q c_q e_q = rho with the SOR coefficients c_q = area /
// staggered distance (SorPipeLine.seq.hpp:30-43) and e = 0 beyond the
// interior (the ghost pressures are fixed during a solve).  Divided by the
// cell volume it is the smoother's form e = (rho / dV + sum cm_q e_q) /
// sum cm_q with per-axis cm = 1 / (D_i Ds_{i-1}), cp = 1 / (D_i Ds_i): the
// boundary cells keep their coupling to the ghost in the diagonal, and the
// smoother reads no neighbour beyond the level.  So one SOR sweep in FP32 is
// the two colour passes of the level-0 smoother with relaxation omega.
int sor_level_setup(cfd_ctx *c, float omega)
{
    const Geo &g = c->g;
    MgLevel &L = c->sor_lev;
    const int n[3] = {g.nxc, g.nyc, g.nzc};
    const MgLevel old = L;
    L = MgLevel{};
    for (int a = 0; a < 3; ++a) L.cm[a] = old.cm[a];
    for (int a = 0; a < 3; ++a) {
        const std::vector<double> &D = c->hraw[3 + a], &Ds = c->hraw[6 + a];
        const int m = n[a];
        std::vector<float> all((size_t)5 * m);
        for (int i = 0; i < m; ++i) {
            const int gi = i + GC;
            const double cm = 1.0 / (D[gi] * Ds[gi - 1]), cp = 1.0 / (D[gi] * Ds[gi]);
            all[i] = (float)cm;
            all[m + i] = (float)cp;
            all[2 * m + i] = (float)(cm + cp);
            all[3 * m + i] = (float)D[gi];
            all[4 * m + i] = (float)(1.0 / D[gi]);
        }
        float *d = const_cast<float *>(L.cm[a]);  // new metrics reuse the tables
        if (!d) CKS(dalloc_t(c, &d, all.size()));
        CK(cudaMemcpy(d, all.data(), all.size() * sizeof(float), cudaMemcpyHostToDevice));
        L.cm[a] = d;
        L.cp[a] = d + m;
        L.sum[a] = d + 2 * m;
        L.w[a] = d + 3 * m;
        L.rw[a] = d + 4 * m;
    }
    L.nx = g.nxc; L.ny = g.nyc; L.nz = g.nzc; L.n = g.n;
    L.x = c->sor_e;
    L.b = c->sor_rho;
    L.om = omega;
    L.pz = 0;
    set_divs(L);
    L.rows2 = false;
    return CFD_OK;
}

// one FP32 SOR sweep (colour 0, then 1) of the correction; returns at once
// when *done
void sor_smooth_sweep(cfd_ctx *c, const int *done)
{
    smooth_launch(c->sor_lev, 0, 0, done, c->s);
    smooth_launch(c->sor_lev, 1, 0, done, c->s);
}

}  // namespace cfd
