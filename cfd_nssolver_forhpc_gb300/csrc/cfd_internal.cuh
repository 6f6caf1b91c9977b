// cfd_internal.cuh -- device-side building blocks shared by the kernels.
//
// Layout: every field keeps the reference's layout (k fastest).  Ghosted
// fields are nx*ny*nz with nx = nx_cal + 4 (two ghost layers, gC = 2,
// inc/grid/structureGrid.hpp:40); compact fields are nx_cal*ny_cal*nz_cal.
//
// Metrics live in per-axis tables of FieldCount rows; every division by a
// cell or staggered width of the reference becomes a multiplication by a
// reciprocal read from these tables (FP64 divides are slow on GB300), and the
// QUICK curvature factors 0.125*D*D/Ds of QuickUnitA/B
// (inc/source/convection_and_difussion.hpp:20-84) are tabulated with the
// reference's own evaluation order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <cstdlib>

namespace cfd {

// ---- programmatic dependent launch ------------------------------------------
// A kernel launched with launch_pdl may start while its predecessor in the
// stream is still running; it calls pdl_wait() before its first global
// memory access (which returns once the predecessor grid has completed and
// its writes are visible), then pdl_allow() so that its own successor may
// begin launching.  A kernel launched normally passes pdl_wait() at once.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_allow() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

// CFDGPU_NO_PDL=1 launches these kernels without the attribute (plain stream order)
inline bool pdl_enabled()
{
    static const bool on = [] {
        const char *e = std::getenv("CFDGPU_NO_PDL");
        return !(e && e[0] == '1');
    }();
    return on;
}

template <class... KArgs, class... Args>
inline void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl_enabled() ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

constexpr int GC = 2;
constexpr int kBlock = 256;
// values per block of the widest grid reduction; the partials buffer of a
// context holds kMaxReduce * red_blocks doubles
constexpr int kMaxReduce = 8;

// Division by a loop-invariant divisor d for dividends below 2^31:
// q = (umulhi(n, m) + n) >> s with s = ceil(log2 d) and
// m = 2^32 (2^s - d) / d + 1 (the round-up method for invariant integer
// division).  Replaces 64-bit integer divides in the row decompositions.
struct FastDiv {
    unsigned int d = 1, m = 1, s = 0;
    FastDiv() = default;
    __host__ explicit FastDiv(unsigned int dv) : d(dv ? dv : 1)
    {
        s = 0;
        while ((1ull << s) < d) ++s;
        m = (unsigned int)(((1ull << 32) * ((1ull << s) - d)) / d + 1);
    }
    __device__ __forceinline__ unsigned int div(unsigned int n) const { return (__umulhi(n, m) + n) >> s; }
};

struct Geo {
    int nx, ny, nz;       // ghosted
    int nxc, nyc, nzc;    // interior
    long long sx;         // ghosted i stride = ny*nz
    int sy;               // ghosted j stride = nz
    long long sxc;        // compact i stride = nyc*nzc
    int syc;              // compact j stride = nzc
    long long ng, n;      // ghosted and compact element counts
    FastDiv fsxc, fsyc;   // division by sxc and syc (n < 2^31)
    int pz;               // 1: periodic in z (the top w face is an unknown, z ghosts wrap)
    FastDiv fsx, fsy;     // division by the ghosted strides sx and sy (ng < 2^31 when used)
};

__host__ __device__ __forceinline__ long long icel(const Geo &g, int i, int j, int k)
{
    return (long long)i * g.sx + (long long)j * g.sy + k;
}
__host__ __device__ __forceinline__ long long icelcal(const Geo &g, int i, int j, int k)
{
    return (long long)(i - GC) * g.sxc + (long long)(j - GC) * g.syc + (k - GC);
}

// Per-axis metric table rows (table[row * n + index], n = ghosted length).
enum AxRow {
    AX_D = 0,   // cell width Dx
    AX_DS,      // staggered width Dxs
    AX_RD,      // 1 / Dx
    AX_RDS,     // 1 / Dxs
    AX_IT,      // face interpolation factor (Dxs*0.5)/Dx  (x_INTRPL, structureGrid.hpp:442)
    AX_CAPP,    // QuickUnitA, Up > 0:  0.125*D[i+1]*D[i+1]/Ds[i]
    AX_CAPN,    //             Up <= 0: 0.125*D[i+1]*D[i+1]/Ds[i+1]
    AX_CANP,    //             Un > 0:  0.125*D[i]*D[i]/Ds[i-1]
    AX_CANN,    //             Un <= 0: 0.125*D[i]*D[i]/Ds[i]
    AX_CBPP,    // QuickUnitB, Up > 0:  0.125*Ds[i]*Ds[i]/D[i]
    AX_CBPN,    //             Up <= 0: 0.125*Ds[i]*Ds[i]/D[i+1]
    AX_CBNP,    //             Un > 0:  0.125*Ds[i-1]*Ds[i-1]/D[i-1]
    AX_CBNN,    //             Un <= 0: 0.125*Ds[i-1]*Ds[i-1]/D[i]
    AX_PM,      // Poisson -face coefficient 1/D[i]/Ds[i-1], zero on the first cell
    AX_PP,      // Poisson +face coefficient 1/D[i]/Ds[i],   zero on the last cell
    AX_RDL,     // 1 / Dx - (float)(1 / Dx): with the FP32 AX_RD row, 1 / Dx as a float pair
    AX_DL,      // Dx - (float)Dx: with the FP32 AX_D row, Dx as a float pair
    AX_ROWS
};

template <class T>
struct Axis {
    const T *t;
    int n;
    __device__ __forceinline__ T operator()(int row, int i) const { return __ldg(t + row * n + i); }
};

template <class T>
struct Metrics {
    Axis<T> x, y, z;
};

// ---- float-float arithmetic ------------------------------------------------
// A value hi + lo of two FP32 numbers with |lo| <= ulp(hi) / 2 carries about
// 48 significant bits.  GB300 issues FP32 operations at many times its FP64
// rate, so kernels of the mixed-precision path that need more than FP32
// accuracy (the Poisson right-hand side, whose divergence of FP32 velocities
// must not lose the digits the FP64 defect correction solves for) use these
// error-free transformations (Knuth's two-sum, the fused multiply-add form of
// Dekker's two-product).  Every rounding step is an explicit _rn intrinsic,
// so the compiler cannot contract or reorder them.
struct ff {
    float hi, lo;
};
// the exact sum a + b as hi + lo
__device__ __forceinline__ ff ff_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
// the exact difference a - b
__device__ __forceinline__ ff ff_two_diff(float a, float b) { return ff_two_sum(a, -b); }
// renormalise s + t when |s| >= |t| (or s == 0)
__device__ __forceinline__ ff ff_fast(float s, float t)
{
    const float h = __fadd_rn(s, t);
    return {h, __fsub_rn(t, __fsub_rn(h, s))};
}
__device__ __forceinline__ ff ff_add(ff a, ff b)
{
    const ff s = ff_two_sum(a.hi, b.hi);
    return ff_fast(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ ff ff_mul(ff a, ff b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    const float e = __fmaf_rn(a.hi, b.hi, -p);  // the exact error of p
    const float t = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
    return ff_fast(p, t);
}
__device__ __forceinline__ ff ff_neg(ff a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }
// a double split into its nearest float and the float nearest the rest
__host__ __device__ inline ff ff_of(double v)
{
    const float h = (float)v;
    return {h, (float)(v - (double)h)};
}

// ---- deterministic grid reductions --------------------------------------
// Each block reduces NV values (warp shuffles, then warps in index order),
// writes them to partials[q * gridDim.x + blockIdx.x], and takes a ticket.
// The last block to arrive sums the partials in block order and returns
// true with the totals in tot[] (valid in every thread of that block).  The
// result does not depend on which block finishes last, so for a fixed launch
// shape the sums are bitwise reproducible.
template <int NV>
__device__ __forceinline__ void warp_sum(double (&v)[NV])
{
#pragma unroll
    for (int q = 0; q < NV; ++q)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], off);
}

// the last block's part of a grid reduction, after every block has written
// its partials and taken its ticket (last: this block's ticket was the last)
template <int NV>
__device__ __forceinline__ bool grid_reduce_tail(bool last, double *partials, unsigned int *counter,
                                                 double (&sm)[32][NV], double (&tot)[NV])
{
    if (!last) return false;
    __threadfence();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
    // four independent chains per thread, so the loads of a large grid's
    // partials are in flight together rather than one after another
    double s[NV];
    const int nb = (int)gridDim.x, bd = (int)blockDim.x;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        const double *pq = partials + q * gridDim.x;
        double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
        int b = threadIdx.x;
        for (; b + 3 * bd < nb; b += 4 * bd) {
            s0 += __ldcg(pq + b);
            s1 += __ldcg(pq + b + bd);
            s2 += __ldcg(pq + b + 2 * bd);
            s3 += __ldcg(pq + b + 3 * bd);
        }
        for (; b < nb; b += bd) s0 += __ldcg(pq + b);
        s[q] = (s0 + s1) + (s2 + s3);
    }
    warp_sum<NV>(s);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) sm[warp][q] = s[q];
    __syncthreads();
    if (warp == 0) {
        double w[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) w[q] = lane < nwarps ? sm[lane][q] : 0.0;
        warp_sum<NV>(w);
        if (lane == 0) {
#pragma unroll
            for (int q = 0; q < NV; ++q) sm[0][q] = w[q];
            *counter = 0u;
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NV; ++q) tot[q] = sm[0][q];
    return true;
}

template <int NV>
__device__ __forceinline__ bool grid_reduce(double (&v)[NV], double *partials,
                                            unsigned int *counter, double (&tot)[NV])
{
    static_assert(NV <= kMaxReduce, "wider than the partials buffer");
    __shared__ double sm[32][NV];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
    warp_sum<NV>(v);
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) sm[warp][q] = v[q];
    __syncthreads();
    if (warp == 0) {
        double w[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) w[q] = lane < nwarps ? sm[lane][q] : 0.0;
        warp_sum<NV>(w);
        if (lane == 0) {
#pragma unroll
            for (int q = 0; q < NV; ++q) partials[q * gridDim.x + blockIdx.x] = w[q];
            __threadfence();
            unsigned int t = atomicAdd(counter, 1u);
            last = (t == gridDim.x - 1);
        }
    }
    __syncthreads();
    return grid_reduce_tail<NV>(last, partials, counter, sm, tot);
}

// The same reduction for FP32 per-thread values: the block's tree runs in
// FP32 (warp shuffles, then the warps in index order; relative error of
// about log2(blockDim) roundings), and only the block totals, the partials,
// are FP64.  GB300 issues FP64 at 1/64 of the FP32 rate, so a double tree
// in every block is a measurable part of a short kernel.
template <int NV>
__device__ __forceinline__ bool grid_reduce_f(float (&v)[NV], double *partials, unsigned int *counter,
                                              double (&tot)[NV])
{
    static_assert(NV <= kMaxReduce, "wider than the partials buffer");
    __shared__ float smf[32][NV];
    __shared__ double sm[32][NV];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], off);
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) smf[warp][q] = v[q];
    __syncthreads();
    if (warp == 0) {
        float w[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) w[q] = lane < nwarps ? smf[lane][q] : 0.f;
#pragma unroll
        for (int q = 0; q < NV; ++q)
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) w[q] += __shfl_down_sync(0xffffffffu, w[q], off);
        if (lane == 0) {
#pragma unroll
            for (int q = 0; q < NV; ++q) partials[q * gridDim.x + blockIdx.x] = (double)w[q];
            __threadfence();
            unsigned int t = atomicAdd(counter, 1u);
            last = (t == gridDim.x - 1);
        }
    }
    __syncthreads();
    return grid_reduce_tail<NV>(last, partials, counter, sm, tot);
}

// The same last-block scheme for maxima (order-independent, so any launch
// shape gives the same result): the last block returns true with tot[].
template <int NV>
__device__ __forceinline__ void warp_max(double (&v)[NV])
{
#pragma unroll
    for (int q = 0; q < NV; ++q)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v[q] = fmax(v[q], __shfl_down_sync(0xffffffffu, v[q], off));
}

template <int NV>
__device__ __forceinline__ bool grid_reduce_max(double (&v)[NV], double *partials, unsigned int *counter,
                                                double (&tot)[NV])
{
    static_assert(NV <= kMaxReduce, "wider than the partials buffer");
    __shared__ double sm[32][NV];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
    warp_max<NV>(v);
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) sm[warp][q] = v[q];
    __syncthreads();
    if (warp == 0) {
        double w[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) w[q] = lane < nwarps ? sm[lane][q] : -INFINITY;
        warp_max<NV>(w);
        if (lane == 0) {
#pragma unroll
            for (int q = 0; q < NV; ++q) partials[q * gridDim.x + blockIdx.x] = w[q];
            __threadfence();
            unsigned int t = atomicAdd(counter, 1u);
            last = (t == gridDim.x - 1);
        }
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double s[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        s[q] = -INFINITY;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
            s[q] = fmax(s[q], __ldcg(partials + q * gridDim.x + b));
    }
    warp_max<NV>(s);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) sm[warp][q] = s[q];
    __syncthreads();
    if (warp == 0) {
        double w[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) w[q] = lane < nwarps ? sm[lane][q] : -INFINITY;
        warp_max<NV>(w);
        if (lane == 0) {
#pragma unroll
            for (int q = 0; q < NV; ++q) sm[0][q] = w[q];
            *counter = 0u;
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NV; ++q) tot[q] = sm[0][q];
    return true;
}

// Block-level max of a non-negative double folded into a global slot with an
// order-independent atomicMax on the bit pattern (non-negative IEEE doubles
// order like their unsigned bit patterns).  NaN propagates as the largest.
__device__ __forceinline__ void grid_max_nonneg(double v, unsigned long long *slot)
{
    __shared__ double sm[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
    unsigned long long b = (v != v) ? 0x7ff8000000000000ull : (unsigned long long)__double_as_longlong(v);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        unsigned long long o = __shfl_down_sync(0xffffffffu, b, off);
        b = o > b ? o : b;
    }
    if (lane == 0) sm[warp] = __longlong_as_double((long long)b);
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = lane < nwarps ? (unsigned long long)__double_as_longlong(sm[lane]) : 0ull;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            unsigned long long o = __shfl_down_sync(0xffffffffu, w, off);
            w = o > w ? o : w;
        }
        if (lane == 0 && w) atomicMax(slot, w);
    }
}

// ---- launch helpers ------------------------------------------------------
inline int blocks_for(long long n, int cap)
{
    long long b = (n + kBlock - 1) / kBlock;
    if (b < 1) b = 1;
    return (int)(b < cap ? b : cap);
}

}  // namespace cfd
