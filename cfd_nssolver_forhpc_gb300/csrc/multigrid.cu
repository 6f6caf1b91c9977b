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
// before the coarse correction and black then red after it, so the V-cycle is
// a symmetric operator and CG keeps its short recurrences.  The coarsest
// level (a few dozen cells) has its mean removed (M is singular, constants
// are its null space) and is relaxed with symmetric sweeps.
//
// Levels above kMgSmall cells run as grid-wide kernels; the remaining small
// levels run inside one single-block kernel that performs their whole sub-
// cycle with block barriers, so a V-cycle is about 10 launches per large
// level plus one.
#include <cmath>
#include <cstring>
#include <vector>

#include "context.h"

using namespace cfd;

namespace {

inline int nblk(long long n) { return (int)((n + kBlock - 1) / kBlock); }

// one cell of the level operator: the neighbour sum and the diagonal of L
__device__ __forceinline__ void mg_cell(const MgLevel &L, const float *__restrict__ x, int i, int j, int k,
                                         long long t, float &nb, float &diag, float &dv)
{
    const long long sx = (long long)L.ny * L.nz, sy = L.nz;
    float s = 0.f;
    if (i > 0) s = fmaf(__ldg(L.cm[0] + i), x[t - sx], s);
    if (i < L.nx - 1) s = fmaf(__ldg(L.cp[0] + i), x[t + sx], s);
    if (j > 0) s = fmaf(__ldg(L.cm[1] + j), x[t - sy], s);
    if (j < L.ny - 1) s = fmaf(__ldg(L.cp[1] + j), x[t + sy], s);
    if (k > 0) s = fmaf(__ldg(L.cm[2] + k), x[t - 1], s);
    if (k < L.nz - 1) s = fmaf(__ldg(L.cp[2] + k), x[t + 1], s);
    nb = s;
    diag = __ldg(L.sum[0] + i) + __ldg(L.sum[1] + j) + __ldg(L.sum[2] + k);
    dv = __ldg(L.w[0] + i) * __ldg(L.w[1] + j) * __ldg(L.w[2] + k);
}

__device__ __forceinline__ void decomp(const MgLevel &L, long long t, int &i, int &j, int &k)
{
    const unsigned u = (unsigned)t;
    const unsigned ii = L.fyz.div(u), r = u - ii * (unsigned)(L.ny * L.nz), jj = L.fz.div(r);
    i = (int)ii;
    j = (int)jj;
    k = (int)(r - jj * (unsigned)L.nz);
}

// one colour of a Gauss-Seidel sweep over cells [t0, n) with stride; with
// zero_init the level starts from x = 0 (neighbours read as 0, the other
// colour written as 0)
__device__ __forceinline__ void smooth_cells(const MgLevel &L, const float *__restrict__ b, float *__restrict__ x,
                                             int color, bool zero_init, long long t0, long long stride)
{
    for (long long t = t0; t < L.n; t += stride) {
        int i, j, k;
        decomp(L, t, i, j, k);
        if (((i + j + k) & 1) != color) {
            if (zero_init) x[t] = 0.f;
            continue;
        }
        float nb, diag, dv;
        if (zero_init) {
            nb = 0.f;
            diag = __ldg(L.sum[0] + i) + __ldg(L.sum[1] + j) + __ldg(L.sum[2] + k);
            dv = __ldg(L.w[0] + i) * __ldg(L.w[1] + j) * __ldg(L.w[2] + k);
        } else {
            mg_cell(L, x, i, j, k, t, nb, diag, dv);
        }
        x[t] = (b[t] / dv + nb) / diag;
    }
}

// coarse b = sum over the children of (b - M x) on the fine level
__device__ __forceinline__ void restrict_cells(const MgLevel &F, const MgLevel &C, const float *__restrict__ bf,
                                               const float *__restrict__ xf, float *__restrict__ bc, long long t0,
                                               long long stride)
{
    const int fx = F.nx / C.nx, fy = F.ny / C.ny, fz = F.nz / C.nz;
    for (long long T = t0; T < C.n; T += stride) {
        int I, J, K;
        decomp(C, T, I, J, K);
        float s = 0.f;
        for (int a = 0; a < fx; ++a)
            for (int b2 = 0; b2 < fy; ++b2)
                for (int c = 0; c < fz; ++c) {
                    const int i = fx * I + a, j = fy * J + b2, k = fz * K + c;
                    const long long t = ((long long)i * F.ny + j) * F.nz + k;
                    float nb, diag, dv;
                    mg_cell(F, xf, i, j, k, t, nb, diag, dv);
                    s += bf[t] - dv * (diag * xf[t] - nb);
                }
        bc[T] = s;
    }
}

// fine x += coarse x of the parent cell
__device__ __forceinline__ void prolong_cells(const MgLevel &F, const MgLevel &C, const float *__restrict__ xc,
                                              float *__restrict__ xf, long long t0, long long stride)
{
    const int fx = F.nx / C.nx, fy = F.ny / C.ny, fz = F.nz / C.nz;
    for (long long t = t0; t < F.n; t += stride) {
        int i, j, k;
        decomp(F, t, i, j, k);
        xf[t] += xc[((long long)(i / fx) * C.ny + j / fy) * C.nz + k / fz];
    }
}

__global__ void __launch_bounds__(kBlock) k_mg_smooth(MgLevel L, const float *b, float *x, int color, int zero_init,
                                                      const int *done)
{
    if (*done) return;
    smooth_cells(L, b, x, color, zero_init != 0, (long long)blockIdx.x * blockDim.x + threadIdx.x,
                 (long long)gridDim.x * blockDim.x);
}

__global__ void __launch_bounds__(kBlock) k_mg_restrict(MgLevel F, MgLevel C, const float *bf, const float *xf,
                                                        float *bc, const int *done)
{
    if (*done) return;
    restrict_cells(F, C, bf, xf, bc, (long long)blockIdx.x * blockDim.x + threadIdx.x,
                   (long long)gridDim.x * blockDim.x);
}

__global__ void __launch_bounds__(kBlock) k_mg_prolong(MgLevel F, MgLevel C, const float *xc, float *xf,
                                                       const int *done)
{
    if (*done) return;
    prolong_cells(F, C, xc, xf, (long long)blockIdx.x * blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
}

constexpr int kSmallThreads = 1024;

// the whole sub-cycle of levels first..last-1 (the coarsest is last-1) in one
// block: pre-smooth and restrict down, relax the coarsest, prolong and
// post-smooth up; block barriers between the phases
__global__ void __launch_bounds__(kSmallThreads) k_mg_small(MgSmall S)
{
    if (*S.done) return;
    const long long t0 = threadIdx.x, st = blockDim.x;
    const int first = S.first, last = S.nlev;
    for (int l = first; l < last - 1; ++l) {
        const MgLevel &L = S.lev[l];
        for (int s = 0; s < S.pre; ++s) {
            smooth_cells(L, L.b, L.x, 0, s == 0, t0, st);
            __syncthreads();
            smooth_cells(L, L.b, L.x, 1, false, t0, st);
            __syncthreads();
        }
        restrict_cells(L, S.lev[l + 1], L.b, L.x, S.lev[l + 1].b, t0, st);
        __syncthreads();
    }
    // coarsest: remove the mean of b (the null space of M), then symmetric
    // sweeps from zero
    {
        const MgLevel &L = S.lev[last - 1];
        __shared__ float red[kSmallThreads / 32];
        float s = 0.f;
        for (long long t = t0; t < L.n; t += st) s += L.b[t];
        for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
        __syncthreads();
        float tot = 0.f;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) tot += red[q];
        const float mean = tot / (float)L.n;
        for (long long t = t0; t < L.n; t += st) L.b[t] -= mean;
        __syncthreads();
        for (int s2 = 0; s2 < S.coarse; ++s2) {
            smooth_cells(L, L.b, L.x, 0, s2 == 0, t0, st);
            __syncthreads();
            smooth_cells(L, L.b, L.x, 1, false, t0, st);
            __syncthreads();
        }
        for (int s2 = 0; s2 < S.coarse; ++s2) {
            smooth_cells(L, L.b, L.x, 1, false, t0, st);
            __syncthreads();
            smooth_cells(L, L.b, L.x, 0, false, t0, st);
            __syncthreads();
        }
    }
    for (int l = last - 2; l >= first; --l) {
        const MgLevel &L = S.lev[l];
        prolong_cells(L, S.lev[l + 1], S.lev[l + 1].x, L.x, t0, st);
        __syncthreads();
        for (int s = 0; s < S.post; ++s) {
            smooth_cells(L, L.b, L.x, 1, false, t0, st);
            __syncthreads();
            smooth_cells(L, L.b, L.x, 0, false, t0, st);
            __syncthreads();
        }
    }
}

// ---- CG with the V-cycle preconditioner -------------------------------------
// h = P r (in place): the Jacobi-scaled residual in the finite-volume form
__global__ void k_mg_h(FvOp<float> F, float *__restrict__ h)
{
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < F.A.n;
         row += (long long)gridDim.x * blockDim.x) {
        const int nz = F.A.nzc, nyz = F.A.nyc * F.A.nzc;
        const int i = (int)(row / nyz), r2 = (int)(row - (long long)i * nyz), j = r2 / nz, k = r2 - j * nz;
        const float dv = __ldg(F.wx + i) * (__ldg(F.wy + j) * __ldg(F.wz + k));
        h[row] = dv * (__ldg(F.sx + i) + (__ldg(F.sy + j) + __ldg(F.sz + k))) * h[row];
    }
}

// rho = h . z; with p0 != null also p0 = z and the solve's initial scalars
__global__ void __launch_bounds__(kBlock)
k_mg_rho(long long n, const float *__restrict__ h, const float *__restrict__ z, float *__restrict__ p0, BicgScal *sc,
         double *partials, unsigned int *counter)
{
    if (!p0 && sc->done) return;
    float pa = 0.f;
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x) {
        const float zv = z[r];
        if (p0) p0[r] = zv;
        pa = fmaf(h[r], zv, pa);
    }
    double acc[1] = {(double)pa}, tot[1];
    if (!grid_reduce<1>(acc, partials, counter, tot) || threadIdx.x != 0) return;
    if (p0) {
        sc->rho = tot[0];
        sc->r0n2 = fabs(tot[0]);
        sc->norm0 = sqrt(fabs(tot[0]));
        sc->iter = 0;
        sc->restart = 0;
        sc->timestep += 1;
        sc->done = tot[0] != 0.0 ? BICG_RUNNING : BICG_ZERO_RHS;
        sc->relres = tot[0] != 0.0 ? 1.0 : 0.0;
        sc->wait_timeout = 0;
        return;
    }
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

// e += alpha p, h -= alpha q (no reduction: rho comes after the V-cycle)
__global__ void __launch_bounds__(kBlock) k_mg_upd(long long n, float *__restrict__ e, const float *__restrict__ p,
                                                   float *__restrict__ h, const float *__restrict__ q, const BicgScal *sc)
{
    if (sc->done) return;
    const float alpha = (float)sc->alpha;
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x) {
        e[r] = fmaf(alpha, p[r], e[r]);
        h[r] = fmaf(-alpha, q[r], h[r]);
    }
}

}  // namespace

namespace cfd {

// host set-up of the level hierarchy below level 0 (the CG's own operator)
int mg_setup(cfd_ctx *c)
{
    Mg &G = c->mg;
    if (G.nlev > 0) return CFD_OK;
    const Geo &g = c->g;
    // level 0: the FP32 finite-volume operator of the CG
    const FvOp<float> F = fv32(c);
    MgLevel L0{};
    L0.nx = g.nxc; L0.ny = g.nyc; L0.nz = g.nzc; L0.n = g.n;
    L0.cm[0] = F.A.cxm; L0.cp[0] = F.A.cxp; L0.sum[0] = F.sx; L0.w[0] = F.wx;
    L0.cm[1] = F.A.cym; L0.cp[1] = F.A.cyp; L0.sum[1] = F.sy; L0.w[1] = F.wy;
    L0.cm[2] = F.A.czm; L0.cp[2] = F.A.czp; L0.sum[2] = F.sz; L0.w[2] = F.wz;
    L0.x = c->w32.r0;  // z
    L0.b = c->r32;     // h
    L0.fyz = FastDiv((unsigned)(g.nyc * g.nzc));
    L0.fz = FastDiv((unsigned)g.nzc);
    G.lev[0] = L0;
    // interior widths (FP64) of level 0, then halve while possible
    std::vector<double> W[3];
    const int n0[3] = {g.nxc, g.nyc, g.nzc};
    for (int a = 0; a < 3; ++a) {
        W[a].resize(n0[a]);
        for (int i = 0; i < n0[a]; ++i) W[a][i] = c->hraw[3 + a][i + GC];
    }
    int nl = 1;
    int n[3] = {g.nxc, g.nyc, g.nzc};
    while (nl < kMgMaxLevels) {
        long long cells = (long long)n[0] * n[1] * n[2];
        if (cells <= 32) break;
        int f[3];
        bool any = false;
        for (int a = 0; a < 3; ++a) {
            f[a] = (n[a] % 2 == 0 && n[a] >= 4) ? 2 : 1;
            any = any || f[a] == 2;
        }
        if (!any) break;
        MgLevel L{};
        std::vector<float> host;
        for (int a = 0; a < 3; ++a) {
            std::vector<double> Wc(n[a] / f[a]);
            for (size_t I = 0; I < Wc.size(); ++I) Wc[I] = f[a] == 2 ? W[a][2 * I] + W[a][2 * I + 1] : W[a][I];
            W[a] = Wc;
            n[a] = (int)Wc.size();
        }
        L.nx = n[0]; L.ny = n[1]; L.nz = n[2];
        L.n = (long long)n[0] * n[1] * n[2];
        L.fyz = FastDiv((unsigned)(n[1] * n[2]));
        L.fz = FastDiv((unsigned)n[2]);
        for (int a = 0; a < 3; ++a) {
            const int m = n[a];
            std::vector<float> cm(m, 0.f), cp(m, 0.f), sm(m, 0.f), w(m, 0.f);
            for (int i = 0; i < m; ++i) {
                w[i] = (float)W[a][i];
                if (i > 0) cm[i] = (float)(1.0 / (W[a][i] * 0.5 * (W[a][i - 1] + W[a][i])));
                if (i < m - 1) cp[i] = (float)(1.0 / (W[a][i] * 0.5 * (W[a][i] + W[a][i + 1])));
                sm[i] = cm[i] + cp[i];
            }
            float *d = nullptr;
            CKS(dalloc_t(c, &d, (size_t)4 * m));
            std::vector<float> all;
            all.insert(all.end(), cm.begin(), cm.end());
            all.insert(all.end(), cp.begin(), cp.end());
            all.insert(all.end(), sm.begin(), sm.end());
            all.insert(all.end(), w.begin(), w.end());
            CK(cudaMemcpy(d, all.data(), all.size() * sizeof(float), cudaMemcpyHostToDevice));
            L.cm[a] = d; L.cp[a] = d + m; L.sum[a] = d + 2 * m; L.w[a] = d + 3 * m;
        }
        CKS(dalloc_t(c, &L.x, (size_t)L.n));
        CKS(dalloc_t(c, &L.b, (size_t)L.n));
        G.lev[nl++] = L;
    }
    G.nlev = nl;
    G.first_small = nl;
    for (int l = 0; l < nl; ++l)
        if (G.lev[l].n <= kMgSmall) {
            G.first_small = l;
            break;
        }
    // usable when there is a coarse level and the coarsest fits the one-block kernel
    G.usable = nl > 1 && G.first_small < nl;
    CKS(dalloc_t(c, &G.never, 1));
    CK(cudaMemset(G.never, 0, sizeof(int)));
    return CFD_OK;
}

// z = V(h): one V-cycle (pre = post = 2 sweeps on the large levels); every
// kernel returns at once when the solve is done
void mg_vcycle(cfd_ctx *c, const int *done)
{
    Mg &G = c->mg;
    const cudaStream_t s = c->s;
    const int fs = G.first_small;
    for (int l = 0; l < fs; ++l) {
        const MgLevel &L = G.lev[l];
        for (int q = 0; q < 2; ++q) {
            k_mg_smooth<<<nblk(L.n), kBlock, 0, s>>>(L, L.b, L.x, 0, q == 0, done);
            k_mg_smooth<<<nblk(L.n), kBlock, 0, s>>>(L, L.b, L.x, 1, 0, done);
        }
        k_mg_restrict<<<nblk(G.lev[l + 1].n), kBlock, 0, s>>>(L, G.lev[l + 1], L.b, L.x, G.lev[l + 1].b, done);
    }
    {
        MgSmall S{};
        S.done = done;
        S.first = fs;
        S.nlev = G.nlev;
        S.pre = 2;
        S.post = 2;
        S.coarse = 24;
        for (int l = 0; l < G.nlev; ++l) S.lev[l] = G.lev[l];
        k_mg_small<<<1, kSmallThreads, 0, s>>>(S);
    }
    for (int l = fs - 1; l >= 0; --l) {
        const MgLevel &L = G.lev[l];
        k_mg_prolong<<<nblk(L.n), kBlock, 0, s>>>(L, G.lev[l + 1], G.lev[l + 1].x, L.x, done);
        for (int q = 0; q < 2; ++q) {
            k_mg_smooth<<<nblk(L.n), kBlock, 0, s>>>(L, L.b, L.x, 1, 0, done);
            k_mg_smooth<<<nblk(L.n), kBlock, 0, s>>>(L, L.b, L.x, 0, 0, done);
        }
    }
    c->launches += 10LL * fs + 1;
}

void mg_h(cfd_ctx *c, float *h)
{
    const FvOp<float> F = fv32(c);
    k_mg_h<<<blocks_for(F.A.n, c->lc.grid_cap), kBlock, 0, c->s>>>(F, h);
}

void mg_rho(cfd_ctx *c, const float *h, const float *z, float *p0, BicgScal *sc)
{
    k_mg_rho<<<c->lc.red_blocks, kBlock, 0, c->s>>>(c->g.n, h, z, p0, sc, c->lc.partials, c->lc.counter);
}

void mg_upd(cfd_ctx *c, float *e, const float *p, float *h, const float *q, const BicgScal *sc)
{
    k_mg_upd<<<blocks_for(c->g.n, c->lc.grid_cap), kBlock, 0, c->s>>>(c->g.n, e, p, h, q, sc);
}

}  // namespace cfd
