// context.h -- the library context (struct cfd_ctx) and the host helpers
// shared by the translation units of the C ABI (api.cu: forward path,
// adjoint_api.cu: discrete adjoint, checkpoints).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/cfdgpu.h"
#include "kernels.h"

namespace cfd {

// records msg as the thread's last error and returns code
int fail(int code, const std::string &msg);

#define CK(...)                                                                            \
    do {                                                                                   \
        cudaError_t e_ = (__VA_ARGS__);                                                    \
        if (e_ != cudaSuccess)                                                             \
            return fail(CFD_ERR_CUDA, std::string(#__VA_ARGS__) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define CKS(...)                        \
    do {                                \
        int st_ = (__VA_ARGS__);        \
        if (st_ != CFD_OK) return st_;  \
    } while (0)

template <class T>
struct Tag {
    using type = T;
};


}  // namespace cfd

struct AdjState;

namespace cfd {
// where a recorded forward step leaves its tape: the velocity T0 at the
// start of the step (3 ghosted fields of the context's velocity type) and the
// pressure the projection of each pass used (interior cells, compact)
struct StepRecord {
    void *T0[3];
    double *x[4];
};

// api.cu: the forward step with an optional tape, the CG-based linear solve
// with caller buffers, FP32 solver tables on demand
int step_recorded(cfd_ctx *c, cfd_step_info *info, const StepRecord *rec);
int linear_solve_cg(cfd_ctx *c, const double *b, double *x, const double *zero, int *iters, double *relres,
                    int *outer);
int ensure_fp32_solver(cfd_ctx *c);
// multigrid.cu: level set-up, V-cycle z = V(h), and the CG pieces around it
int mg_setup(cfd_ctx *c);
bool mg_vcycle(cfd_ctx *c, const int *done, BicgScal *rho_sc = nullptr);
bool mg_fuses_rho(const Mg &G);
int mg_grid_levels(const Mg &G);
int sor_level_setup(cfd_ctx *c, float omega);
void sor_smooth_sweep(cfd_ctx *c, const int *done);
void mg_h(cfd_ctx *c, float *h, const double *rn2, BicgScal *sc);
void mg_time_part(cfd_ctx *c, int part);
long long mg_vcycle_launches(const Mg &G);
void mg_rho(cfd_ctx *c, const float *h, const float *z, float *p0, BicgScal *sc);
void mg_upd(cfd_ctx *c, float *e, const float *p, float *h, const float *q, BicgScal *sc,
            const float *p2 = nullptr);
// adjoint_api.cu: releases the host side of the adjoint state
void adj_free(AdjState *a);

}  // namespace cfd

struct cfd_ctx {
    cfd_config cfg{};
    cfd::Geo g{};
    bool fp32 = false;
    cudaStream_t s = nullptr;
    cfd::cfd_launch_ctx lc{};
    std::vector<void *> allocs;

    // state (velocity type T = double or float)
    void *vel[3][3] = {};  // [slot 0/1/2 = T0/T1/T3][component]
    void *cdbuf[3] = {};   // the step's one convection-diffusion of T0 (predictor-corrector method)
    void *eta = nullptr, *f = nullptr, *src = nullptr;
    double *p = nullptr, *x = nullptr, *b = nullptr, *jp = nullptr;
    double *staging = nullptr;  // FP64 staging for conversions (mixed precision)

    // metrics: raw arrays (X,Y,Z,Dx,Dy,Dz,Dxs,Dys,Dzs) and per-axis tables
    double *raw = nullptr;
    double *rawp[9] = {};
    double *tab64[3] = {};
    float *tab32[3] = {};
    bool metrics = false;
    std::vector<double> hraw[9];

    // Poisson operators
    double *spe_c[3] = {};
    float *spe_c32[3] = {};
    float *jp32 = nullptr;
    float *jp32lo = nullptr;  // jp - jp32 as a float: jp as a float pair (mixed path's right-hand side)
    int *ell_cols = nullptr;
    double *ell_vals = nullptr;
    float *ell_vals32 = nullptr;

    // BiCGSTAB work
    cfd::BicgVecs<double> w64{};
    cfd::BicgVecs<float> w32{};
    double *px1 = nullptr, *px2 = nullptr;
    float *r32 = nullptr, *e32 = nullptr;
    float *p_alt = nullptr, *ap_alt = nullptr;  // second p/ap pair of the fused FP32 iteration
    float *fv_sum[3] = {};                      // per-axis [cm + cp | interior width] (FP32), CG inner solve
    float *cg_ip = nullptr;                     // 1 / diag(M) (FP32) of the CG inner solve
    cfd::CgTma cgtma{};                         // tensor maps of the TMA-fed CG stencil
    cfd::Mg mg{};                               // multigrid levels of the MG-preconditioned CG
    cfd::BicgScal sc_init{}, sc_in_init{};  // scalars of a fresh solver (cfd_start restores them)
    cfd::BicgScal *sc = nullptr, *sc_in = nullptr, *sc_t = nullptr, *h_sc = nullptr;
    cfd::OuterScal *os = nullptr, *h_os = nullptr;  // the defect correction's state (graph 6)
    cfd::OuterCfg outer_cfg[2] = {};                // ... the sweep parameters graphs 6 and 7 were built with
    const double *outer_b[2] = {};                  // ... and their right-hand side and solution buffers
    double *outer_x[2] = {};
    bool outer_graph = true;  // the mixed defect correction as one graph where it applies
    // warm start of the defect-correction solves of a step: per pass the
    // solutions of that pass in the last two steps (warm_n of them), from
    // which the next one starts by linear extrapolation in time
    double *warm_hist[4][3] = {};  // oldest first
    int warm_n[4] = {};
    bool warm_extrap = true;
    int warm_order = 1;  // 1: linear extrapolation (two steps), 2: quadratic (three)
    // [0] FP64 BiCGSTAB, [1] FP32 inner BiCGSTAB, [2] fused FP32 BiCGSTAB, [3] FP32 CG
    // [4] multigrid-preconditioned CG, [5] red-black SOR, [6] the mixed defect
    // correction around the multigrid CG (outer loop and inner solves) for the
    // context's own b and x, [7] the same for caller buffers (adjoint solves)
    static constexpr int kGraphs = 8;
    cudaGraphExec_t graph[kGraphs] = {};
    long long graph_batch[kGraphs] = {};  // shape key of each cached graph

    // SOR
    double *sor_cf = nullptr, *sor_rhs = nullptr;  // colour-split SOR coefficients and right-hand side
    cfd::SorAcc *sor_acc = nullptr;
    // mixed-precision SOR: the FP32 correction and its right-hand side (the
    // FP64 residual, both compact); null where the sweeps stay FP64
    float *sor_e = nullptr, *sor_rho = nullptr;
    cfd::MgLevel sor_lev{};  // the FP32 sweeps as the level-0 smoother (sor_level_setup)

    // scalars: [0] rhs mean, [1..2] cd/cl, [3] residual norm^2, [4] dot
    double *dscal = nullptr, *h_scal = nullptr;
    unsigned long long *dmax = nullptr, *h_max = nullptr;

    long long loop = 1;
    double time = 0.0;
    bool use_graphs = true;
    bool device_loops = true;  // solve loops as graph WHILE nodes (else host-polled graph batches)
    int debug = 0;
    bool fused = true;  // fused FP32 inner iterations (SPE operator)
    long long launches = 0;  // kernels issued by the step and solver paths
    int test_trip_cap = 0;   // > 0: cap on the body runs of every solve loop (cfd_set_test_limits)
    double vol_total = 0.0;  // interior volume of the grid (set with the metrics)
    // > 0: the inner tolerance of a defect-correction sweep is loosened to
    // inner_adapt * tol / (the relative residual before it) when that is
    // larger than inner_tol (at most 0.5): the last sweep stops once it has
    // the digits the outer test needs
    double inner_adapt = 0.2;
    bool div_check = false;  // cfd_set_step_divergence_check
    double last_div[3] = {-1.0, -1.0, -1.0};  // its result for the last step

    // inflow profile: per-j Dirichlet value of u on the x-min face (nullptr:
    // the scalar bc_dir[0][0]); a parameter of the adjoint
    double *inflow = nullptr;
    double *inflow_buf = nullptr;

    // monitors: reduction outputs (8 doubles) and the running extremes of
    // get_Cfl (the reference's simuClass::U_max / U_min / cfl_max persist
    // across calls), reset by cfd_start
    double *mon = nullptr;
    void *vis = nullptr;  // Smagorinsky eddy viscosity (compact, T), LES contexts only
    double run_umax[3] = {-1e10, -1e10, -1e10}, run_umin[3] = {1e10, 1e10, 1e10}, cfl_max = 0.0;
    AdjState *adj = nullptr;  // discrete-adjoint state (cfd_adj_enable)
};

namespace cfd {

template <class T>
T *dv(cfd_ctx *c, int slot, int comp)
{
    return static_cast<T *>(c->vel[slot][comp]);
}

inline int slot_index(int slot)
{
    return slot == CFD_SLOT_T0 ? 0 : slot == CFD_SLOT_T1 ? 1 : slot == CFD_SLOT_T3 ? 2 : -1;
}

inline int dalloc(cfd_ctx *c, void **p, size_t bytes)
{
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(CFD_ERR_NOMEM, std::string("cudaMalloc(") + std::to_string(bytes) +
                                       "): " + cudaGetErrorString(e));
    }
    c->allocs.push_back(*p);
    return CFD_OK;
}

template <class P>
inline int dalloc_t(cfd_ctx *c, P **p, size_t count)
{
    return dalloc(c, reinterpret_cast<void **>(p), count * sizeof(P));
}

template <class Fn>
auto dispatch(cfd_ctx *c, Fn &&fn)
{
    if (c->fp32) return fn(Tag<float>{});
    return fn(Tag<double>{});
}

template <class T>
Metrics<T> metrics_of(cfd_ctx *c);
template <>
inline Metrics<double> metrics_of<double>(cfd_ctx *c)
{
    return {{c->tab64[0], c->g.nx}, {c->tab64[1], c->g.ny}, {c->tab64[2], c->g.nz}};
}
template <>
inline Metrics<float> metrics_of<float>(cfd_ctx *c)
{
    return {{c->tab32[0], c->g.nx}, {c->tab32[1], c->g.ny}, {c->tab32[2], c->g.nz}};
}

inline SpeOp<double> spe64(cfd_ctx *c)
{
    const Geo &g = c->g;
    return {c->spe_c[0], c->spe_c[0] + g.nxc, c->spe_c[1], c->spe_c[1] + g.nyc, c->spe_c[2],
            c->spe_c[2] + g.nzc, c->jp, g.nxc, g.nyc, g.nzc, g.sxc, g.n, g.fsxc, FastDiv((unsigned int)g.nzc),
            g.pz};
}
inline SpeOp<float> spe32(cfd_ctx *c)
{
    const Geo &g = c->g;
    return {c->spe_c32[0], c->spe_c32[0] + g.nxc, c->spe_c32[1], c->spe_c32[1] + g.nyc, c->spe_c32[2],
            c->spe_c32[2] + g.nzc, c->jp32, g.nxc, g.nyc, g.nzc, g.sxc, g.n, g.fsxc,
            FastDiv((unsigned int)g.nzc), g.pz};
}
// interior cell widths of axis a (FP32 metric table row AX_D from the first
// interior cell)
inline const float *fv_width_src(cfd_ctx *c, int a)
{
    const int n[3] = {c->g.nx, c->g.ny, c->g.nz};
    return c->tab32[a] + (size_t)AX_D * n[a] + GC;
}

inline FvOp<float> fv32(cfd_ctx *c)
{
    const Geo &g = c->g;
    FvOp<float> F;
    F.A = spe32(c);
    F.wx = c->fv_sum[0] + g.nxc;
    F.wy = c->fv_sum[1] + g.nyc;
    F.wz = c->fv_sum[2] + g.nzc;
    F.sx = c->fv_sum[0];
    F.sy = c->fv_sum[1];
    F.sz = c->fv_sum[2];
    return F;
}
inline EllOp<double> ell64(cfd_ctx *c) { return {c->ell_cols, c->ell_vals, c->g.n}; }
inline EllOp<float> ell32(cfd_ctx *c) { return {c->ell_cols, c->ell_vals32, c->g.n}; }

// Per-axis tables (row-major [AX_ROWS][n]) from the cell and staggered
// widths, with the reference's evaluation order for every factor.
inline std::vector<double> axis_table(const std::vector<double> &D, const std::vector<double> &Ds)
{
    const int n = (int)D.size();
    std::vector<double> t((size_t)AX_ROWS * n, 0.0);
    auto T = [&](int r, int i) -> double & { return t[(size_t)r * n + i]; };
    for (int i = 0; i < n; ++i) {
        T(AX_D, i) = D[i];
        T(AX_DS, i) = Ds[i];
        T(AX_RD, i) = 1.0 / D[i];
        T(AX_RDS, i) = 1.0 / Ds[i];
        T(AX_IT, i) = (Ds[i] * 0.5) / D[i];
        if (i + 1 < n) {
            T(AX_CAPP, i) = 0.125 * D[i + 1] * D[i + 1] / Ds[i];
            T(AX_CAPN, i) = 0.125 * D[i + 1] * D[i + 1] / Ds[i + 1];
            T(AX_CBPN, i) = 0.125 * Ds[i] * Ds[i] / D[i + 1];
            T(AX_PP, i) = 1.0 / D[i] / Ds[i];
        }
        if (i >= 1) {
            T(AX_CANP, i) = 0.125 * D[i] * D[i] / Ds[i - 1];
            T(AX_CBNP, i) = 0.125 * Ds[i - 1] * Ds[i - 1] / D[i - 1];
            T(AX_CBNN, i) = 0.125 * Ds[i - 1] * Ds[i - 1] / D[i];
            T(AX_PM, i) = 1.0 / D[i] / Ds[i - 1];
        }
        T(AX_CANN, i) = 0.125 * D[i] * D[i] / Ds[i];
        T(AX_CBPP, i) = 0.125 * Ds[i] * Ds[i] / D[i];
        // low parts of 1 / D and D (float-float arithmetic of the mixed path)
        T(AX_RDL, i) = (double)(float)(T(AX_RD, i) - (double)(float)T(AX_RD, i));
        T(AX_DL, i) = (double)(float)(D[i] - (double)(float)D[i]);
    }
    return t;
}

inline BcTab bc_tab(const cfd_ctx *c)
{
    BcTab bc;
    for (int q = 0; q < 18; ++q) {
        bc.dir[q] = c->cfg.bc_dir[q / 3][q % 3];
        bc.num[q] = c->cfg.bc_num[q / 3][q % 3];
    }
    bc.inflow = c->inflow;
    bc.skip_outflow = 0;
    return bc;
}

inline int check_ctx(cfd_ctx *c)
{
    if (!c) return fail(CFD_ERR_ARG, "null context");
    return CFD_OK;
}

inline int need_metrics(cfd_ctx *c)
{
    CKS(check_ctx(c));
    if (!c->metrics) return fail(CFD_ERR_STATE, "grid metrics not set (cfd_grid_uniform / cfd_set_metrics)");
    return CFD_OK;
}

inline int check_slot(int slot)
{
    if (slot_index(slot) < 0) return fail(CFD_ERR_ARG, "velocity slot must be 0 (T0), 1 (T1) or 3 (T3)");
    return CFD_OK;
}

}  // namespace cfd
