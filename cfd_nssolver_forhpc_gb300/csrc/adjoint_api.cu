// adjoint_api.cu -- C ABI of the discrete adjoint (include/cfdgpu.h):
// adjoint state, kernel-level adjoint entry points, the step tape with its
// replay, checkpoints of the forward state, and the checkpointed reverse
// time stepping of the mean-drag objective.
//
// The adjoint of one predictor-corrector step (RUN_CPU_PC_METHOD.hpp:287-627;
// the plain driver is the one-pass case) runs the forward operations in
// reverse:
//   Cd/Cl -> BC_staggered_copy -> BC_staggered_main -> (T0 = T3) ->
//   for pass 3..0: [src += dt f] -> update_UandF -> Pressure_transform ->
//                  solve -> createBMatrix -> source add -> ConvectionDifussion
//   -> (src = 0)
// Every pass reads the convection-diffusion of the same T0, so the adjoints
// of its four outputs are summed and transposed once per step.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "context.h"

using namespace cfd;

struct Checkpoint {
    void *T[2][3] = {};  // T0, T1
    double *p = nullptr, *x = nullptr, *px1 = nullptr, *px2 = nullptr;
    BicgScal *sc = nullptr, *sc_in = nullptr;
    long long loop = 1;
    double time = 0.0;
    bool valid = false;
};

struct AdjState {
    double *a0[3] = {}, *a1[3] = {}, *a3[3] = {}, *acd[3] = {};
    double *ax = nullptr, *ab = nullptr, *aw = nullptr, *bp = nullptr, *zero = nullptr, *pint = nullptr;
    double *af = nullptr, *asrc = nullptr, *aeta = nullptr, *ainflow = nullptr;
    double *red = nullptr;
    // warm start of the adjoint Poisson solve of pass k: its solutions of the
    // two steps after this one (the reverse sweep's previous two), extrapolated
    double *awh[4][2] = {};
    int awn[4] = {};
    // replay of one step (forward velocity type)
    void *snap[4][3] = {};
    void *rT3[3] = {};
    void *rf = nullptr, *rsrc = nullptr;
    double *rp = nullptr;
    // tape
    int tape_len = 0;
    std::vector<void *> tape_T0;     // [pos * 3 + q]
    std::vector<double *> tape_x;    // [pos * 4 + pass]
    std::vector<long long> tape_loop;
    std::vector<Checkpoint> ck;
    long long solve_iters = 0;
    // the checkpointed run of cfd_adj_forward, reversed by cfd_adj_reverse
    cfd_adj_run_config run{};
    int run_nseg = 0;
    bool run_ready = false;
};

namespace cfd {
void adj_free(AdjState *a) { delete a; }
}

namespace {

int need_adj(cfd_ctx *c)
{
    CKS(need_metrics(c));
    if (!c->adj) return fail(CFD_ERR_STATE, "adjoint not enabled (cfd_adj_enable)");
    return CFD_OK;
}

size_t adj_count(const cfd_ctx *c, int field)
{
    if (field >= CFD_ADJ_U0 && field <= CFD_ADJ_CDW) return (size_t)c->g.ng;
    if (field == CFD_ADJ_X || field == CFD_ADJ_B) return (size_t)c->g.n;
    if (field == CFD_ADJ_F || field == CFD_ADJ_SRC) return (size_t)(3 * c->g.n);
    if (field == CFD_ADJ_ETA) return (size_t)c->g.ng;
    if (field == CFD_ADJ_INFLOW) return (size_t)c->g.nyc;
    return 0;
}

double *adj_ptr(cfd_ctx *c, int field)
{
    AdjState &A = *c->adj;
    if (field >= CFD_ADJ_U0 && field <= CFD_ADJ_W0) return A.a0[field - CFD_ADJ_U0];
    if (field >= CFD_ADJ_U1 && field <= CFD_ADJ_W1) return A.a1[field - CFD_ADJ_U1];
    if (field >= CFD_ADJ_U3 && field <= CFD_ADJ_W3) return A.a3[field - CFD_ADJ_U3];
    if (field >= CFD_ADJ_CDU && field <= CFD_ADJ_CDW) return A.acd[field - CFD_ADJ_CDU];
    switch (field) {
    case CFD_ADJ_X: return A.ax;
    case CFD_ADJ_B: return A.ab;
    case CFD_ADJ_F: return A.af;
    case CFD_ADJ_SRC: return A.asrc;
    case CFD_ADJ_ETA: return A.aeta;
    case CFD_ADJ_INFLOW: return A.ainflow;
    default: return nullptr;
    }
}

int zero_adjoint(cfd_ctx *c)
{
    AdjState &A = *c->adj;
    for (int f = CFD_ADJ_U0; f <= CFD_ADJ_INFLOW; ++f)
        CK(cudaMemsetAsync(adj_ptr(c, f), 0, adj_count(c, f) * sizeof(double), c->s));
    CK(cudaMemsetAsync(A.aw, 0, (size_t)c->g.n * sizeof(double), c->s));
    for (int &k : A.awn) k = 0;
    A.solve_iters = 0;
    return CFD_OK;
}

int alloc_tape(cfd_ctx *c, int len)
{
    AdjState &A = *c->adj;
    const Geo &g = c->g;
    const size_t ts = c->fp32 ? sizeof(float) : sizeof(double);
    const int old = A.tape_len;
    A.tape_T0.resize((size_t)len * 3, nullptr);
    A.tape_x.resize((size_t)len * 4, nullptr);
    A.tape_loop.resize((size_t)len, 0);
    for (int pos = old; pos < len; ++pos) {
        for (int q = 0; q < 3; ++q) CKS(dalloc(c, &A.tape_T0[(size_t)pos * 3 + q], (size_t)g.ng * ts));
        for (int k = 0; k < 4; ++k) CKS(dalloc_t(c, &A.tape_x[(size_t)pos * 4 + k], (size_t)g.n));
    }
    A.tape_len = len;
    return CFD_OK;
}

// adjoint Poisson solve: ab = A^-T ax on the range of the operator.  pass >= 0:
// the solve of that pass in the reverse sweep, started from the same pass's
// solutions of the two steps after this one extrapolated (the forward's warm
// start run backwards in time; CFDGPU_WARM=prev: the previous solve's)
int adj_solve(cfd_ctx *c, int *iters, double *relres, int pass = -1)
{
    AdjState &A = *c->adj;
    const Metrics<double> m = metrics_of<double>(c);
    const long long n = c->g.n;
    launch_adj_solve_in(c->lc, c->g, m, c->jp, A.ax, A.red, A.bp);
    c->launches += 2;
    CK(cudaGetLastError());
    const bool warm = pass >= 0 && pass < 4 && c->warm_extrap;
    if (warm && !A.awh[pass][0]) {
        for (int q = 0; q < 2; ++q) CKS(dalloc_t(c, &A.awh[pass][q], (size_t)n));
        A.awn[pass] = 0;
    }
    if (warm && A.awn[pass] >= 2) {
        launch_extrapolate(c->lc, n, A.aw, A.awh[pass][0], A.awh[pass][1]);
        c->launches += 1;
        CK(cudaGetLastError());
    } else if (warm && A.awn[pass] == 1) {
        CK(cudaMemcpyAsync(A.aw, A.awh[pass][1], (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, c->s));
    }
    int it = 0, outer = 0;
    double rr = 0.0;
    const int st = linear_solve_cg(c, A.bp, A.aw, A.zero, &it, &rr, &outer);
    if (st != CFD_OK && st != CFD_ERR_NOCONV) return st;
    if (warm && st == CFD_OK) {
        std::swap(A.awh[pass][0], A.awh[pass][1]);
        CK(cudaMemcpyAsync(A.awh[pass][1], A.aw, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, c->s));
        A.awn[pass] = std::min(2, A.awn[pass] + 1);
    }
    launch_adj_solve_out(c->lc, c->g, m, c->jp, A.aw, A.red, A.ab);
    c->launches += 2;
    CK(cudaGetLastError());
    A.solve_iters += it;
    if (iters) *iters = it;
    if (relres) *relres = rr;
    return st;
}

template <class T>
T *tape_T0(AdjState &A, int pos, int q)
{
    return static_cast<T *>(A.tape_T0[(size_t)pos * 3 + q]);
}

// Reverse of the step recorded at tape position pos.
template <class T>
int adj_step_t(cfd_ctx *c, int pos, double wcd, double wcl, cfd_adj_step_info *info)
{
    AdjState &A = *c->adj;
    const Geo &g = c->g;
    const cudaStream_t s = c->s;
    const bool pc = c->cfg.method == CFD_METHOD_PC;
    const bool aligned = c->cfg.aligned_source != 0;
    const int npass = pc ? 4 : 1;
    const Metrics<T> mT = metrics_of<T>(c);
    const Metrics<double> m = metrics_of<double>(c);
    const double dt = c->cfg.dt, nudt = (1.0 / c->cfg.re) * c->cfg.dt;
    const T dtT = (T)dt, nudtT = (T)nudt;
    const size_t fb = (size_t)g.ng * sizeof(T);
    const T *T0[3] = {tape_T0<T>(A, pos, 0), tape_T0<T>(A, pos, 1), tape_T0<T>(A, pos, 2)};
    double *const *X = &A.tape_x[(size_t)pos * 4];
    const T *eta = static_cast<const T *>(c->eta);
    T *rsrc = static_cast<T *>(A.rsrc), *rf = static_cast<T *>(A.rf);
    auto S = [&](int k, int q) { return static_cast<T *>(A.snap[k][q]); };
    auto R3 = [&](int q) { return static_cast<T *>(A.rT3[q]); };

    // replay: T1 of every pass (the scrambled source coupling accumulates in
    // elements the convection-diffusion does not write, so passes chain)
    if (pc) CK(cudaMemsetAsync(rsrc, 0, (size_t)(3 * g.n) * sizeof(T), s));
    for (int k = 0; k < npass; ++k) {
        for (int q = 0; q < 3; ++q)
            CK(cudaMemcpyAsync(S(k, q), k == 0 ? T0[q] : S(k - 1, q), fb, cudaMemcpyDeviceToDevice, s));
        launch_convdiff<T>(s, g, mT, dtT, nudtT, T0[0], T0[1], T0[2], S(k, 0), S(k, 1), S(k, 2),
                           (pc && aligned && k > 0) ? rsrc : nullptr);
        if (pc && !aligned) launch_src_add<T>(c->lc, g, 0, S(k, 0), S(k, 1), S(k, 2), rsrc);
        launch_transform(s, g, X[k], A.rp);
        launch_update_uf<T>(s, g, mT, dt, (T)(1.0 / dt), A.rp, eta, S(k, 0), S(k, 1), S(k, 2), R3(0), R3(1),
                            R3(2), rf);
        if (pc && k < npass - 1) launch_src_accumulate<T>(c->lc, 3 * g.n, dtT, rsrc, rf);
        c->launches += 3 + ((pc && !aligned) ? 1 : 0) + ((pc && k < npass - 1) ? 1 : 0);
    }
    CK(cudaGetLastError());

    // reverse
    launch_adj_bc_copy(s, g, A.a0[0], A.a0[1], A.a0[2], A.a1[0], A.a1[1], A.a1[2]);
    launch_adj_bc_main(s, g, bc_tab(c), A.a0[0], A.a0[1], A.a0[2], A.ainflow);
    c->launches += 4;
    cfd_adj_step_info loc{};
    int st = CFD_OK;
    for (int k = npass - 1; k >= 0; --k) {
        UfAdjArgs U{};
        U.x = X[k];
        for (int d = 0; d < 3; ++d) {
            U.a3[d] = k == npass - 1 ? A.a0[d] : nullptr;  // T0 = T3 after the last pass
            U.a1[d] = A.a1[d];
        }
        U.af = nullptr;
        U.asrc = (pc && k < npass - 1) ? A.asrc : nullptr;
        U.src_dt = dt;
        U.wcd = k == npass - 1 ? wcd : 0.0;
        U.wcl = k == npass - 1 ? wcl : 0.0;
        U.lz = c->cfg.lz;
        U.ax = A.ax;
        U.aeta = A.aeta;
        launch_adj_update_uf<T>(s, g, m, dt, U, S(k, 0), S(k, 1), S(k, 2), eta);
        c->launches += 1;
        if (k == npass - 1)
            for (int q = 0; q < 3; ++q) CK(cudaMemsetAsync(A.a0[q], 0, (size_t)g.ng * sizeof(double), s));
        if (A.tape_loop[pos] > 1) {  // the pressure was solved in this step (pLoopIni)
            const int s2 = adj_solve(c, &loc.iters[k], &loc.relres[k], k);
            if (s2 != CFD_OK && s2 != CFD_ERR_NOCONV) return s2;
            if (s2 != CFD_OK) st = s2;
            launch_adj_rhs(c->lc, g, m, 1.0 / dt, c->jp, A.ab, c->cfg.compat_rhs != 0, A.red, A.a1[0], A.a1[1],
                           A.a1[2]);
            c->launches += c->cfg.compat_rhs ? 2 : 1;
        }
        CK(cudaMemsetAsync(A.ax, 0, (size_t)g.n * sizeof(double), s));
        if (pc && !aligned) {
            launch_adj_src_add_ref(c->lc, g.n, A.a1[0], A.a1[1], A.a1[2], A.asrc);
            c->launches += 1;
        }
        launch_adj_cd_gather(s, g, A.a1[0], A.a1[1], A.a1[2], A.acd[0], A.acd[1], A.acd[2],
                             (pc && aligned && k > 0) ? A.asrc : nullptr);
        c->launches += 1;
        CK(cudaGetLastError());
    }
    if (pc) CK(cudaMemsetAsync(A.asrc, 0, (size_t)(3 * g.n) * sizeof(double), s));
    launch_adj_convdiff<T>(s, g, m, dt, nudt, T0[0], T0[1], T0[2], A.acd[0], A.acd[1], A.acd[2], A.a0[0], A.a0[1],
                           A.a0[2]);
    c->launches += 1;
    for (int q = 0; q < 3; ++q) CK(cudaMemsetAsync(A.acd[q], 0, (size_t)g.ng * sizeof(double), s));
    CK(cudaGetLastError());
    if (info) *info = loc;
    return st;
}

int ck_save(cfd_ctx *c, int slot)
{
    AdjState &A = *c->adj;
    Checkpoint &k = A.ck[slot];
    const Geo &g = c->g;
    const size_t fb = (size_t)g.ng * (c->fp32 ? sizeof(float) : sizeof(double));
    for (int sl = 0; sl < 2; ++sl)
        for (int q = 0; q < 3; ++q)
            CK(cudaMemcpyAsync(k.T[sl][q], c->vel[sl][q], fb, cudaMemcpyDeviceToDevice, c->s));
    CK(cudaMemcpyAsync(k.p, c->p, (size_t)g.ng * sizeof(double), cudaMemcpyDeviceToDevice, c->s));
    CK(cudaMemcpyAsync(k.x, c->x, (size_t)g.n * sizeof(double), cudaMemcpyDeviceToDevice, c->s));
    if (c->px1) CK(cudaMemcpyAsync(k.px1, c->px1, (size_t)g.n * sizeof(double), cudaMemcpyDeviceToDevice, c->s));
    if (c->px2) CK(cudaMemcpyAsync(k.px2, c->px2, (size_t)g.n * sizeof(double), cudaMemcpyDeviceToDevice, c->s));
    CK(cudaMemcpyAsync(k.sc, c->sc, sizeof(BicgScal), cudaMemcpyDeviceToDevice, c->s));
    CK(cudaMemcpyAsync(k.sc_in, c->sc_in, sizeof(BicgScal), cudaMemcpyDeviceToDevice, c->s));
    k.loop = c->loop;
    k.time = c->time;
    k.valid = true;
    return CFD_OK;
}

int ck_load(cfd_ctx *c, int slot)
{
    AdjState &A = *c->adj;
    Checkpoint &k = A.ck[slot];
    if (!k.valid) return fail(CFD_ERR_STATE, "checkpoint slot was never saved");
    for (int &q : c->warm_n) q = 0;  // a checkpoint holds no warm-start history
    const Geo &g = c->g;
    const size_t fb = (size_t)g.ng * (c->fp32 ? sizeof(float) : sizeof(double));
    for (int sl = 0; sl < 2; ++sl)
        for (int q = 0; q < 3; ++q)
            CK(cudaMemcpyAsync(c->vel[sl][q], k.T[sl][q], fb, cudaMemcpyDeviceToDevice, c->s));
    CK(cudaMemcpyAsync(c->p, k.p, (size_t)g.ng * sizeof(double), cudaMemcpyDeviceToDevice, c->s));
    CK(cudaMemcpyAsync(c->x, k.x, (size_t)g.n * sizeof(double), cudaMemcpyDeviceToDevice, c->s));
    if (c->px1) CK(cudaMemcpyAsync(c->px1, k.px1, (size_t)g.n * sizeof(double), cudaMemcpyDeviceToDevice, c->s));
    if (c->px2) CK(cudaMemcpyAsync(c->px2, k.px2, (size_t)g.n * sizeof(double), cudaMemcpyDeviceToDevice, c->s));
    CK(cudaMemcpyAsync(c->sc, k.sc, sizeof(BicgScal), cudaMemcpyDeviceToDevice, c->s));
    CK(cudaMemcpyAsync(c->sc_in, k.sc_in, sizeof(BicgScal), cudaMemcpyDeviceToDevice, c->s));
    c->loop = k.loop;
    c->time = k.time;
    return CFD_OK;
}

int ck_alloc(cfd_ctx *c, int count)
{
    AdjState &A = *c->adj;
    const Geo &g = c->g;
    const size_t fb = (size_t)g.ng * (c->fp32 ? sizeof(float) : sizeof(double));
    const int old = (int)A.ck.size();
    if (count <= old) return CFD_OK;
    CK(cudaStreamSynchronize(c->s));
    A.ck.resize(count);
    for (int i = old; i < count; ++i) {
        Checkpoint &k = A.ck[i];
        for (int sl = 0; sl < 2; ++sl)
            for (int q = 0; q < 3; ++q) CKS(dalloc(c, &k.T[sl][q], fb));
        CKS(dalloc_t(c, &k.p, (size_t)g.ng));
        CKS(dalloc_t(c, &k.x, (size_t)g.n));
        if (c->px1) CKS(dalloc_t(c, &k.px1, (size_t)g.n));
        if (c->px2) CKS(dalloc_t(c, &k.px2, (size_t)g.n));
        CKS(dalloc_t(c, &k.sc, 1));
        CKS(dalloc_t(c, &k.sc_in, 1));
    }
    return CFD_OK;
}

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

// ============================================================================
extern "C" {

int cfd_set_inflow_profile(cfd_ctx *c, const double *u_in, size_t ny)
{
    CKS(check_ctx(c));
    if (!u_in) {
        c->inflow = nullptr;
        return CFD_OK;
    }
    if (ny != (size_t)c->g.nyc) return fail(CFD_ERR_ARG, "inflow profile needs ny_cal values");
    if (!c->inflow_buf) {
        CK(cudaStreamSynchronize(c->s));
        CKS(dalloc_t(c, &c->inflow_buf, ny));
    }
    c->inflow = c->inflow_buf;
    CK(cudaMemcpyAsync(c->inflow, u_in, ny * sizeof(double), cudaMemcpyHostToDevice, c->s));
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_adj_enable(cfd_ctx *c, int tape_len)
{
    CKS(need_metrics(c));
    if (c->cfg.solver == CFD_SOLVER_SOR_RB)
        return fail(CFD_ERR_ARG, "the adjoint needs a Krylov pressure solver (SPE or ELL)");
    if (c->cfg.les_smagorinsky) return fail(CFD_ERR_ARG, "the adjoint does not cover the Smagorinsky model");
    if (c->cfg.conv_outflow_uc > 0.0)
        return fail(CFD_ERR_ARG, "the adjoint does not cover the convective outflow condition");
    if (c->cfg.periodic_z) return fail(CFD_ERR_ARG, "the adjoint does not cover periodic z");
    if (tape_len < 1) return fail(CFD_ERR_ARG, "tape_len must be at least 1");
    if (c->adj) {
        if (tape_len > c->adj->tape_len) CKS(alloc_tape(c, tape_len));
        return CFD_OK;
    }
    CKS(ensure_fp32_solver(c));
    const Geo &g = c->g;
    const size_t ts = c->fp32 ? sizeof(float) : sizeof(double);
    c->adj = new AdjState();
    AdjState &A = *c->adj;
    for (int q = 0; q < 3; ++q) {
        CKS(dalloc_t(c, &A.a0[q], (size_t)g.ng));
        CKS(dalloc_t(c, &A.a1[q], (size_t)g.ng));
        CKS(dalloc_t(c, &A.a3[q], (size_t)g.ng));
        CKS(dalloc_t(c, &A.acd[q], (size_t)g.ng));
        CKS(dalloc(c, &A.rT3[q], (size_t)g.ng * ts));
        for (int k = 0; k < 4; ++k) CKS(dalloc(c, &A.snap[k][q], (size_t)g.ng * ts));
    }
    CKS(dalloc_t(c, &A.ax, (size_t)g.n));
    CKS(dalloc_t(c, &A.ab, (size_t)g.n));
    CKS(dalloc_t(c, &A.aw, (size_t)g.n));
    CKS(dalloc_t(c, &A.bp, (size_t)g.n));
    CKS(dalloc_t(c, &A.zero, (size_t)g.n));
    CKS(dalloc_t(c, &A.pint, (size_t)g.n));
    CKS(dalloc_t(c, &A.af, (size_t)(3 * g.n)));
    CKS(dalloc_t(c, &A.asrc, (size_t)(3 * g.n)));
    CKS(dalloc_t(c, &A.aeta, (size_t)g.ng));
    CKS(dalloc_t(c, &A.ainflow, (size_t)g.nyc));
    CKS(dalloc_t(c, &A.red, 8));
    CKS(dalloc(c, &A.rf, (size_t)(3 * g.n) * ts));
    CKS(dalloc(c, &A.rsrc, (size_t)(3 * g.n) * ts));
    CKS(dalloc_t(c, &A.rp, (size_t)g.ng));
    CK(cudaMemsetAsync(A.zero, 0, (size_t)g.n * sizeof(double), c->s));
    CK(cudaMemsetAsync(A.rp, 0, (size_t)g.ng * sizeof(double), c->s));
    CKS(zero_adjoint(c));
    CKS(alloc_tape(c, tape_len));
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_adj_zero(cfd_ctx *c)
{
    CKS(need_adj(c));
    CKS(zero_adjoint(c));
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

size_t cfd_adj_field_count(cfd_ctx *c, int field)
{
    if (!c) return 0;
    return adj_count(c, field);
}

int cfd_adj_upload(cfd_ctx *c, int field, const double *host, size_t count)
{
    CKS(need_adj(c));
    const size_t n = adj_count(c, field);
    if (n == 0) return fail(CFD_ERR_ARG, "unknown adjoint field");
    if (!host || count != n) return fail(CFD_ERR_ARG, "adjoint upload: null host array or wrong element count");
    CK(cudaMemcpyAsync(adj_ptr(c, field), host, n * sizeof(double), cudaMemcpyHostToDevice, c->s));
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_adj_download(cfd_ctx *c, int field, double *host, size_t count)
{
    CKS(need_adj(c));
    const size_t n = adj_count(c, field);
    if (n == 0) return fail(CFD_ERR_ARG, "unknown adjoint field");
    if (!host || count != n) return fail(CFD_ERR_ARG, "adjoint download: null host array or wrong element count");
    CK(cudaMemcpyAsync(host, adj_ptr(c, field), n * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_adj_convection_diffusion(cfd_ctx *c, int src_slot)
{
    CKS(need_adj(c));
    CKS(check_slot(src_slot));
    const int a = slot_index(src_slot);
    AdjState &A = *c->adj;
    const double dt = c->cfg.dt, nudt = (1.0 / c->cfg.re) * c->cfg.dt;
    dispatch(c, [&](auto tag) {
        using T = typename decltype(tag)::type;
        launch_adj_convdiff<T>(c->s, c->g, metrics_of<double>(c), dt, nudt, dv<T>(c, a, 0), dv<T>(c, a, 1),
                               dv<T>(c, a, 2), A.acd[0], A.acd[1], A.acd[2], A.a0[0], A.a0[1], A.a0[2]);
        return 0;
    });
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_adj_update_uf(cfd_ctx *c, int src_slot, double wcd, double wcl)
{
    CKS(need_adj(c));
    CKS(check_slot(src_slot));
    const int a = slot_index(src_slot);
    AdjState &A = *c->adj;
    launch_gather_interior(c->s, c->g, c->p, A.pint);
    UfAdjArgs U{};
    U.x = A.pint;
    for (int d = 0; d < 3; ++d) {
        U.a3[d] = A.a3[d];
        U.a1[d] = A.a1[d];
    }
    U.af = A.af;
    U.asrc = nullptr;
    U.src_dt = 0.0;
    U.wcd = wcd;
    U.wcl = wcl;
    U.lz = c->cfg.lz;
    U.ax = A.ax;
    U.aeta = A.aeta;
    dispatch(c, [&](auto tag) {
        using T = typename decltype(tag)::type;
        launch_adj_update_uf<T>(c->s, c->g, metrics_of<double>(c), c->cfg.dt, U, dv<T>(c, a, 0), dv<T>(c, a, 1),
                                dv<T>(c, a, 2), static_cast<const T *>(c->eta));
        return 0;
    });
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_adj_create_b(cfd_ctx *c)
{
    CKS(need_adj(c));
    AdjState &A = *c->adj;
    launch_adj_rhs(c->lc, c->g, metrics_of<double>(c), 1.0 / c->cfg.dt, c->jp, A.ab, c->cfg.compat_rhs != 0, A.red,
                   A.a1[0], A.a1[1], A.a1[2]);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_adj_pressure_solve(cfd_ctx *c, int *iters, double *relres)
{
    CKS(need_adj(c));
    const int st = adj_solve(c, iters, relres);
    CK(cudaStreamSynchronize(c->s));
    return st;
}

int cfd_adj_add_source(cfd_ctx *c)
{
    CKS(need_adj(c));
    AdjState &A = *c->adj;
    if (c->cfg.aligned_source)
        launch_adj_src_add_aligned(c->s, c->g, A.a1[0], A.a1[1], A.a1[2], A.asrc);
    else
        launch_adj_src_add_ref(c->lc, c->g.n, A.a1[0], A.a1[1], A.a1[2], A.asrc);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_adj_bc_main(cfd_ctx *c)
{
    CKS(need_adj(c));
    AdjState &A = *c->adj;
    launch_adj_bc_main(c->s, c->g, bc_tab(c), A.a0[0], A.a0[1], A.a0[2], A.ainflow);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_adj_bc_copy(cfd_ctx *c)
{
    CKS(need_adj(c));
    AdjState &A = *c->adj;
    launch_adj_bc_copy(c->s, c->g, A.a0[0], A.a0[1], A.a0[2], A.a1[0], A.a1[1], A.a1[2]);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_step_record(cfd_ctx *c, int pos, cfd_step_info *info)
{
    CKS(need_adj(c));
    AdjState &A = *c->adj;
    if (pos < 0 || pos >= A.tape_len) return fail(CFD_ERR_ARG, "tape position out of range");
    StepRecord rec{};
    for (int q = 0; q < 3; ++q) rec.T0[q] = A.tape_T0[(size_t)pos * 3 + q];
    for (int k = 0; k < 4; ++k) rec.x[k] = A.tape_x[(size_t)pos * 4 + k];
    A.tape_loop[pos] = c->loop;
    return step_recorded(c, info, &rec);
}

int cfd_adj_step(cfd_ctx *c, int pos, double wcd, double wcl, cfd_adj_step_info *info)
{
    CKS(need_adj(c));
    AdjState &A = *c->adj;
    if (pos < 0 || pos >= A.tape_len || A.tape_loop[pos] < 1)
        return fail(CFD_ERR_ARG, "tape position out of range or never recorded");
    const int st = dispatch(c, [&](auto tag) {
        using T = typename decltype(tag)::type;
        return adj_step_t<T>(c, pos, wcd, wcl, info);
    });
    CK(cudaStreamSynchronize(c->s));
    return st;
}

int cfd_adj_finish(cfd_ctx *c)
{
    CKS(need_adj(c));
    AdjState &A = *c->adj;
    launch_adj_bc_copy(c->s, c->g, A.a0[0], A.a0[1], A.a0[2], A.a1[0], A.a1[1], A.a1[2]);
    launch_adj_bc_main(c->s, c->g, bc_tab(c), A.a0[0], A.a0[1], A.a0[2], A.ainflow);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_checkpoint_alloc(cfd_ctx *c, int count)
{
    CKS(need_adj(c));
    if (count < 1) return fail(CFD_ERR_ARG, "checkpoint count must be positive");
    return ck_alloc(c, count);
}

int cfd_checkpoint_save(cfd_ctx *c, int slot)
{
    CKS(need_adj(c));
    if (slot < 0 || slot >= (int)c->adj->ck.size()) return fail(CFD_ERR_ARG, "checkpoint slot out of range");
    CKS(ck_save(c, slot));
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_checkpoint_load(cfd_ctx *c, int slot)
{
    CKS(need_adj(c));
    if (slot < 0 || slot >= (int)c->adj->ck.size()) return fail(CFD_ERR_ARG, "checkpoint slot out of range");
    CKS(ck_load(c, slot));
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_adj_forward(cfd_ctx *c, const cfd_adj_run_config *cfg, cfd_adj_run_result *out)
{
    CKS(need_adj(c));
    if (!cfg || !out) return fail(CFD_ERR_ARG, "null argument");
    AdjState &A = *c->adj;
    const int first = cfg->first, last = cfg->last, L = cfg->interval;
    if (first < 1 || last < first) return fail(CFD_ERR_ARG, "need 1 <= first <= last");
    if (L < 1 || L > A.tape_len) return fail(CFD_ERR_ARG, "interval must be in [1, tape_len]");
    if (c->loop != 1) return fail(CFD_ERR_STATE, "the checkpointed run starts right after cfd_start");
    const int nseg = (last + L - 1) / L;
    CKS(ck_alloc(c, nseg + 1));
    A.run_ready = false;
    *out = cfd_adj_run_result{};
    out->checkpoints = nseg;

    CK(cudaStreamSynchronize(c->s));
    const double t0 = now_s();
    std::vector<double> cd((size_t)last + 1, 0.0);
    int st = CFD_OK;
    for (int n = 1; n <= last; ++n) {
        if ((n - 1) % L == 0) CKS(ck_save(c, (n - 1) / L));
        cfd_step_info info{};
        const int s2 = step_recorded(c, &info, nullptr);
        if (s2 != CFD_OK && s2 != CFD_ERR_NOCONV) return s2;
        if (s2 != CFD_OK) st = s2;
        cd[n] = info.cd;
        for (int k = 0; k < 4; ++k) out->forward_iters += info.iters[k];
    }
    CKS(ck_save(c, nseg));  // the final state, restored after the reverse sweep
    CK(cudaStreamSynchronize(c->s));
    out->forward_seconds = now_s() - t0;
    double J = 0.0;
    for (int n = first; n <= last; ++n) J += cd[n];
    out->J = J / (double)(last - first + 1);
    A.run = *cfg;
    A.run_nseg = nseg;
    A.run_ready = true;
    return st;
}

int cfd_adj_reverse(cfd_ctx *c, cfd_adj_run_result *out)
{
    CKS(need_adj(c));
    AdjState &A = *c->adj;
    if (!A.run_ready) return fail(CFD_ERR_STATE, "cfd_adj_reverse needs a completed cfd_adj_forward");
    const int first = A.run.first, last = A.run.last, L = A.run.interval, nseg = A.run_nseg;
    const double w = 1.0 / (double)(last - first + 1);
    CK(cudaStreamSynchronize(c->s));
    const double t0 = now_s();
    int st = CFD_OK;
    CKS(zero_adjoint(c));
    for (int seg = nseg - 1; seg >= 0; --seg) {
        CKS(ck_load(c, seg));
        const int n0 = seg * L + 1, n1 = std::min(last, n0 + L - 1);
        for (int n = n0; n <= n1; ++n) {
            const int pos = n - n0;
            StepRecord rec{};
            for (int q = 0; q < 3; ++q) rec.T0[q] = A.tape_T0[(size_t)pos * 3 + q];
            for (int k = 0; k < 4; ++k) rec.x[k] = A.tape_x[(size_t)pos * 4 + k];
            A.tape_loop[pos] = c->loop;
            cfd_step_info info{};
            const int s2 = step_recorded(c, &info, &rec);
            if (s2 != CFD_OK && s2 != CFD_ERR_NOCONV) return s2;
        }
        for (int n = n1; n >= n0; --n) {
            const double wn = (n >= first && n <= last) ? w : 0.0;
            const int s2 = dispatch(c, [&](auto tag) {
                using T = typename decltype(tag)::type;
                return adj_step_t<T>(c, n - n0, wn, 0.0, nullptr);
            });
            if (s2 != CFD_OK && s2 != CFD_ERR_NOCONV) return s2;
            if (s2 != CFD_OK) st = s2;
        }
    }
    // cfd_start's boundary conditions
    launch_adj_bc_copy(c->s, c->g, A.a0[0], A.a0[1], A.a0[2], A.a1[0], A.a1[1], A.a1[2]);
    launch_adj_bc_main(c->s, c->g, bc_tab(c), A.a0[0], A.a0[1], A.a0[2], A.ainflow);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    const double t1 = now_s();
    CKS(ck_load(c, nseg));
    CK(cudaStreamSynchronize(c->s));
    if (out) {
        out->adjoint_seconds = t1 - t0;
        out->adjoint_iters = A.solve_iters;
        out->checkpoints = nseg;
    }
    return st;
}

int cfd_adj_mean_drag(cfd_ctx *c, const cfd_adj_run_config *cfg, cfd_adj_run_result *out)
{
    if (!out) return fail(CFD_ERR_ARG, "null argument");
    const int s1 = cfd_adj_forward(c, cfg, out);
    if (s1 != CFD_OK && s1 != CFD_ERR_NOCONV) return s1;
    const int s2 = cfd_adj_reverse(c, out);
    if (s2 != CFD_OK) return s2;
    return s1;
}

}  // extern "C"
