// api.cu -- the C ABI of include/cfdgpu.h: context, device memory, metric
// tables, and the host orchestration of the time step and of the iterative
// solvers (BiCGSTAB with device-resident scalars replayed from a CUDA graph,
// red-black SOR, mixed-precision defect correction).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "context.h"

using namespace cfd;

namespace {

thread_local std::string g_err;

}  // namespace

namespace cfd {
int fail(int code, const std::string &msg)
{
    g_err = msg;
    return code;
}
int set_last_error(int code, const std::string &msg) { return fail(code, msg); }
}  // namespace cfd

namespace {

size_t field_count(const cfd_ctx *c, int field)
{
    if (field >= CFD_FIELD_U0 && field <= CFD_FIELD_ETA) return (size_t)c->g.ng;
    if (field == CFD_FIELD_F || field == CFD_FIELD_SRC) return (size_t)(3 * c->g.n);
    if (field >= CFD_FIELD_X && field <= CFD_FIELD_JP) return (size_t)c->g.n;
    if (field == CFD_FIELD_VIS) return c->vis ? (size_t)c->g.n : 0;
    return 0;
}

// device pointer and whether it holds velocity-type (T) data
void *field_ptr(cfd_ctx *c, int field, bool &is_t)
{
    is_t = false;
    if (field <= CFD_FIELD_W3) {
        is_t = true;
        return c->vel[field / 3][field % 3];
    }
    switch (field) {
    case CFD_FIELD_P: return c->p;
    case CFD_FIELD_ETA: is_t = true; return c->eta;
    case CFD_FIELD_F: is_t = true; return c->f;
    case CFD_FIELD_SRC: is_t = true; return c->src;
    case CFD_FIELD_X: return c->x;
    case CFD_FIELD_B: return c->b;
    case CFD_FIELD_JP: return c->jp;
    case CFD_FIELD_VIS: is_t = true; return c->vis;
    default: return nullptr;
    }
}

// ---- solvers ----------------------------------------------------------------

// Trip cap of a solve loop: enough body runs for the iteration cap, lowered
// by cfd_set_test_limits.
int trip_cap(const cfd_ctx *c, long long want)
{
    long long cap = std::min<long long>(want, 1 << 30);
    if (c->test_trip_cap > 0) cap = std::min<long long>(cap, c->test_trip_cap);
    return (int)cap;
}

// One CUDA graph per solve: head() (the solve's set-up and first steps),
// then a WHILE node whose body is body() followed by the loop condition
// (k_loop_cond), so the whole solve runs on the device and the host waits
// once.  The graph is rebuilt when `key` (its shape) changes.
template <class Head, class Body>
int while_graph(cfd_ctx *c, int gi, long long key, BicgScal *sc, int cap, Head &&head, Body &&body)
{
    cudaGraphExec_t &ge = c->graph[gi];
    if (ge && c->graph_batch[gi] == key) return CFD_OK;
    if (ge) { cudaGraphExecDestroy(ge); ge = nullptr; }
    cudaGraph_t g = nullptr;
    CK(cudaGraphCreate(&g, 0));
    std::string what;
    cudaError_t e = cudaSuccess;
    do {
        cudaGraphConditionalHandle h;
        if ((e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault)) != cudaSuccess) { what = "handle"; break; }
        if ((e = cudaStreamBeginCaptureToGraph(c->s, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) { what = "capture"; break; }
        head();
        launch_loop_cond(c->s, h, sc, cap, 1);
        cudaStreamCaptureStatus cs;
        const cudaGraphNode_t *deps = nullptr;
        size_t nd = 0;
        e = cudaStreamGetCaptureInfo(c->s, &cs, nullptr, nullptr, &deps, nullptr, &nd);
        std::vector<cudaGraphNode_t> last(deps, deps + (e == cudaSuccess ? nd : 0));
        cudaGraph_t cap_g = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(c->s, &cap_g);
        if (e != cudaSuccess || e2 != cudaSuccess) { e = e != cudaSuccess ? e : e2; what = "capture"; break; }
        cudaGraphNodeParams p{};
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = h;
        p.conditional.type = cudaGraphCondTypeWhile;
        p.conditional.size = 1;
        cudaGraphNode_t wn;
        if ((e = cudaGraphAddNode(&wn, g, last.data(), nullptr, last.size(), &p)) != cudaSuccess) { what = "while node"; break; }
        if ((e = cudaStreamBeginCaptureToGraph(c->s, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                               cudaStreamCaptureModeThreadLocal)) != cudaSuccess) { what = "body capture"; break; }
        body();
        launch_loop_cond(c->s, h, sc, cap, 0);
        if ((e = cudaStreamEndCapture(c->s, &cap_g)) != cudaSuccess) { what = "body capture"; break; }
        if ((e = cudaGraphInstantiate(&ge, g, 0)) != cudaSuccess) { ge = nullptr; what = "instantiate"; break; }
    } while (false);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(CFD_ERR_CUDA, "solve graph (" + what + "): " + cudaGetErrorString(e));
    c->graph_batch[gi] = key;
    return CFD_OK;
}

// launch a solve graph and wait for it; `what` names the solve in errors
int run_while_graph(cfd_ctx *c, int gi, BicgScal *sc, long long launches_head, long long launches_body,
                    const char *what)
{
    CK(cudaGraphLaunch(c->graph[gi], c->s));
    CK(cudaMemcpyAsync(c->h_sc, sc, sizeof(BicgScal), cudaMemcpyDeviceToHost, c->s));
    CK(cudaStreamSynchronize(c->s));
    c->launches += launches_head + 1 + (long long)c->h_sc->loop_trips * (launches_body + 1);
    if (c->debug > 1)
        std::fprintf(stderr, "[cfdgpu] %s graph %d: trips %d done %d iter %d relres %.3e restarts %d\n", what, gi,
                     c->h_sc->loop_trips, c->h_sc->done, c->h_sc->iter, c->h_sc->relres, c->h_sc->restarts);
    if (c->h_sc->wait_timeout) return fail(CFD_ERR_TIMEOUT, "a bounded wait of the TMA pipeline gave up");
    if (c->h_sc->done == BICG_RUNNING) return fail(CFD_ERR_TIMEOUT, std::string(what) + " did not report completion");
    return CFD_OK;
}

// A graph of body() alone (no condition), replayed by the host until the
// solve reports completion: the form used when device loops are off.
template <class Body>
int batch_graph(cfd_ctx *c, int gi, long long key, Body &&body)
{
    cudaGraphExec_t &ge = c->graph[gi];
    if (ge && c->graph_batch[gi] == key) return CFD_OK;
    if (ge) { cudaGraphExecDestroy(ge); ge = nullptr; }
    cudaGraph_t gr = nullptr;
    CK(cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal));
    body();
    cudaError_t e = cudaStreamEndCapture(c->s, &gr);
    if (e != cudaSuccess) return fail(CFD_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&ge, gr, 0);
    cudaGraphDestroy(gr);
    if (e != cudaSuccess) { ge = nullptr; return fail(CFD_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e)); }
    c->graph_batch[gi] = key;
    return CFD_OK;
}

template <class Op, class V>
int bicg_run(cfd_ctx *c, const Op &A, const V *b, V *x, const BicgVecs<V> &w, V *px1, V *px2,
             BicgScal *sc, int which_graph)
{
    const int batch = c->cfg.check_every;
    const int cap = trip_cap(c, (long long)c->cfg.p_iter_max / batch + 3);
    auto iterations = [&] { for (int q = 0; q < batch; ++q) launch_bicg_iteration<Op, V>(c->lc, A, x, w, sc); };
    if (c->use_graphs && c->device_loops) {
        CKS(while_graph(
            c, which_graph, ((long long)cap << 20) | batch, sc, cap,
            [&] { launch_bicg_init<Op, V>(c->lc, A, b, x, w, px1, px2, sc); },
            [&] { for (int q = 0; q < batch; ++q) launch_bicg_iteration<Op, V>(c->lc, A, x, w, sc); }));
        return run_while_graph(c, which_graph, sc, 1, 5LL * batch, "BiCGSTAB");
    }
    if (c->use_graphs) CKS(batch_graph(c, which_graph, -batch, iterations));
    launch_bicg_init<Op, V>(c->lc, A, b, x, w, px1, px2, sc);
    c->launches += 1;
    CK(cudaGetLastError());
    for (long long nb = 0;; ++nb) {
        c->launches += 5LL * batch;
        if (c->use_graphs) CK(cudaGraphLaunch(c->graph[which_graph], c->s));
        else iterations();
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(c->h_sc, sc, sizeof(BicgScal), cudaMemcpyDeviceToHost, c->s));
        CK(cudaStreamSynchronize(c->s));
        if (c->debug > 1)
            std::fprintf(stderr, "[cfdgpu] batch %lld: done %d iter %d relres %.3e rho %.3e alpha %.3e "
                         "omega %.3e beta %.3e restart %d\n", nb, c->h_sc->done, c->h_sc->iter,
                         c->h_sc->relres, c->h_sc->rho, c->h_sc->alpha, c->h_sc->omega, c->h_sc->beta,
                         c->h_sc->restart);
        if (c->h_sc->done != BICG_RUNNING) break;
        if (nb >= cap) return fail(CFD_ERR_TIMEOUT, "BiCGSTAB did not report completion");
    }
    return CFD_OK;
}

// Runs an inner solve whose first iteration is issued directly and whose
// later iterations come in pairs (the pair brings the alternating buffers
// back): prologue(), then pair(0), pair(1) while the solve runs -- inside
// one graph (a WHILE node over `pairs` pairs) or, without graphs, polled
// from the host after every `pairs` pairs.
// single: the body is one iteration, pair(0) (its kernels alternate their
// buffers at run time).
template <class Pro, class Pair>
int run_pairs(cfd_ctx *c, int gi, BicgScal *sc, Pro &&prologue, Pair &&pair, int launches_prologue,
              int launches_pair, int pairs_req = 0, bool single = false)
{
    const int pairs = pairs_req > 0 ? pairs_req : (c->cfg.check_every + 1) / 2;
    const int per_body = single ? 1 : 2 * pairs;
    const int cap = trip_cap(c, (long long)c->cfg.p_iter_max / per_body + 3);
    auto body = [&] {
        if (single) {
            pair(0);
            return;
        }
        for (int q = 0; q < pairs; ++q) {
            pair(0);
            pair(1);
        }
    };
    if (c->use_graphs && c->device_loops) {
        CKS(while_graph(c, gi, ((long long)cap << 20) | (single ? 0 : pairs), sc, cap, prologue, body));
        return run_while_graph(c, gi, sc, launches_prologue, (long long)launches_pair * per_body, "inner solve");
    }
    if (c->use_graphs) CKS(batch_graph(c, gi, -(single ? 0 : pairs) - 1, body));
    prologue();
    c->launches += launches_prologue;
    CK(cudaGetLastError());
    for (long long nb = 0;; ++nb) {
        CK(cudaMemcpyAsync(c->h_sc, sc, sizeof(BicgScal), cudaMemcpyDeviceToHost, c->s));
        CK(cudaStreamSynchronize(c->s));
        if (c->h_sc->wait_timeout) return fail(CFD_ERR_TIMEOUT, "a bounded wait of the TMA pipeline gave up");
        if (c->h_sc->done != BICG_RUNNING) break;
        if (nb >= cap) return fail(CFD_ERR_TIMEOUT, "inner solve did not report completion");
        c->launches += (long long)launches_pair * per_body;
        if (c->use_graphs) CK(cudaGraphLaunch(c->graph[gi], c->s));
        else body();
        CK(cudaGetLastError());
    }
    return CFD_OK;
}

// FP32 inner BiCGSTAB with the fused kernels (SPE operator, jp formed on the fly)
int bicg_run_fused(cfd_ctx *c, const SpeOp<float> &Ainit, const SpeOp<float> &A, const float *b, float *x,
                   BicgScal *sc)
{
    return run_pairs(
        c, 2, sc,
        [&] {
            launch_bicg_init<SpeOp<float>, float>(c->lc, Ainit, b, x, c->w32, nullptr, nullptr, sc);
            launch_bicg_fused_iteration<float>(c->lc, A, x, c->w32, c->p_alt, c->ap_alt, sc, 0, true);
        },
        [&](int from) { launch_bicg_fused_iteration<float>(c->lc, A, x, c->w32, c->p_alt, c->ap_alt, sc, from, false); },
        4, 3);
}

// FP32 Jacobi-preconditioned CG on M e = P r (h = r32 in, scaled in place)
int cg_run(cfd_ctx *c, const FvOp<float> &F, float *h, float *e, BicgScal *sc)
{
    return run_pairs(
        c, 3, sc,
        [&] {
            launch_cg_init(c->lc, F, h, c->w32.p1, sc);
            launch_cg_iteration(c->lc, F, c->cg_ip, e, h, c->w32.r0, c->w32.p1, c->p_alt, c->w32.ap, sc, 0, true,
                                &c->cgtma);
        },
        [&](int from) {
            launch_cg_iteration(c->lc, F, c->cg_ip, e, h, c->w32.r0, c->w32.p1, c->p_alt, c->w32.ap, sc, from,
                                false, &c->cgtma);
        },
        3, 2);
}

// FP32 CG on M e = P r preconditioned by one multigrid V-cycle per iteration
// (multigrid.cu): z = V(h), rho = h.z, p0 = z, the first stencil launch
// (pn, q, alpha) and update (e, h, the stopping test); then per iteration a
// V-cycle and rho', the stencil launch and the update.  The loop body is one
// iteration ending with its stopping test, so the loop condition after it
// sees the test at once and no launches run dead after convergence (a dead
// V-cycle is some thirty launches); the stencil launch and the update
// alternate the two p buffers at run time (sc->pp) to make that possible.
static void cg_mg_prologue(cfd_ctx *c, const FvOp<float> &F, float *h, float *e, BicgScal *sc)
{
    float *z = c->w32.r0, *q = c->w32.ap;
    mg_h(c, h, c->dscal + 3, sc);
    mg_vcycle(c, c->mg.never);
    mg_rho(c, h, z, c->w32.p1, sc);
    launch_cg_pq_mg(c->lc, F, &c->cgtma, z, c->w32.p1, c->p_alt, q, sc, 0, true);
    mg_upd(c, e, c->w32.p1, h, q, sc);
}

static void cg_mg_iteration(cfd_ctx *c, const FvOp<float> &F, float *h, float *e, BicgScal *sc)
{
    float *z = c->w32.r0, *q = c->w32.ap;
    // V-cycle, then rho' = h . z (fused into the V-cycle's last launch where it can be)
    if (!mg_vcycle(c, &sc->done, sc)) mg_rho(c, h, z, nullptr, sc);
    launch_cg_pq_mg(c->lc, F, &c->cgtma, z, c->w32.p1, c->p_alt, q, sc, 0, false, true);
    mg_upd(c, e, c->w32.p1, h, q, sc, c->p_alt);
}

// launches of the prologue and of one iteration
static int cg_mg_launches(const cfd_ctx *c, bool prologue)
{
    const int v = (int)mg_vcycle_launches(c->mg), fr = mg_fuses_rho(c->mg) ? 1 : 0;
    return prologue ? v + 4 : v + 3 - fr;
}

int cg_run_mg(cfd_ctx *c, const FvOp<float> &F, float *h, float *e, BicgScal *sc)
{
    return run_pairs(
        c, 4, sc, [&] { cg_mg_prologue(c, F, h, e, sc); }, [&](int) { cg_mg_iteration(c, F, h, e, sc); },
        cg_mg_launches(c, true), cg_mg_launches(c, false), 1, true);
}

// The graphs bake in the buffers and operator of the context; they are
// captured for the configured operator only.
template <class Op>
int solve64(cfd_ctx *c, const Op &A, int *iters, double *relres)
{
    CKS(bicg_run<Op, double>(c, A, c->b, c->x, c->w64, c->px1, c->px2, c->sc, 0));
    int st = CFD_OK;
    if (c->h_sc->done == BICG_CAPPED) {
        launch_bicg_nan_reset<double>(c->lc, c->g.n, c->x, c->px1, c->px2, c->sc);
        c->launches += 2;
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(c->h_sc, c->sc, sizeof(BicgScal), cudaMemcpyDeviceToHost, c->s));
        CK(cudaStreamSynchronize(c->s));
        st = fail(CFD_ERR_NOCONV, "BiCGSTAB reached its iteration cap");
    }
    if (iters) *iters = c->h_sc->iter;
    if (relres) *relres = c->h_sc->relres;
    return st;
}

void residual64(cfd_ctx *c, const SpeOp<double> &A, const double *b, const double *x, float *r32, double *out,
                double *bout = nullptr)
{
    launch_residual64<float>(c->lc, A, b, x, r32, out, bout);
}
void residual64(cfd_ctx *c, const EllOp<double> &A, const double *b, const double *x, float *r32, double *out,
                double *bout = nullptr)
{
    launch_residual64_ell<float>(c->lc, A, b, x, r32, out, bout);
}

// The defect correction of solve_mixed as one CUDA graph (SPE operator,
// multigrid-CG inner solve): the first residual and the outer state
// (k_outer_start), then a WHILE node whose body is one sweep -- e = 0, the
// inner solve (its prologue and its own WHILE node, nested), the outer
// bookkeeping (k_outer_inner_done), the correction, the new residual and the
// outer condition (k_outer_next).  A Poisson solve is then one graph launch
// and one wait, where the host loop waits twice a sweep.  Graph slot 6 for
// the context's b and x, 7 for caller buffers; rebuilt when the buffers, the
// trip caps or the sweep parameters change.
static bool same_cfg(const OuterCfg &a, const OuterCfg &b)
{
    return a.tol == b.tol && a.inner_tol == b.inner_tol && a.adapt == b.adapt && a.max_outer == b.max_outer &&
           a.cap == b.cap;
}

int mixed_graph(cfd_ctx *c, int gi, const SpeOp<double> &A64, const double *b, double *x, const OuterCfg &cfg,
                int cap_in)
{
    cudaGraphExec_t &ge = c->graph[gi];
    const int slot = gi - 6;
    const long long key = ((long long)cap_in << 20) | 1;
    if (ge && c->graph_batch[gi] == key && same_cfg(c->outer_cfg[slot], cfg) && c->outer_b[slot] == b &&
        c->outer_x[slot] == x)
        return CFD_OK;
    if (ge) { cudaGraphExecDestroy(ge); ge = nullptr; }
    const FvOp<float> F = fv32(c);
    const long long n = c->g.n;
    cudaGraph_t g = nullptr;
    CK(cudaGraphCreate(&g, 0));
    std::string what;
    cudaError_t e = cudaSuccess;
    bool capturing = false;
    // end the capture into a graph, returning its last nodes
    auto end = [&](std::vector<cudaGraphNode_t> &last) {
        cudaStreamCaptureStatus cs;
        const cudaGraphNode_t *deps = nullptr;
        size_t nd = 0;
        cudaError_t e1 = cudaStreamGetCaptureInfo(c->s, &cs, nullptr, nullptr, &deps, nullptr, &nd);
        last.assign(deps, deps + (e1 == cudaSuccess ? nd : 0));
        cudaGraph_t cg = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(c->s, &cg);
        capturing = false;
        return e1 != cudaSuccess ? e1 : e2;
    };
    auto begin = [&](cudaGraph_t into, const cudaGraphNode_t *deps, size_t nd) {
        const cudaError_t e1 = cudaStreamBeginCaptureToGraph(c->s, into, deps, nullptr, nd,
                                                             cudaStreamCaptureModeThreadLocal);
        capturing = e1 == cudaSuccess;
        return e1;
    };
    auto add_while = [&](cudaGraph_t into, cudaGraphConditionalHandle h, const std::vector<cudaGraphNode_t> &deps,
                         cudaGraphNode_t *node, cudaGraph_t *body) {
        cudaGraphNodeParams p{};
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = h;
        p.conditional.type = cudaGraphCondTypeWhile;
        p.conditional.size = 1;
        const cudaError_t e1 = cudaGraphAddNode(node, into, deps.data(), nullptr, deps.size(), &p);
        if (e1 == cudaSuccess) *body = p.conditional.phGraph_out[0];
        return e1;
    };
    do {
        std::vector<cudaGraphNode_t> last;
        cudaGraphConditionalHandle ho, hi;
        if ((e = cudaGraphConditionalHandleCreate(&ho, g, 0, cudaGraphCondAssignDefault)) != cudaSuccess) { what = "handle"; break; }
        if ((e = begin(g, nullptr, 0)) != cudaSuccess) { what = "capture"; break; }
        residual64(c, A64, b, x, c->r32, c->dscal + 3, c->dscal + 4);
        launch_outer_start(c->s, ho, c->os, c->dscal + 3, c->sc_in, cfg);
        if ((e = end(last)) != cudaSuccess) { what = "capture"; break; }
        cudaGraphNode_t wo, wi;
        cudaGraph_t gb = nullptr, gib = nullptr;
        if ((e = add_while(g, ho, last, &wo, &gb)) != cudaSuccess) { what = "outer while node"; break; }
        if ((e = cudaGraphConditionalHandleCreate(&hi, gb, 0, cudaGraphCondAssignDefault)) != cudaSuccess) { what = "inner handle"; break; }
        if ((e = begin(gb, nullptr, 0)) != cudaSuccess) { what = "sweep capture"; break; }
        cudaMemsetAsync(c->e32, 0, (size_t)n * sizeof(float), c->s);
        cg_mg_prologue(c, F, c->r32, c->e32, c->sc_in);
        launch_loop_cond(c->s, hi, c->sc_in, cap_in, 1);
        if ((e = end(last)) != cudaSuccess) { what = "sweep capture"; break; }
        if ((e = add_while(gb, hi, last, &wi, &gib)) != cudaSuccess) { what = "inner while node"; break; }
        if ((e = begin(gib, nullptr, 0)) != cudaSuccess) { what = "inner capture"; break; }
        cg_mg_iteration(c, F, c->r32, c->e32, c->sc_in);
        launch_loop_cond(c->s, hi, c->sc_in, cap_in, 0);
        if ((e = end(last)) != cudaSuccess) { what = "inner capture"; break; }
        if ((e = begin(gb, &wi, 1)) != cudaSuccess) { what = "sweep capture"; break; }
        launch_outer_inner_done(c->s, c->os, c->sc_in);
        launch_correct_gated(c->lc, n, x, c->e32, &c->sc_in->rhs_scale, c->os);
        residual64(c, A64, b, x, c->r32, c->dscal + 3);
        launch_outer_next(c->s, ho, c->os, c->dscal + 3, c->sc_in, cfg);
        if ((e = end(last)) != cudaSuccess) { what = "sweep capture"; break; }
        if ((e = cudaGraphInstantiate(&ge, g, 0)) != cudaSuccess) { ge = nullptr; what = "instantiate"; break; }
    } while (false);
    if (capturing) {
        cudaGraph_t cg = nullptr;
        cudaStreamEndCapture(c->s, &cg);
    }
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(CFD_ERR_CUDA, "defect-correction graph (" + what + "): " + cudaGetErrorString(e));
    }
    c->graph_batch[gi] = key;
    c->outer_cfg[slot] = cfg;
    c->outer_b[slot] = b;
    c->outer_x[slot] = x;
    return CFD_OK;
}

int solve_mixed_graph(cfd_ctx *c, const SpeOp<double> &A64, const double *b, double *x, int *iters, double *relres,
                      int *outer, bool zero_x_if_zero_rhs)
{
    OuterCfg cfg{};
    cfg.tol = c->cfg.p_criteria;
    cfg.inner_tol = c->cfg.inner_tol;
    cfg.adapt = c->inner_adapt;
    cfg.max_outer = c->cfg.max_outer;
    cfg.cap = trip_cap(c, (long long)c->cfg.max_outer + 2);
    const int cap_in = trip_cap(c, (long long)c->cfg.p_iter_max + 3);
    const int gi = (b == c->b && x == c->x) ? 6 : 7;
    CKS(mixed_graph(c, gi, A64, b, x, cfg, cap_in));
    CK(cudaGraphLaunch(c->graph[gi], c->s));
    CK(cudaMemcpyAsync(c->h_os, c->os, sizeof(OuterScal), cudaMemcpyDeviceToHost, c->s));
    CK(cudaMemcpyAsync(c->h_sc, c->sc_in, sizeof(BicgScal), cudaMemcpyDeviceToHost, c->s));
    CK(cudaStreamSynchronize(c->s));
    const OuterScal o = *c->h_os;
    c->launches += 2 + (long long)o.loop_trips * (cg_mg_launches(c, true) + 5) +
                   (long long)o.inner_trips * (cg_mg_launches(c, false) + 1);
    if (o.state == OUTER_ZERO_RHS) {
        if (zero_x_if_zero_rhs) CK(cudaMemsetAsync(x, 0, (size_t)c->g.n * sizeof(double), c->s));
        if (iters) *iters = 0;
        if (relres) *relres = 0.0;
        if (outer) *outer = 0;
        return CFD_OK;
    }
    if (o.state == OUTER_INNER_WAIT) return fail(CFD_ERR_TIMEOUT, "a bounded wait of the TMA pipeline gave up");
    if (o.state == OUTER_INNER_CAP) return fail(CFD_ERR_TIMEOUT, "inner solve did not report completion");
    if (iters) *iters = o.iters;
    if (relres) *relres = o.rel;
    if (outer) *outer = o.sweeps;
    switch (o.state) {
    case OUTER_CONVERGED: return CFD_OK;
    case OUTER_CAPPED: return fail(CFD_ERR_NOCONV, "defect correction reached its sweep cap");
    case OUTER_DIVERGED: return fail(CFD_ERR_NOCONV, "FP32 inner solve diverged");
    case OUTER_NONFINITE: return fail(CFD_ERR_NAN, "non-finite Poisson residual");
    default: return fail(CFD_ERR_TIMEOUT, "defect correction did not report completion");
    }
}

// Mixed precision: FP64 defect correction around FP32 BiCGSTAB solves.
//   r = b - A x (FP64, written as FP32);  stop when |r|/|b| < tol
//   solve A e = r in FP32 to inner_tol (e from 0);  x += e (FP64)
template <class Op64, class Op32>
int solve_mixed(cfd_ctx *c, const Op64 &A64, const Op32 &A32, const double *b, double *x, const double *zero,
                int inner, int *iters, double *relres, int *outer, bool zero_x_if_zero_rhs = false)
{
    const long long n = c->g.n;
    if constexpr (std::is_same<Op64, SpeOp<double>>::value && std::is_same<Op32, SpeOp<float>>::value) {
        if (inner == CFD_INNER_MG && c->mg.usable && c->use_graphs && c->device_loops && c->outer_graph &&
            !c->debug) {
            const int st = solve_mixed_graph(c, A64, b, x, iters, relres, outer, zero_x_if_zero_rhs);
            // where the CUDA runtime cannot build the graph (nested conditional nodes):
            // the host loop from here on
            if (st != CFD_ERR_CUDA || c->graph[(b == c->b && x == c->x) ? 6 : 7]) return st;
            c->outer_graph = false;
        }
    }
    // the first residual (from the warm start) also gives |b|^2, the
    // reference norm of the stopping test
    (void)zero;
    residual64(c, A64, b, x, c->r32, c->dscal + 3, c->dscal + 4);
    c->launches += 1;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(c->h_scal, c->dscal, 8 * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    CK(cudaStreamSynchronize(c->s));
    const double norm0 = std::sqrt(c->h_scal[4]);
    int total = 0, sweeps = 0;
    double rel = 0.0;
    if (norm0 == 0.0) {
        if (zero_x_if_zero_rhs) CK(cudaMemsetAsync(x, 0, (size_t)n * sizeof(double), c->s));
        if (iters) *iters = 0;
        if (relres) *relres = 0.0;
        if (outer) *outer = 0;
        return CFD_OK;
    }
    int st = CFD_OK;
    for (bool first = true;; first = false) {
        if (!first) {
            residual64(c, A64, b, x, c->r32, c->dscal + 3);
            c->launches += 1;
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(c->h_scal, c->dscal, 8 * sizeof(double), cudaMemcpyDeviceToHost, c->s));
            CK(cudaStreamSynchronize(c->s));
        }
        rel = std::sqrt(c->h_scal[3]) / norm0;
        if (rel < c->cfg.p_criteria || !std::isfinite(rel)) break;
        if (sweeps >= c->cfg.max_outer) { st = fail(CFD_ERR_NOCONV, "defect correction reached its sweep cap"); break; }
        CK(cudaMemsetAsync(c->e32, 0, (size_t)n * sizeof(float), c->s));
        if (c->inner_adapt > 0.0) {
            const double want = std::min(0.5, c->inner_adapt * c->cfg.p_criteria / rel);
            launch_set_tol(c->s, c->sc_in, std::max(c->cfg.inner_tol, want));
            c->launches += 1;
        }
        if constexpr (std::is_same<Op32, SpeOp<float>>::value) {
            SpeOp<float> Afly = A32;
            Afly.jp = nullptr;
            if (inner == CFD_INNER_MG && c->mg.usable) CKS(cg_run_mg(c, fv32(c), c->r32, c->e32, c->sc_in));
            else if (inner == CFD_INNER_CG || inner == CFD_INNER_MG) CKS(cg_run(c, fv32(c), c->r32, c->e32, c->sc_in));
            else if (c->fused) CKS(bicg_run_fused(c, A32, Afly, c->r32, c->e32, c->sc_in));
            else CKS((bicg_run<Op32, float>(c, A32, c->r32, c->e32, c->w32, nullptr, nullptr, c->sc_in, 1)));
        } else {
            CKS((bicg_run<Op32, float>(c, A32, c->r32, c->e32, c->w32, nullptr, nullptr, c->sc_in, 1)));
        }
        total += c->h_sc->iter;
        if (!(c->h_sc->relres < 1.0)) {
            // the inner solve diverged: keep x, report
            st = fail(CFD_ERR_NOCONV, "FP32 inner solve diverged");
            ++sweeps;
            break;
        }
        if (c->debug)
            std::fprintf(stderr, "[cfdgpu] outer %d rel %.3e | inner done %d iter %d relres %.3e norm0 %.3e "
                         "rho %.3e alpha %.3e omega %.3e\n", sweeps, rel, c->h_sc->done, c->h_sc->iter,
                         c->h_sc->relres, c->h_sc->norm0, c->h_sc->rho, c->h_sc->alpha, c->h_sc->omega);
        // the multigrid-CG solved for r / |r|
        const bool scaled = inner == CFD_INNER_MG && c->mg.usable && std::is_same<Op32, SpeOp<float>>::value;
        launch_correct<float>(c->lc, n, x, c->e32, scaled ? &c->sc_in->rhs_scale : nullptr);
        c->launches += 1;
        CK(cudaGetLastError());
        ++sweeps;
    }
    if (!std::isfinite(rel)) st = fail(CFD_ERR_NAN, "non-finite Poisson residual");
    if (iters) *iters = total;
    if (relres) *relres = rel;
    if (outer) *outer = sweeps;
    return st;
}

int poisson_solve(cfd_ctx *c, int *iters, double *relres, int *outer)
{
    if (outer) *outer = 0;
    const bool ell = c->cfg.solver == CFD_SOLVER_BICG_ELL;
    if (c->cfg.precision == CFD_PREC_MIXED || c->cfg.precision == CFD_PREC_FP64_DC) {
        const int inner = c->cfg.inner_solver;
        if (c->cfg.precision == CFD_PREC_FP64_DC) CKS(ensure_fp32_solver(c));
        if (inner == CFD_INNER_MG) CKS(mg_setup(c));
        if (ell) return solve_mixed(c, ell64(c), ell32(c), c->b, c->x, c->w64.r0, inner, iters, relres, outer);
        return solve_mixed(c, spe64(c), spe32(c), c->b, c->x, c->w64.r0, inner, iters, relres, outer);
    }
    if (ell) return solve64(c, ell64(c), iters, relres);
    return solve64(c, spe64(c), iters, relres);
}

// SorPipeLine_seq (SorPipeLine.seq.hpp:48-117) in red-black order: the
// right-hand side from velocity slot si, then sweeps until the max change
// is at most the tolerance or p_sor_iter_max sweeps ran, all on the device
// (graph 5: a WHILE node over check_every sweeps; host-polled batches when
// device loops are off).  iters = sweeps - 1 and err = the last max change,
// as the reference reports them.
//
// Mixed-precision contexts sweep in FP32 inside an FP64 defect correction:
// each loop body is one FP64 sweep (whose max change is the reference's stop
// test, unchanged), the FP64 change of a Jacobi step at every cell, 4 x
// check_every FP32 sweeps on the correction, and p += correction.  The FP32
// sweeps count towards p_sor_iter_max, which is tested at the FP64 sweeps
// (a capped solve can run up to one body's FP32 sweeps past it).
template <class T>
int sor_solve_t(cfd_ctx *c, int si, int *iters, double *err)
{
    const Geo &g = c->g;
    const Metrics<double> m = metrics_of<double>(c);
    const int itmax = c->cfg.p_sor_iter_max;
    const bool mixed = c->sor_e != nullptr;
    const int batch = c->cfg.check_every, inner = 4 * batch;
    const int cap = trip_cap(c, mixed ? (long long)itmax / (inner + 1) + 3 : (long long)itmax / batch + 3);
    const double omega = c->cfg.p_sor_omega, tol = c->cfg.p_criteria;
    auto head = [&]() -> int {
        if (mixed) CK(cudaMemsetAsync(c->sor_e, 0, (size_t)g.n * sizeof(float), c->s));
        launch_sor_rhs_rb<T>(c->s, g, m, 1.0 / c->cfg.dt, dv<T>(c, si, 0), dv<T>(c, si, 1), dv<T>(c, si, 2),
                             c->sor_rhs, c->sc, c->sor_acc);
        return CFD_OK;
    };
    auto body = [&] {
        if (mixed) {
            launch_sor_rb_sweep(c->s, g, c->sor_cf, c->sor_rhs, c->p, omega, tol, itmax, c->sc, c->sor_acc);
            launch_sor_residual(c->s, g, c->sor_cf, c->sor_rhs, c->p, c->sor_rho, c->sc);
            for (int q = 0; q < inner; ++q) sor_smooth_sweep(c, &c->sc->done);
            launch_sor_correct(c->s, g, c->p, c->sor_e, inner, c->sc);
            return;
        }
        for (int q = 0; q < batch; ++q)
            launch_sor_rb_sweep(c->s, g, c->sor_cf, c->sor_rhs, c->p, omega, tol, itmax, c->sc, c->sor_acc);
    };
    const long long body_launches = mixed ? 4LL + 2LL * inner : 2LL * batch;
    const long long key = ((long long)cap << 20) | ((long long)batch << 4) | (mixed ? 8 : 0) | si;
    if (c->use_graphs && c->device_loops) {
        CKS(while_graph(c, 5, key, c->sc, cap, head, body));
        CKS(run_while_graph(c, 5, c->sc, mixed ? 2 : 1, body_launches, "SOR"));
    } else {
        if (c->use_graphs) CKS(batch_graph(c, 5, -key, body));
        CKS(head());
        c->launches += 1;
        for (long long nb = 0;; ++nb) {
            if (nb >= cap) return fail(CFD_ERR_TIMEOUT, "SOR did not report completion");
            if (c->use_graphs) CK(cudaGraphLaunch(c->graph[5], c->s));
            else body();
            c->launches += body_launches;
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(c->h_sc, c->sc, sizeof(BicgScal), cudaMemcpyDeviceToHost, c->s));
            CK(cudaStreamSynchronize(c->s));
            if (c->h_sc->done != BICG_RUNNING) break;
        }
    }
    if (iters) *iters = c->h_sc->iter - 1;
    if (err) *err = c->h_sc->relres;
    return CFD_OK;
}

// Warm start of pass k's Poisson solve (mixed and FP64-defect-correction
// contexts): the reference starts every solve from the previous one's
// solution (the previous pass's), which at 512x256x32 leaves an initial
// relative residual of 0.3 to 50; pass k's own solutions of the last two
// steps, extrapolated linearly in time, start it far closer, so the
// defect correction needs fewer sweeps.  The converged solution is the same
// to the solver tolerance.  CFDGPU_WARM=prev keeps the reference's start.
static bool warm_applies(const cfd_ctx *c)
{
    return c->warm_extrap && c->cfg.solver != CFD_SOLVER_SOR_RB &&
           (c->cfg.precision == CFD_PREC_MIXED || c->cfg.precision == CFD_PREC_FP64_DC);
}

static int warm_start(cfd_ctx *c, int k)
{
    if (!warm_applies(c) || k < 0 || k >= 4) return CFD_OK;
    const long long n = c->g.n;
    const int keep = c->warm_order + 1;  // solutions the extrapolation reads
    if (!c->warm_hist[k][0]) {
        for (int q = 0; q < keep; ++q)
            if (dalloc_t(c, &c->warm_hist[k][q], (size_t)n) != CFD_OK) {
                c->warm_extrap = false;  // no room: the reference's start
                cudaGetLastError();
                return CFD_OK;
            }
        c->warm_n[k] = 0;
    }
    double *const *h = c->warm_hist[k];  // the newest is h[keep - 1]
    if (c->warm_n[k] >= 3 && keep == 3) {
        launch_extrapolate(c->lc, n, c->x, h[0], h[1], h[2]);
        c->launches += 1;
        CK(cudaGetLastError());
    } else if (c->warm_n[k] >= 2) {
        launch_extrapolate(c->lc, n, c->x, h[keep - 2], h[keep - 1]);
        c->launches += 1;
        CK(cudaGetLastError());
    } else if (c->warm_n[k] == 1) {
        CK(cudaMemcpyAsync(c->x, h[keep - 1], (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, c->s));
    }
    return CFD_OK;
}

static int warm_store(cfd_ctx *c, int k)
{
    if (!warm_applies(c) || k < 0 || k >= 4 || !c->warm_hist[k][0]) return CFD_OK;
    const int keep = c->warm_order + 1;
    double **h = c->warm_hist[k];
    double *oldest = h[0];
    for (int q = 0; q + 1 < keep; ++q) h[q] = h[q + 1];
    h[keep - 1] = oldest;
    CK(cudaMemcpyAsync(h[keep - 1], c->x, (size_t)c->g.n * sizeof(double), cudaMemcpyDeviceToDevice, c->s));
    c->warm_n[k] = std::min(keep, c->warm_n[k] + 1);
    return CFD_OK;
}

// rhs_done: the pass kernel already formed b (and its compatibility projection)
template <class T>
int pressure_step(cfd_ctx *c, int si, int *iters, double *relres, int *outer, bool rhs_done = false)
{
    const Geo &g = c->g;
    if (c->cfg.solver == CFD_SOLVER_SOR_RB) {
        if (outer) *outer = 0;
        return sor_solve_t<T>(c, si, iters, relres);
    }
    if (!rhs_done) {
        launch_rhs<T>(c->lc, g, metrics_of<double>(c), 1.0 / c->cfg.dt, c->jp, dv<T>(c, si, 0),
                      dv<T>(c, si, 1), dv<T>(c, si, 2), c->b, c->cfg.compat_rhs != 0, c->dscal + 0);
        c->launches += c->cfg.compat_rhs ? 2 : 1;
    }
    CK(cudaGetLastError());
    int st = poisson_solve(c, iters, relres, outer);
    if (st != CFD_OK && st != CFD_ERR_NOCONV) return st;
    launch_transform(c->s, g, c->x, c->p);
    c->launches += 1;
    CK(cudaGetLastError());
    return st;
}

template <class T>
int step_t(cfd_ctx *c, cfd_step_info *info, const StepRecord *rec)
{
    const Geo &g = c->g;
    const Metrics<T> m = metrics_of<T>(c);
    const bool pc = c->cfg.method == CFD_METHOD_PC;
    const bool aligned = c->cfg.aligned_source != 0;
    const T dt = (T)c->cfg.dt, nudt = (T)((1.0 / c->cfg.re) * c->cfg.dt);
    T *u0 = dv<T>(c, 0, 0), *v0 = dv<T>(c, 0, 1), *w0 = dv<T>(c, 0, 2);
    T *u1 = dv<T>(c, 1, 0), *v1 = dv<T>(c, 1, 1), *w1 = dv<T>(c, 1, 2);
    T *u3 = dv<T>(c, 2, 0), *v3 = dv<T>(c, 2, 1), *w3 = dv<T>(c, 2, 2);
    T *src = static_cast<T *>(c->src), *f = static_cast<T *>(c->f);
    const int npass = pc ? 4 : 1;
    int st = CFD_OK;
    cfd_step_info loc{};
    if (rec)
        for (int q = 0; q < 3; ++q)
            CK(cudaMemcpyAsync(rec->T0[q], c->vel[0][q], (size_t)g.ng * sizeof(T), cudaMemcpyDeviceToDevice, c->s));
    if (pc) CK(cudaMemsetAsync(src, 0, (size_t)(3 * g.n) * sizeof(T), c->s));
    T *vis = static_cast<T *>(c->vis);
    if (vis) {  // SmagorinskyModel of T0 (the same in every pass of the step)
        launch_smagorinsky<T>(c->s, g, metrics_of<double>(c), u0, v0, w0, vis);
        c->launches += 1;
    }
    // predictor-corrector: every pass starts with ConvectionDifussion(T0 -> T1)
    // of the same T0 (RUN_CPU_PC_METHOD.hpp:304, 455); it is evaluated once
    T *C[3] = {static_cast<T *>(c->cdbuf[0]), static_cast<T *>(c->cdbuf[1]), static_cast<T *>(c->cdbuf[2])};
    if (pc) {
        launch_convdiff<T>(c->s, g, m, dt, nudt, u0, v0, w0, C[0], C[1], C[2], nullptr, vis, (T)(1.0 / c->cfg.re));
        c->launches += 1;
    }
    const bool krylov = c->cfg.solver != CFD_SOLVER_SOR_RB;
    for (int pass = 0; pass < npass; ++pass) {
        bool rhs_done = false;
        if (pc) {
            // T1 = C + source, and the pass's Poisson right-hand side
            PassArgs<T> A{};
            for (int q = 0; q < 3; ++q) A.C[q] = C[q];
            A.T1[0] = u1; A.T1[1] = v1; A.T1[2] = w1;
            A.src = src;
            A.src_mode = pass == 0 ? 0 : (aligned ? 2 : 1);
            A.jp = c->jp;
            A.jph = c->jp32;
            A.jpl = c->jp32lo;
            A.ddt = 1.0 / c->cfg.dt;
            rhs_done = krylov && c->loop > 1;
            A.b = rhs_done ? c->b : nullptr;
            A.partials = rhs_done && c->cfg.compat_rhs ? c->lc.partials : nullptr;
            A.counter = c->lc.counter;
            A.mean = c->dscal + 0;
            A.vol = c->vol_total;
            const bool ghosts = !aligned && pass > 0;
            launch_pass<T>(c->lc, g, metrics_of<double>(c), metrics_of<float>(c), A, ghosts);
            c->launches += 1 + (ghosts ? 1 : 0) + (A.partials ? 1 : 0);
        } else {
            launch_convdiff<T>(c->s, g, m, dt, nudt, u0, v0, w0, u1, v1, w1, nullptr, vis, (T)(1.0 / c->cfg.re));
            c->launches += 1;
        }
        if (g.pz) {  // the divergence at the first cell reads w on face 1 = the top face
            launch_sync_z<T>(c->s, g, u1, v1, w1);
            c->launches += 1;
        }
        CK(cudaGetLastError());
        if (c->loop > 1) {
            CKS(warm_start(c, pass));
            int s2 = pressure_step<T>(c, 1, &loc.iters[pass], &loc.relres[pass], &loc.outer[pass], rhs_done);
            if (s2 != CFD_OK && s2 != CFD_ERR_NOCONV) return s2;
            if (s2 != CFD_OK) st = s2;
            if (s2 == CFD_OK) CKS(warm_store(c, pass));
        }
        if (g.pz) {  // the top w face's pressure gradient reads p above it
            launch_sync_z<double>(c->s, g, c->p, nullptr, nullptr);
            c->launches += 1;
        }
        if (rec) {
            launch_gather_interior(c->s, g, c->p, rec->x[pass]);
            c->launches += 1;
        }
        if (c->div_check && pass == npass - 1 && c->loop > 1) {
            // T2 = u* - dt grad p of the last pass, before the boundary update
            // rewrites T1's faces
            CK(cudaMemsetAsync(c->dmax, 0, 3 * sizeof(unsigned long long), c->s));
            launch_div_projected<T>(c->lc, g, metrics_of<double>(c), c->cfg.dt, c->p, u1, v1, w1,
                                    c->cfg.compat_rhs ? c->dscal + 0 : nullptr, c->dmax, true);
            CK(cudaMemcpyAsync(c->h_max, c->dmax, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->s));
            c->launches += 1;
        }
        if (pc) {
            // the predictor passes feed f into the source; the final pass
            // stores f and reduces the drag and lift
            const bool last = pass == npass - 1;
            launch_update_pass<T>(c->lc, g, m, metrics_of<double>(c), c->cfg.dt, c->p, static_cast<T *>(c->eta),
                                  u1, v1, w1, u3, v3, w3, f, last, last ? nullptr : src, c->cfg.lz,
                                  last ? c->dscal + 1 : nullptr);
            c->launches += 1;
        } else {
            launch_update_uf<T>(c->s, g, m, c->cfg.dt, (T)(1.0 / c->cfg.dt), c->p, static_cast<T *>(c->eta),
                                u1, v1, w1, u3, v3, w3, f);
            c->launches += 1;
        }
        CK(cudaGetLastError());
    }
    const size_t bytes = (size_t)g.ng * sizeof(T);
    const bool conv = c->cfg.conv_outflow_uc > 0.0;
    if (conv) {  // convective outflow from the old T0 into T3, before T0 <- T3
        launch_bc_convective<T>(c->lc, g, metrics_of<double>(c), c->cfg.dt, c->cfg.conv_outflow_uc, u0, v0, w0,
                                u3, v3, w3, c->dscal + 6);
        c->launches += 2;
        CK(cudaGetLastError());
    }
    for (int q = 0; q < 3; ++q)
        CK(cudaMemcpyAsync(c->vel[0][q], c->vel[2][q], bytes, cudaMemcpyDeviceToDevice, c->s));
    BcTab bc = bc_tab(c);
    bc.skip_outflow = conv ? 1 : 0;
    launch_bc_main<T>(c->s, g, bc, u0, v0, w0, c->p);
    launch_bc_copy<T>(c->s, g, u0, v0, w0, u1, v1, w1);
    if (!pc) launch_cdcl<T>(c->lc, g, metrics_of<double>(c), c->cfg.lz, f, c->dscal + 1);
    c->launches += 3 + 1 + (pc ? 0 : 1);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(c->h_scal, c->dscal, 8 * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    CK(cudaStreamSynchronize(c->s));
    loc.cd = c->h_scal[1];
    loc.cl = c->h_scal[2];
    if (c->div_check && c->loop > 1) std::memcpy(c->last_div, c->h_max, sizeof(c->last_div));
    c->loop += 1;
    c->time += c->cfg.dt;
    loc.loop = c->loop;
    loc.time = c->time;
    if (info) *info = loc;
    return st;
}

}  // namespace

namespace cfd {

int step_recorded(cfd_ctx *c, cfd_step_info *info, const StepRecord *rec)
{
    return dispatch(c, [&](auto tag) {
        using T = typename decltype(tag)::type;
        return step_t<T>(c, info, rec);
    });
}

// FP64 defect correction around the FP32 CG inner solve for A x = b with
// caller buffers (the adjoint Poisson solves): same tolerances as the
// forward solve, residual with the FP64 matrix-free operator; b = 0 gives
// x = 0 (the warm start is dropped)
int linear_solve_cg(cfd_ctx *c, const double *b, double *x, const double *zero, int *iters, double *relres,
                    int *outer)
{
    int inner = CFD_INNER_CG;
    if (c->cfg.inner_solver == CFD_INNER_MG) {
        CKS(mg_setup(c));
        inner = CFD_INNER_MG;
    }
    return solve_mixed(c, spe64(c), spe32(c), b, x, zero, inner, iters, relres, outer, true);
}

// FP32 operator tables and CG buffers in an FP64 context (for the adjoint
// solves); a mixed-precision context has them already
int ensure_fp32_solver(cfd_ctx *c)
{
    if (!c->metrics) return fail(CFD_ERR_STATE, "grid metrics not set (cfd_grid_uniform / cfd_set_metrics)");
    if (c->cg_ip && c->w32.r0 && c->r32) return CFD_OK;
    const Geo &g = c->g;
    const long long n = g.n;
    const int nc[3] = {g.nxc, g.nyc, g.nzc};
    CK(cudaStreamSynchronize(c->s));
    if (!c->w32.r0) CKS(dalloc_t(c, &c->w32.r0, n));
    if (!c->w32.p1) CKS(dalloc_t(c, &c->w32.p1, n));
    if (!c->w32.ap) CKS(dalloc_t(c, &c->w32.ap, n));
    if (!c->p_alt) CKS(dalloc_t(c, &c->p_alt, n));
    if (!c->r32) CKS(dalloc_t(c, &c->r32, n));
    if (!c->e32) CKS(dalloc_t(c, &c->e32, n));
    if (!c->jp32) CKS(dalloc_t(c, &c->jp32, n));
    for (int a = 0; a < 3; ++a) {
        if (!c->spe_c32[a]) CKS(dalloc_t(c, &c->spe_c32[a], 2 * (size_t)nc[a]));
        if (!c->fv_sum[a]) CKS(dalloc_t(c, &c->fv_sum[a], 2 * (size_t)nc[a]));
    }
    if (!c->cg_ip) CKS(dalloc_t(c, &c->cg_ip, n));
    for (int a = 0; a < 3; ++a) {
        launch_convert<double, float>(c->lc, 2LL * nc[a], c->spe_c[a], c->spe_c32[a]);
        launch_fv_axes(c->s, nc[a], c->spe_c32[a], fv_width_src(c, a), c->fv_sum[a]);
    }
    launch_convert<double, float>(c->lc, n, c->jp, c->jp32);
    launch_cg_ip(c->lc, fv32(c), c->cg_ip);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cg_tma_setup(c->cgtma, fv32(c), c->w32.r0, c->r32, c->w32.p1, c->p_alt, sms > 0 ? sms : 148,
                 c->lc.red_blocks);
    return CFD_OK;
}

}  // namespace cfd

namespace {

int build_tables(cfd_ctx *c)
{
    // new metrics: the multigrid levels and their graph are rebuilt on demand
    if (c->graph[4]) {
        cudaGraphExecDestroy(c->graph[4]);
        c->graph[4] = nullptr;
    }
    c->mg.nlev = 0;
    c->mg.usable = false;
    const Geo &g = c->g;
    const int n[3] = {g.nx, g.ny, g.nz};
    for (int a = 0; a < 3; ++a) {
        std::vector<double> t = axis_table(c->hraw[3 + a], c->hraw[6 + a]);
        CK(cudaMemcpyAsync(c->tab64[a], t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice, c->s));
        std::vector<float> t32(t.begin(), t.end());
        CK(cudaMemcpyAsync(c->tab32[a], t32.data(), t32.size() * sizeof(float), cudaMemcpyHostToDevice, c->s));
        CK(cudaStreamSynchronize(c->s));
    }
    for (int q = 0; q < 9; ++q)
        CK(cudaMemcpyAsync(c->rawp[q], c->hraw[q].data(), c->hraw[q].size() * sizeof(double),
                           cudaMemcpyHostToDevice, c->s));
    {
        // the interior volume: the product of the interior lengths
        double len[3] = {0.0, 0.0, 0.0};
        for (int a = 0; a < 3; ++a)
            for (int i = GC; i < n[a] - GC; ++i) len[a] += c->hraw[3 + a][i];
        c->vol_total = len[0] * len[1] * len[2];
    }
    // operators
    launch_spe_setup(c->s, g, c->rawp[3], c->rawp[4], c->rawp[5], c->rawp[6], c->rawp[7], c->rawp[8],
                     c->spe_c[0], c->spe_c[1], c->spe_c[2], c->jp);
    if (c->cfg.solver == CFD_SOLVER_BICG_ELL)
        launch_ell_assemble(c->s, g, c->rawp[3], c->rawp[4], c->rawp[5], c->rawp[6], c->rawp[7],
                            c->rawp[8], c->ell_cols, c->ell_vals, c->jp);
    if (c->sor_cf)
        launch_sor_coef_rb(c->s, g, c->rawp[3], c->rawp[4], c->rawp[5], c->rawp[6], c->rawp[7], c->rawp[8],
                           c->sor_cf);
    if (c->sor_e) CKS(sor_level_setup(c, (float)c->cfg.p_sor_omega));
    // FP32 copies of the operator, each only where the context holds one (a
    // mixed-precision SOR context has none; FP64 contexts get them when a
    // defect-correction solve first needs them)
    for (int a = 0; a < 3; ++a) {
        const int na = a == 0 ? g.nxc : a == 1 ? g.nyc : g.nzc;
        if (!c->spe_c32[a]) continue;
        launch_convert<double, float>(c->lc, 2LL * na, c->spe_c[a], c->spe_c32[a]);
        if (c->fv_sum[a]) launch_fv_axes(c->s, na, c->spe_c32[a], fv_width_src(c, a), c->fv_sum[a]);
    }
    if (c->jp32) launch_convert<double, float>(c->lc, g.n, c->jp, c->jp32);
    if (c->jp32lo) launch_split_lo(c->lc, g.n, c->jp, c->jp32lo);
    if (c->cg_ip) launch_cg_ip(c->lc, fv32(c), c->cg_ip);
    if (c->ell_vals32) launch_convert<double, float>(c->lc, 7 * g.n, c->ell_vals, c->ell_vals32);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    c->metrics = true;
    return CFD_OK;
}

void free_ctx(cfd_ctx *c)
{
    if (!c) return;
    for (auto &ge : c->graph)
        if (ge) cudaGraphExecDestroy(ge);
    if (c->s) cudaStreamSynchronize(c->s);
    for (void *p : c->allocs) cudaFree(p);
    if (c->h_sc) cudaFreeHost(c->h_sc);
    if (c->h_os) cudaFreeHost(c->h_os);
    if (c->h_scal) cudaFreeHost(c->h_scal);
    if (c->h_max) cudaFreeHost(c->h_max);
    adj_free(c->adj);
    if (c->s) cudaStreamDestroy(c->s);
    delete c;
}

}  // namespace

// ============================================================================
extern "C" {

int cfd_abi_version(void) { return CFDGPU_ABI_VERSION; }

const char *cfd_last_error(void) { return g_err.c_str(); }

int cfd_config_default(cfd_config *cfg, int nx, int ny, int nz)
{
    if (!cfg) return fail(CFD_ERR_ARG, "null config");
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->nx_cal = nx;
    cfg->ny_cal = ny;
    cfg->nz_cal = nz;
    cfg->lx = 1.0;
    cfg->ly = 1.0;
    cfg->lz = 1.0;
    cfg->re = 40.0;      // src/CFD_MX.cpp:39
    cfg->dt = 0.002;     // src/CFD_MX.cpp:37
    cfg->method = CFD_METHOD_PC;
    cfg->solver = CFD_SOLVER_BICG_SPE;
    cfg->precision = CFD_PREC_FP64;
    cfg->p_criteria = 1e-3;   // simuClass.hpp:74
    cfg->p_iter_max = 5000;   // bicgstabRe2.hpp:57
    cfg->p_sor_omega = 1.8;   // simuClass.hpp:78
    cfg->p_sor_iter_max = 5000;
    cfg->aligned_source = 0;
    cfg->compat_rhs = 0;
    cfg->check_every = 16;
    cfg->inner_tol = 1e-3;
    cfg->inner_solver = CFD_INNER_MG;
    cfg->max_outer = 30;
    cfg->conv_outflow_uc = 0.0;
    cfg->les_smagorinsky = 0;
    return CFD_OK;
}

int cfd_create(const cfd_config *cfg, cfd_ctx **out)
{
    if (!cfg || !out) return fail(CFD_ERR_ARG, "null argument");
    *out = nullptr;
    const cfd_config &k = *cfg;
    if (k.nx_cal < 4 || k.ny_cal < 4 || k.nz_cal < 4)
        return fail(CFD_ERR_ARG, "every interior dimension must be at least 4");
    const long long n = (long long)k.nx_cal * k.ny_cal * k.nz_cal;
    if (n >= (1LL << 31) - 1) return fail(CFD_ERR_ARG, "grid too large for 32-bit ELL column indices");
    if (!(k.lx > 0 && k.ly > 0 && k.lz > 0)) return fail(CFD_ERR_ARG, "domain lengths must be positive");
    if (!(k.dt > 0) || !(k.re > 0)) return fail(CFD_ERR_ARG, "dt and re must be positive");
    if (!(k.p_criteria > 0) || k.p_iter_max < 1 || k.p_sor_iter_max < 1)
        return fail(CFD_ERR_ARG, "solver tolerance and iteration caps must be positive");
    if (k.solver != CFD_SOLVER_BICG_SPE && k.solver != CFD_SOLVER_BICG_ELL && k.solver != CFD_SOLVER_SOR_RB)
        return fail(CFD_ERR_ARG, "unknown solver");
    if (k.method != CFD_METHOD_PC && k.method != CFD_METHOD_PLAIN) return fail(CFD_ERR_ARG, "unknown method");
    if (k.precision != CFD_PREC_FP64 && k.precision != CFD_PREC_MIXED && k.precision != CFD_PREC_FP64_DC)
        return fail(CFD_ERR_ARG, "unknown precision");
    if (k.check_every < 1 || k.check_every > 4096) return fail(CFD_ERR_ARG, "check_every out of range");
    if (k.les_smagorinsky != 0 && k.les_smagorinsky != 1) return fail(CFD_ERR_ARG, "les_smagorinsky must be 0 or 1");
    if (k.inner_solver != CFD_INNER_CG && k.inner_solver != CFD_INNER_BICGSTAB && k.inner_solver != CFD_INNER_MG)
        return fail(CFD_ERR_ARG, "unknown inner solver");
    if (!(k.conv_outflow_uc >= 0.0) || !std::isfinite(k.conv_outflow_uc))
        return fail(CFD_ERR_ARG, "conv_outflow_uc must be finite and >= 0");
    if (k.conv_outflow_uc > 0.0 && !(k.conv_outflow_uc * k.dt <= 0.5 * 1e300))
        return fail(CFD_ERR_ARG, "conv_outflow_uc out of range");
    if (k.precision != CFD_PREC_FP64 && (!(k.inner_tol > 0 && k.inner_tol < 1) || k.max_outer < 1))
        return fail(CFD_ERR_ARG, "mixed precision needs 0 < inner_tol < 1 and max_outer >= 1");
    if (k.precision == CFD_PREC_FP64_DC && k.solver != CFD_SOLVER_BICG_SPE)
        return fail(CFD_ERR_ARG, "CFD_PREC_FP64_DC solves with the matrix-free SPE operator only");
    if (k.periodic_z != 0 && k.periodic_z != 1) return fail(CFD_ERR_ARG, "periodic_z must be 0 or 1");
    if (k.periodic_z && k.solver == CFD_SOLVER_SOR_RB)
        return fail(CFD_ERR_ARG, "periodic z needs a Krylov solver (SPE or ELL), not SOR");
    if (k.solver == CFD_SOLVER_SOR_RB && k.nx_cal > 65535)
        return fail(CFD_ERR_ARG, "the SOR sweeps take at most 65535 cells in x");

    cfd_ctx *c = new cfd_ctx();
    c->cfg = k;
    c->fp32 = k.precision == CFD_PREC_MIXED;
    Geo &g = c->g;
    g.nxc = k.nx_cal; g.nyc = k.ny_cal; g.nzc = k.nz_cal;
    g.nx = g.nxc + 2 * GC; g.ny = g.nyc + 2 * GC; g.nz = g.nzc + 2 * GC;
    g.sx = (long long)g.ny * g.nz; g.sy = g.nz;
    g.sxc = (long long)g.nyc * g.nzc; g.syc = g.nzc;
    g.ng = (long long)g.nx * g.ny * g.nz;
    g.n = n;
    g.fsxc = FastDiv((unsigned int)g.sxc);
    g.fsyc = FastDiv((unsigned int)g.syc);
    g.fsx = FastDiv((unsigned int)g.sx);
    g.fsy = FastDiv((unsigned int)g.sy);
    g.pz = k.periodic_z;
    if (const char *e = std::getenv("CFDGPU_NO_GRAPH")) c->use_graphs = !(e[0] == '1');
    if (const char *e = std::getenv("CFDGPU_SOLVE_LOOP")) c->device_loops = std::strcmp(e, "host") != 0;
    if (const char *e = std::getenv("CFDGPU_DEBUG")) c->debug = std::atoi(e);
    if (const char *e = std::getenv("CFDGPU_NO_FUSED")) c->fused = !(e[0] == '1');
    if (const char *e = std::getenv("CFDGPU_INNER_ADAPT")) c->inner_adapt = std::max(0.0, std::atof(e));
    if (const char *e = std::getenv("CFDGPU_OUTER_LOOP")) c->outer_graph = std::strcmp(e, "host") != 0;
    if (const char *e = std::getenv("CFDGPU_WARM")) {
        c->warm_extrap = std::strcmp(e, "prev") != 0;
        if (std::strcmp(e, "quadratic") == 0) c->warm_order = 2;
    }

    int st = CFD_OK;
    auto bail = [&](int code) { free_ctx(c); return code; };
    cudaError_t e = cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(fail(CFD_ERR_CUDA, std::string("stream: ") + cudaGetErrorString(e)));
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 148;
    const size_t ts = c->fp32 ? sizeof(float) : sizeof(double);
#define AL(ptr, bytes) \
    if ((st = dalloc(c, reinterpret_cast<void **>(&(ptr)), (bytes))) != CFD_OK) return bail(st)
    for (int sl = 0; sl < 3; ++sl)
        for (int q = 0; q < 3; ++q) AL(c->vel[sl][q], (size_t)g.ng * ts);
    if (k.method == CFD_METHOD_PC)
        for (int q = 0; q < 3; ++q) AL(c->cdbuf[q], (size_t)g.ng * ts);
    AL(c->eta, (size_t)g.ng * ts);
    AL(c->f, (size_t)(3 * n) * ts);
    AL(c->src, (size_t)(3 * n) * ts);
    AL(c->p, (size_t)g.ng * sizeof(double));
    AL(c->x, (size_t)n * sizeof(double));
    AL(c->b, (size_t)n * sizeof(double));
    AL(c->jp, (size_t)n * sizeof(double));
    AL(c->raw, (size_t)(3 * (g.nx + g.ny + g.nz) + 3) * sizeof(double));
    {
        double *q = c->raw;
        const int len[9] = {g.nx + 1, g.ny + 1, g.nz + 1, g.nx, g.ny, g.nz, g.nx, g.ny, g.nz};
        for (int a = 0; a < 9; ++a) { c->rawp[a] = q; q += len[a]; c->hraw[a].assign(len[a], 0.0); }
    }
    const int na[3] = {g.nx, g.ny, g.nz};
    const int nc[3] = {g.nxc, g.nyc, g.nzc};
    for (int a = 0; a < 3; ++a) {
        AL(c->tab64[a], (size_t)AX_ROWS * na[a] * sizeof(double));
        AL(c->tab32[a], (size_t)AX_ROWS * na[a] * sizeof(float));
        AL(c->spe_c[a], (size_t)2 * nc[a] * sizeof(double));
    }
    const bool bicg = k.solver != CFD_SOLVER_SOR_RB;
    if (k.solver == CFD_SOLVER_BICG_ELL) {
        AL(c->ell_cols, (size_t)(7 * n) * sizeof(int));
        AL(c->ell_vals, (size_t)(7 * n) * sizeof(double));
    }
    if (bicg && !c->fp32) {
        AL(c->w64.r0, n * 8); AL(c->w64.r1, n * 8); AL(c->w64.p1, n * 8);
        AL(c->w64.s1, n * 8); AL(c->w64.ap, n * 8); AL(c->w64.as, n * 8);
        AL(c->px1, n * 8); AL(c->px2, n * 8);
    }
    if (bicg && c->fp32) {
        AL(c->w64.r0, n * 8);  // FP64 zero vector for |b| in the defect correction
        AL(c->w32.r0, n * 4); AL(c->w32.r1, n * 4); AL(c->w32.p1, n * 4);
        AL(c->w32.s1, n * 4); AL(c->w32.ap, n * 4); AL(c->w32.as, n * 4);
        AL(c->r32, n * 4); AL(c->e32, n * 4);
        AL(c->p_alt, n * 4); AL(c->ap_alt, n * 4);
        for (int a = 0; a < 3; ++a) AL(c->spe_c32[a], (size_t)2 * nc[a] * sizeof(float));
        for (int a = 0; a < 3; ++a) AL(c->fv_sum[a], 2 * (size_t)nc[a] * sizeof(float));
        AL(c->cg_ip, n * 4);
        AL(c->jp32, n * 4);
        AL(c->jp32lo, n * 4);
        if (k.solver == CFD_SOLVER_BICG_ELL) AL(c->ell_vals32, (size_t)(7 * n) * sizeof(float));
    }
    if (!bicg) {
        AL(c->sor_cf, (size_t)(14 * sor_slots(g)) * sizeof(double));
        AL(c->sor_rhs, (size_t)(2 * sor_slots(g)) * sizeof(double));
        AL(c->sor_acc, sizeof(SorAcc));
        bool sweeps32 = c->fp32;
        if (const char *e = std::getenv("CFDGPU_SOR_FP32")) sweeps32 = sweeps32 && e[0] != '0';
        if (sweeps32) {
            AL(c->sor_e, (size_t)g.n * sizeof(float));
            AL(c->sor_rho, (size_t)g.n * sizeof(float));
        }
    }
    AL(c->sc, sizeof(BicgScal));
    AL(c->sc_in, sizeof(BicgScal));
    AL(c->sc_t, sizeof(BicgScal));
    AL(c->os, sizeof(OuterScal));
    AL(c->dscal, 8 * sizeof(double));
    AL(c->mon, 8 * sizeof(double));
    if (k.les_smagorinsky) AL(c->vis, (size_t)n * ts);
    AL(c->dmax, 3 * sizeof(unsigned long long));
    const int red_blocks = blocks_for(n, sms * 8);
    AL(c->lc.partials, (size_t)kMaxReduce * red_blocks * sizeof(double));
    AL(c->lc.counter, sizeof(unsigned int));
    // the largest field crossing the boundary: ghosted, or f / src (3 x compact)
    if (c->fp32) AL(c->staging, (size_t)std::max<long long>(g.ng, 3 * g.n) * sizeof(double));
#undef AL
    if (cudaMallocHost(reinterpret_cast<void **>(&c->h_sc), sizeof(BicgScal)) != cudaSuccess ||
        cudaMallocHost(reinterpret_cast<void **>(&c->h_os), sizeof(OuterScal)) != cudaSuccess ||
        cudaMallocHost(reinterpret_cast<void **>(&c->h_scal), 8 * sizeof(double)) != cudaSuccess ||
        cudaMallocHost(reinterpret_cast<void **>(&c->h_max), 3 * sizeof(unsigned long long)) != cudaSuccess) {
        cudaGetLastError();
        return bail(fail(CFD_ERR_NOMEM, "pinned host allocation failed"));
    }
    c->lc.s = c->s;
    c->lc.red_blocks = red_blocks;
    c->lc.grid_cap = sms * 16;
    c->lc.cg_grid = cg_resident_grid(sms, red_blocks);
    if (c->cg_ip) cg_tma_setup(c->cgtma, fv32(c), c->w32.r0, c->r32, c->w32.p1, c->p_alt, sms, red_blocks);

    // zero everything, then the reference's initial values
    e = cudaMemsetAsync(c->lc.counter, 0, sizeof(unsigned int), c->s);
    BicgScal h{};
    h.tol = k.p_criteria;
    h.restart_tol = 1e-7 * k.p_criteria;  // pRestartFactor_ (bicgstabRe2.hpp:39-42)
    h.maxit = k.p_iter_max;
    BicgScal hin{};
    hin.tol = k.inner_tol;
    hin.restart_tol = 1e-7 * k.inner_tol;
    hin.maxit = k.p_iter_max;
    hin.restart_rel = 1e-5;
    c->sc_init = h;
    c->sc_in_init = hin;
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->sc, &h, sizeof(h), cudaMemcpyHostToDevice, c->s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->sc_in, &hin, sizeof(hin), cudaMemcpyHostToDevice, c->s);
    const size_t zero_bytes[] = {(size_t)g.ng * ts, (size_t)(3 * n) * ts, (size_t)n * 8};
    for (int sl = 0; sl < 3 && e == cudaSuccess; ++sl)
        for (int q = 0; q < 3 && e == cudaSuccess; ++q) e = cudaMemsetAsync(c->vel[sl][q], 0, zero_bytes[0], c->s);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->eta, 0, zero_bytes[0], c->s);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->f, 0, zero_bytes[1], c->s);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->src, 0, zero_bytes[1], c->s);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->p, 0, (size_t)g.ng * 8, c->s);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->x, 0, zero_bytes[2], c->s);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->b, 0, zero_bytes[2], c->s);
    if (e == cudaSuccess && c->px1) e = cudaMemsetAsync(c->px1, 0, zero_bytes[2], c->s);
    if (e == cudaSuccess && c->px2) e = cudaMemsetAsync(c->px2, 0, zero_bytes[2], c->s);
    if (e == cudaSuccess && c->w64.r0) e = cudaMemsetAsync(c->w64.r0, 0, zero_bytes[2], c->s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->s);
    if (e != cudaSuccess) return bail(fail(CFD_ERR_CUDA, std::string("init: ") + cudaGetErrorString(e)));
    *out = c;
    return CFD_OK;
}

int cfd_destroy(cfd_ctx *c)
{
    if (!c) return CFD_OK;
    free_ctx(c);
    return CFD_OK;
}

int cfd_sync(cfd_ctx *c)
{
    CKS(check_ctx(c));
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_grid_uniform(cfd_ctx *c)
{
    CKS(check_ctx(c));
    const Geo &g = c->g;
    const int n[3] = {g.nx, g.ny, g.nz};
    const double L[3] = {c->cfg.lx, c->cfg.ly, c->cfg.lz};
    // grid::init_uniform (structureGrid.hpp:409-440)
    for (int a = 0; a < 3; ++a) {
        const double d = L[a] / (n[a] - 2.0 * GC);
        std::vector<double> &P = c->hraw[a];
        P[0] = 0.0 - 2.0 * d;
        for (int i = 1; i < n[a] + 1; ++i) P[i] = P[i - 1] + d;
        c->hraw[3 + a].assign(n[a], d);
        c->hraw[6 + a].assign(n[a], d);
    }
    return build_tables(c);
}

int cfd_set_metrics(cfd_ctx *c, const double *X, const double *Y, const double *Z, const double *Dx,
                    const double *Dy, const double *Dz, const double *Dxs, const double *Dys,
                    const double *Dzs)
{
    CKS(check_ctx(c));
    const double *in[9] = {X, Y, Z, Dx, Dy, Dz, Dxs, Dys, Dzs};
    for (int q = 0; q < 9; ++q) {
        if (!in[q]) return fail(CFD_ERR_ARG, "null metric array");
        std::memcpy(c->hraw[q].data(), in[q], c->hraw[q].size() * sizeof(double));
    }
    for (int q = 3; q < 9; ++q)
        for (double v : c->hraw[q])
            if (!(v > 0) || !std::isfinite(v)) return fail(CFD_ERR_ARG, "cell widths must be positive and finite");
    return build_tables(c);
}

size_t cfd_field_count(cfd_ctx *c, int field)
{
    if (!c) return 0;
    return field_count(c, field);
}

// the device address of a host buffer of `bytes` bytes that starts on a
// 16-byte boundary and that the GPU can address as a whole (registered and
// mapped, or any memory on systems with address translation such as Grace),
// else null.  The first and the last byte must both map, contiguously: a
// buffer of which only the head lies in a registration goes through copies.
static void *mapped_host(const void *host, size_t bytes)
{
    if ((reinterpret_cast<uintptr_t>(host) & 15u) != 0 || bytes == 0) return nullptr;
    void *dev = nullptr, *dev_last = nullptr;
    const char *last = static_cast<const char *>(host) + (bytes - 1);
    if (cudaHostGetDevicePointer(&dev, const_cast<void *>(host), 0) != cudaSuccess ||
        cudaHostGetDevicePointer(&dev_last, const_cast<char *>(last), 0) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (static_cast<char *>(dev_last) - static_cast<char *>(dev) != (ptrdiff_t)(bytes - 1)) return nullptr;
    return (reinterpret_cast<uintptr_t>(dev) & 15u) == 0 ? dev : nullptr;
}

int cfd_upload(cfd_ctx *c, int field, const double *host, size_t count)
{
    CKS(check_ctx(c));
    if (field < 0 || field >= CFD_FIELD_COUNT) return fail(CFD_ERR_ARG, "unknown field");
    if (!host) return fail(CFD_ERR_ARG, "null host pointer");
    const size_t want = field_count(c, field);
    if (count != want)
        return fail(CFD_ERR_ARG, "element count " + std::to_string(count) + " != " + std::to_string(want));
    bool is_t;
    void *d = field_ptr(c, field, is_t);
    if (const double *hd = static_cast<const double *>(mapped_host(host, count * sizeof(double)))) {
        // host buffer the GPU addresses directly: one kernel reads it over the
        // host link (190 GB/s on GB300), converting on the way
        if (is_t && c->fp32) launch_link_copy<double, float>(c->lc, (long long)count, hd, static_cast<float *>(d));
        else launch_link_copy<double, double>(c->lc, (long long)count, hd, static_cast<double *>(d));
        CK(cudaGetLastError());
    } else if (is_t && c->fp32) {
        CK(cudaMemcpyAsync(c->staging, host, count * sizeof(double), cudaMemcpyHostToDevice, c->s));
        launch_convert<double, float>(c->lc, (long long)count, c->staging, static_cast<float *>(d));
        CK(cudaGetLastError());
    } else {
        CK(cudaMemcpyAsync(d, host, count * sizeof(double), cudaMemcpyHostToDevice, c->s));
    }
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_download(cfd_ctx *c, int field, double *host, size_t count)
{
    CKS(check_ctx(c));
    if (field < 0 || field >= CFD_FIELD_COUNT) return fail(CFD_ERR_ARG, "unknown field");
    if (!host) return fail(CFD_ERR_ARG, "null host pointer");
    const size_t want = field_count(c, field);
    if (count != want)
        return fail(CFD_ERR_ARG, "element count " + std::to_string(count) + " != " + std::to_string(want));
    bool is_t;
    void *d = field_ptr(c, field, is_t);
    // downloads stay on the copy engines: kernel writes over the host link
    // measured 79 GB/s on GB300 against the copy path's better total
    if (is_t && c->fp32) {
        launch_convert<float, double>(c->lc, (long long)count, static_cast<float *>(d), c->staging);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(host, c->staging, count * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    } else {
        CK(cudaMemcpyAsync(host, d, count * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    }
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_host_register(void *host, size_t bytes)
{
    if (!host || !bytes) return fail(CFD_ERR_ARG, "null or empty host buffer");
    CK(cudaHostRegister(host, bytes, cudaHostRegisterMapped | cudaHostRegisterPortable));
    return CFD_OK;
}

int cfd_host_mapped(const void *host)
{
    return mapped_host(host, 1) ? 1 : 0;
}

int cfd_host_mapped_range(const void *host, size_t bytes)
{
    return mapped_host(host, bytes) ? 1 : 0;
}

int cfd_host_unregister(void *host)
{
    if (!host) return fail(CFD_ERR_ARG, "null host buffer");
    CK(cudaHostUnregister(host));
    return CFD_OK;
}

int cfd_init_uniform(cfd_ctx *c, double ui, double vi, double wi)
{
    CKS(check_ctx(c));
    const double val[3] = {ui, vi, wi};
    dispatch(c, [&](auto tag) {
        using T = typename decltype(tag)::type;
        for (int sl = 0; sl < 3; ++sl)
            for (int q = 0; q < 3; ++q) launch_fill<T>(c->lc, c->g.ng, dv<T>(c, sl, q), (T)val[q]);
        return 0;
    });
    CK(cudaMemsetAsync(c->p, 0, (size_t)c->g.ng * sizeof(double), c->s));
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_start(cfd_ctx *c)
{
    CKS(need_metrics(c));
    const size_t ts = c->fp32 ? 4 : 8;
    for (int sl = 1; sl < 3; ++sl)
        for (int q = 0; q < 3; ++q)
            CK(cudaMemcpyAsync(c->vel[sl][q], c->vel[0][q], (size_t)c->g.ng * ts, cudaMemcpyDeviceToDevice, c->s));
    // a fresh solver state: zero warm start and the initial scalars, so a
    // context restarted with cfd_start repeats a fresh context's run
    CK(cudaMemsetAsync(c->x, 0, (size_t)c->g.n * sizeof(double), c->s));
    if (c->px1) CK(cudaMemsetAsync(c->px1, 0, (size_t)c->g.n * sizeof(double), c->s));
    if (c->px2) CK(cudaMemsetAsync(c->px2, 0, (size_t)c->g.n * sizeof(double), c->s));
    CK(cudaMemcpyAsync(c->sc, &c->sc_init, sizeof(BicgScal), cudaMemcpyHostToDevice, c->s));
    CK(cudaMemcpyAsync(c->sc_in, &c->sc_in_init, sizeof(BicgScal), cudaMemcpyHostToDevice, c->s));
    CKS(cfd_bc_main(c, CFD_SLOT_T0));
    CKS(cfd_bc_copy(c, CFD_SLOT_T0, CFD_SLOT_T1));
    c->loop = 1;
    for (int &k : c->warm_n) k = 0;  // the warm-start history starts over
    c->time = 0.0;
    for (int q = 0; q < 3; ++q) {
        c->run_umax[q] = -1e10;
        c->run_umin[q] = 1e10;
    }
    c->cfl_max = 0.0;
    return CFD_OK;
}

int cfd_convection_diffusion(cfd_ctx *c, int src_slot, int dst_slot)
{
    CKS(need_metrics(c));
    CKS(check_slot(src_slot));
    CKS(check_slot(dst_slot));
    if (src_slot == dst_slot) return fail(CFD_ERR_ARG, "source and destination slots must differ");
    const int a = slot_index(src_slot), b = slot_index(dst_slot);
    dispatch(c, [&](auto tag) {
        using T = typename decltype(tag)::type;
        if (c->vis) launch_smagorinsky<T>(c->s, c->g, metrics_of<double>(c), dv<T>(c, a, 0), dv<T>(c, a, 1),
                                          dv<T>(c, a, 2), static_cast<T *>(c->vis));
        launch_convdiff<T>(c->s, c->g, metrics_of<T>(c), (T)c->cfg.dt, (T)((1.0 / c->cfg.re) * c->cfg.dt),
                           dv<T>(c, a, 0), dv<T>(c, a, 1), dv<T>(c, a, 2), dv<T>(c, b, 0), dv<T>(c, b, 1),
                           dv<T>(c, b, 2), nullptr, static_cast<T *>(c->vis), (T)(1.0 / c->cfg.re));
        return 0;
    });
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_add_source(cfd_ctx *c, int slot)
{
    CKS(check_ctx(c));
    CKS(check_slot(slot));
    const int a = slot_index(slot);
    dispatch(c, [&](auto tag) {
        using T = typename decltype(tag)::type;
        launch_src_add<T>(c->lc, c->g, c->cfg.aligned_source, dv<T>(c, a, 0), dv<T>(c, a, 1), dv<T>(c, a, 2),
                          static_cast<T *>(c->src));
        return 0;
    });
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_accumulate_source(cfd_ctx *c)
{
    CKS(check_ctx(c));
    dispatch(c, [&](auto tag) {
        using T = typename decltype(tag)::type;
        launch_src_accumulate<T>(c->lc, 3 * c->g.n, (T)c->cfg.dt, static_cast<T *>(c->src),
                                 static_cast<T *>(c->f));
        return 0;
    });
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_clear_source(cfd_ctx *c)
{
    CKS(check_ctx(c));
    CK(cudaMemsetAsync(c->src, 0, (size_t)(3 * c->g.n) * (c->fp32 ? 4 : 8), c->s));
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_create_b(cfd_ctx *c, int slot, double *mean)
{
    CKS(need_metrics(c));
    CKS(check_slot(slot));
    const int a = slot_index(slot);
    const bool compat = c->cfg.compat_rhs != 0;
    dispatch(c, [&](auto tag) {
        using T = typename decltype(tag)::type;
        launch_rhs<T>(c->lc, c->g, metrics_of<double>(c), 1.0 / c->cfg.dt, c->jp, dv<T>(c, a, 0),
                      dv<T>(c, a, 1), dv<T>(c, a, 2), c->b, compat, c->dscal + 0);
        return 0;
    });
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(c->h_scal, c->dscal, 8 * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    CK(cudaStreamSynchronize(c->s));
    if (mean) *mean = compat ? c->h_scal[0] : 0.0;
    return CFD_OK;
}

int cfd_bicgstab(cfd_ctx *c, int *iters, double *relres)
{
    CKS(need_metrics(c));
    if (c->cfg.solver == CFD_SOLVER_SOR_RB) return fail(CFD_ERR_STATE, "context was created for SOR");
    return poisson_solve(c, iters, relres, nullptr);
}

int cfd_apply_operator(cfd_ctx *c)
{
    CKS(need_metrics(c));
    if (c->cfg.solver == CFD_SOLVER_BICG_ELL) launch_apply(c->lc, ell64(c), c->x, c->b);
    else launch_apply(c->lc, spe64(c), c->x, c->b);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_pressure_transform(cfd_ctx *c)
{
    CKS(check_ctx(c));
    launch_transform(c->s, c->g, c->x, c->p);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_sor(cfd_ctx *c, int slot, int *iters, double *err)
{
    CKS(need_metrics(c));
    CKS(check_slot(slot));
    if (c->cfg.solver != CFD_SOLVER_SOR_RB) return fail(CFD_ERR_STATE, "context was not created for SOR");
    const int a = slot_index(slot);
    return dispatch(c, [&](auto tag) {
        using T = typename decltype(tag)::type;
        return sor_solve_t<T>(c, a, iters, err);
    });
}

int cfd_update_uf(cfd_ctx *c, int src_slot, int dst_slot)
{
    CKS(need_metrics(c));
    CKS(check_slot(src_slot));
    CKS(check_slot(dst_slot));
    const int a = slot_index(src_slot), b = slot_index(dst_slot);
    dispatch(c, [&](auto tag) {
        using T = typename decltype(tag)::type;
        launch_update_uf<T>(c->s, c->g, metrics_of<T>(c), c->cfg.dt, (T)(1.0 / c->cfg.dt), c->p,
                            static_cast<T *>(c->eta), dv<T>(c, a, 0), dv<T>(c, a, 1), dv<T>(c, a, 2),
                            dv<T>(c, b, 0), dv<T>(c, b, 1), dv<T>(c, b, 2), static_cast<T *>(c->f));
        return 0;
    });
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_cdcl(cfd_ctx *c, double *cd, double *cl)
{
    CKS(need_metrics(c));
    dispatch(c, [&](auto tag) {
        using T = typename decltype(tag)::type;
        launch_cdcl<T>(c->lc, c->g, metrics_of<double>(c), c->cfg.lz, static_cast<T *>(c->f), c->dscal + 1);
        return 0;
    });
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(c->h_scal, c->dscal, 8 * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    CK(cudaStreamSynchronize(c->s));
    if (cd) *cd = c->h_scal[1];
    if (cl) *cl = c->h_scal[2];
    return CFD_OK;
}

int cfd_bc_main(cfd_ctx *c, int slot)
{
    CKS(check_ctx(c));
    CKS(check_slot(slot));
    const int a = slot_index(slot);
    const BcTab bc = bc_tab(c);
    dispatch(c, [&](auto tag) {
        using T = typename decltype(tag)::type;
        launch_bc_main<T>(c->s, c->g, bc, dv<T>(c, a, 0), dv<T>(c, a, 1), dv<T>(c, a, 2), c->p);
        return 0;
    });
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_bc_copy(cfd_ctx *c, int from_slot, int to_slot)
{
    CKS(check_ctx(c));
    CKS(check_slot(from_slot));
    CKS(check_slot(to_slot));
    const int a = slot_index(from_slot), b = slot_index(to_slot);
    dispatch(c, [&](auto tag) {
        using T = typename decltype(tag)::type;
        launch_bc_copy<T>(c->s, c->g, dv<T>(c, a, 0), dv<T>(c, a, 1), dv<T>(c, a, 2), dv<T>(c, b, 0),
                          dv<T>(c, b, 1), dv<T>(c, b, 2));
        return 0;
    });
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_copy_velocity(cfd_ctx *c, int from_slot, int to_slot)
{
    CKS(check_ctx(c));
    CKS(check_slot(from_slot));
    CKS(check_slot(to_slot));
    const int a = slot_index(from_slot), b = slot_index(to_slot);
    const size_t bytes = (size_t)c->g.ng * (c->fp32 ? 4 : 8);
    for (int q = 0; q < 3; ++q)
        CK(cudaMemcpyAsync(c->vel[b][q], c->vel[a][q], bytes, cudaMemcpyDeviceToDevice, c->s));
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_eta_cylinder_z(cfd_ctx *c, double cx, double cy, double radius, int nsub)
{
    CKS(need_metrics(c));
    if (nsub < 0 || nsub > 4096 || !(radius > 0)) return fail(CFD_ERR_ARG, "bad cylinder parameters");
    double *eta64 = c->fp32 ? c->staging : static_cast<double *>(c->eta);
    CK(cudaMemsetAsync(eta64, 0, (size_t)c->g.ng * sizeof(double), c->s));
    launch_eta_cylinder_z(c->s, c->g, c->rawp[0], c->rawp[1], c->rawp[3], c->rawp[4], cx, cy, radius, nsub,
                          nsub > 0 ? std::pow((double)nsub, -2.0) : 0.0, eta64);
    if (c->fp32) launch_convert<double, float>(c->lc, c->g.ng, eta64, static_cast<float *>(c->eta));
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_step(cfd_ctx *c, cfd_step_info *info)
{
    CKS(need_metrics(c));
    return dispatch(c, [&](auto tag) {
        using T = typename decltype(tag)::type;
        return step_t<T>(c, info, nullptr);
    });
}

int cfd_div_inf(cfd_ctx *c, int slot, double *out)
{
    CKS(need_metrics(c));
    CKS(check_slot(slot));
    if (!out) return fail(CFD_ERR_ARG, "null output");
    const int a = slot_index(slot);
    CK(cudaMemsetAsync(c->dmax, 0, sizeof(unsigned long long), c->s));
    dispatch(c, [&](auto tag) {
        using T = typename decltype(tag)::type;
        launch_div_inf<T>(c->lc, c->g, metrics_of<double>(c), dv<T>(c, a, 0), dv<T>(c, a, 1), dv<T>(c, a, 2),
                          c->dmax);
        return 0;
    });
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(c->h_max, c->dmax, sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->s));
    CK(cudaStreamSynchronize(c->s));
    std::memcpy(out, c->h_max, sizeof(double));
    return CFD_OK;
}

int cfd_div_projected(cfd_ctx *c, int slot, double *div_inf, double *dev_inf)
{
    CKS(need_metrics(c));
    CKS(check_slot(slot));
    const int a = slot_index(slot);
    CK(cudaMemsetAsync(c->dmax, 0, 2 * sizeof(unsigned long long), c->s));
    const double *mean = c->cfg.compat_rhs ? c->dscal + 0 : nullptr;
    dispatch(c, [&](auto tag) {
        using T = typename decltype(tag)::type;
        launch_div_projected<T>(c->lc, c->g, metrics_of<double>(c), c->cfg.dt, c->p, dv<T>(c, a, 0),
                                dv<T>(c, a, 1), dv<T>(c, a, 2), mean, c->dmax);
        return 0;
    });
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(c->h_max, c->dmax, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->s));
    CK(cudaStreamSynchronize(c->s));
    if (div_inf) std::memcpy(div_inf, c->h_max, sizeof(double));
    if (dev_inf) std::memcpy(dev_inf, c->h_max + 1, sizeof(double));
    return CFD_OK;
}

int cfd_cfl(cfd_ctx *c, int slot, cfd_cfl_info *out)
{
    CKS(need_metrics(c));
    CKS(check_slot(slot));
    if (!out) return fail(CFD_ERR_ARG, "null output");
    const int a = slot_index(slot);
    dispatch(c, [&](auto tag) {
        using T = typename decltype(tag)::type;
        launch_cfl<T>(c->lc, c->g, metrics_of<double>(c), dv<T>(c, a, 0), dv<T>(c, a, 1), dv<T>(c, a, 2), c->mon);
        return 0;
    });
    c->launches += 1;
    CK(cudaGetLastError());
    double h[7];
    CK(cudaMemcpyAsync(h, c->mon, sizeof(h), cudaMemcpyDeviceToHost, c->s));
    CK(cudaStreamSynchronize(c->s));
    out->cfl = h[0] * c->cfg.dt;
    c->cfl_max = std::max(c->cfl_max, out->cfl);
    out->cfl_max = c->cfl_max;
    for (int q = 0; q < 3; ++q) {
        c->run_umax[q] = std::max(c->run_umax[q], h[1 + 2 * q]);
        c->run_umin[q] = std::min(c->run_umin[q], -h[2 + 2 * q]);
        out->u_max[q] = c->run_umax[q];
        out->u_min[q] = c->run_umin[q];
    }
    // simuClass::timestepper (simuClass.hpp:185-199) with its default factors
    const double re = c->cfg.re, cfl_factor = 0.05, grid_fo_factor = 0.15, dt_min = 1e-12;
    double dt = 1e10;
    for (int q = 0; q < 3; ++q) dt = std::min(dt, cfl_factor / (re * out->u_max[q] * out->u_max[q]));
    for (int q = 0; q < 3; ++q) dt = std::min(dt, grid_fo_factor * 0.5 * re * out->u_min[q] * out->u_min[q]);
    out->dt_next = dt < dt_min ? dt_min : dt;
    return CFD_OK;
}

int cfd_smagorinsky(cfd_ctx *c, int slot)
{
    CKS(need_metrics(c));
    CKS(check_slot(slot));
    if (!c->vis) return fail(CFD_ERR_STATE, "the context was created without les_smagorinsky");
    const int a = slot_index(slot);
    dispatch(c, [&](auto tag) {
        using T = typename decltype(tag)::type;
        launch_smagorinsky<T>(c->s, c->g, metrics_of<double>(c), dv<T>(c, a, 0), dv<T>(c, a, 1), dv<T>(c, a, 2),
                              static_cast<T *>(c->vis));
        return 0;
    });
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_steady_max(cfd_ctx *c, int slot_new, int slot_old, double *out)
{
    CKS(need_metrics(c));
    CKS(check_slot(slot_new));
    CKS(check_slot(slot_old));
    if (!out) return fail(CFD_ERR_ARG, "null output");
    const int a = slot_index(slot_new), b = slot_index(slot_old);
    dispatch(c, [&](auto tag) {
        using T = typename decltype(tag)::type;
        launch_steady_max<T>(c->lc, c->g, dv<T>(c, a, 0), dv<T>(c, a, 1), dv<T>(c, a, 2), dv<T>(c, b, 0),
                             dv<T>(c, b, 1), dv<T>(c, b, 2), c->mon);
        return 0;
    });
    c->launches += 1;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, c->mon, 3 * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_sync_periodic_z(cfd_ctx *c, int slot)
{
    CKS(check_ctx(c));
    if (!c->g.pz) return fail(CFD_ERR_STATE, "the context is not periodic in z");
    if (slot == -1) {
        launch_sync_z<double>(c->s, c->g, c->p, nullptr, nullptr);
    } else {
        CKS(check_slot(slot));
        const int a = slot_index(slot);
        dispatch(c, [&](auto tag) {
            using T = typename decltype(tag)::type;
            launch_sync_z<T>(c->s, c->g, dv<T>(c, a, 0), dv<T>(c, a, 1), dv<T>(c, a, 2));
            return 0;
        });
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->s));
    return CFD_OK;
}

int cfd_set_clock(cfd_ctx *c, long long loop, double time)
{
    CKS(check_ctx(c));
    if (loop < 1 || !std::isfinite(time)) return fail(CFD_ERR_ARG, "loop must be >= 1 and time finite");
    c->loop = loop;
    c->time = time;
    for (int &k : c->warm_n) k = 0;  // a restored state: no history
    return CFD_OK;
}

int cfd_get_clock(cfd_ctx *c, long long *loop, double *time)
{
    CKS(check_ctx(c));
    if (loop) *loop = c->loop;
    if (time) *time = c->time;
    return CFD_OK;
}

int cfd_set_step_divergence_check(cfd_ctx *c, int on)
{
    CKS(check_ctx(c));
    c->div_check = on != 0;
    for (double &v : c->last_div) v = -1.0;
    return CFD_OK;
}

int cfd_step_divergence(cfd_ctx *c, double *out3)
{
    CKS(check_ctx(c));
    if (!out3) return fail(CFD_ERR_ARG, "null output");
    if (!c->div_check) return fail(CFD_ERR_STATE, "the step divergence check is off");
    std::memcpy(out3, c->last_div, sizeof(c->last_div));
    return CFD_OK;
}

int cfd_set_test_limits(cfd_ctx *c, int loop_trip_cap, long long tma_wait_limit)
{
    CKS(check_ctx(c));
    c->test_trip_cap = loop_trip_cap > 0 ? loop_trip_cap : 0;
    c->cgtma.wait_limit = tma_wait_limit >= 0 ? tma_wait_limit : (1LL << 24);
    // the cached solve graphs hold the old cap and limit as launch arguments
    for (int q = 0; q < cfd_ctx::kGraphs; ++q) {
        if (c->graph[q]) cudaGraphExecDestroy(c->graph[q]);
        c->graph[q] = nullptr;
        c->graph_batch[q] = 0;
    }
    return CFD_OK;
}

int cfd_launch_count(cfd_ctx *c, long long *count)
{
    CKS(check_ctx(c));
    if (!count) return fail(CFD_ERR_ARG, "null output");
    *count = c->launches;
    return CFD_OK;
}

int cfd_stream(cfd_ctx *c, void **stream)
{
    CKS(check_ctx(c));
    if (!stream) return fail(CFD_ERR_ARG, "null output");
    *stream = (void *)c->s;
    return CFD_OK;
}

int cfd_time_kernels(cfd_ctx *c, int reps, double *ms, int nms)
{
    CKS(need_metrics(c));
    if (!ms || nms < 1 || reps < 1) return fail(CFD_ERR_ARG, "bad arguments");
    for (int k = 0; k < nms && k < CFD_KERNEL_COUNT; ++k) ms[k] = -1.0;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    auto timed = [&](int id, auto &&launch) -> int {
        launch();  // warm-up launch
        CK(cudaEventRecord(e0, c->s));
        for (int r = 0; r < reps; ++r) launch();
        CK(cudaEventRecord(e1, c->s));
        CK(cudaEventSynchronize(e1));
        CK(cudaGetLastError());
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, e0, e1));
        if (id < nms) ms[id] = (double)t / reps;
        return CFD_OK;
    };
    // scratch scalars: never converge, never cap
    BicgScal hs{};
    hs.norm0 = 1.0; hs.rho = 1.0; hs.alpha = 0.5; hs.omega = 0.5; hs.beta = 0.5;
    hs.tol = 0.0; hs.restart_tol = 0.0; hs.maxit = 0x7fffffff; hs.timestep = 1;
    hs.r0n2 = 1.0; hs.rhs_scale = 1.0;
    CK(cudaMemcpyAsync(c->sc_t, &hs, sizeof(hs), cudaMemcpyHostToDevice, c->s));
    int st = CFD_OK;
    const Geo &g = c->g;
    const int G = c->lc.red_blocks;
    if (c->cfg.solver != CFD_SOLVER_SOR_RB) {
        auto run = [&](auto A, auto *x, auto &w) -> int {
            using V = std::remove_pointer_t<decltype(x)>;
            cfd_launch_ctx &lc = c->lc;
            int s2 = CFD_OK;
            if ((s2 = timed(CFD_KERNEL_BICG_AP, [&] { launch_bicg_iteration_part<decltype(A), V>(lc, A, x, w, c->sc_t, 0); })) != CFD_OK) return s2;
            if ((s2 = timed(CFD_KERNEL_BICG_S, [&] { launch_bicg_iteration_part<decltype(A), V>(lc, A, x, w, c->sc_t, 1); })) != CFD_OK) return s2;
            if ((s2 = timed(CFD_KERNEL_BICG_AS, [&] { launch_bicg_iteration_part<decltype(A), V>(lc, A, x, w, c->sc_t, 2); })) != CFD_OK) return s2;
            if ((s2 = timed(CFD_KERNEL_BICG_XR, [&] { launch_bicg_iteration_part<decltype(A), V>(lc, A, x, w, c->sc_t, 3); })) != CFD_OK) return s2;
            return timed(CFD_KERNEL_BICG_P, [&] { launch_bicg_iteration_part<decltype(A), V>(lc, A, x, w, c->sc_t, 4); });
        };
        (void)G;
        if (c->fp32) {
            float *xs = c->e32;
            CK(cudaMemsetAsync(xs, 0, (size_t)g.n * sizeof(float), c->s));
            st = c->cfg.solver == CFD_SOLVER_BICG_ELL ? run(ell32(c), xs, c->w32) : run(spe32(c), xs, c->w32);
        } else {
            double *xs = c->px2;
            CK(cudaMemcpyAsync(xs, c->x, (size_t)g.n * sizeof(double), cudaMemcpyDeviceToDevice, c->s));
            st = c->cfg.solver == CFD_SOLVER_BICG_ELL ? run(ell64(c), xs, c->w64) : run(spe64(c), xs, c->w64);
            CK(cudaMemcpyAsync(c->px2, c->px1, (size_t)g.n * sizeof(double), cudaMemcpyDeviceToDevice, c->s));
        }
        if (st != CFD_OK) return st;
        if (c->fp32 && c->cfg.solver == CFD_SOLVER_BICG_SPE) {
            const FvOp<float> F = fv32(c);
            CK(cudaMemcpyAsync(c->sc_t, &hs, sizeof(hs), cudaMemcpyHostToDevice, c->s));
            CK(cudaMemsetAsync(c->e32, 0, (size_t)g.n * sizeof(float), c->s));
            if ((st = timed(CFD_KERNEL_CG_PQ, [&] {
                     launch_cg_part(c->lc, F, c->cg_ip, c->e32, c->r32, c->w32.r0, c->w32.p1, c->p_alt, c->w32.ap,
                                    c->sc_t, 0, &c->cgtma);
                 })) != CFD_OK)
                return st;
            if ((st = timed(CFD_KERNEL_CG_UPD, [&] {
                     launch_cg_part(c->lc, F, c->cg_ip, c->e32, c->r32, c->w32.r0, c->w32.p1, c->p_alt, c->w32.ap,
                                    c->sc_t, 1);
                 })) != CFD_OK)
                return st;
            if ((st = timed(CFD_KERNEL_RESIDUAL64, [&] {
                     residual64(c, spe64(c), c->b, c->x, c->r32, c->dscal + 5);
                 })) != CFD_OK)
                return st;
            if (c->cfg.inner_solver == CFD_INNER_MG) {
                CKS(mg_setup(c));
                if (c->mg.usable) {
                    const int ids[6] = {CFD_KERNEL_MG_SMOOTH, CFD_KERNEL_MG_RESTRICT, CFD_KERNEL_MG_PROLONG,
                                        CFD_KERNEL_MG_COARSE, CFD_KERNEL_MG_VCYCLE, CFD_KERNEL_MG_SWEEP};
                    for (int part = 0; part < 6; ++part)
                        if (!((part < 3 || part == 5) && mg_grid_levels(c->mg) == 0) &&
                            !(part == 5 && c->mg.lev[0].sweep_tj == 0))
                            if ((st = timed(ids[part], [&] { mg_time_part(c, part); })) != CFD_OK) return st;
                    if ((st = timed(CFD_KERNEL_MG_UPD, [&] {
                             mg_upd(c, c->e32, c->w32.p1, c->r32, c->w32.ap, c->sc_t);
                         })) != CFD_OK)
                        return st;
                    if ((st = timed(CFD_KERNEL_MG_RHO, [&] { mg_rho(c, c->r32, c->w32.r0, nullptr, c->sc_t); })) !=
                        CFD_OK)
                        return st;
                }
            }
        }
    }
    if (c->cfg.solver == CFD_SOLVER_SOR_RB) {
        // sweeps of a copy of p (in T3, or in the FP64 staging buffer of a
        // mixed context) with a tolerance that never stops them
        double *ps = c->fp32 ? c->staging : dv<double>(c, 2, 0);
        CK(cudaMemcpyAsync(ps, c->p, (size_t)g.ng * sizeof(double), cudaMemcpyDeviceToDevice, c->s));
        if ((st = timed(CFD_KERNEL_SOR_SWEEP, [&] {
                 launch_sor_rb_sweep(c->s, g, c->sor_cf, c->sor_rhs, ps, c->cfg.p_sor_omega, -1.0, 0x7fffffff,
                                     c->sc_t, c->sor_acc);
             })) != CFD_OK)
            return st;
        if (c->sor_e && (st = timed(CFD_KERNEL_SOR32_SWEEP, [&] { sor_smooth_sweep(c, &c->sc_t->done); })) != CFD_OK)
            return st;
        if (c->sor_e) CK(cudaMemsetAsync(c->sor_e, 0, (size_t)g.n * sizeof(float), c->s));
    }
    st = dispatch(c, [&](auto tag) -> int {
        using T = typename decltype(tag)::type;
        const Metrics<T> m = metrics_of<T>(c);
        int s2;
        // T3 is scratch here: convection-diffusion T0 -> T3, projection T1 -> T3
        if ((s2 = timed(CFD_KERNEL_CONVDIFF, [&] {
                 launch_convdiff<T>(c->s, g, m, (T)c->cfg.dt, (T)((1.0 / c->cfg.re) * c->cfg.dt), dv<T>(c, 0, 0),
                                    dv<T>(c, 0, 1), dv<T>(c, 0, 2), dv<T>(c, 2, 0), dv<T>(c, 2, 1), dv<T>(c, 2, 2),
                                    nullptr);
             })) != CFD_OK)
            return s2;
        if ((s2 = timed(CFD_KERNEL_UPDATE_UF, [&] {
                 launch_update_uf<T>(c->s, g, m, c->cfg.dt, (T)(1.0 / c->cfg.dt), c->p, static_cast<T *>(c->eta),
                                     dv<T>(c, 1, 0), dv<T>(c, 1, 1), dv<T>(c, 1, 2), dv<T>(c, 2, 0),
                                     dv<T>(c, 2, 1), dv<T>(c, 2, 2), static_cast<T *>(c->f));
             })) != CFD_OK)
            return s2;
        if (c->cfg.method == CFD_METHOD_PC) {
            // a middle pass of the fused step (source in the reference's
            // index convention, right-hand side with the compatibility sums),
            // T1 and T3 both scratch: the pass writes T3 from the stored
            // convection-diffusion, the update reads T3 and writes T1
            PassArgs<T> A{};
            for (int q = 0; q < 3; ++q) {
                A.C[q] = static_cast<const T *>(c->cdbuf[q]);
                A.T1[q] = dv<T>(c, 2, q);
            }
            A.src = static_cast<const T *>(c->src);
            A.src_mode = c->cfg.aligned_source ? 2 : 1;
            A.jp = c->jp;
            A.jph = c->jp32;
            A.jpl = c->jp32lo;
            A.ddt = 1.0 / c->cfg.dt;
            const bool krylov = c->cfg.solver != CFD_SOLVER_SOR_RB;
            A.b = krylov ? c->b : nullptr;
            A.partials = krylov && c->cfg.compat_rhs ? c->lc.partials : nullptr;
            A.counter = c->lc.counter;
            A.mean = c->dscal + 7;
            A.vol = c->vol_total;
            if ((s2 = timed(CFD_KERNEL_PASS, [&] {
                     launch_pass<T>(c->lc, g, metrics_of<double>(c), metrics_of<float>(c), A, false);
                 })) != CFD_OK)
                return s2;
            if ((s2 = timed(CFD_KERNEL_UPDATE_PASS, [&] {
                     launch_update_pass<T>(c->lc, g, m, metrics_of<double>(c), c->cfg.dt, c->p,
                                           static_cast<T *>(c->eta), dv<T>(c, 2, 0), dv<T>(c, 2, 1), dv<T>(c, 2, 2),
                                           dv<T>(c, 1, 0), dv<T>(c, 1, 1), dv<T>(c, 1, 2), static_cast<T *>(c->f),
                                           false, static_cast<T *>(c->src), c->cfg.lz, nullptr);
                 })) != CFD_OK)
                return s2;
        }
        if (c->cfg.solver != CFD_SOLVER_SOR_RB) {
            if ((s2 = timed(CFD_KERNEL_RHS, [&] {
                     launch_rhs<T>(c->lc, g, metrics_of<double>(c), 1.0 / c->cfg.dt, c->jp, dv<T>(c, 1, 0),
                                   dv<T>(c, 1, 1), dv<T>(c, 1, 2), c->b, c->cfg.compat_rhs != 0, c->dscal + 0);
                 })) != CFD_OK)
                return s2;
        }
        return CFD_OK;
    });
    if (st != CFD_OK) return st;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return CFD_OK;
}

}  // extern "C"
