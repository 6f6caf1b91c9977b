// kernels.h -- host-side launch interface of the kernels (flow.cu, poisson.cu).
#pragma once

#include <cuda_runtime.h>

#include <cuda.h>

#include "cfd_internal.cuh"

namespace cfd {

struct BcTab {
    double dir[18];
    double num[18];
    // optional per-j Dirichlet value of u on the x-min face (interior j,
    // nyc entries) replacing dir[0]
    const double *inflow;
    // 1: the x-max face's velocities were set by the convective outflow
    // condition (k_bc_conv), so the table leaves them alone
    int skip_outflow;
};

// What a launcher needs besides its arguments: the stream, the fixed shape
// of reduction launches (so sums are reproducible) and their scratch.
struct cfd_launch_ctx {
    cudaStream_t s;
    int red_blocks;         // grid size of every reducing launch
    int grid_cap;           // cap for grid-stride elementwise launches
    int cg_grid;            // resident-block grid of the CG inner kernels (<= red_blocks)
    double *partials;       // kMaxReduce * red_blocks doubles
    unsigned int *counter;  // last-block ticket, zero between launches
};

// ---- flow.cu ----
template <class T>
void launch_convdiff(cudaStream_t s, const Geo &g, const Metrics<T> &m, T dt, T nudt, const T *u0,
                     const T *v0, const T *w0, T *u1, T *v1, T *w1, const T *src_aligned,
                     const T *vis = nullptr, T nu = T(0));
// Smagorinsky eddy viscosity (compact) of (u, v, w)
template <class T>
void launch_smagorinsky(cudaStream_t s, const Geo &g, const Metrics<double> &m, const T *u, const T *v,
                        const T *w, T *vis);
template <class T>
void launch_src_add(cfd_launch_ctx &c, const Geo &g, int aligned, T *u1, T *v1, T *w1, const T *src);
template <class T>
void launch_src_accumulate(cfd_launch_ctx &c, long long n3, T dt, T *src, const T *f);
// One predictor-corrector pass from the step's single convection-diffusion
// C: T1 = C (+ the source), and (b != nullptr) the Poisson right-hand side
// with the compatibility projection (partials != nullptr); flow.cu.
template <class T>
struct PassArgs {
    const T *C[3];
    T *T1[3];
    const T *src;
    int src_mode;            // 0 none, 1 the reference's index convention, 2 aligned
    const double *jp;
    const float *jph, *jpl;  // mixed path: jp as a float pair
    double ddt;
    double *b;
    double *partials;
    unsigned int *counter;
    double *mean;
    double vol;  // total interior volume (the compatibility mean's denominator)
    ff mddt;     // -ddt as a float pair (set by launch_pass)
};
template <class T>
void launch_pass(cfd_launch_ctx &c, const Geo &g, const Metrics<double> &m, const Metrics<float> &m32,
                 const PassArgs<T> &A, bool ghosts);
// update_UandF of one pass with src += dt f (src != nullptr), f stored
// (store_f) and Cd/Cl reduced into cdcl[0..1] (cdcl != nullptr)
template <class T>
void launch_update_pass(cfd_launch_ctx &c, const Geo &g, const Metrics<T> &m, const Metrics<double> &m64, double dt,
                        const double *p, const T *eta, const T *u1, const T *v1, const T *w1, T *u3, T *v3, T *w3,
                        T *f, bool store_f, T *src, double lz, double *cdcl);
// lo[t] = the low float of a[t] as a float pair
void launch_split_lo(cfd_launch_ctx &c, long long n, const double *a, float *lo);
template <class T>
void launch_rhs(cfd_launch_ctx &c, const Geo &g, const Metrics<double> &m, double ddt,
                const double *jp, const T *u1, const T *v1, const T *w1, double *b, bool compat,
                double *mean);
void launch_transform(cudaStream_t s, const Geo &g, const double *x, double *p);
template <class T>
void launch_update_uf(cudaStream_t s, const Geo &g, const Metrics<T> &m, double dt, T rdt,
                      const double *p, const T *eta, const T *u1, const T *v1, const T *w1, T *u3,
                      T *v3, T *w3, T *f);
template <class T>
void launch_cdcl(cfd_launch_ctx &c, const Geo &g, const Metrics<double> &m, double lz, const T *f,
                 double *out2);
template <class T>
void launch_bc_main(cudaStream_t s, const Geo &g, const BcTab &bc, T *u, T *v, T *w, double *p);
template <class T>
void launch_bc_copy(cudaStream_t s, const Geo &g, const T *uo, const T *vo, const T *wo, T *u, T *v,
                    T *w);
void launch_eta_cylinder_z(cudaStream_t s, const Geo &g, const double *X, const double *Y,
                           const double *Dx, const double *Dy, double cx, double cy, double radius,
                           int nsub, double scale, double *eta);
template <class T>
void launch_div_inf(cfd_launch_ctx &c, const Geo &g, const Metrics<double> &m, const T *u,
                    const T *v, const T *w, unsigned long long *slot);
template <class T>
void launch_div_projected(cfd_launch_ctx &c, const Geo &g, const Metrics<double> &m, double dt,
                          const double *p, const T *u1, const T *v1, const T *w1, const double *mean,
                          unsigned long long *slot2, bool with_ustar = false);
template <class T>
void launch_fill(cfd_launch_ctx &c, long long n, T *a, T val);
template <class A, class B>
void launch_convert(cfd_launch_ctx &c, long long n, const A *a, B *b);
// element copy with conversion where a or b is the device mapping of a
// registered host buffer (16-byte aligned)
template <class A, class B>
void launch_link_copy(cfd_launch_ctx &c, long long n, const A *a, B *b);

// ---- poisson.cu ----

// Matrix-free Jacobi-scaled 7-point operator (SPE_matrix1 with jp_on_):
// (A x)_r = x_r - jp_r * (sum over the six neighbours of c_nb x_nb), with the
// per-axis coefficients zeroed on the faces where the neighbour does not
// exist (SPE_sparseMatrix1.hpp:126-144).
template <class V>
struct SpeOp {
    const V *cxm, *cxp, *cym, *cyp, *czm, *czp;  // interior-length axes
    const V *jp;                                  // compact
    int nxc, nyc, nzc;
    long long sxc;
    long long n;
    FastDiv fsxc, fnzc;                           // division by sxc and nzc
    int pz;                                       // 1: the z neighbours wrap (periodic z);
                                                  // czm[0] and czp[nzc - 1] are then non-zero
};

// The finite-volume form M = D_V L of the same operator (D_V = cell
// volumes): (M x)_r = dV_r (diag_r x_r - sum c_nb x_nb), symmetric positive
// semi-definite, with Jacobi preconditioner P_r = dV_r diag_r.  wx/wy/wz are
// the interior cell widths, sx/sy/sz the per-axis sums cm + cp.
template <class V>
struct FvOp {
    SpeOp<V> A;
    const V *wx, *wy, *wz;
    const V *sx, *sy, *sz;
};

// ELL operator, slot-major: vals[s * n + row], cols[s * n + row], s < 7
template <class V>
struct EllOp {
    const int *cols;
    const V *vals;
    long long n;
};

// Device scalars of one BiCGSTAB solve (the locals of bicgstabRe2::solve
// plus its persistent counters).
struct BicgScal {
    double norm0, rho, alpha, omega, beta, relres, tol, restart_tol;
    // restart_rel > 0 selects the scale-invariant restart of the FP32 inner
    // solves: restart when |r1.r0| < restart_rel |r1| |r0| (r0n2 = |r0|^2),
    // re-seeding the shadow residual with r1 and rho with |r1|^2.
    // restart_rel == 0 keeps bicgstabRe2's absolute rule.
    double restart_rel, r0n2;
    int iter, done, restart, timestep, maxit, restarts, total_iters, nonfinite;
    int wait_timeout;  // a bounded device wait (TMA pipeline) gave up
    int loop_trips;    // body runs of the solve's device-side loop (graph WHILE node)
    double rhs_scale;  // the multigrid-CG solves for rhs / rhs_scale; the correction multiplies back
    double qz;         // q . z of the CG stencil launch (flexible beta: h_new . z_old = rho - alpha q . z)
    int pp;            // multigrid CG with one iteration per loop body: which of its two p buffers holds p
};
enum { BICG_RUNNING = 0, BICG_CONVERGED = 1, BICG_CAPPED = 2, BICG_ZERO_RHS = 3 };

// Work vectors of one BiCGSTAB instance (precision V).
template <class V>
struct BicgVecs {
    V *r0, *r1, *p1, *s1, *ap, *as;
};

// convective outflow at the x-max face (extension; the reference has only the
// Dirichlet/Neumann table): from the old field (u0, v0, w0) the outflow face
// u and the ghost v, w move by first-order upwind with speed uc, into the new
// field (u3, v3, w3); then u on that face is scaled so that its flux equals
// the inflow face's (scale_out = flux in / flux out)
template <class T>
void launch_bc_convective(cfd_launch_ctx &c, const Geo &g, const Metrics<double> &m, double dt, double uc,
                          const T *u0, const T *v0, const T *w0, T *u3, T *v3, T *w3, double *scale_out);

// the WHILE condition of a solve loop inside one CUDA graph: continue while
// sc->done is BICG_RUNNING, no bounded wait gave up and the body has run
// fewer than cap times; first != 0 is the check after the head (resets the
// trip count)
void launch_loop_cond(cudaStream_t s, cudaGraphConditionalHandle h, BicgScal *sc, int cap, int first);
// sc->tol = tol, in stream order
void launch_set_tol(cudaStream_t s, BicgScal *sc, double tol);

// The mixed defect correction as one CUDA graph (api.cu, solve_mixed_graph):
// the outer loop's state on the device.  `state` ends as one of OUTER_*.
struct OuterScal {
    double norm0, rel;  // |b| and the last |r| / |b|
    int sweeps, iters, inner_trips, loop_trips, state;
};
enum {
    OUTER_RUNNING = 0, OUTER_CONVERGED = 1, OUTER_CAPPED = 2, OUTER_DIVERGED = 3, OUTER_NONFINITE = 4,
    OUTER_INNER_WAIT = 5, OUTER_INNER_CAP = 6, OUTER_ZERO_RHS = 7
};
// the sweep parameters the graph bakes in
struct OuterCfg {
    double tol, inner_tol, adapt;  // outer tolerance, inner tolerance floor, adaptive factor (0: off)
    int max_outer, cap;            // sweep cap, trip cap of the outer loop
};
// after the first residual (norm2[0] = |r|^2, norm2[1] = |b|^2): the state,
// the first inner tolerance and the WHILE condition
void launch_outer_start(cudaStream_t s, cudaGraphConditionalHandle h, OuterScal *os, const double *norm2,
                        BicgScal *sc_in, OuterCfg cfg);
// after an inner solve: its iterations and trips, and whether it failed
void launch_outer_inner_done(cudaStream_t s, OuterScal *os, const BicgScal *sc_in);
// after the correction and the new residual (norm2[0] = |r|^2): the next
// sweep's inner tolerance and the WHILE condition
void launch_outer_next(cudaStream_t s, cudaGraphConditionalHandle h, OuterScal *os, const double *norm2,
                       BicgScal *sc_in, OuterCfg cfg);
// x = 2 h1 - h0 (h2 null: linear) or 3 h2 - 3 h1 + h0 (quadratic): the
// extrapolation in time of a pass's solution
void launch_extrapolate(cfd_launch_ctx &c, long long n, double *x, const double *h0, const double *h1,
                        const double *h2 = nullptr);
// x += scale e unless the defect correction has stopped (os->state)
void launch_correct_gated(cfd_launch_ctx &c, long long n, double *x, const float *e, const double *scale,
                          const OuterScal *os);

// periodic z: the z ghost planes of up to three fields (null fields skipped)
template <class T>
void launch_sync_z(cudaStream_t s, const Geo &g, T *a0, T *a1, T *a2);

void launch_spe_setup(cudaStream_t s, const Geo &g, const double *Dx, const double *Dy,
                      const double *Dz, const double *Dxs, const double *Dys, const double *Dzs,
                      double *cx, double *cy, double *cz, double *jp);
void launch_ell_assemble(cudaStream_t s, const Geo &g, const double *Dx, const double *Dy,
                         const double *Dz, const double *Dxs, const double *Dys, const double *Dzs,
                         int *cols, double *vals, double *jp);

template <class Op>
void launch_apply(cfd_launch_ctx &c, const Op &A, const double *x, double *r);

// one BiCGSTAB solve: init kernel then the iteration kernels (bicgstabRe2.hpp:93-189)
template <class Op, class V>
void launch_bicg_init(cfd_launch_ctx &c, const Op &A, const V *b, V *x, const BicgVecs<V> &w,
                      V *px1, V *px2, BicgScal *sc);
template <class Op, class V>
void launch_bicg_iteration(cfd_launch_ctx &c, const Op &A, V *x, const BicgVecs<V> &w, BicgScal *sc);
// fused FP32 iteration of the mixed-precision inner solves (SPE operator):
// k_bicg_pap (p update + SpMV), k_bicg_sas (s update + SpMV), k_bicg_xr;
// p/ap alternate between (w.p1, w.ap) and (p_alt, ap_alt)
template <class V>
void launch_bicg_fused_iteration(cfd_launch_ctx &c, const SpeOp<V> &A, V *x, const BicgVecs<V> &w,
                                 V *p_alt, V *ap_alt, BicgScal *sc, int from, bool first);
// FP32 Jacobi-preconditioned CG on M e = P r (the mixed-precision inner
// solve): init, first M p, then (fused p update + M p, update) pairs
void launch_cg_init(cfd_launch_ctx &c, const FvOp<float> &F, float *h, float *p, BicgScal *sc);
// TMA-fed variant of the CG stencil kernel: tensor maps of the z, p and p_alt
// vectors ([nxc][nyc][nzc] FP32, boxes of one (j, k) tile plane with halo),
// built when nzc is a multiple of 4 (16-byte row strides)
struct CgTma {
    bool ok = false;
    int TK = 0, TJ = 0, grid = 0;
    size_t smem = 0;
    bool form_z = false;     // z = h / P formed in the stencil kernel (no z vector)
    long long wait_limit = 1LL << 24;  // try-waits before a pipeline wait gives up
    CUtensorMap zh, p, palt;  // z (or the residual h when form_z), p, p_alt
    CUtensorMap zv;           // the z vector (read by the multigrid-preconditioned CG)
};
// builds the maps for the given buffers; false when TMA cannot be used
bool cg_tma_setup(CgTma &t, const FvOp<float> &F, const float *z, const float *h, const float *p,
                  const float *p_alt, int sms, int red_blocks);
void launch_cg_iteration(cfd_launch_ctx &c, const FvOp<float> &F, const float *iP, float *e, float *h, float *z,
                         float *p, float *p_alt, float *q, BicgScal *sc, int from, bool first,
                         const CgTma *tma = nullptr);
// one full wave of the CG inner kernels on this device, capped at red_blocks
int cg_resident_grid(int sms, int red_blocks);
// one stencil launch of the multigrid-preconditioned CG: pn = z + beta p
// (first: pn = p0), q = M pn, alpha; z is a vector (the V-cycle's output).
// p is read from P[from] and pn written to the other buffer, or, with dyn
// (not first), from buffer sc->pp of (p, p_alt) at run time
void launch_cg_pq_mg(cfd_launch_ctx &c, const FvOp<float> &F, const CgTma *tma, float *z, float *p, float *p_alt,
                     float *q, BicgScal *sc, int from, bool first, bool dyn = false);
// iP = 1 / diag(M), once per context
void launch_cg_ip(cfd_launch_ctx &c, const FvOp<float> &F, float *iP);
void launch_fv_axes(cudaStream_t s, int n, const float *c, const float *width, float *out);
// one CG kernel (0 = fused p update + M p, 1 = update), for timing
void launch_cg_part(cfd_launch_ctx &c, const FvOp<float> &F, const float *iP, float *e, float *h, float *z,
                    float *p, float *pn, float *q, BicgScal *sc, int part, const CgTma *tma = nullptr);
// one kernel of the iteration (0 ap, 1 s, 2 as, 3 xr, 4 p), for timing
template <class Op, class V>
void launch_bicg_iteration_part(cfd_launch_ctx &c, const Op &A, V *x, const BicgVecs<V> &w, BicgScal *sc,
                                int part);
template <class V>
void launch_bicg_nan_reset(cfd_launch_ctx &c, long long n, V *x, const V *px1, const V *px2,
                           BicgScal *sc);

// SorPipeLine (SorPipeLine.seq.hpp:30-117) in red-black order, colour-split.
// Colour c holds the cells with i + j + k + c even; in the row (i, j) they
// sit at k = GC + ((i + j + GC + c) & 1) + 2 m, m < sor_pairs(g) (the last
// slot of a row is unused when its colour has one cell fewer).  Slot
// h = ((i - GC) nyc + (j - GC)) sor_pairs + m of colour c holds
//   cf[(c * 7 + q) * nh + h], q = 0..5: face area / staggered distance
//     towards +x, -x, +y, -y, +z, -z; q = 6: -1 / (their sum);
//   rhs[c * nh + h]: mass change / dt,
// with nh = nxc nyc sor_pairs: every access of a sweep to them is coalesced.
inline long long sor_pairs(const Geo &g) { return (g.nzc + 1) / 2; }
inline long long sor_slots(const Geo &g) { return (long long)g.nxc * g.nyc * sor_pairs(g); }
// running maxima of |change| of the two colours and the last-block ticket
struct SorAcc {
    unsigned long long mx[2];
    unsigned int ticket, pad;
};
void launch_sor_coef_rb(cudaStream_t s, const Geo &g, const double *Dx, const double *Dy, const double *Dz,
                        const double *Dxs, const double *Dys, const double *Dzs, double *cf);
// the right-hand side from (u1, v1, w1); its first thread also starts a solve:
// sc->done = running, sc->iter = 0 sweeps, acc cleared
template <class T>
void launch_sor_rhs_rb(cudaStream_t s, const Geo &g, const Metrics<double> &m, double rdt, const T *u1,
                       const T *v1, const T *w1, double *rhs, BicgScal *sc, SorAcc *acc);
// one sweep (both colours) of p += omega (p_new - p); after the sweep the
// do-while test of SorPipeLine.seq.hpp:112 (max |change| > tol and
// sweeps < itmax) runs on the device: sc->iter = sweeps so far, and when the
// test fails sc->relres = the last max change and sc->done is set.  Sweeps
// issued after that return at once.
void launch_sor_rb_sweep(cudaStream_t s, const Geo &g, const double *cf, const double *rhs, double *p,
                         double omega, double tol, int itmax, BicgScal *sc, SorAcc *acc);
// one colour alone, for timing
void launch_sor_rb_colour(cudaStream_t s, const Geo &g, const double *cf, const double *rhs, double *p,
                          double omega, double tol, int itmax, int colour, BicgScal *sc, SorAcc *acc);
// Mixed-precision SOR: FP32 sweeps on the correction inside an FP64 defect
// correction.  rho = sum_q c_q p_q - rhs - (sum c) p at every cell (FP64,
// stored FP32, icelCal order), the right-hand side of the correction
// equation (sum c) e - sum_q c_q e_q = rho (e = 0 beyond the interior), which
// the level-0 smoother sweeps in FP32 (sor_smooth_sweep, multigrid.cu); then
// p += e, e = 0, and sc->iter += the FP32 sweeps run.  All return at once
// when sc->done.
void launch_sor_residual(cudaStream_t s, const Geo &g, const double *cf, const double *rhs, const double *p,
                         float *rho, const BicgScal *sc);
void launch_sor_correct(cudaStream_t s, const Geo &g, double *p, float *e, int sweeps, BicgScal *sc);

// mixed precision pieces
template <class V>
void launch_residual64(cfd_launch_ctx &c, const SpeOp<double> &A, const double *b, const double *x,
                       V *r32, double *norm2_out, double *bnorm2_out = nullptr);
template <class V>
void launch_residual64_ell(cfd_launch_ctx &c, const EllOp<double> &A, const double *b,
                           const double *x, V *r32, double *norm2_out, double *bnorm2_out = nullptr);
template <class V>
void launch_correct(cfd_launch_ctx &c, long long n, double *x, const V *e, const double *scale = nullptr);


// monitors (flow.cu): out[7] = {max c, max u, -min u, max v, -min v, max w, -min w}
template <class T>
void launch_cfl(cfd_launch_ctx &c, const Geo &g, const Metrics<double> &m, const T *u, const T *v, const T *w,
                double *out);
template <class T>
void launch_steady_max(cfd_launch_ctx &c, const Geo &g, const T *ua, const T *va, const T *wa, const T *ub,
                       const T *vb, const T *wb, double *out);

// ---- adjoint.cu (discrete adjoint; adjoint arrays are FP64) ----
struct UfAdjArgs {
    const double *x;      // pressure at interior cells (compact)
    const double *a3[3];  // adjoint of T3 (ghosted), read only; may be null
    const double *af;     // adjoint of f (compact 3N), may be null
    const double *asrc;   // adjoint of src (3N), may be null
    double src_dt;        // dt of src += dt f
    double wcd, wcl, lz;  // drag/lift weights of the objective
    double *a1[3];        // adjoint of T1 (ghosted), +=
    double *ax;           // adjoint of x (compact), +=
    double *aeta;         // adjoint of eta (ghosted), +=
};
template <class T>
void launch_adj_convdiff(cudaStream_t s, const Geo &g, const Metrics<double> &m, double dt, double nudt,
                         const T *u0, const T *v0, const T *w0, const double *lu, const double *lv,
                         const double *lw, double *au, double *av, double *aw);
template <class T>
void launch_adj_update_uf(cudaStream_t s, const Geo &g, const Metrics<double> &m, double dt,
                          const UfAdjArgs &A, const T *u1, const T *v1, const T *w1, const T *eta);
void launch_adj_rhs(cfd_launch_ctx &c, const Geo &g, const Metrics<double> &m, double ddt, const double *jp,
                    const double *lb, bool compat, double *red, double *au, double *av, double *aw);
void launch_adj_solve_in(cfd_launch_ctx &c, const Geo &g, const Metrics<double> &m, const double *jp,
                         const double *lx, double *red, double *bp);
void launch_adj_solve_out(cfd_launch_ctx &c, const Geo &g, const Metrics<double> &m, const double *jp,
                          const double *w, double *red, double *lb);
void launch_adj_bc_main(cudaStream_t s, const Geo &g, const BcTab &bc, double *au, double *av, double *aw,
                        double *ainflow);
void launch_adj_bc_copy(cudaStream_t s, const Geo &g, double *a0u, double *a0v, double *a0w, double *a1u,
                        double *a1v, double *a1w);
void launch_adj_src_add_ref(cfd_launch_ctx &c, long long n, const double *a1u, const double *a1v,
                            const double *a1w, double *asrc);
void launch_adj_src_add_aligned(cudaStream_t s, const Geo &g, const double *a1u, const double *a1v,
                                const double *a1w, double *asrc);
void launch_adj_cd_gather(cudaStream_t s, const Geo &g, double *a1u, double *a1v, double *a1w, double *cu,
                          double *cv, double *cw, double *asrc);
void launch_gather_interior(cudaStream_t s, const Geo &g, const double *p, double *x);
void launch_adj_add(cfd_launch_ctx &c, long long n, double *a, const double *b);


// ---- multigrid.cu: V-cycle preconditioner of the FP32 inner CG ----
constexpr int kMgMaxLevels = 10;
constexpr long long kMgSmall = 4096;  // levels at or below this size run in one block (larger ones as tiles)
struct MgLevel {
    int nx, ny, nz;
    long long n;
    FastDiv fyz, fz;      // division by ny*nz and nz
    FastDiv fyh, fh;      // division by ny*(nz/2) and nz/2 (cell pairs along k, nz even)
    FastDiv fyq, fq;      // division by ny*(nz/4) and nz/4 (cell quads along k, nz % 4 == 0)
    FastDiv fy2q;         // division by (ny/2)*(nz/4) (pairs of quads in j, ny even)
    const float *cm[3], *cp[3], *sum[3], *w[3];  // per axis: -face, +face, cm + cp, width
    const float *rw[3];   // per axis: 1 / width
    float *x, *b;
    const float *rv, *rg;  // per cell 1 / dV and 1 / diag (small-level kernel only)
    float *xalt;           // second x buffer of a grid-wide level (fused sweeps ping-pong)
    int sweep_tj, sweep_ci;  // fused sweep tiling: j rows and i planes per block (0: not fused)
    bool quads;           // the float4 smoother applies (nz % 4 == 0, aligned arrays)
    int pz;               // 1: periodic in z (nz even: red-black stays a two-colouring)
    float om;             // smoother relaxation: x += om (x_gs - x); 1 is Gauss-Seidel
    bool rows2;           // colour launches run k_mg_smooth4x2 (two j rows a thread)
    int march;            // > 0: ... k_mg_smooth4m instead, marching this many x planes a thread
};
// A grid-wide level whose smoothing phases run as tiles with a recomputed
// halo (multigrid.cu, k_mg_tile): tx == 0 where the level runs colour launches
struct MgTile {
    int tx, ty, h, sweeps;  // interior tile, halo (2 sweeps), sweeps of a phase
    int wx, wy, n4;         // tile extent with halo, quads along k
    int tiles_y;            // tiles along y
    FastDiv fn4, fwy;       // division by n4 and wy
};
constexpr int kMgSmallSmem = 200 * 1024;  // shared-memory bytes for the small levels' x and b
struct MgSmall {
    int first, nlev, pre, post;
    const int *done;
    const float *cinv;   // dense inverse of the coarsest operator (regularised, symmetric), n x n
    const float *image;  // the static part of the shared-memory layout, copied in at the start
    int image_floats;    // its size (a multiple of 4)
    int cinv_off;        // shared-memory float offset of the dense inverse, -1: read it from global
    int rv_off[kMgMaxLevels];   // per small level: per-cell 1 / dV, then 1 / diag
    int tab_off[kMgMaxLevels];  // ... its axis tables (per axis cm, cp, sum, w, 1 / w)
    int off[kMgMaxLevels];      // ... its x, then b (not part of the image)
    MgLevel lev[kMgMaxLevels];
};
// The coarse levels first..nlev-1 of a V-cycle in one thread-block cluster
// of kClusterCtas CTAs (multigrid.cu, k_mg_cluster): CTA r owns the x planes
// [r nx / C, (r + 1) nx / C) of every level in its shared memory, reads its
// neighbours' boundary planes through distributed shared memory, and the
// phases are separated by cluster barriers.
constexpr int kClusterCtas = 8;
constexpr int kClusterThreads = 1024;
constexpr int kMgClusterSmem = 200 * 1024;  // shared memory a CTA may use for its slabs
struct MgCluster {
    int first, nlev, pre, post;
    const int *done;
    const float *cinv;           // dense inverse of the coarsest level (global), nc x nc
    int off[kMgMaxLevels];       // per level: shared-memory float offset of the slab's x, then its b
    int part_off;                // CTA partial sums (the coarsest level's mean)
    MgLevel lev[kMgMaxLevels];
};
struct Mg {
    int nlev = 0, first_small = 0;
    int first_cluster = 0;   // > 0: levels from it on run in k_mg_cluster (else the small kernel)
    int cluster_smem = 0;    // its dynamic shared memory per CTA (bytes)
    int sweeps = 2;  // smoothing sweeps per level, before and after the coarse correction
    int sweeps0 = 2; // ... on the finest level
    int small_sweeps = 2;  // ... on the levels inside the single-block kernel
    bool transfer4 = true; // float4-row restriction / prolongation where the levels allow
    bool rows2 = true;     // colour launches of large float4 levels with even ny: two j rows a thread
    bool cluster = false;  // the coarse levels in one thread-block cluster where they partition;
                           // measured slower than the launches and the small kernel it replaces
    MgTile tile[kMgMaxLevels] = {};  // per grid-wide level: its phases as tiles (tx > 0)
    MgTile tile_r[kMgMaxLevels] = {};      // ... split phases: the launch that ends with the restriction
    bool tile_split[kMgMaxLevels] = {};    // ... the phases run one sweep a launch
    // the exact separable solve of the coarsest level (fast diagonalisation,
    // multigrid.cu): fd_level > 0 is that level, solved in place of the small
    // levels below it
    int fd_level = 0;
    float *fd_v[3] = {};   // per axis: n x n eigenvectors (row i: component i of every mode)
    float *fd_l[3] = {};   // per axis: the eigenvalues, ascending
    bool fd_null = false;  // the mode (0, 0, 0) spans the null space (dropped)
    int fuse_from = kMgMaxLevels;  // from this level down, the first pre-sweep from zero and the
                                   // prolongation + first post-colour each in one pass (float4
                                   // levels); off by default
    int pairs = 1;   // CG iteration pairs per loop body (graph replay) of the inner solve
    float *cinv = nullptr;
    bool usable = false;
    int *never = nullptr;  // a device flag that stays 0 (the ungated V-cycle)
    int small_smem = 0;    // dynamic shared memory of the small-level kernel (bytes)
    bool cinv_smem = false;  // the dense inverse is staged in that shared memory
    float *image = nullptr;  // static part of that shared memory (inverse, per-cell and axis tables)
    int image_floats = 0;
    MgLevel lev[kMgMaxLevels];
};

}  // namespace cfd
