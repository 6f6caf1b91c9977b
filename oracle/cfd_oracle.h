/*
 * cfd_oracle.h -- CPU FP64 restatement of the CFD_NSsolver_forHPC time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This oracle is the checker for the CUDA
 * library: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it.  The product path never calls it.
 *
 * Parity pinning: every function here is checked against the reference's own
 * headers (compiled from a patched scratch copy by oracle/build_ref.py) on
 * seeded inputs, and against the golden fixtures in tests/golden/ that were
 * generated from the reference by tests/golden/make_golden.py.
 *
 * Array conventions follow the reference exactly:
 *   ghosted arrays (u, v, w, p, eta): icel(i,j,k) = i*ny*nz + j*nz + k with
 *     nx = nxCal + 4 etc.  (inc/grid/structureGrid.hpp:159)
 *   compact arrays (b, x, jp, f, src): icelCal(i,j,k) = (i-2)*nyCal*nzCal +
 *     (j-2)*nzCal + (k-2)  (inc/grid/structureGrid.hpp:182)
 *   f and src hold 3 compact components back to back (u, v, w).
 */
#ifndef CFD_ORACLE_H
#define CFD_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nxc, nyc, nzc;           /* interior cells (grid::nxCal, nyCal, nzCal) */
    int nx, ny, nz;              /* ghosted sizes = interior + 4 */
    double lx, ly, lz;
    const double *X, *Y, *Z;     /* node coordinates, length n+1 */
    const double *Dx, *Dy, *Dz;  /* cell widths, ghosted length */
    const double *Dxs, *Dys, *Dzs; /* staggered widths, ghosted length */
    int periodic_z;              /* 1: periodic in z (extension; the reference is Neumann-only
                                    in z); z spacing uniform across the periodic face */
} og_grid;

/* ---- grid generation (structureGrid.hpp:409-440, :326-405, :506-559) ---- */
void og_grid_uniform(int nxc, int nyc, int nzc, double lx, double ly, double lz,
                     double *X, double *Y, double *Z, double *Dx, double *Dy, double *Dz,
                     double *Dxs, double *Dys, double *Dzs);

/* ---- K1: QUICK convection + diffusion, explicit Euler ---- */
void og_convdiff(const og_grid *g, double dt, double nu,
                 const double *u0, const double *v0, const double *w0,
                 double *u1, double *v1, double *w1);

/* ---- predictor-corrector source coupling ---- */
void og_src_add(const og_grid *g, int aligned, double *u1, double *v1, double *w1,
                const double *src);
void og_src_accumulate(const og_grid *g, double dt, double *src, const double *f);

/* ---- K2: Poisson right-hand side ---- */
void og_rhs(const og_grid *g, double dt, const double *jp,
            const double *u1, const double *v1, const double *w1, double *b);
double og_rhs_compat(const og_grid *g, double dt, const double *jp,
                     const double *u1, const double *v1, const double *w1, double *b);

/* ---- matrix-free operator (SPE_sparseMatrix1.hpp) ---- */
void og_spe_setup(const og_grid *g, double *xm, double *xp, double *ym, double *yp,
                  double *zm, double *zp, double *val, double *jp);
void og_spe_spmv(int nxc, int nyc, int nzc,
                 const double *xm, const double *xp, const double *ym, const double *yp,
                 const double *zm, const double *zp, const double *jp,
                 const double *x, double *r);

/* ---- ELL operator (PressureMatrix.hpp + ELL_sparseMatrix.hpp) ---- */
void og_ell_assemble(const og_grid *g, int *cols, double *vals, double *jp);
void og_ell_spmv(long long n, const int *cols, const double *vals, const double *x, double *r);

/* ---- BiCGSTAB (bicgstabRe2.hpp) ---- */
typedef struct og_bicg og_bicg;
og_bicg *og_bicg_create(long long n, double tol, int maxit);
void og_bicg_destroy(og_bicg *s);
/* kind 0 = matrix-free SPE operator, 1 = ELL operator */
void og_bicg_set_spe(og_bicg *s, int nxc, int nyc, int nzc,
                     const double *xm, const double *xp, const double *ym, const double *yp,
                     const double *zm, const double *zp, const double *jp);
void og_bicg_set_ell(og_bicg *s, const int *cols, const double *vals);
/* the SPE operator wraps in z (periodic z, extension) */
void og_bicg_set_periodic_z(og_bicg *s, int periodic_z);
int og_bicg_solve(og_bicg *s, const double *b, double *x, int *iters, double *relres);
void og_bicg_counters(const og_bicg *s, int *timestep, int *total_iters, int *restarts,
                      int *resets);

/* ---- SOR (SorPipeLine.seq.hpp) and its red-black reordering ---- */
void og_sor_coef(const og_grid *g, double *cf);
void og_sor_rhs(const og_grid *g, double dt, const double *u1, const double *v1,
                const double *w1, double *cf);
void og_sor_seq(const og_grid *g, double omega, double tol, int itmax, const double *cf,
                double *p, int *iters, double *err);
void og_sor_redblack(const og_grid *g, double omega, double tol, int itmax,
                     const double *cf, double *p, int *iters, double *err);

/* ---- K5: projection + direct forcing (updateUandF.hpp) ---- */
void og_pressure_transform(const og_grid *g, const double *x, double *p);
void og_update_uf(const og_grid *g, double dt, const double *p, const double *eta,
                  const double *u1, const double *v1, const double *w1,
                  double *u3, double *v3, double *w3, double *f);
void og_cdcl(const og_grid *g, const double *f, double *cd, double *cl);

/* ---- K6: boundary conditions (Boundary_Condition.hpp, updateBC.hpp) ---- */
void og_bc_main(const og_grid *g, const double *dir, const double *num,
                double *u, double *v, double *w, double *p);
void og_bc_copy(const og_grid *g, const double *uo, const double *vo, const double *wo,
                double *u, double *v, double *w);

/* ---- immersed body (setEta.hpp) ---- */
/* nsub >= 1: the reference's nsub x nsub sub-sampling of cut cells;
   nsub == 0: the exact area fraction (extension, og_disc_rect_area) */
void og_eta_cylinder_z(const og_grid *g, double cx, double cy, double radius, int nsub,
                       double *eta);
/* area of the disc of radius r at the origin inside [x0, x1] x [y0, y1] */
double og_disc_rect_area(double x0, double x1, double y0, double y1, double r);

/* ---- diagnostics ---- */
double og_div_inf(const og_grid *g, const double *u, const double *v, const double *w);

/* ---- LES (source/smagorinskyModel.hpp:31-78): eddy viscosity per cell,
   compact; og_convdiff_les uses nu + vis[cell] in the diffusion ---- */
void og_smagorinsky(const og_grid *g, const double *u, const double *v, const double *w, double *vis);
void og_convdiff_les(const og_grid *g, double dt, double nu, const double *vis,
                     const double *u0, const double *v0, const double *w0,
                     double *u1, double *v1, double *w1);

/* ---- monitors (analyses/cfl.hpp:3-80, simuClass.hpp:185-199,
        analyses/CheckSteadystate.hpp:166-215) ---- */
/* cfl = dt * max over cells of (u/Dxs + v/Dys + w/Dzs) (signed, last normal
   face skipped); umax/umin[3] are updated in place (running extremes, the
   reference never resets them), *cfl_max likewise. */
double og_cfl(const og_grid *g, double dt, const double *u, const double *v, const double *w,
              double *umax, double *umin, double *cfl_max);
/* timestepper: min(cflFactor/(Re U^2) over umax, gridFoFactor 0.5 Re U^2
   over umin), at least dt_min */
double og_timestepper(double re, const double *umax, const double *umin, double cfl_factor,
                      double grid_fo_factor, double dt_min);
/* max(0, max over interior of (new - old)) per component */
void og_steady_max(const og_grid *g, const double *u0, const double *v0, const double *w0,
                   const double *u3, const double *v3, const double *w3, double *out3);
double og_dot(const double *a, const double *b, long long n);

/* ---- whole time step (RUN_CPU_PC_METHOD.hpp:287-627, RUN_CPU.hpp:290-462) ---- */
typedef struct {
    int method;        /* 0 = predictor-corrector (default driver), 1 = plain */
    int solver;        /* 0 = BiCGSTAB SPE, 1 = BiCGSTAB ELL, 2 = SOR lexicographic,
                          3 = SOR red-black */
    int aligned_src;   /* 0 = reference index convention, 1 = aligned */
    int compat;        /* subtract the volume-weighted RHS mean before each solve */
    double dt, nu, tol, omega;
    int maxit, sor_maxit;
    double conv_uc;    /* > 0: convective outflow at the x-max face (extension, see og_bc_convective) */
} og_step_cfg;

/* Convective outflow at the x-max face (an extension: the reference has only
   the Dirichlet/Neumann table).  For every interior (j, k), from the old field
   (u0, v0, w0): u on the outflow face nx-3 moves by first-order upwind,
   u_b - C (u_b - u_{b-1}) with C = uc dt / Dx[nx-3], and v, w in the ghost
   cell nx-2 likewise with C = uc dt / Dxs[nx-3]; results go to the new field
   (u3, v3, w3).  Then u on the face is scaled by (inflow flux) / (outflow
   flux), the fluxes being sums of u times Dy Dz over the inflow face (u0 at
   face 1) and the outflow face, and the outer ghosts take the face values. */
void og_bc_convective(const og_grid *g, double dt, double uc, const double *u0, const double *v0,
                      const double *w0, double *u3, double *v3, double *w3);
/* periodic z (g->periodic_z): ghost planes k = 0, 1 take planes k + nzc and
   k = nz-2, nz-1 take k - nzc, over the whole x-y plane; for w, a face
   variable, face nz-3 is the same face as face 1 and is an unknown */
void og_periodic_z(const og_grid *g, double *a);
/* og_bc_main that leaves the x-max face's velocities alone when skip_outflow */
void og_bc_main_ex(const og_grid *g, const double *dir, const double *num, double *u, double *v,
                   double *w, double *p, int skip_outflow);

typedef struct og_sim og_sim;
og_sim *og_sim_create(const og_grid *g, const og_step_cfg *cfg, const double *dir,
                      const double *num, const double *eta);
void og_sim_destroy(og_sim *s);
/* fields: 0..2 T0 u,v,w; 3..5 T1; 6..8 T3; 9 p; 10 eta; 11 f (3N); 12 src (3N);
   13 x (N); 14 b (N); 15 jp (N) */
double *og_sim_field(og_sim *s, int which);
void og_sim_init(og_sim *s, double ui, double vi, double wi);
/* first boundary update: T1 = T3 = T0, BC on T0 and p, boundary copy T0 -> T1 */
void og_sim_start(og_sim *s);
/* one time step; loop counter starts at 1.  Outputs per-pass iterations and
   the last pass's Cd/Cl. */
int og_sim_step(og_sim *s, int *iters4, double *err4, double *cd, double *cl);
long long og_sim_loop(const og_sim *s);
void og_sim_set_loop(og_sim *s, long long loop);

#ifdef __cplusplus
}
#endif
#endif
