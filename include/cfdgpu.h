/*
 * cfdgpu.h -- C ABI of the GB300 time step for the CFD_NSsolver_forHPC
 * staggered-grid Navier-Stokes / direct-forcing immersed-boundary solver.
 *
 * One context owns one device-resident simulation: the velocity triplets T0,
 * T1, T3, the pressure p, the volume fraction eta, the forcing f, the
 * predictor-corrector source, and the Poisson system (b, x, jp and the
 * operator).  Arrays cross this boundary in the reference's own layouts:
 *
 *   ghosted   icel(i,j,k)    = i*ny*nz + j*nz + k, nx = nx_cal + 4, ...
 *             (inc/grid/structureGrid.hpp:159)
 *   compact   icelCal(i,j,k) = (i-2)*ny_cal*nz_cal + (j-2)*nz_cal + (k-2)
 *             (inc/grid/structureGrid.hpp:182)
 *   f, src    three compact components back to back (u, v, w)
 *
 * so a host array of the reference (std::vector<double>::data()) is uploaded
 * or downloaded with one copy.  Every call returns CFD_OK (0) or a negative
 * cfd_status; cfd_last_error() describes the last failure of the calling
 * thread.  A context is used by one host thread at a time; all its work is
 * ordered on one CUDA stream.
 *
 * Each entry point names the reference function (file:line) it replaces.
 */
#ifndef CFDGPU_H
#define CFDGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CFDGPU_ABI_VERSION 1

typedef struct cfd_ctx cfd_ctx;

typedef enum {
    CFD_OK = 0,
    CFD_ERR_ARG = -1,     /* invalid argument (null pointer, size, slot, enum) */
    CFD_ERR_CUDA = -2,    /* a CUDA runtime call failed */
    CFD_ERR_NOMEM = -3,   /* device allocation failed */
    CFD_ERR_NOCONV = -4,  /* iterative solver hit its iteration cap */
    CFD_ERR_NAN = -5,     /* non-finite values found */
    CFD_ERR_TIMEOUT = -6, /* a bounded device wait gave up */
    CFD_ERR_STATE = -7    /* call not valid in the context's current state */
} cfd_status;

/* Poisson solver (inc/controlPanel.hpp:17-23 selects these at compile time) */
typedef enum {
    CFD_SOLVER_BICG_SPE = 0, /* bicgstabRe2 over the matrix-free SPE_matrix1 operator */
    CFD_SOLVER_BICG_ELL = 1, /* bicgstabRe2 over the ELL matrix of createPressureMatrix */
    CFD_SOLVER_SOR_RB = 3    /* SorPipeLine finite-volume SOR, red-black ordered */
} cfd_solver_kind;

typedef enum {
    CFD_METHOD_PC = 0,   /* runSeqOmp_predictionMethod (inc/run/RUN_CPU_PC_METHOD.hpp:9) */
    CFD_METHOD_PLAIN = 1 /* runSeqOmp (inc/run/RUN_CPU.hpp:11) */
} cfd_method;

typedef enum {
    CFD_PREC_FP64 = 0,  /* everything in FP64, as the reference */
    CFD_PREC_MIXED = 1, /* FP32 fields, FP32 convection-diffusion and inner Krylov
                           iterations; FP64 defect correction of the Poisson
                           residual, FP64 dots and FP64 divergence check */
    CFD_PREC_FP64_DC = 2 /* FP64 fields and flow kernels, as CFD_PREC_FP64, with the
                           mixed path's Poisson solve (FP64 defect correction
                           around the FP32 inner solver): an extension that
                           separates what FP32 fields buy from what the solver buys */
} cfd_precision;

/* Inner solver of the mixed-precision defect correction (matrix-free SPE
   operator; the ELL operator always uses BiCGSTAB). */
typedef enum {
    CFD_INNER_CG = 0,       /* FP32 Jacobi-preconditioned CG on the symmetric
                               finite-volume form M = D_V L of the operator */
    CFD_INNER_BICGSTAB = 1, /* FP32 BiCGSTAB on the Jacobi-scaled operator, restarted
                               when |r1.r0| < 1e-5 |r1||r0| */
    CFD_INNER_MG = 2        /* default: FP32 flexible CG on the finite-volume form
                               preconditioned by a geometric multigrid V-cycle (SPE
                               operator; falls back to Jacobi-PCG where the grid does not
                               coarsen to at most 256 cells) */
} cfd_inner_solver;

/* Velocity slots: the reference's T0 (old), T1 (predicted u*), T3 (new). */
enum { CFD_SLOT_T0 = 0, CFD_SLOT_T1 = 1, CFD_SLOT_T3 = 3 };

/* Field handles for upload/download. */
typedef enum {
    CFD_FIELD_U0 = 0, CFD_FIELD_V0, CFD_FIELD_W0, /* T0 (ghosted) */
    CFD_FIELD_U1, CFD_FIELD_V1, CFD_FIELD_W1,     /* T1 (ghosted) */
    CFD_FIELD_U3, CFD_FIELD_V3, CFD_FIELD_W3,     /* T3 (ghosted) */
    CFD_FIELD_P,                                  /* pressure::p (ghosted) */
    CFD_FIELD_ETA,                                /* DfibArray::eta (ghosted) */
    CFD_FIELD_F,                                  /* DfibArray::f (3 x compact) */
    CFD_FIELD_SRC,                                /* PC source_termF (3 x compact) */
    CFD_FIELD_X,                                  /* MxClass::X_result (compact) */
    CFD_FIELD_B,                                  /* MxClass::matB (compact) */
    CFD_FIELD_JP,                                 /* grid::jp Jacobi scaling (compact) */
    CFD_FIELD_VIS,                                /* velocity::Viseff eddy viscosity (compact, LES) */
    CFD_FIELD_COUNT
} cfd_field;

typedef struct {
    int nx_cal, ny_cal, nz_cal; /* interior cells, grid::nxCal.. (structureGrid.hpp:44-46) */
    double lx, ly, lz;          /* domain lengths (structureGrid.hpp:34) */
    double re;                  /* simuClass::set_Re (simuClass.hpp:39) */
    double dt;                  /* simuClass::set_dt (simuClass.hpp:108) */
    int method;                 /* cfd_method */
    int solver;                 /* cfd_solver_kind */
    int precision;              /* cfd_precision */
    double p_criteria;          /* simuClass::p_criteria, solver tolerance (simuClass.hpp:74) */
    int p_iter_max;             /* bicgstabRe2 iters_max_ (bicgstabRe2.hpp:57) */
    double p_sor_omega;         /* simuClass::p_sor_omega (simuClass.hpp:78) */
    int p_sor_iter_max;         /* simuClass::p_sor_iter_max (simuClass.hpp:80) */
    int aligned_source;         /* 0: add the PC source with the reference's compact
                                   index into the ghosted array (RUN_CPU_PC_METHOD.hpp:314);
                                   1: add it at the cell it belongs to */
    int compat_rhs;             /* 1: subtract the volume-weighted mean of the unscaled
                                   Poisson RHS (makes the singular Neumann system
                                   consistent; needed for tolerances below ~1e-6) */
    double bc_dir[6][3];        /* Dirichlet table Dir[face][component] */
    double bc_num[6][3];        /* Neumann table Num[face][component]
                                   (Boundary_Condition.hpp:4-31) */
    int check_every;            /* BiCGSTAB iterations per loop body of the device-side
                                   solve loop (per host poll without graphs) (>= 1) */
    double inner_tol;           /* mixed precision: relative tolerance of each FP32
                                   inner solve inside the FP64 defect correction */
    int max_outer;              /* mixed precision: defect-correction sweeps cap */
    int inner_solver;           /* mixed precision: cfd_inner_solver */
    int les_smagorinsky;        /* 1: Smagorinsky eddy viscosity added to nu in the diffusion
                                   (source/smagorinskyModel.hpp:31, TERBULENCE_SMAGORINSKY) */
    double conv_outflow_uc;     /* > 0: convective outflow at the x-max face with this speed
                                   (first-order upwind of u on the face and of v, w in the ghost
                                   cells, outflow flux scaled to the inflow flux at the end of
                                   every step); 0: the Dirichlet/Neumann table (the reference's) */
    int periodic_z;             /* 1: periodic in z (an extension; the reference's table has
                                   only Dirichlet/Neumann faces, Boundary_Condition.hpp:4-31):
                                   the two ghost planes at each z end take the interior planes
                                   one period away, the top w face is an unknown like the
                                   others, and the Poisson operators wrap in z.  The Krylov
                                   solvers only (not SOR); no adjoint. */
} cfd_config;

typedef struct {
    long long loop;      /* simuClass::loop after the step */
    double time;         /* simuClass::time after the step */
    int iters[4];        /* per pass: solver iterations (simuClass::iters) */
    double relres[4];    /* per pass: relative residual / SOR change (simuClass::error) */
    int outer[4];        /* per pass: defect-correction sweeps (mixed precision) */
    double cd, cl;       /* drag and lift of the final pass (Delay_IO_CD_CL) */
} cfd_step_info;

/* ---- lifetime ---------------------------------------------------------- */
int cfd_abi_version(void);
const char *cfd_last_error(void);
/* Fill *cfg with the reference defaults for an nx x ny x nz interior grid. */
int cfd_config_default(cfd_config *cfg, int nx_cal, int ny_cal, int nz_cal);
int cfd_create(const cfd_config *cfg, cfd_ctx **out);
int cfd_destroy(cfd_ctx *ctx);
int cfd_sync(cfd_ctx *ctx);

/* ---- grid and state ---------------------------------------------------- */
/* grid::init_uniform (structureGrid.hpp:409-440) computed on the host */
int cfd_grid_uniform(cfd_ctx *ctx);
/* Metrics of any staggered grid: X,Y,Z have n+1 nodes, the rest n (ghosted). */
int cfd_set_metrics(cfd_ctx *ctx, const double *X, const double *Y, const double *Z,
                    const double *Dx, const double *Dy, const double *Dz,
                    const double *Dxs, const double *Dys, const double *Dzs);
/* count must equal the field's element count (ghosted, compact or 3 x compact). */
int cfd_upload(cfd_ctx *ctx, int field, const double *host, size_t count);
int cfd_download(cfd_ctx *ctx, int field, double *host, size_t count);
size_t cfd_field_count(cfd_ctx *ctx, int field);
/* Page-lock and map a host buffer (cudaHostRegister, mapped).  cfd_upload
   reads a host buffer the GPU can address (registered and mapped, or any host
   memory on systems with address translation such as Grace) that starts on a
   16-byte boundary with one kernel over the host link, conversion to FP32
   fields included; other buffers, and every download, go through copies.
   Both forms give identical data. */
int cfd_host_register(void *host, size_t bytes);
int cfd_host_unregister(void *host);
/* 1 when the GPU can address this byte of host memory, else 0. */
int cfd_host_mapped(const void *host);
/* 1 when cfd_upload reads a buffer of `bytes` bytes at `host` by the direct
   kernel path (aligned, first and last byte mapped contiguously), else 0. */
int cfd_host_mapped_range(const void *host, size_t bytes);
/* velocity::iniU (physicalVariables.hpp:53) on T0, T1, T3 and p = 0
   (RUN_CPU_PC_METHOD.hpp:84-89) */
int cfd_init_uniform(cfd_ctx *ctx, double ui, double vi, double wi);
/* First boundary update: T1 = T3 = T0, BC_staggered_main(T0, p),
   BC_staggered_copy(T0 -> T1)  (RUN_CPU_PC_METHOD.hpp:114-119) */
int cfd_start(cfd_ctx *ctx);

/* simuClass::loop and simuClass::time (simuClass.hpp:92-94): the step
   counter (the first step, loop 1, solves no Poisson equation) and the time.
   Setting them restarts a run from fields uploaded from elsewhere (another
   context, another precision, a Plot3D file), and drops the history the
   mixed path's warm start extrapolates from (cfd_step). */
int cfd_set_clock(cfd_ctx *ctx, long long loop, double time);
int cfd_get_clock(cfd_ctx *ctx, long long *loop, double *time);

/* ---- the hot-path operators --------------------------------------------- */
/* ConvectionDifussion(simu, T[src], T[dst]) (convection_and_difussion.hpp:168) */
int cfd_convection_diffusion(cfd_ctx *ctx, int src_slot, int dst_slot);
/* T[slot] += source_termF (RUN_CPU_PC_METHOD.hpp:309-316) */
int cfd_add_source(cfd_ctx *ctx, int slot);
/* source_termF += dt * Dfib.f (RUN_CPU_PC_METHOD.hpp:393-401) */
int cfd_accumulate_source(cfd_ctx *ctx);
/* source_termF = 0 (RUN_CPU_PC_METHOD.hpp:290) */
int cfd_clear_source(cfd_ctx *ctx);
/* createBMatrix_omp(T[slot], Mx) (b_matrix.hpp:51), plus the compatibility
   projection when cfg.compat_rhs is set; *mean receives the removed mean
   (may be NULL) */
int cfd_create_b(cfd_ctx *ctx, int slot, double *mean);
/* bicgstabRe2::operator()(Mx.matB, Mx.X_result) (bicgstabRe2.hpp:46, 93-189);
   returns CFD_ERR_NOCONV when the cap was hit (x then got the NaN reset of
   lines 143-163).  In mixed precision this is the FP64 defect correction. */
int cfd_bicgstab(cfd_ctx *ctx, int *iters, double *relres);
/* B = A X with the configured operator (SPE_matrix1::multiply_omp,
   SPE_sparseMatrix1.hpp:259, or ELL_matrix::multiply_omp, ELL_sparseMatrix.hpp:478) */
int cfd_apply_operator(cfd_ctx *ctx);
/* Pressure_transform_X_result (Transform.hpp:8-24) */
int cfd_pressure_transform(cfd_ctx *ctx);
/* SorPipeLine (SorPipeLine.seq.hpp:4-122) on T[slot], red-black ordered */
int cfd_sor(cfd_ctx *ctx, int slot, int *iters, double *err);
/* update_UandF_omp(Dfib, simu, p, T[src], T[dst]) (updateUandF.hpp:95-190) */
int cfd_update_uf(cfd_ctx *ctx, int src_slot, int dst_slot);
/* virtualF_Int + Delay_IO_CD_CL's coefficients (virtualForceIntergrator.hpp:5-37,
   120-127) from the current f */
int cfd_cdcl(cfd_ctx *ctx, double *cd, double *cl);
/* BC_staggered_main(T[slot], p) (Boundary_Condition.hpp:37-175) */
int cfd_bc_main(cfd_ctx *ctx, int slot);
/* BC_staggered_copy(T[from] -> T[to]) (updateBC.hpp:6-111) */
int cfd_bc_copy(cfd_ctx *ctx, int from_slot, int to_slot);
/* velocity::copy_omp (physicalVariables.hpp:84-102) */
int cfd_copy_velocity(cfd_ctx *ctx, int from_slot, int to_slot);
/* Periodic z (cfg.periodic_z): copy the interior planes one period away into
   the z ghost planes of velocity slot `slot`, or of the pressure when slot is
   -1.  cfd_step does this after each convection-diffusion pass (T1) and
   after each pressure transform (p); cfd_bc_main does it for its slot and p. */
int cfd_sync_periodic_z(cfd_ctx *ctx, int slot);
/* DFIB_CylinderZ (setEta.hpp:136-204) with explicit centre and radius: cut
   cells sub-sampled nsub x nsub as the reference does (nsub >= 1), or their
   exact area fraction (nsub == 0, an extension) */
int cfd_eta_cylinder_z(cfd_ctx *ctx, double cx, double cy, double radius, int nsub);
/* One iteration of the main loop of the configured driver
   (RUN_CPU_PC_METHOD.hpp:287-627 or RUN_CPU.hpp:290-462, without IO).  The
   FP64 path starts each Poisson solve from the previous solve's solution, as
   the reference does; the mixed and FP64-defect-correction paths start pass
   k from its own solutions of the two previous steps, extrapolated linearly
   in time (environment CFDGPU_WARM=prev: the reference's start). */
int cfd_step(cfd_ctx *ctx, cfd_step_info *info);
/* max |div T[slot]| over interior cells, FP64 */
int cfd_div_inf(cfd_ctx *ctx, int slot, double *out);
/* Divergence of the projected field T2 = u* - dt grad p that update_UandF
   forms (updateUandF.hpp:136, 158, 179), with u* = T[slot] and the current p,
   using the reference's face rules (boundary faces and the skipped last
   normal faces are not projected).  *div_inf = max |div T2|; *dev_inf =
   max |div T2 + dt * m| where m is the RHS mean removed by the last
   compatibility projection (0 when compat_rhs is off): the part of the
   divergence a converged pressure solve is responsible for.  FP64. */
int cfd_div_projected(cfd_ctx *ctx, int slot, double *div_inf, double *dev_inf);

/* Divergence check inside cfd_step (no counterpart in the reference).  With
   on != 0, every later cfd_step that solves a Poisson equation measures, after
   the last pass's solve and before the boundary update rewrites T1's faces,
   what cfd_div_projected measures on T1: out3[0] = max |div T2|, out3[1] =
   max |div T2 + dt m| (the part a converged solve answers for), and out3[2] =
   max |div u*|, the divergence the projection had to remove.  One extra FP64
   reduction per step.  cfd_step_divergence returns the last step's values
   (-1 before the first such step). */
int cfd_set_step_divergence_check(cfd_ctx *ctx, int on);
int cfd_step_divergence(cfd_ctx *ctx, double *out3);

/* ---- instrumentation ---------------------------------------------------- */
/* Number of kernels the context has issued from the time-step and solver
   paths (cfd_step, cfd_bicgstab, cfd_sor and what they call), counting every
   kernel node of a replayed CUDA graph, including Krylov iterations queued
   past convergence that return at once. */
int cfd_launch_count(cfd_ctx *ctx, long long *count);

/* Test hooks (no counterpart in the reference).  Every device-side wait of
   the solvers is bounded, so that a lost copy or a solve that never reports
   completion ends with CFD_ERR_TIMEOUT instead of hanging the GPU; these
   lower the bounds so tests can make them run out on purpose:
     loop_trip_cap > 0   caps the body runs of every device-side solve loop
                         (a CUDA-graph WHILE node); a solve still running at
                         the cap returns CFD_ERR_TIMEOUT.  0 restores the
                         default (enough runs for cfg.p_iter_max iterations).
     tma_wait_limit >= 0 is the number of try-waits after which a wait of the
                         TMA pipeline of the FP32 CG stencil gives up (0: at
                         once).  The block then issues no more copies, waits
                         out those in flight and skips the rest of its work;
                         the solve returns CFD_ERR_TIMEOUT.  < 0 restores the
                         default (2^24).
   The state of the solve that timed out is undefined; the context stays
   usable. */
int cfd_set_test_limits(cfd_ctx *ctx, int loop_trip_cap, long long tma_wait_limit);

/* The context's CUDA stream (a cudaStream_t), for callers that record events
   or order their own work on it. */
int cfd_stream(cfd_ctx *ctx, void **stream);

/* Kernels timed by cfd_time_kernels, in ms[] order. */
typedef enum {
    CFD_KERNEL_BICG_AP = 0,  /* ap = A p1 and ap.r0            (bicgstabRe2.hpp:120-121) */
    CFD_KERNEL_BICG_S,       /* s = r1 - alpha ap              (:122-124) */
    CFD_KERNEL_BICG_AS,      /* as = A s, as.s and as.as       (:126-128) */
    CFD_KERNEL_BICG_XR,      /* x, r1 update, |r1|^2 and r1.r0 (:130-138, 167) */
    CFD_KERNEL_BICG_P,       /* p1 = r1 + beta (p1 - omega ap) (:172-176) */
    CFD_KERNEL_CONVDIFF,     /* ConvectionDifussion */
    CFD_KERNEL_UPDATE_UF,    /* update_UandF_omp */
    CFD_KERNEL_RHS,          /* createBMatrix_omp (+ compatibility mean) */
    CFD_KERNEL_SOR_SWEEP,    /* one red + one black SOR sweep */
    CFD_KERNEL_CG_PQ,        /* mixed precision: p = z + beta p, q = M p, p.q (FP32) */
    CFD_KERNEL_CG_UPD,       /* mixed precision: e, h, z update and h.z (FP32) */
    CFD_KERNEL_RESIDUAL64,   /* mixed precision: FP64 residual b - A x of the defect correction */
    CFD_KERNEL_MG_SMOOTH,    /* multigrid: one colour of a Gauss-Seidel sweep on the finest level */
    CFD_KERNEL_MG_RESTRICT,  /* multigrid: residual of the finest level summed to the next */
    CFD_KERNEL_MG_PROLONG,   /* multigrid: coarse correction added to the finest level */
    CFD_KERNEL_MG_COARSE,    /* multigrid: the coarse solve (the separable solve of the coarsest
                                level, or the single-block sub-cycle of the small levels) */
    CFD_KERNEL_MG_VCYCLE,    /* multigrid: one whole V-cycle (all its launches) */
    CFD_KERNEL_MG_UPD,       /* multigrid CG: e, h update */
    CFD_KERNEL_MG_RHO,       /* multigrid CG: h.z and the scalar update */
    CFD_KERNEL_MG_SWEEP,     /* multigrid: one fused red-black sweep on the finest level */
    CFD_KERNEL_PASS,         /* predictor-corrector pass: T1 = C + source and the right-hand side */
    CFD_KERNEL_UPDATE_PASS,  /* predictor-corrector pass: update_UandF with src += dt f */
    CFD_KERNEL_SOR32_SWEEP,  /* mixed precision: one red + one black FP32 sweep on the SOR correction */
    CFD_KERNEL_COUNT
} cfd_kernel_id;

/* Mean device time (ms) of one launch of each hot kernel, measured with CUDA
   events around `reps` back-to-back launches on the context stream.  The
   Krylov kernels run on the solver's scratch vectors and a scratch copy of
   x, the SOR sweep on a copy of p; the flow kernels write T3 and the
   predictor-corrector source, both rewritten by the next step before they
   are read.  Call it between steps.  ms[k] < 0 marks a kernel the context
   does not use.  nms is the length of ms (at most CFD_KERNEL_COUNT
   entries are written). */
int cfd_time_kernels(cfd_ctx *ctx, int reps, double *ms, int nms);

/* ---- allocation-free drag and lift ------------------------------------- */
/* No counterpart in the reference.  The same drag and lift as cfd_cdcl, for
   callers that cannot allocate device memory: an application whose own pool
   owns the GPU's memory and forbids allocations outside it, or a loop that
   cannot afford the device-wide synchronisation a cudaMalloc may cause.
   The caller passes device arrays: Dx, Dy, Dz (ghosted widths, nx_cal+4 ...
   entries) and f (3 x compact forcing, DfibArray::f layout); cd and cl are
   host outputs.  The work is ordered on `stream` (a cudaStream_t, NULL for
   the default stream), which is synchronised before returning.
   Nothing is allocated by the call: the scratch is one file-scope device
   array of about 1 MiB that every GPU that loads the library keeps until the
   process exits.  With lazy module loading (the CUDA default) that array
   comes into existence when the library's device code is first loaded on a
   device, which the first call on that device may do; a caller whose pool
   takes the GPU's memory should make one call (or create any context)
   before handing the memory to its pool.  At most CFD_NOALLOC_MAX_CELLS
   interior cells; larger grids return CFD_ERR_ARG.  Each call outside stream
   capture looks up the array's device address with the device current (a
   device reset moves it); a call during capture reuses the last address
   found on that device, so make the first call before any capture.  Every
   call uses the same scratch: calls that overlap on the GPU (other streams,
   other host threads) race and must be serialised. */
#define CFD_NOALLOC_MAX_CELLS 268435456
int cfd_cdcl_noalloc(int nx_cal, int ny_cal, int nz_cal, double lz, const double *Dx,
                     const double *Dy, const double *Dz, const double *f, double *cd, double *cl,
                     void *stream);


/* ---- inflow profile -------------------------------------------------------
   Per-j Dirichlet value of u on the x-min face (ny_cal values, interior j in
   order), replacing the scalar bc_dir[0][0] in BC_staggered_main
   (Boundary_Condition.hpp:72-76, face 0, component u).  u_in = NULL restores
   the scalar.  The profile is a parameter of the discrete adjoint below.   */
int cfd_set_inflow_profile(cfd_ctx *ctx, const double *u_in, size_t ny_cal);

/* ---- discrete adjoint -------------------------------------------------------
   No counterpart in the reference: the reverse-mode derivative of the time
   step, kernel by kernel.  Adjoint arrays are FP64 in every context and use
   the forward layouts; each cfd_adj_* kernel entry applies the transpose of
   the linearised forward function named beside it to the adjoint fields.
   Supported for the Krylov solvers (SPE, ELL); the adjoint Poisson solves use
   FP64 defect correction around FP32 CG on the finite-volume operator, to the
   forward tolerance.                                                        */
typedef enum {
    CFD_ADJ_U0 = 0, CFD_ADJ_V0, CFD_ADJ_W0, /* adjoint of T0 (ghosted)                  */
    CFD_ADJ_U1, CFD_ADJ_V1, CFD_ADJ_W1,     /* adjoint of T1 (ghosted)                  */
    CFD_ADJ_U3, CFD_ADJ_V3, CFD_ADJ_W3,     /* adjoint of T3 (ghosted)                  */
    CFD_ADJ_CDU, CFD_ADJ_CDV, CFD_ADJ_CDW,  /* adjoint of the convection-diffusion
                                               output (ghosted)                         */
    CFD_ADJ_X,                              /* adjoint of x / interior p (compact)      */
    CFD_ADJ_B,                              /* adjoint of b (compact)                   */
    CFD_ADJ_F,                              /* adjoint of f (compact, 3 components)     */
    CFD_ADJ_SRC,                            /* adjoint of source_termF (compact, 3)     */
    CFD_ADJ_ETA,                            /* gradient w.r.t. eta (ghosted)            */
    CFD_ADJ_INFLOW                          /* gradient w.r.t. the inflow profile (ny)  */
} cfd_adj_field;

/* Allocates the adjoint state and a tape of tape_len steps (needs metrics).  */
int cfd_adj_enable(cfd_ctx *ctx, int tape_len);
int cfd_adj_zero(cfd_ctx *ctx);                      /* every adjoint field = 0 */
size_t cfd_adj_field_count(cfd_ctx *ctx, int field);
int cfd_adj_upload(cfd_ctx *ctx, int field, const double *host, size_t count);
int cfd_adj_download(cfd_ctx *ctx, int field, double *host, size_t count);

/* Kernel adjoints (transposes of the forward entry points' linearisations):
   ADJ_T0 += (d ConvectionDifussion(slot) / d slot)^T ADJ_CD       (cfd_convection_diffusion) */
int cfd_adj_convection_diffusion(cfd_ctx *ctx, int src_slot);
/* ADJ_T1, ADJ_X, ADJ_ETA += transpose of update_UandF(slot) applied to
   (ADJ_T3, ADJ_F + the drag/lift weights: J += wcd Cd + wcl Cl)   (cfd_update_uf + cfd_cdcl) */
int cfd_adj_update_uf(cfd_ctx *ctx, int src_slot, double wcd, double wcl);
/* ADJ_T1 += createBMatrix^T ADJ_B (with the compatibility projection when
   cfg.compat_rhs)                                                  (cfd_create_b) */
int cfd_adj_create_b(cfd_ctx *ctx);
/* ADJ_B = A^-T ADJ_X on the range of the singular operator         (cfd_bicgstab) */
int cfd_adj_pressure_solve(cfd_ctx *ctx, int *iters, double *relres);
/* ADJ_SRC += adjoint of the PC source coupling of ADJ_T1           (cfd_add_source) */
int cfd_adj_add_source(cfd_ctx *ctx);
/* ADJ_T0 (in place) and ADJ_INFLOW: BC_staggered_main^T            (cfd_bc_main) */
int cfd_adj_bc_main(cfd_ctx *ctx);
/* ADJ_T0 += ADJ_T1 on the copied faces, which are cleared          (cfd_bc_copy) */
int cfd_adj_bc_copy(cfd_ctx *ctx);

/* Tape.  cfd_step_record is cfd_step that also stores the step's input
   velocity and the pressure of each pass at tape position pos (0 <= pos <
   tape_len).  cfd_adj_step reverses the step recorded at pos: it replays the
   passes from the tape (no Poisson solves) in adjoint-owned buffers, then
   applies the adjoint of every operation of the step in reverse order; the
   objective's weights on that step's drag and lift are wcd, wcl.  The
   forward state of the context is not modified.  cfd_adj_finish applies the
   adjoint of cfd_start's boundary conditions after the first step.         */
typedef struct {
    int iters[4];     /* adjoint Poisson solve iterations (FP32 inner) per pass */
    double relres[4]; /* final FP64 relative residuals                         */
} cfd_adj_step_info;
int cfd_step_record(cfd_ctx *ctx, int pos, cfd_step_info *info);
int cfd_adj_step(cfd_ctx *ctx, int pos, double wcd, double wcl, cfd_adj_step_info *info);
int cfd_adj_finish(cfd_ctx *ctx);

/* Checkpoints of the forward state (T0, T1, p, x, solver scalars, step
   counter), device-resident.  cfd_checkpoint_alloc sizes the store.        */
int cfd_checkpoint_alloc(cfd_ctx *ctx, int count);
int cfd_checkpoint_save(cfd_ctx *ctx, int slot);
int cfd_checkpoint_load(cfd_ctx *ctx, int slot);

/* Gradient of the time-averaged drag J = mean(Cd over steps first..last)
   (step n = the n-th step after cfd_start) with respect to eta and the
   inflow profile, by checkpointed reverse time stepping.
   cfd_adj_forward runs `last` steps from a context right after cfd_start,
   saving a checkpoint every `interval` steps, and returns J.
   cfd_adj_reverse recomputes each segment on the tape (interval <= tape_len)
   and reverses it, last segment first; the gradients are left in ADJ_ETA and
   ADJ_INFLOW and the context in the state after step `last`.
   cfd_adj_mean_drag runs both.                                             */
typedef struct {
    int first, last;  /* averaging window (inclusive); the run has `last` steps */
    int interval;     /* checkpoint interval = segment length (<= tape_len)     */
} cfd_adj_run_config;
typedef struct {
    double J;                 /* the objective                                  */
    double forward_seconds;   /* the forward run with checkpoints               */
    double adjoint_seconds;   /* recompute + reverse sweep                      */
    long long forward_iters;  /* forward Poisson iterations                     */
    long long adjoint_iters;  /* adjoint Poisson iterations (FP32 inner)        */
    int checkpoints;
} cfd_adj_run_result;
int cfd_adj_forward(cfd_ctx *ctx, const cfd_adj_run_config *cfg, cfd_adj_run_result *out);
int cfd_adj_reverse(cfd_ctx *ctx, cfd_adj_run_result *out);
int cfd_adj_mean_drag(cfd_ctx *ctx, const cfd_adj_run_config *cfg, cfd_adj_run_result *out);


/* ---- stretched grid ------------------------------------------------------------
   The reference's default "non_uniform-SML" grid (grid::unit_SML,
   grid::init_nonuniform_SML, structureGrid.hpp:326-405; ghosts as
   init_gC_dx, :506-559): per axis a fine region of fine_cells cells over
   fine_fraction of the length, centred and shifted by offset cells, coarse
   cells either side; fine_cells = 0 gives a uniform axis.  cfd_sml_default
   fills the reference's settings (0.3, 0.3, 0.5; 100, 100, 0; -4, 0, 0).
   cfd_sml_metrics computes the arrays on the host (X..Z: n+1 nodes, widths:
   n, ghosted); cfd_grid_sml applies them to a context (cfd_set_metrics).   */
typedef struct {
    double fine_fraction[3];
    int fine_cells[3];
    int offset[3];
} cfd_sml_config;
int cfd_sml_default(cfd_sml_config *cfg);
int cfd_sml_metrics(int nx_cal, int ny_cal, int nz_cal, double lx, double ly, double lz,
                    const cfd_sml_config *cfg, double *X, double *Y, double *Z, double *Dx, double *Dy,
                    double *Dz, double *Dxs, double *Dys, double *Dzs);
int cfd_grid_sml(cfd_ctx *ctx, const cfd_sml_config *cfg);

/* SmagorinskyModel (source/smagorinskyModel.hpp:31): eddy viscosity of
   velocity slot `slot` into CFD_FIELD_VIS (contexts created with
   les_smagorinsky = 1; the step and cfd_convection_diffusion call it on T0). */
int cfd_smagorinsky(cfd_ctx *ctx, int slot);

/* ---- monitors ----------------------------------------------------------------
   cfd_cfl: get_Cfl (analyses/cfl.hpp:3) of velocity slot `slot`: cfl = dt *
   max over cells of the signed sum u/Dxs + v/Dys + w/Dzs (last normal face
   skipped, as the reference does).  u_max/u_min and cfl_max are running
   values since cfd_start, as the reference's simuClass keeps them; dt_next is
   simuClass::timestepper (simuClass.hpp:185) with its default factors
   (cflFactor 0.05, gridFoFactor 0.15, dtMin 1e-12) on those extremes.
   cfd_steady_max: CheckSteadyStatebyMaxVal_omp (analyses/CheckSteadystate.hpp:
   166): out[c] = max(0, max over interior cells of (new - old)).           */
typedef struct {
    double cfl, cfl_max;
    double u_max[3], u_min[3];
    double dt_next;
} cfd_cfl_info;
int cfd_cfl(cfd_ctx *ctx, int slot, cfd_cfl_info *out);
int cfd_steady_max(cfd_ctx *ctx, int slot_new, int slot_old, double *out3);

/* ---- Plot3D files and the FP64 state file ----------------------------------
   Plot3D as the reference writes it: single block, whole grid, native-endian
   int32/float32, no record markers, i fastest.
     cfd_write_plot3d_x  OutputPlot3D_Xfile (io/Plot3D/xfileWrite.hpp:6): cell
                         centres Xc = (X[i+2] + X[i+3]) / 2 etc.
     cfd_write_plot3d_q  OutputPLOT3D_Qfile (io/Plot3D/qfile.hpp:7): header
                         (0, 0, Re, time), then p, the cell-centred u, v, w
                         (face pairs averaged) and eta of velocity slot `slot`;
                         formed on the GPU, one copy to the host.
     cfd_plot3d_q_host   the same file from ghosted FP64 host arrays.
     cfd_read_plot3d_q   QfileRead (io/Plot3D/qfileRead.hpp:6): cond[4] = (mach,
                         alpha, Re, time); ghosted FP64 p, u, v, w, eta with the
                         staggered faces rebuilt as the average of the two
                         adjacent centres (the last face of a line takes the
                         last centre), ghosts zero.
   cfd_save_state / cfd_load_state: no counterpart in the reference; a bitwise
   restart file of T0, T1, T3, eta, p, x, the solver scalars, the step counter,
   the time and the inflow profile.                                          */
int cfd_write_plot3d_x(cfd_ctx *ctx, const char *path);
int cfd_write_plot3d_q(cfd_ctx *ctx, int slot, const char *path);
int cfd_plot3d_q_host(const char *path, int nx_cal, int ny_cal, int nz_cal, double re, double time,
                      const double *p, const double *u, const double *v, const double *w, const double *eta);
int cfd_read_plot3d_q(const char *path, int nx_cal, int ny_cal, int nz_cal, double *cond, double *p,
                      double *u, double *v, double *w, double *eta);
int cfd_save_state(cfd_ctx *ctx, const char *path);
int cfd_load_state(cfd_ctx *ctx, const char *path);

#ifdef __cplusplus
}
#endif
#endif /* CFDGPU_H */
