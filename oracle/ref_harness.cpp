// ref_harness.cpp -- drives the reference's own hot-path functions.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_ref.py compiles this file against
// a patched scratch copy of the reference headers (grid size, lengths, BC
// table and cylinder centre are compile-time constants there) into
// oracle/_ref/<config>/libref.so.  The tests use it to pin the C oracle, the
// golden-fixture script uses it to produce tests/golden/, and bench.py's
// reference arm uses ref_pc_run to time the reference's CPU path.
//
// Every entry point copies host arrays into the reference's own state
// objects, calls one reference function unchanged, and copies the result out.
#include "controlPanel.hpp"
#include "run/general.hpp"

#include <chrono>
#include <cstring>
#include <memory>
#include <unistd.h>

namespace {

struct Harness {
    grid gA;
    simuClass simu;
    calDomain Lo;
    shareMenory ShareM;
    velocity T0, T1, T3;
    pressure t1;
    DfibArray Dfib;
    MxClass Mx;   // SPE operator, RHS and solution (MxClass, PressureClass.hpp:24)
    MxClass MxE;  // ELL operator
    SORcoefficient Sor;
    std::unique_ptr<solver::bicgstabRe2<SPE_type>> spe;
    std::unique_ptr<solver::bicgstabRe2<ELL_type>> ell;
    std::vector<double> jp_spe, jp_ell, src;
    bool sor_ready = false;
};

Harness *H = nullptr;

size_t ng() { return (size_t)H->gA.iceltot; }
size_t nc() { return (size_t)H->gA.iceltotCal; }

void put(std::vector<double> &dst, const double *src, size_t n)
{
    if (src) std::memcpy(dst.data(), src, n * sizeof(double));
}
void get(double *dst, const std::vector<double> &src, size_t n)
{
    if (dst) std::memcpy(dst, src.data(), n * sizeof(double));
}

// The compatibility extension also used by the oracle (og_rhs_compat):
// remove the volume-weighted mean of the unscaled RHS from Mx.matB.
void compat_hook(MxClass &Mx, const std::vector<double> &jp)
{
    grid &gA = H->gA;
    velocity &T1 = H->T1;
    const double ddt = 1.0 / H->simu.dt;
    double sdv = 0.0, sdvd = 0.0;
    for (int i = gA.gC; i < gA.nx - gA.gC; ++i)
        for (int j = gA.gC; j < gA.ny - gA.gC; ++j)
            for (int k = gA.gC; k < gA.nz - gA.gC; ++k) {
                auto ic = gA.icel(i, j, k);
                double vol = gA.Dx[i] * gA.Dy[j] * gA.Dz[k];
                double d = -ddt * ((T1.u[ic] - T1.u[gA.icel(i - 1, j, k)]) / gA.Dx[i]
                                   + (T1.v[ic] - T1.v[gA.icel(i, j - 1, k)]) / gA.Dy[j]
                                   + (T1.w[ic] - T1.w[gA.icel(i, j, k - 1)]) / gA.Dz[k]);
                sdvd += vol * d;
                sdv += vol;
            }
    const double mean = sdvd / sdv;
    for (size_t r = 0; r < Mx.matB.size(); ++r) Mx.matB[r] = Mx.matB[r] - jp[r] * mean;
}

}  // namespace

extern "C" {

// OpenMP thread count of the reference's loops.  BC_staggered_main races
// between its `omp for nowait` face loops (Boundary_Condition.hpp:72-142)
// when more than one thread runs it; parity checks use 1.
void ref_set_threads(int n) { omp_set_num_threads(n > 0 ? n : 1); }

void ref_dims(int *nxc, int *nyc, int *nzc, double *lens)
{
    grid g;
    *nxc = g.nxCal;
    *nyc = g.nyCal;
    *nzc = g.nzCal;
    lens[0] = g.lx;
    lens[1] = g.ly;
    lens[2] = g.lz;
}

// Mirrors the set-up part of runSeqOmp_predictionMethod
// (inc/run/RUN_CPU_PC_METHOD.hpp:61-179) without file IO.
void ref_setup(double dt, double re, double tol, int with_eta)
{
    delete H;
    H = new Harness();
    simuClass &simu = H->simu;
    grid &gA = H->gA;
    simu.set_time_max(1e30);
    simu.set_dt(dt);
    simu.set_Re(re);
    simu.p_criteria = tol;
    simu.Locality = 1;
    simu.loop = 1;
    std::vector<int> gs{gA.nx, gA.ny, gA.nz}, dims{1, 1, 1};
    H->Lo.initTable(gs, dims);
    H->Lo.initLocal(0, 0, 0);
    resize_variable(gA, H->t1, H->T0, H->T1, H->T3, H->Dfib);
    H->T0.iniU(1.0, 0.0, 0.0);
    H->T1.iniU(1.0, 0.0, 0.0);
    H->T3.iniU(1.0, 0.0, 0.0);
    H->t1.init_p(0.0);
    generateGride(simu, H->ShareM, H->Lo, gA);
    H->Mx.X_result.resize(gA.iceltotCal, 0.0);
    H->MxE.X_result.resize(gA.iceltotCal, 0.0);
    H->Mx.matA_spe.resize(gA.nxCal, gA.nyCal, gA.nzCal);
    H->Mx.matA_spe.setupPressure(gA.gC, gA.Dx, gA.Dy, gA.Dz, gA.Dxs, gA.Dys, gA.Dzs);
    H->jp_spe = H->Mx.matA_spe.set_Jp_pc();
    H->spe.reset(new solver::bicgstabRe2<SPE_type>(H->Mx.matA_spe));
    H->spe->setTolerance(tol);
    createPressureMatrix(H->MxE, simu, H->Lo, gA);
    H->jp_ell = gA.jp;
    H->ell.reset(new solver::bicgstabRe2<ELL_type>(H->MxE.matA_ell));
    H->ell->setTolerance(tol);
    gA.jp = H->jp_spe;
    std::fill(H->Dfib.eta.begin(), H->Dfib.eta.end(), 0.0);
    if (with_eta) DFIB_CylinderZ(H->Dfib, H->Lo, gA);
    H->src.assign(3 * nc(), 0.0);
}

void ref_grid(double *X, double *Y, double *Z, double *Dx, double *Dy, double *Dz, double *Dxs,
              double *Dys, double *Dzs)
{
    grid &g = H->gA;
    get(X, g.X, g.nx + 1);
    get(Y, g.Y, g.ny + 1);
    get(Z, g.Z, g.nz + 1);
    get(Dx, g.Dx, g.nx);
    get(Dy, g.Dy, g.ny);
    get(Dz, g.Dz, g.nz);
    get(Dxs, g.Dxs, g.nx);
    get(Dys, g.Dys, g.ny);
    get(Dzs, g.Dzs, g.nz);
}

void ref_eta(double *eta) { get(eta, H->Dfib.eta, ng()); }
void ref_set_eta(const double *eta) { put(H->Dfib.eta, eta, ng()); }
void ref_jp(double *jp_spe, double *jp_ell)
{
    get(jp_spe, H->jp_spe, nc());
    get(jp_ell, H->jp_ell, nc());
}

// ConvectionDifussion (inc/source/convection_and_difussion.hpp:168)
void ref_convdiff(const double *u0, const double *v0, const double *w0, double *u1, double *v1,
                  double *w1)
{
    put(H->T0.u, u0, ng()); put(H->T0.v, v0, ng()); put(H->T0.w, w0, ng());
    put(H->T1.u, u1, ng()); put(H->T1.v, v1, ng()); put(H->T1.w, w1, ng());
    ConvectionDifussion(H->simu, H->T0, H->T1, H->Lo, H->gA);
    get(u1, H->T1.u, ng()); get(v1, H->T1.v, ng()); get(w1, H->T1.w, ng());
}

// createBMatrix_omp (inc/matrix/b_matrix.hpp:51); kind 0 = SPE jp, 1 = ELL jp
void ref_rhs(int kind, const double *u1, const double *v1, const double *w1, double *b)
{
    put(H->T1.u, u1, ng()); put(H->T1.v, v1, ng()); put(H->T1.w, w1, ng());
    H->gA.jp = kind ? H->jp_ell : H->jp_spe;
    createBMatrix_omp(H->T1, H->Mx, H->simu, H->Lo, H->gA);
    get(b, H->Mx.matB, nc());
}

// SPE_matrix1::multiply_omp (inc/matrix/SPE_sparseMatrix1.hpp:259)
void ref_spe_spmv(const double *x, double *r)
{
    std::vector<double> xv(x, x + nc()), rv(nc());
    H->Mx.matA_spe.multiply_omp(xv, rv);
    get(r, rv, nc());
}

// ELL_matrix::multiply_omp (inc/matrix/ELL_sparseMatrix.hpp:478)
void ref_ell_spmv(const double *x, double *r)
{
    std::vector<double> xv(x, x + nc()), rv(nc());
    H->MxE.matA_ell.multiply_omp(xv, rv);
    get(r, rv, nc());
}

// bicgstabRe2::solve (inc/solver/bicgstabRe2.hpp:93) with the persistent
// solver object of the chosen operator; x is the warm start in, solution out.
void ref_bicg(int kind, const double *b, double *x, int *iters, double *relres)
{
    std::vector<double> bv(b, b + nc()), xv(x, x + nc());
    std::pair<int, double> r = kind ? (*H->ell)(bv, xv) : (*H->spe)(bv, xv);
    *iters = r.first;
    *relres = r.second;
    get(x, xv, nc());
}

// SorPipeLine_seq (inc/pressure/solver/SorPipeLine.seq.hpp:4).  The
// coefficient block is built on the first call (the reference builds it when
// simu.loop == 1).  p is the ghosted pressure, in/out.
void ref_sor_seq(const double *u1, const double *v1, const double *w1, double *p, double omega,
                 double tol, int itmax, int *iters, double *err)
{
    put(H->T1.u, u1, ng()); put(H->T1.v, v1, ng()); put(H->T1.w, w1, ng());
    put(H->t1.p, p, ng());
    simuClass &simu = H->simu;
    size_t keep = simu.loop;
    if (!H->sor_ready) { simu.loop = 1; H->sor_ready = true; }
    simu.p_sor_omega = omega;
    simu.p_criteria = tol;
    simu.p_sor_iter_max = (size_t)itmax;
    SorPipeLine_seq(H->Sor, simu, H->T1, H->t1, H->Lo, H->gA);
    simu.loop = keep;
    *iters = simu.iters;
    *err = simu.error;
    get(p, H->t1.p, ng());
}

// update_UandF_omp (inc/dfib/updateUandF.hpp:95); f is in/out (skipped
// faces keep their value)
void ref_update_uf(const double *p, const double *u1, const double *v1, const double *w1,
                   double *u3, double *v3, double *w3, double *f)
{
    put(H->t1.p, p, ng());
    put(H->T1.u, u1, ng()); put(H->T1.v, v1, ng()); put(H->T1.w, w1, ng());
    put(H->T3.u, u3, ng()); put(H->T3.v, v3, ng()); put(H->T3.w, w3, ng());
    put(H->Dfib.f, f, 3 * nc());
    update_UandF_omp(H->Dfib, H->simu, H->t1, H->T1, H->T3, H->Lo, H->gA);
    get(u3, H->T3.u, ng()); get(v3, H->T3.v, ng()); get(w3, H->T3.w, ng());
    get(f, H->Dfib.f, 3 * nc());
}

// virtualF_Int + the Cd/Cl formula of Delay_IO_CD_CL
// (inc/dfib/virtualForceIntergrator.hpp:5, 120-127), without the file IO
void ref_cdcl(const double *f, double *cd, double *cl)
{
    put(H->Dfib.f, f, 3 * nc());
    virtualF_Int(H->Dfib, H->Lo, H->gA, 0);
    virtualF_Int(H->Dfib, H->Lo, H->gA, 1);
    *cd = -2.0 * H->Dfib.ValSum[0] / H->gA.lz;
    *cl = -2.0 * H->Dfib.ValSum[1] / H->gA.lz;
}

// BC_staggered_main (inc/BoundaryCondition/Boundary_Condition.hpp:37)
void ref_bc_main(double *u, double *v, double *w, double *p)
{
    put(H->T0.u, u, ng()); put(H->T0.v, v, ng()); put(H->T0.w, w, ng());
    put(H->t1.p, p, ng());
    BC_staggered_main(H->Lo, H->T0, H->t1, H->gA);
    get(u, H->T0.u, ng()); get(v, H->T0.v, ng()); get(w, H->T0.w, ng());
    get(p, H->t1.p, ng());
}

// BC_staggered_copy (inc/BoundaryCondition/updateBC.hpp:6)
void ref_bc_copy(const double *uo, const double *vo, const double *wo, double *u, double *v,
                 double *w)
{
    put(H->T0.u, uo, ng()); put(H->T0.v, vo, ng()); put(H->T0.w, wo, ng());
    put(H->T1.u, u, ng()); put(H->T1.v, v, ng()); put(H->T1.w, w, ng());
    BC_staggered_copy(H->Lo, H->T0, H->T1, H->gA);
    get(u, H->T1.u, ng()); get(v, H->T1.v, ng()); get(w, H->T1.w, ng());
}

// ---- whole-run driver ------------------------------------------------------
// The initial state: T0 = given fields (or (1,0,0) when null), then
// T1 = T3 = T0 and the first boundary update (RUN_CPU_PC_METHOD.hpp:114-119).
void ref_pc_start(const double *u0, const double *v0, const double *w0)
{
    put(H->T0.u, u0, ng()); put(H->T0.v, v0, ng()); put(H->T0.w, w0, ng());
    H->T1.u = H->T3.u = H->T0.u;
    H->T1.v = H->T3.v = H->T0.v;
    H->T1.w = H->T3.w = H->T0.w;
    BC_staggered_main(H->Lo, H->T0, H->t1, H->gA);
    BC_staggered_copy(H->Lo, H->T0, H->T1, H->gA);
}

// nsteps iterations of the main loop of runSeqOmp_predictionMethod
// (method 0, RUN_CPU_PC_METHOD.hpp:287-627) or runSeqOmp (method 1,
// RUN_CPU.hpp:290-462), IO removed.  solver: 0 = BiCGSTAB SPE, 1 = BiCGSTAB
// ELL, 2 = SorPipeLine_seq.  Per step: Cd, Cl, the 4 per-pass iteration
// counts and the wall time of the step.
void ref_pc_run(int nsteps, int method, int solver, int compat, double *cd, double *cl,
                int *iters4, double *wall)
{
    Harness &h = *H;
    grid &gA = h.gA;
    simuClass &simu = h.simu;
    calDomain &Lo = h.Lo;
    auto pressure_solve = [&](int pass, int s) {
        if (simu.loop > 1) {
            if (solver <= 1) {
                gA.jp = solver ? h.jp_ell : h.jp_spe;
                createBMatrix_omp(h.T1, h.Mx, simu, Lo, gA);
                if (compat) compat_hook(h.Mx, gA.jp);
                if (solver)
                    std::tie(simu.iters, simu.error) = (*h.ell)(h.Mx.matB, h.Mx.X_result);
                else
                    std::tie(simu.iters, simu.error) = (*h.spe)(h.Mx.matB, h.Mx.X_result);
                Pressure_transform_X_result(h.t1, h.Mx, Lo, gA);
            } else {
                size_t keep = simu.loop;
                if (!h.sor_ready) { simu.loop = 1; h.sor_ready = true; }
                SorPipeLine_seq(h.Sor, simu, h.T1, h.t1, Lo, gA);
                simu.loop = keep;
            }
            iters4[s * 4 + pass] = simu.iters;
        } else {
            iters4[s * 4 + pass] = 0;
        }
    };
    for (int s = 0; s < nsteps; ++s) {
        auto t0 = std::chrono::steady_clock::now();
        int npass = method == 0 ? 4 : 1;
        if (method == 0) std::fill(h.src.begin(), h.src.end(), 0.0);
        for (int pass = 0; pass < npass; ++pass) {
            ConvectionDifussion(simu, h.T0, h.T1, Lo, gA);
            if (method == 0) {
                for (int whichDim = 0; whichDim < 3; whichDim++)
                    for (auto i = Lo.i_begin; i < Lo.i_endof; ++i)
                        for (auto j = Lo.j_begin; j < Lo.j_endof; ++j)
                            for (auto k = Lo.k_begin; k < Lo.k_endof; ++k)
                                h.T1.U(whichDim)[gA.icelCal(i, j, k)] +=
                                    h.src[gA.icelCal(i, j, k) + gA.iceltotCal * whichDim];
            }
            pressure_solve(pass, s);
            update_UandF_omp(h.Dfib, simu, h.t1, h.T1, h.T3, Lo, gA);
            if (method == 0 && pass < 3) {
                for (int whichDim = 0; whichDim < 3; whichDim++)
                    for (auto i = Lo.i_begin; i < Lo.i_endof; ++i)
                        for (auto j = Lo.j_begin; j < Lo.j_endof; ++j)
                            for (auto k = Lo.k_begin; k < Lo.k_endof; ++k)
                                h.src[gA.icelCal(i, j, k) + gA.iceltotCal * whichDim] +=
                                    simu.dt * h.Dfib.f[gA.icelCal(i, j, k) + gA.iceltotCal * whichDim];
            }
        }
        for (int pass = npass; pass < 4; ++pass) iters4[s * 4 + pass] = 0;
        h.T0.copy_omp(h.T3);
        BC_staggered_main(Lo, h.T0, h.t1, gA);
        BC_staggered_copy(Lo, h.T0, h.T1, gA);
        virtualF_Int(h.Dfib, Lo, gA, 0);
        virtualF_Int(h.Dfib, Lo, gA, 1);
        cd[s] = -2.0 * h.Dfib.ValSum[0] / gA.lz;
        cl[s] = -2.0 * h.Dfib.ValSum[1] / gA.lz;
        simu.finishloop();
        wall[s] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
}

// Read back the state after ref_pc_run: T0 (u,v,w), p, f (3N), x (N).
void ref_state(double *u, double *v, double *w, double *p, double *f, double *x)
{
    get(u, H->T0.u, ng()); get(v, H->T0.v, ng()); get(w, H->T0.w, ng());
    get(p, H->t1.p, ng());
    get(f, H->Dfib.f, 3 * nc());
    get(x, H->Mx.X_result, nc());
}


// The reference's Plot3D writers and reader (io/Plot3D/*.hpp).  They write to
// mx_out/ under the current directory, so the harness changes into `dir`
// (which must hold an mx_out/ directory) around the call.
int ref_plot3d_x(const char *dir)
{
    char cwd[4096];
    if (!getcwd(cwd, sizeof(cwd)) || chdir(dir) != 0) return -1;
    OutputPlot3D_Xfile(H->simu, H->gA);
    return chdir(cwd);
}

int ref_plot3d_q(const char *dir, int io, double time, const double *p, const double *u, const double *v,
                 const double *w, const double *eta)
{
    char cwd[4096];
    if (!getcwd(cwd, sizeof(cwd)) || chdir(dir) != 0) return -1;
    put(H->t1.p, p, ng());
    put(H->T3.u, u, ng());
    put(H->T3.v, v, ng());
    put(H->T3.w, w, ng());
    put(H->Dfib.eta, eta, ng());
    H->simu.currentFile = (size_t)io;
    H->simu.set_time(time);
    OutputPLOT3D_Qfile(H->Dfib, H->simu, H->t1, H->T3, H->gA);
    return chdir(cwd);
}

// QfileRead: cond = (mach, alpha, Re, time), ghosted p, u, v, w, eta
void ref_plot3d_read(const char *path, double *cond, double *p, double *u, double *v, double *w, double *eta)
{
    auto [nb, mach, alpha, reyn, time, dp, du, dv, dw, deta] = QfileRead(H->gA, std::string(path));
    (void)nb;
    cond[0] = mach;
    cond[1] = alpha;
    cond[2] = reyn;
    cond[3] = time;
    get(p, dp, ng());
    get(u, du, ng());
    get(v, dv, ng());
    get(w, dw, ng());
    get(eta, deta, ng());
}

// get_Cfl (analyses/cfl.hpp:3) for one field: the running extremes are reset
// first, so the returned cfl, U_max and U_min are this call's
void ref_cfl(const double *u, const double *v, const double *w, double *cfl, double *umax, double *umin)
{
    put(H->T0.u, u, ng());
    put(H->T0.v, v, ng());
    put(H->T0.w, w, ng());
    H->simu.U_max.clear();
    H->simu.U_min.clear();
    H->simu.cfl_max = -1e300;
    get_Cfl(H->T0, H->Lo, H->gA, H->simu);
    *cfl = H->simu.cfl_max;
    for (int q = 0; q < 3; ++q) {
        umax[q] = H->simu.U_max[q];
        umin[q] = H->simu.U_min[q];
    }
}

// simuClass::timestepper (simuClass.hpp:185) with the given extremes
double ref_timestepper(const double *umax, const double *umin)
{
    H->simu.U_max.assign(umax, umax + 3);
    H->simu.U_min.assign(umin, umin + 3);
    H->simu.timestepper();
    return H->simu.dt_next;
}

// CheckSteadyStatebyMaxVal_omp (analyses/CheckSteadystate.hpp:166)
void ref_steady(const double *u0, const double *v0, const double *w0, const double *u3, const double *v3,
                const double *w3, double *out)
{
    put(H->T0.u, u0, ng());
    put(H->T0.v, v0, ng());
    put(H->T0.w, w0, ng());
    put(H->T3.u, u3, ng());
    put(H->T3.v, v3, ng());
    put(H->T3.w, w3, ng());
    auto [a, b, c] = CheckSteadyStatebyMaxVal_omp(H->simu, H->ShareM, H->T0, H->T3, H->Lo, H->gA);
    out[0] = a;
    out[1] = b;
    out[2] = c;
}

#ifdef TERBULENCE_SMAGORINSKY
// SmagorinskyModel (source/smagorinskyModel.hpp:31) of (u, v, w): the eddy
// viscosity per cell (compact); ref_convdiff then uses it for T0
void ref_smagorinsky(const double *u, const double *v, const double *w, double *vis)
{
    put(H->T0.u, u, ng());
    put(H->T0.v, v, ng());
    put(H->T0.w, w, ng());
    SmagorinskyModel(H->ShareM, H->simu, H->T0, H->t1, H->Lo, H->gA);
    get(vis, H->T0.Viseff, nc());
}
#endif

}  // extern "C"
