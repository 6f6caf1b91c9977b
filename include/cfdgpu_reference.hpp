// cfdgpu_reference.hpp -- C++ drop-in layer for the reference's run drivers.
//
// The reference's GPU design (inc/ocl/*) overloads each hot-path function
// with a leading context argument, e.g.
//   CenterQuickScheme_OCL(OCLstruct&, ..., velocity&, velocity&, calDomain&, grid&)
//   (inc/ocl/convection_difussion_ocl.hpp:5)
// and keeps the state in device buffers owned by that context, reading it
// back only for IO (inc/run/RUN_GPU.hpp:511-526).  This header provides the
// same pattern for the CUDA library: a CUDAstruct that owns a cfd_ctx and
// knows which of the driver's objects live in which device slot, and one
// *_CUDA function per reference function, with the reference's parameter
// list after the context.  A run driver switches with `#if defined(PC_CUDA)`.
//
// Templates keep this header free of the reference's own headers: Simu,
// Vel, Pre, Dfib, Mx, Dom and Grid are the reference's simuClass, velocity,
// pressure, DfibArray, MxClass, calDomain and grid.
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "cfdgpu.h"

struct CUDAstruct {
    cfd_ctx *ctx = nullptr;
    const void *T[3] = {nullptr, nullptr, nullptr};  // driver's T0, T1, T3 objects
    int last_iters = 0;
    double last_error = 0.0;

    CUDAstruct() = default;
    CUDAstruct(const CUDAstruct &) = delete;
    CUDAstruct &operator=(const CUDAstruct &) = delete;
    ~CUDAstruct() { cfd_destroy(ctx); }

    static void check(int st, const char *what)
    {
        if (st != CFD_OK && st != CFD_ERR_NOCONV)
            throw std::runtime_error(std::string(what) + ": " + cfd_last_error());
    }

    // Create the context from the driver's grid and simulation settings and
    // register which velocity object is T0, T1 and T3.  compat_rhs = 1 adds
    // the compatibility projection of the Poisson right-hand side (an
    // extension; needed for tolerances below ~1e-6, see cfd_config).
    template <class Grid, class Simu, class Vel>
    void init(Grid &gA, Simu &simu, const Vel &T0, const Vel &T1, const Vel &T3, int solver,
              const double dir[6][3], const double num[6][3], int method = CFD_METHOD_PC,
              int compat_rhs = 0)
    {
        cfd_config cfg;
        check(cfd_config_default(&cfg, gA.nxCal, gA.nyCal, gA.nzCal), "cfd_config_default");
        cfg.lx = gA.lx; cfg.ly = gA.ly; cfg.lz = gA.lz;
        cfg.re = simu.Re;
        cfg.dt = simu.dt;
        cfg.p_criteria = simu.p_criteria;
        cfg.p_iter_max = (int)simu.p_iterMax;
        cfg.p_sor_omega = simu.p_sor_omega;
        cfg.p_sor_iter_max = (int)simu.p_sor_iter_max;
        cfg.solver = solver;
        cfg.method = method;
        cfg.compat_rhs = compat_rhs;
        for (int b = 0; b < 6; ++b)
            for (int c = 0; c < 3; ++c) { cfg.bc_dir[b][c] = dir[b][c]; cfg.bc_num[b][c] = num[b][c]; }
        check(cfd_create(&cfg, &ctx), "cfd_create");
        check(cfd_set_metrics(ctx, gA.X.data(), gA.Y.data(), gA.Z.data(), gA.Dx.data(), gA.Dy.data(),
                              gA.Dz.data(), gA.Dxs.data(), gA.Dys.data(), gA.Dzs.data()),
              "cfd_set_metrics");
        T[0] = &T0; T[1] = &T1; T[2] = &T3;
    }

    template <class Vel>
    int slot(const Vel &v) const
    {
        if (&v == T[0]) return CFD_SLOT_T0;
        if (&v == T[1]) return CFD_SLOT_T1;
        if (&v == T[2]) return CFD_SLOT_T3;
        throw std::invalid_argument("velocity object not registered with CUDAstruct::init");
    }

    // host <-> device at IO points (the OCL layer's read-back)
    template <class Vel>
    void upload(const Vel &v)
    {
        const int s = slot(v) == CFD_SLOT_T3 ? 6 : 3 * slot(v);
        check(cfd_upload(ctx, s + 0, v.u.data(), v.u.size()), "upload u");
        check(cfd_upload(ctx, s + 1, v.v.data(), v.v.size()), "upload v");
        check(cfd_upload(ctx, s + 2, v.w.data(), v.w.size()), "upload w");
    }
    template <class Vel>
    void download(Vel &v)
    {
        const int s = slot(v) == CFD_SLOT_T3 ? 6 : 3 * slot(v);
        check(cfd_download(ctx, s + 0, v.u.data(), v.u.size()), "download u");
        check(cfd_download(ctx, s + 1, v.v.data(), v.v.size()), "download v");
        check(cfd_download(ctx, s + 2, v.w.data(), v.w.size()), "download w");
    }
    void upload(int field, const std::vector<double> &a)
    {
        check(cfd_upload(ctx, field, a.data(), a.size()), "upload");
    }
    void download(int field, std::vector<double> &a)
    {
        check(cfd_download(ctx, field, a.data(), a.size()), "download");
    }
};

// ConvectionDifussion (inc/source/convection_and_difussion.hpp:168)
template <class Simu, class Vel, class Dom, class Grid>
bool ConvectionDifussion_CUDA(CUDAstruct &cu, Simu &, Vel &oldVel, Vel &curtVel, const Dom &, Grid &)
{
    CUDAstruct::check(cfd_convection_diffusion(cu.ctx, cu.slot(oldVel), cu.slot(curtVel)),
                      "ConvectionDifussion");
    return true;
}

// createBMatrix_omp (inc/matrix/b_matrix.hpp:51)
template <class Vel, class Mx, class Simu, class Dom, class Grid>
void createBMatrix_CUDA(CUDAstruct &cu, Vel &T1, Mx &, Simu &, Dom &, Grid &)
{
    CUDAstruct::check(cfd_create_b(cu.ctx, cu.slot(T1), nullptr), "createBMatrix");
}

// bicgstabRe2::operator() (inc/solver/bicgstabRe2.hpp:46) on Mx.matB / Mx.X_result
inline std::pair<int, double> pSolver_CUDA(CUDAstruct &cu)
{
    int it = 0;
    double res = 0.0;
    CUDAstruct::check(cfd_bicgstab(cu.ctx, &it, &res), "bicgstab");
    return {it, res};
}

// Pressure_transform_X_result (inc/pressure/Transform.hpp:8)
template <class Pre, class Mx, class Dom, class Grid>
void Pressure_transform_X_result_CUDA(CUDAstruct &cu, Pre &, Mx &, Dom &, Grid &)
{
    CUDAstruct::check(cfd_pressure_transform(cu.ctx), "Pressure_transform_X_result");
}

// SorPipeLine_omp / _seq (inc/pressure/solver/SorPipeLine.omp.hpp:7), red-black
template <class Sor, class Simu, class Vel, class Pre, class Dom, class Grid>
bool SorPipeLine_CUDA(CUDAstruct &cu, Sor &, Simu &simu, Vel &T1, Pre &, Dom &, Grid &)
{
    int it = 0;
    double err = 0.0;
    CUDAstruct::check(cfd_sor(cu.ctx, cu.slot(T1), &it, &err), "SorPipeLine");
    simu.iters = it;
    simu.error = err;
    return true;
}

// update_UandF_omp (inc/dfib/updateUandF.hpp:95)
template <class Dfib, class Simu, class Pre, class Vel, class Dom, class Grid>
void update_UandF_CUDA(CUDAstruct &cu, Dfib &, const Simu &, const Pre &, const Vel &oldVel,
                       Vel &curtVel, const Dom &, Grid &)
{
    CUDAstruct::check(cfd_update_uf(cu.ctx, cu.slot(oldVel), cu.slot(curtVel)), "update_UandF");
}

// BC_staggered_main (inc/BoundaryCondition/Boundary_Condition.hpp:37)
template <class Dom, class Vel, class Pre, class Grid>
bool BC_staggered_main_CUDA(CUDAstruct &cu, Dom &, Vel &vel, Pre &, Grid &)
{
    CUDAstruct::check(cfd_bc_main(cu.ctx, cu.slot(vel)), "BC_staggered_main");
    return true;
}

// BC_staggered_copy (inc/BoundaryCondition/updateBC.hpp:6)
template <class Dom, class Vel, class Grid>
bool BC_staggered_copy_CUDA(CUDAstruct &cu, const Dom &, const Vel &oldVel, Vel &currtVel, Grid &)
{
    CUDAstruct::check(cfd_bc_copy(cu.ctx, cu.slot(oldVel), cu.slot(currtVel)), "BC_staggered_copy");
    return true;
}

// velocity::copy_omp (inc/physicalVariables.hpp:84): dst.copy_omp(src)
template <class Vel>
void copy_vel_CUDA(CUDAstruct &cu, Vel &dst, const Vel &src)
{
    CUDAstruct::check(cfd_copy_velocity(cu.ctx, cu.slot(src), cu.slot(dst)), "copy_omp");
}

// Delay_IO_CD_CL's drag/lift (inc/dfib/virtualForceIntergrator.hpp:108), no file IO
template <class Simu, class Dom, class Dfib, class Grid>
std::pair<double, double> Delay_IO_CD_CL_CUDA(CUDAstruct &cu, Simu &simu, Dom &, Dfib &, Grid &)
{
    double cd = 0.0, cl = 0.0;
    CUDAstruct::check(cfd_cdcl(cu.ctx, &cd, &cl), "Delay_IO_CD_CL");
    simu.cd[simu.loop % simu.delayIO] = cd;
    simu.cl[simu.loop % simu.delayIO] = cl;
    return {cd, cl};
}

// DFIB_CylinderZ (inc/dfib/setEta.hpp:136) with the reference's hard-coded
// centre (6.5, ly/2) and radius 0.5 unless given
template <class Dfib, class Dom, class Grid>
void DFIB_CylinderZ_CUDA(CUDAstruct &cu, Dfib &, Dom &, Grid &gA, double cx = 6.5, double radius = 0.5)
{
    CUDAstruct::check(cfd_eta_cylinder_z(cu.ctx, cx, gA.ly / 2.0, radius, 100), "DFIB_CylinderZ");
}

// One iteration of the driver's main loop (RUN_CPU_PC_METHOD.hpp:287-627)
template <class Simu>
cfd_step_info step_CUDA(CUDAstruct &cu, Simu &simu)
{
    cfd_step_info info;
    CUDAstruct::check(cfd_step(cu.ctx, &info), "step");
    simu.iters = info.iters[3];
    simu.error = info.relres[3];
    simu.finishloop();
    return info;
}
