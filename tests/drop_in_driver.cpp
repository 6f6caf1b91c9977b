// The reference's predictor-corrector main loop (RUN_CPU_PC_METHOD.hpp:287-627)
// with every hot-path call switched to the CUDA drop-in of
// include/cfdgpu_reference.hpp, as a `#if defined(PC_CUDA)` branch of a run
// driver would be written.  Compiled (not run) by tests/test_reference_shim.py
// against the reference's own headers to prove the signatures line up.
#include "controlPanel.hpp"
#include "run/general.hpp"

#include "cfdgpu_reference.hpp"

bool runCuda_predictionMethod(grid &gA, simuClass &simu, const double dir[6][3], const double num[6][3])
{
    DfibArray Dfib;
    pressure t1;
    velocity T0, T1, T3;
    SORcoefficient Sor;
    MxClass Mx;
    calDomain globalDomain;
    std::vector<int> grid_size{gA.nx, gA.ny, gA.nz}, dims{1, 1, 1};
    globalDomain.initTable(grid_size, dims);
    globalDomain.initLocal(0, 0, 0);
    resize_variable(gA, t1, T0, T1, T3, Dfib);
    T0.iniU(1.0, 0.0, 0.0);
    generateGride(simu, globalDomain, gA);

    CUDAstruct cu;
    cu.init(gA, simu, T0, T1, T3, CFD_SOLVER_BICG_SPE, dir, num);
    cu.upload(T0);
    cu.upload(T1);
    cu.upload(T3);
    BC_staggered_main_CUDA(cu, globalDomain, T0, t1, gA);
    BC_staggered_copy_CUDA(cu, globalDomain, T0, T1, gA);
    DFIB_CylinderZ_CUDA(cu, Dfib, globalDomain, gA);

    for (simu.loop = 1; simu.get_finishloop(); simu.finishloop()) {
        cfd_clear_source(cu.ctx);
        for (int pass = 0; pass < 4; ++pass) {
            ConvectionDifussion_CUDA(cu, simu, T0, T1, globalDomain, gA);
            cfd_add_source(cu.ctx, CFD_SLOT_T1);
            if (simu.loop > 1) {
                createBMatrix_CUDA(cu, T1, Mx, simu, globalDomain, gA);
                std::tie(simu.iters, simu.error) = pSolver_CUDA(cu);
                Pressure_transform_X_result_CUDA(cu, t1, Mx, globalDomain, gA);
            }
            update_UandF_CUDA(cu, Dfib, simu, t1, T1, T3, globalDomain, gA);
            if (pass < 3) cfd_accumulate_source(cu.ctx);
        }
        copy_vel_CUDA(cu, T0, T3);
        BC_staggered_main_CUDA(cu, globalDomain, T0, t1, gA);
        BC_staggered_copy_CUDA(cu, globalDomain, T0, T1, gA);
        auto cdcl = Delay_IO_CD_CL_CUDA(cu, simu, globalDomain, Dfib, gA);
        (void)cdcl;
        if (simu.get_writefile()) {
            cu.download(T3);
            cu.download(CFD_FIELD_P, t1.p);
        }
    }
    return true;
}
