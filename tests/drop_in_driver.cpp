// The reference's predictor-corrector main loop (RUN_CPU_PC_METHOD.hpp:287-627)
// with every hot-path call switched to the CUDA drop-in of
// include/cfdgpu_reference.hpp, as a `#if defined(PC_CUDA)` branch of a run
// driver would be written.  tests/test_reference_shim.py type-checks it
// against the reference's own headers; with CFDGPU_DROP_IN_MAIN defined it
// is also a program (tests/test_gpu_drop_in.py links it to libcfdgpu.so and
// runs it on the GPU), whose main() sets the simulation up as the reference's
// driver does and prints the drag and lift of every step on lines tagged CDCL
// (the reference's own set-up code prints to stdout too).
#include "controlPanel.hpp"
#include "run/general.hpp"

#include "cfdgpu_reference.hpp"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <utility>
#include <vector>

// u0, v0, w0: initial T0 fields (ghosted; null: iniU(1, 0, 0)); cx: the
// cylinder centre; out: drag and lift of every step
bool runCuda_predictionMethod(grid &gA, simuClass &simu, const double dir[6][3], const double num[6][3],
                              int nsteps, double cx, const double *u0, const double *v0, const double *w0,
                              int compat_rhs, std::vector<std::pair<double, double>> &out)
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
    if (u0 && v0 && w0) {
        T0.u.assign(u0, u0 + T0.u.size());
        T0.v.assign(v0, v0 + T0.v.size());
        T0.w.assign(w0, w0 + T0.w.size());
    }
    T1 = T0;
    T3 = T0;
    t1.init_p(0.0);
    generateGride(simu, globalDomain, gA);

    CUDAstruct cu;
    cu.init(gA, simu, T0, T1, T3, CFD_SOLVER_BICG_SPE, dir, num, CFD_METHOD_PC, compat_rhs);
    cu.upload(T0);
    cu.upload(T1);
    cu.upload(T3);
    BC_staggered_main_CUDA(cu, globalDomain, T0, t1, gA);
    BC_staggered_copy_CUDA(cu, globalDomain, T0, T1, gA);
    DFIB_CylinderZ_CUDA(cu, Dfib, globalDomain, gA, cx);

    simu.loop = 1;
    for (int s = 0; s < nsteps; ++s) {
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
        out.push_back(Delay_IO_CD_CL_CUDA(cu, simu, globalDomain, Dfib, gA));
        simu.finishloop();
    }
    cu.download(T0);
    cu.download(CFD_FIELD_P, t1.p);
    return true;
}

#ifdef CFDGPU_DROP_IN_MAIN
// usage: drop_in <steps> <dt> <re> <tol> <cx> <bc table file: 18 Dir, 18 Num>
//                [<u0> <v0> <w0>: raw FP64 ghosted fields]
static std::vector<double> read_raw(const char *path, size_t n)
{
    std::vector<double> a(n);
    std::ifstream f(path, std::ios::binary);
    if (!f.read(reinterpret_cast<char *>(a.data()), (std::streamsize)(n * sizeof(double)))) {
        std::fprintf(stderr, "cannot read %zu doubles from %s\n", n, path);
        std::exit(2);
    }
    return a;
}

int main(int argc, char **argv)
{
    if (argc != 7 && argc != 10) {
        std::fprintf(stderr, "usage: %s steps dt re tol cx bc_file [u0 v0 w0]\n", argv[0]);
        return 2;
    }
    const int steps = std::atoi(argv[1]);
    simuClass simu;
    simu.set_time_max(1e30);
    simu.set_dt(std::atof(argv[2]));
    simu.set_Re(std::atof(argv[3]));
    simu.p_criteria = std::atof(argv[4]);
    simu.Locality = 1;
    const double cx = std::atof(argv[5]);
    double dir[6][3], num[6][3];
    std::ifstream bc(argv[6]);
    for (int q = 0; q < 18; ++q) bc >> dir[q / 3][q % 3];
    for (int q = 0; q < 18; ++q) bc >> num[q / 3][q % 3];
    if (!bc) {
        std::fprintf(stderr, "cannot read the BC table from %s\n", argv[6]);
        return 2;
    }
    grid gA;
    std::vector<double> u0, v0, w0;
    if (argc == 10) {
        const size_t ng = (size_t)gA.nx * gA.ny * gA.nz;
        u0 = read_raw(argv[7], ng);
        v0 = read_raw(argv[8], ng);
        w0 = read_raw(argv[9], ng);
    }
    std::vector<std::pair<double, double>> cdcl;
    try {
        runCuda_predictionMethod(gA, simu, dir, num, steps, cx, u0.empty() ? nullptr : u0.data(),
                                 v0.empty() ? nullptr : v0.data(), w0.empty() ? nullptr : w0.data(), 1, cdcl);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "drop-in run failed: %s\n", e.what());
        return 1;
    }
    for (size_t s = 0; s < cdcl.size(); ++s)
        std::printf("CDCL %zu %.17g %.17g\n", s + 1, cdcl[s].first, cdcl[s].second);
    return 0;
}
#endif
