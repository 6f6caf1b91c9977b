// plot3d.cu -- the reference's on-disk formats and a bitwise state file.
//
// Plot3D (inc/io/Plot3D/xfileWrite.hpp:6-61, qfile.hpp:7-104,
// qfileRead.hpp:6-95): single block, whole 3-D grid, native-endian 32-bit
// integers and floats with no record markers, i running fastest.
//   .x  Nblock nx ny nz | Xc (nx*ny*nz) | Yc | Zc       (cell centres)
//   .q  Nblock nx ny nz | mach alpha Re time | p | uc | vc | wc | eta
// uc = (u[i-1] + u[i]) / 2 is the cell-centred velocity (each staggered face
// pair averaged in FP64, then rounded to float), the same for v, w.  The .q
// reader returns ghosted FP64 arrays and rebuilds the staggered faces as
// QfileRead does: face i = (centre i + centre i+1) / 2 (the pair summed in
// float), the last face of each line taking the last centre.  Plot3D output
// is lossy (float, centred); the state file below is the bitwise restart.
//
// The context writer forms the five fields on the GPU in file order (one
// kernel, one copy to the host); the host writer serves callers whose fields
// are already on the host and produces the same bytes.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "context.h"

using namespace cfd;

namespace {

// five float fields (p, uc, vc, wc, eta) of the file, i fastest
template <class T>
__global__ void k_plot3d_q(Geo g, const double *__restrict__ p, const T *__restrict__ u, const T *__restrict__ v,
                           const T *__restrict__ w, const T *__restrict__ eta, float *__restrict__ out)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.n) return;
    const int i = (int)(t % g.nxc), rest = (int)(t / g.nxc);
    const int j = rest % g.nyc, k = rest / g.nyc;
    const long long ic = icel(g, i + GC, j + GC, k + GC);
    out[t] = (float)p[ic];
    out[g.n + t] = (float)(0.5 * ((double)u[ic - g.sx] + (double)u[ic]));
    out[2 * g.n + t] = (float)(0.5 * ((double)v[ic - g.sy] + (double)v[ic]));
    out[3 * g.n + t] = (float)(0.5 * ((double)w[ic - 1] + (double)w[ic]));
    out[4 * g.n + t] = (float)eta[ic];
}

struct File {
    FILE *f = nullptr;
    explicit File(const char *path, const char *mode) : f(std::fopen(path, mode)) {}
    ~File()
    {
        if (f) std::fclose(f);
    }
};

int write_all(FILE *f, const void *p, size_t bytes, const char *path)
{
    if (bytes && std::fwrite(p, 1, bytes, f) != bytes) return fail(CFD_ERR_ARG, std::string("write failed: ") + path);
    return CFD_OK;
}

int read_all(FILE *f, void *p, size_t bytes, const char *path)
{
    if (bytes && std::fread(p, 1, bytes, f) != bytes)
        return fail(CFD_ERR_ARG, std::string("file too short or unreadable: ") + path);
    return CFD_OK;
}

int write_q(const char *path, int nx, int ny, int nz, double re, double time, const float *fields)
{
    File F(path, "wb");
    if (!F.f) return fail(CFD_ERR_ARG, std::string("cannot open for writing: ") + path);
    const int head[4] = {1, nx, ny, nz};
    const float cond[4] = {0.0f, 0.0f, (float)re, (float)time};
    CKS(write_all(F.f, head, sizeof(head), path));
    CKS(write_all(F.f, cond, sizeof(cond), path));
    return write_all(F.f, fields, (size_t)5 * nx * ny * nz * sizeof(float), path);
}

// state file: magic, version, dims, precision, loop, time, then the arrays
constexpr char kStateMagic[8] = {'C', 'F', 'D', 'G', 'P', 'U', 'S', '2'};

struct StateHeader {
    char magic[8];
    int nxc, nyc, nzc, fp32;
    long long loop;
    double time;
    int has_inflow, pad;
};

}  // namespace

extern "C" {

int cfd_write_plot3d_x(cfd_ctx *c, const char *path)
{
    CKS(need_metrics(c));
    if (!path) return fail(CFD_ERR_ARG, "null path");
    const Geo &g = c->g;
    const int nc[3] = {g.nxc, g.nyc, g.nzc};
    std::vector<float> centre[3];
    for (int a = 0; a < 3; ++a) {  // structureGrid.hpp:295: Xc = (X[i+gC] + X[i+gC+1]) / 2
        const std::vector<double> &X = c->hraw[a];
        centre[a].resize(nc[a]);
        for (int i = 0; i < nc[a]; ++i) centre[a][i] = (float)((X[i + GC] + X[i + GC + 1]) / 2.0);
    }
    const size_t n = (size_t)g.n;
    std::vector<float> buf(3 * n);
    for (int k = 0; k < g.nzc; ++k)
        for (int j = 0; j < g.nyc; ++j)
            for (int i = 0; i < g.nxc; ++i) {
                const size_t t = ((size_t)k * g.nyc + j) * g.nxc + i;
                buf[t] = centre[0][i];
                buf[n + t] = centre[1][j];
                buf[2 * n + t] = centre[2][k];
            }
    File F(path, "wb");
    if (!F.f) return fail(CFD_ERR_ARG, std::string("cannot open for writing: ") + path);
    const int head[4] = {1, g.nxc, g.nyc, g.nzc};
    CKS(write_all(F.f, head, sizeof(head), path));
    return write_all(F.f, buf.data(), buf.size() * sizeof(float), path);
}

int cfd_write_plot3d_q(cfd_ctx *c, int slot, const char *path)
{
    CKS(need_metrics(c));
    CKS(check_slot(slot));
    if (!path) return fail(CFD_ERR_ARG, "null path");
    const Geo &g = c->g;
    const int a = slot_index(slot);
    float *d = nullptr;
    CK(cudaStreamSynchronize(c->s));
    CK(cudaMalloc(reinterpret_cast<void **>(&d), (size_t)5 * g.n * sizeof(float)));
    dispatch(c, [&](auto tag) {
        using T = typename decltype(tag)::type;
        k_plot3d_q<T><<<(unsigned)((g.n + kBlock - 1) / kBlock), kBlock, 0, c->s>>>(
            g, c->p, dv<T>(c, a, 0), dv<T>(c, a, 1), dv<T>(c, a, 2), static_cast<const T *>(c->eta), d);
        return 0;
    });
    std::vector<float> host((size_t)5 * g.n);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(host.data(), d, host.size() * sizeof(float), cudaMemcpyDeviceToHost, c->s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->s);
    cudaFree(d);
    if (e != cudaSuccess) return fail(CFD_ERR_CUDA, std::string("plot3d q: ") + cudaGetErrorString(e));
    return write_q(path, g.nxc, g.nyc, g.nzc, c->cfg.re, c->time, host.data());
}

int cfd_plot3d_q_host(const char *path, int nxc, int nyc, int nzc, double re, double time, const double *p,
                      const double *u, const double *v, const double *w, const double *eta)
{
    if (!path || !p || !u || !v || !w || !eta) return fail(CFD_ERR_ARG, "null argument");
    if (nxc < 1 || nyc < 1 || nzc < 1) return fail(CFD_ERR_ARG, "grid dimensions must be positive");
    const long long nx = nxc + 2 * GC, ny = nyc + 2 * GC, nz = nzc + 2 * GC;
    const size_t n = (size_t)nxc * nyc * nzc;
    auto I = [&](long long i, long long j, long long k) { return (i * ny + j) * nz + k; };
    std::vector<float> buf(5 * n);
    for (int k = 0; k < nzc; ++k)
        for (int j = 0; j < nyc; ++j)
            for (int i = 0; i < nxc; ++i) {
                const size_t t = ((size_t)k * nyc + j) * nxc + i;
                const long long ic = I(i + GC, j + GC, k + GC);
                buf[t] = (float)p[ic];
                buf[n + t] = (float)(0.5 * (u[I(i + GC - 1, j + GC, k + GC)] + u[ic]));
                buf[2 * n + t] = (float)(0.5 * (v[I(i + GC, j + GC - 1, k + GC)] + v[ic]));
                buf[3 * n + t] = (float)(0.5 * (w[I(i + GC, j + GC, k + GC - 1)] + w[ic]));
                buf[4 * n + t] = (float)eta[ic];
            }
    return write_q(path, nxc, nyc, nzc, re, time, buf.data());
}

int cfd_read_plot3d_q(const char *path, int nxc, int nyc, int nzc, double *cond, double *p, double *u, double *v,
                      double *w, double *eta)
{
    if (!path || !cond || !p || !u || !v || !w || !eta) return fail(CFD_ERR_ARG, "null argument");
    File F(path, "rb");
    if (!F.f) return fail(CFD_ERR_ARG, std::string("cannot open for reading: ") + path);
    int head[4];
    float fc[4];
    CKS(read_all(F.f, head, sizeof(head), path));
    if (head[0] != 1 || head[1] != nxc || head[2] != nyc || head[3] != nzc)
        return fail(CFD_ERR_ARG, std::string("Plot3D q header does not match the grid: ") + path);
    CKS(read_all(F.f, fc, sizeof(fc), path));
    for (int q = 0; q < 4; ++q) cond[q] = fc[q];
    const size_t n = (size_t)nxc * nyc * nzc;
    std::vector<float> buf(5 * n);
    CKS(read_all(F.f, buf.data(), buf.size() * sizeof(float), path));
    const long long nx = nxc + 2 * GC, ny = nyc + 2 * GC, nz = nzc + 2 * GC;
    const size_t ng = (size_t)(nx * ny * nz);
    for (double *a : {p, u, v, w, eta}) std::memset(a, 0, ng * sizeof(double));
    auto I = [&](long long i, long long j, long long k) { return (i * ny + j) * nz + k; };
    auto D = [&](int field, int i, int j, int k) {  // file value at interior (i, j, k), zero-based
        return buf[(size_t)field * n + ((size_t)k * nyc + j) * nxc + i];
    };
    // the pair is summed in float, as QfileRead's float vectors do, then halved in FP64
    auto face = [&](int field, int i, int j, int k, int i2, int j2, int k2) {
        const float s = D(field, i, j, k) + D(field, i2, j2, k2);
        return (double)s / 2.0;
    };
    for (int k = 0; k < nzc; ++k)
        for (int j = 0; j < nyc; ++j)
            for (int i = 0; i < nxc; ++i) {
                const long long ic = I(i + GC, j + GC, k + GC);
                p[ic] = D(0, i, j, k);
                eta[ic] = D(4, i, j, k);
                u[ic] = i == nxc - 1 ? D(1, i, j, k) : face(1, i, j, k, i + 1, j, k);
                v[ic] = j == nyc - 1 ? D(2, i, j, k) : face(2, i, j, k, i, j + 1, k);
                w[ic] = k == nzc - 1 ? D(3, i, j, k) : face(3, i, j, k, i, j, k + 1);
            }
    return CFD_OK;
}

int cfd_save_state(cfd_ctx *c, const char *path)
{
    CKS(check_ctx(c));
    if (!path) return fail(CFD_ERR_ARG, "null path");
    const Geo &g = c->g;
    const size_t ts = c->fp32 ? sizeof(float) : sizeof(double);
    StateHeader h{};
    std::memcpy(h.magic, kStateMagic, 8);
    h.nxc = g.nxc; h.nyc = g.nyc; h.nzc = g.nzc; h.fp32 = c->fp32 ? 1 : 0;
    h.loop = c->loop; h.time = c->time; h.has_inflow = c->inflow ? 1 : 0;
    // device arrays in file order: T0, T1, T3 (3 each), eta, p, x, solver
    // scalars, inflow (T3's ghost corners reach T0 through the T0 = T3 copy)
    std::vector<unsigned char> buf;
    auto add = [&](const void *dptr, size_t bytes) -> int {
        const size_t off = buf.size();
        buf.resize(off + bytes);
        CK(cudaMemcpyAsync(buf.data() + off, dptr, bytes, cudaMemcpyDeviceToHost, c->s));
        return CFD_OK;
    };
    CK(cudaStreamSynchronize(c->s));
    for (int sl = 0; sl < 3; ++sl)
        for (int q = 0; q < 3; ++q) CKS(add(c->vel[sl][q], (size_t)g.ng * ts));
    CKS(add(c->eta, (size_t)g.ng * ts));
    CKS(add(c->p, (size_t)g.ng * sizeof(double)));
    CKS(add(c->x, (size_t)g.n * sizeof(double)));
    CKS(add(c->sc, sizeof(BicgScal)));
    CKS(add(c->sc_in, sizeof(BicgScal)));
    if (c->inflow) CKS(add(c->inflow, (size_t)g.nyc * sizeof(double)));
    CK(cudaStreamSynchronize(c->s));
    File F(path, "wb");
    if (!F.f) return fail(CFD_ERR_ARG, std::string("cannot open for writing: ") + path);
    CKS(write_all(F.f, &h, sizeof(h), path));
    return write_all(F.f, buf.data(), buf.size(), path);
}

int cfd_load_state(cfd_ctx *c, const char *path)
{
    CKS(check_ctx(c));
    if (!path) return fail(CFD_ERR_ARG, "null path");
    const Geo &g = c->g;
    const size_t ts = c->fp32 ? sizeof(float) : sizeof(double);
    File F(path, "rb");
    if (!F.f) return fail(CFD_ERR_ARG, std::string("cannot open for reading: ") + path);
    StateHeader h{};
    CKS(read_all(F.f, &h, sizeof(h), path));
    if (std::memcmp(h.magic, kStateMagic, 8) != 0) return fail(CFD_ERR_ARG, std::string("not a state file: ") + path);
    if (h.nxc != g.nxc || h.nyc != g.nyc || h.nzc != g.nzc || h.fp32 != (c->fp32 ? 1 : 0))
        return fail(CFD_ERR_ARG, "state file grid or precision does not match the context");
    size_t bytes = (size_t)10 * g.ng * ts + (size_t)g.ng * sizeof(double) + (size_t)g.n * sizeof(double) +
                   2 * sizeof(BicgScal) + (h.has_inflow ? (size_t)g.nyc * sizeof(double) : 0);
    std::vector<unsigned char> buf(bytes);
    CKS(read_all(F.f, buf.data(), bytes, path));
    if (h.has_inflow && !c->inflow_buf) {
        CK(cudaStreamSynchronize(c->s));
        CKS(dalloc_t(c, &c->inflow_buf, (size_t)g.nyc));
    }
    size_t off = 0;
    auto take = [&](void *dptr, size_t n) -> int {
        CK(cudaMemcpyAsync(dptr, buf.data() + off, n, cudaMemcpyHostToDevice, c->s));
        off += n;
        return CFD_OK;
    };
    for (int sl = 0; sl < 3; ++sl)
        for (int q = 0; q < 3; ++q) CKS(take(c->vel[sl][q], (size_t)g.ng * ts));
    CKS(take(c->eta, (size_t)g.ng * ts));
    CKS(take(c->p, (size_t)g.ng * sizeof(double)));
    CKS(take(c->x, (size_t)g.n * sizeof(double)));
    CKS(take(c->sc, sizeof(BicgScal)));
    CKS(take(c->sc_in, sizeof(BicgScal)));
    if (h.has_inflow) CKS(take(c->inflow_buf, (size_t)g.nyc * sizeof(double)));
    c->inflow = h.has_inflow ? c->inflow_buf : nullptr;
    CK(cudaStreamSynchronize(c->s));
    c->loop = h.loop;
    c->time = h.time;
    return CFD_OK;
}

}  // extern "C"
