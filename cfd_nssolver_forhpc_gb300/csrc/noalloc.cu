// noalloc.cu -- drag and lift without any device allocation.
//
// cfd_cdcl (api.cu) reduces inside a context whose scratch was allocated by
// cfd_create.  cfd_cdcl_noalloc is for callers that cannot allocate device
// memory at all: an application that hands the whole GPU to its own memory
// pool and forbids allocations outside it, or a time-critical loop in which
// cudaMalloc's implicit device-wide synchronisation is not acceptable.  The
// caller passes its own device arrays; the only scratch is the file-scope
// array below, which every GPU that loads this library keeps until exit.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "../../include/cfdgpu.h"
#include "cfd_internal.cuh"

namespace cfd {
// defined in api.cu: sets the message cfd_last_error() returns
int set_last_error(int code, const std::string &msg);
}

namespace {

using namespace cfd;

// One partial (x and y sums) per chunk of kChunk cells, a ticket, and the
// two results: 16 B x 65536 + 256 B of header, about 1 MiB.
constexpr int kChunk = 4096;
constexpr int kMaxChunks = CFD_NOALLOC_MAX_CELLS / kChunk;

struct NoallocScratch {
    unsigned int ticket;
    unsigned int pad[63];
    double result[2];
    double pad2[30];
    double partial[2 * kMaxChunks];
};

static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

// Device address of g_noalloc_scratch per device, looked up with that
// device current (the host-side symbol is only a stand-in for it).  The
// lookup is repeated on every call made outside stream capture, so a device
// reset (which reloads the module at a new address) cannot leave a stale
// address behind; a call made during capture uses the last address found.
std::mutex g_mu;
NoallocScratch *g_addr[64] = {};


// Each block sums one chunk of kChunk cells in a fixed order, so the partials
// and the final sum do not depend on scheduling.
__global__ void __launch_bounds__(kBlock)
k_cdcl_noalloc(Geo g, const double *__restrict__ Dx, const double *__restrict__ Dy,
               const double *__restrict__ Dz, double lz, const double *__restrict__ f,
               NoallocScratch *s)
{
    const long long lo = (long long)blockIdx.x * kChunk;
    const long long hi = lo + kChunk < g.n ? lo + kChunk : g.n;
    double acc[2] = {0.0, 0.0};
    for (long long t = lo + threadIdx.x; t < hi; t += blockDim.x) {
        const long long i = t / g.sxc;
        const long long rem = t - i * g.sxc;
        const int j = (int)(rem / g.nzc), k = (int)(rem - (long long)j * g.nzc);
        const double vol = Dx[i + GC] * Dy[j + GC] * Dz[k + GC];
        acc[0] += f[t] * vol;
        acc[1] += f[g.n + t] * vol;
    }
    double tot[2];
    // grid_reduce writes partials[q * gridDim.x + blockIdx.x] and resets the
    // ticket when the last block has summed them
    if (grid_reduce<2>(acc, s->partial, &s->ticket, tot) && threadIdx.x == 0) {
        s->result[0] = -2.0 * tot[0] / lz;
        s->result[1] = -2.0 * tot[1] / lz;
    }
}

}  // namespace

extern "C" int cfd_cdcl_noalloc(int nx_cal, int ny_cal, int nz_cal, double lz, const double *Dx,
                                const double *Dy, const double *Dz, const double *f, double *cd,
                                double *cl, void *stream)
{
    if (nx_cal < 1 || ny_cal < 1 || nz_cal < 1 || !(lz > 0) || !Dx || !Dy || !Dz || !f || !cd || !cl) {
        return cfd::set_last_error(CFD_ERR_ARG, "cfd_cdcl_noalloc: invalid argument");
    }
    const long long n = (long long)nx_cal * ny_cal * nz_cal;
    if (n > CFD_NOALLOC_MAX_CELLS) {
        return cfd::set_last_error(CFD_ERR_ARG, "cfd_cdcl_noalloc: " + std::to_string(n) +
                                                    " cells exceed the scratch limit of " +
                                                    std::to_string((long long)CFD_NOALLOC_MAX_CELLS) +
                                                    " (CFD_NOALLOC_MAX_CELLS)");
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) {
        return cfd::set_last_error(CFD_ERR_CUDA, std::string("cfd_cdcl_noalloc: cudaGetDevice: ") +
                                                     cudaGetErrorString(e));
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(st, &cap);
    if (e != cudaSuccess) {
        return cfd::set_last_error(CFD_ERR_CUDA, std::string("cfd_cdcl_noalloc: cudaStreamIsCapturing: ") +
                                                     cudaGetErrorString(e));
    }
    NoallocScratch *s = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_addr[dev] || cap == cudaStreamCaptureStatusNone) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                return cfd::set_last_error(CFD_ERR_CUDA, std::string("cfd_cdcl_noalloc: cudaGetSymbolAddress: ") +
                                                             cudaGetErrorString(e));
            }
            g_addr[dev] = static_cast<NoallocScratch *>(p);
        }
        s = g_addr[dev];
    }
    Geo g{};
    g.nxc = nx_cal; g.nyc = ny_cal; g.nzc = nz_cal;
    g.nx = nx_cal + 2 * GC; g.ny = ny_cal + 2 * GC; g.nz = nz_cal + 2 * GC;
    g.sx = (long long)g.ny * g.nz; g.sy = g.nz;
    g.sxc = (long long)ny_cal * nz_cal; g.syc = nz_cal;
    g.ng = (long long)g.nx * g.ny * g.nz; g.n = n;
    // the ticket must start at zero (a call aborted mid-way could leave it set)
    e = cudaMemsetAsync(&s->ticket, 0, sizeof(unsigned int), st);
    if (e == cudaSuccess) {
        const int blocks = (int)((n + kChunk - 1) / kChunk);
        k_cdcl_noalloc<<<blocks, kBlock, 0, st>>>(g, Dx, Dy, Dz, lz, f, s);
        e = cudaGetLastError();
    }
    double out[2] = {0.0, 0.0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, s->result, sizeof(out), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        return cfd::set_last_error(CFD_ERR_CUDA, std::string("cfd_cdcl_noalloc: ") + cudaGetErrorString(e));
    }
    *cd = out[0];
    *cl = out[1];
    return CFD_OK;
}
