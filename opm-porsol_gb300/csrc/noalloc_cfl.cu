// noalloc_cfl.cu -- porsol_transport_cfl_noalloc: the viscous CFL time step of the transport
// solver, computed without allocating any device memory.
//
// Who needs it: callers that may not allocate device memory at the moment they need the
// step bound, for example a simulator whose device memory is owned by its own pool allocator
// (a cudaMalloc behind the pool's back would fragment or exceed the budget the pool manages).
// The transport handle (porsol_transport_*) allocates its buffers at init; this entry point
// takes the caller's device arrays and uses a fixed scratch array compiled into the library
// instead.
//
// Scratch: s_cfl_scratch, a file-scope __device__ array of CFL_MAX_BLOCKS per-block minima
// and flags plus the final result.  Every GPU that loads the library holds it
// until the process exits (256 KiB).  Each call writes every slot it later reads, so nothing has to
// start at zero; calls that overlap on the GPU share the array and race.
#include <cuda_runtime.h>

#include <mutex>

#include "porsol_gpu.h"

namespace {

constexpr int CFL_THREADS = 256;
constexpr int CFL_MAX_BLOCKS = 16384;                       // 4,194,304 cells at most
constexpr int CFL_MAX_CELLS = CFL_MAX_BLOCKS * CFL_THREADS;

// [0, CFL_MAX_BLOCKS): per-block minimum of the local step; [CFL_MAX_BLOCKS, 2*CFL_MAX_BLOCKS):
// per-block flag (1.0 when a cell's step is exactly zero); [2*CFL_MAX_BLOCKS]: result;
// [2*CFL_MAX_BLOCKS + 1]: zero-step flag of the whole grid.
constexpr int CFL_SCRATCH = 2 * CFL_MAX_BLOCKS + 2;
static __device__ __align__(256) double s_cfl_scratch[CFL_SCRATCH];

// Per-device address of s_cfl_scratch, looked up once per device context.  The address belongs
// to the module loaded into that context: after cudaDeviceReset (or a primary-context release)
// the module is loaded again, possibly elsewhere, so each cached address is kept together with
// the context it was looked up in and is looked up again when the current context differs.
constexpr int MAX_DEVICES = 64;
std::mutex g_mutex;
double* g_scratch[MAX_DEVICES] = {nullptr};
void* g_context[MAX_DEVICES] = {nullptr};

// cuCtxGetCurrent from the driver through the runtime (no link-time dependency on libcuda).
using CtxGetCurrent = int (*)(void**);
CtxGetCurrent ctx_get_current()
{
    static const CtxGetCurrent fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<CtxGetCurrent>(p);
    }();
    return fn;
}

void* current_context()
{
    void* c = nullptr;
    const CtxGetCurrent fn = ctx_get_current();
    if (!fn || fn(&c) != 0) return nullptr;
    return c;
}

// Stage 1 -- the per-cell bound of findCFLtimeVelocity (CflCalculator.hpp:55-88):
// cfl_factor |c| phi_c / max(sum of outfluxes, sum of influxes); one minimum per block.
__global__ void __launch_bounds__(CFL_THREADS) k_cfl_blocks(int nc, const int* __restrict__ facepos,
                                                            const double* __restrict__ flux,
                                                            const double* __restrict__ vol,
                                                            const double* __restrict__ poro, double fac,
                                                            double* __restrict__ scratch)
{
    __shared__ double smin[CFL_THREADS / 32];
    __shared__ int szero[CFL_THREADS / 32];
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double dt = 1e100;
    int zero = 0;
    if (c < nc) {
        double fp = 0.0, fn = 0.0;
        for (int hf = facepos[c]; hf < facepos[c + 1]; ++hf) {
            const double f = flux[hf];
            if (f > 0) fp += f;
            else fn -= f;
        }
        const double loc = (fac * vol[c] * poro[c]) / fmax(fn, fp);
        zero = loc == 0.0;
        if (loc >= 0.0) dt = loc;   // NaN never wins the comparison in the reference
    }
    for (int o = 16; o > 0; o >>= 1) {
        dt = fmin(dt, __shfl_xor_sync(0xffffffffu, dt, o));
        zero |= __shfl_xor_sync(0xffffffffu, zero, o);
    }
    if ((threadIdx.x & 31) == 0) {
        smin[threadIdx.x >> 5] = dt;
        szero[threadIdx.x >> 5] = zero;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = smin[0];
        int z = szero[0];
        for (int w = 1; w < CFL_THREADS / 32; ++w) {
            m = fmin(m, smin[w]);
            z |= szero[w];
        }
        scratch[blockIdx.x] = m;
        scratch[CFL_MAX_BLOCKS + blockIdx.x] = z ? 1.0 : 0.0;
    }
}

// Stage 2 -- minimum over the block minima (order-independent, so the result is exact).
__global__ void __launch_bounds__(CFL_THREADS) k_cfl_final(int nblocks, double* __restrict__ scratch)
{
    __shared__ double smin[CFL_THREADS / 32];
    __shared__ double szero[CFL_THREADS / 32];
    double m = 1e100, z = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
        m = fmin(m, scratch[b]);
        z = fmax(z, scratch[CFL_MAX_BLOCKS + b]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
        z = fmax(z, __shfl_xor_sync(0xffffffffu, z, o));
    }
    if ((threadIdx.x & 31) == 0) {
        smin[threadIdx.x >> 5] = m;
        szero[threadIdx.x >> 5] = z;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double mm = smin[0], zz = szero[0];
        for (int w = 1; w < CFL_THREADS / 32; ++w) {
            mm = fmin(mm, smin[w]);
            zz = fmax(zz, szero[w]);
        }
        scratch[2 * CFL_MAX_BLOCKS] = mm;
        scratch[2 * CFL_MAX_BLOCKS + 1] = zz;
    }
}

// Address of the scratch array on the current device.  The first call on a device (and the
// first call after its context was replaced) looks it up with cudaGetSymbolAddress; the host
// symbol s_cfl_scratch itself is only a host-side stand-in and is never passed to a kernel.
cudaError_t scratch_on_current_device(double** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mutex);
    void* ctx = current_context();
    if (!g_scratch[dev] || !ctx || ctx != g_context[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, s_cfl_scratch);   // also makes the device's context current
        if (e != cudaSuccess) return e;
        g_scratch[dev] = static_cast<double*>(p);
        g_context[dev] = current_context();
    }
    *out = g_scratch[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" int porsol_transport_cfl_noalloc(int num_cells, const int* cell_facepos, const double* outflux,
                                            const double* cell_volume, const double* porosity, double cfl_factor,
                                            double* dt, void* stream)
{
    if (num_cells < 1 || num_cells > CFL_MAX_CELLS || !cell_facepos || !outflux || !cell_volume || !porosity || !dt)
        return PORSOL_ERR_BAD_ARG;
    double* scratch = nullptr;
    if (scratch_on_current_device(&scratch) != cudaSuccess) return PORSOL_ERR_CUDA;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nblocks = (num_cells + CFL_THREADS - 1) / CFL_THREADS;
    k_cfl_blocks<<<nblocks, CFL_THREADS, 0, s>>>(num_cells, cell_facepos, outflux, cell_volume, porosity, cfl_factor,
                                                 scratch);
    k_cfl_final<<<1, CFL_THREADS, 0, s>>>(nblocks, scratch);
    if (cudaGetLastError() != cudaSuccess) return PORSOL_ERR_CUDA;
    double res[2];
    if (cudaMemcpyAsync(res, scratch + 2 * CFL_MAX_BLOCKS, sizeof(res), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return PORSOL_ERR_CUDA;
    *dt = res[0];
    return res[1] != 0.0 ? PORSOL_ERR_CFL : PORSOL_OK;
}
