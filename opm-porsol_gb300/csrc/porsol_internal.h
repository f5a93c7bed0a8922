// porsol_internal.h -- shared host/device declarations of the GB300 porsol library.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <atomic>

#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <type_traits>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "porsol_gpu.h"

namespace porsol {

// ------------------------------------------------------------------ errors
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define PORSOL_CUDA(call)                                                                   \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            throw ::porsol::Error(PORSOL_ERR_CUDA, std::string(#call " failed: ") +          \
                                                        cudaGetErrorString(e_));            \
    } while (0)

#define PORSOL_REQUIRE(cond, code, msg)                      \
    do {                                                     \
        if (!(cond)) throw ::porsol::Error((code), (msg));    \
    } while (0)

// Device status bits written by kernels (atomicOr) and mapped to porsol_status on the host.
enum : int {
    ST_NONFINITE = 1,     // NaN/Inf or non-positive pivot/mobility sum
    ST_BREAKDOWN = 2,     // Krylov breakdown (zero curvature)
    ST_SAT_RANGE = 4,     // saturation outside [-0.001, 1.001]
    ST_CFL_ZERO = 8,      // CFL step of zero
    ST_TIMEOUT = 16,      // bounded wait gave up
    ST_BAD_INDEX = 32,    // index check failed
};

// ------------------------------------------------------------------ host vectors
// Allocator whose resize() leaves plain values uninitialised: the large host arrays of the
// structure build are written in full by parallel loops, so the serial zero fill of a
// std::vector (and its single-threaded first touch of every page) is skipped.
template <class T>
struct DefaultInitAlloc : std::allocator<T> {
    template <class U>
    struct rebind {
        using other = DefaultInitAlloc<U>;
    };
    DefaultInitAlloc() = default;
    template <class U>
    DefaultInitAlloc(const DefaultInitAlloc<U>&) noexcept
    {
    }
    template <class U>
    void construct(U* p) noexcept(std::is_nothrow_default_constructible<U>::value)
    {
        ::new (static_cast<void*>(p)) U;
    }
    template <class U, class... Args>
    void construct(U* p, Args&&... args)
    {
        ::new (static_cast<void*>(p)) U(std::forward<Args>(args)...);
    }
};
template <class T>
using HVec = std::vector<T, DefaultInitAlloc<T>>;

// ------------------------------------------------------------------ device buffers
template <class T>
struct DBuf {
    // Grow-only device buffer: alloc() keeps the allocation when it is large enough, so
    // repeated setups of the same size (every solve) do no cudaMalloc/cudaFree.
    T* p = nullptr;
    size_t n = 0;    // elements in use
    size_t cap = 0;  // elements allocated
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : p(o.p), n(o.n), cap(o.cap) { o.p = nullptr; o.n = o.cap = 0; }
    DBuf& operator=(DBuf&& o) noexcept
    {
        if (this != &o) {
            release();
            p = o.p; n = o.n; cap = o.cap;
            o.p = nullptr; o.n = o.cap = 0;
        }
        return *this;
    }
    ~DBuf() { release(); }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = cap = 0;
    }
    void alloc(size_t cnt)
    {
        if (cnt <= cap && p) {
            n = cnt;
            return;
        }
        release();
        if (cnt == 0) return;
        PORSOL_CUDA(cudaMalloc(&p, cnt * sizeof(T)));
        n = cap = cnt;
    }
    void upload(const T* h, size_t cnt, cudaStream_t s)
    {
        alloc(cnt);
        if (cnt) PORSOL_CUDA(cudaMemcpyAsync(p, h, cnt * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    template <class A>
    void upload(const std::vector<T, A>& h, cudaStream_t s)
    {
        upload(h.data(), h.size(), s);
    }
    void download(T* h, size_t cnt, cudaStream_t s) const
    {
        if (cnt) PORSOL_CUDA(cudaMemcpyAsync(h, p, cnt * sizeof(T), cudaMemcpyDeviceToHost, s));
    }
    void zero(cudaStream_t s)
    {
        if (n) PORSOL_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
    }
};

// ------------------------------------------------------------------ sparse matrices
// Sliced ELLPACK with slice height 32 (one warp): row r lives in slice r/32, lane r%32;
// entry t of row r is at slice_ptr[r/32] + 32*t + r%32.  Entries of a row are sorted by
// column; padding entries carry col = row and value 0.
constexpr int SELL_C = 32;

struct SellPattern {
    int n = 0;          // rows
    int nslices = 0;
    long long nent = 0; // stored entries incl. padding
    HVec<int> h_slice_ptr, h_col, h_rowlen;
    DBuf<int> slice_ptr, col, rowlen, diag;   // diag: slot index of the diagonal
    // the columns again as 16-bit offsets from the row (padding 0), when every stored column lies
    // within 32767 rows of its row (upload() decides; off16 stays empty otherwise): the CG's
    // matrix-vector products then read 2 instead of 4 bytes of index per entry
    DBuf<short> off16;
    bool has_off16() const { return off16.p != nullptr && off16.n == size_t(nent); }
    void upload(cudaStream_t s);
};

template <class T>
struct SellMatrix {
    const SellPattern* pat = nullptr;
    DBuf<T> val;
};

// Build a SELL pattern from CSR with sorted columns.  csr2sell[k] = slot of CSR entry k.
void build_sell(int n, const HVec<int>& rowptr, const HVec<int>& col, SellPattern& P, HVec<int>* csr2sell);

// ------------------------------------------------------------------ profiling
enum ProfKernel { PK_SPMV64 = 0, PK_SPMV32 = 1, PK_ASSEMBLE = 2, PK_RECOVER = 3, PK_VCYCLE = 4, PK_CHEB = 5, PK_COUNT = 6 };

struct Profiler {
    bool on = false;
    int launches[PK_COUNT] = {0};
    double ms[PK_COUNT] = {0};
    double bytes[PK_COUNT] = {0};
    struct Pending { cudaEvent_t a, b; int k; double bytes; };
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> pool;
    cudaEvent_t get();
    void begin(cudaStream_t s, int k, double bytes, cudaEvent_t* out_a);
    void end(cudaStream_t s, int k, double bytes, cudaEvent_t a);
    void collect();    // synchronises on pending events
    void reset();
    ~Profiler();
};

struct ProfScope {
    Profiler& P;
    cudaStream_t s;
    int k;
    double bytes;
    cudaEvent_t a = nullptr;
    ProfScope(Profiler& p, cudaStream_t st, int kern, double b) : P(p), s(st), k(kern), bytes(b)
    {
        if (P.on) P.begin(s, k, bytes, &a);
    }
    ~ProfScope()
    {
        if (P.on && a) P.end(s, k, bytes, a);
    }
};

// ------------------------------------------------------------------ tracing
// NVTX range for the duration of a scope (header-only NVTX 3: a no-op unless a profiler such as
// Nsight Systems or Nsight Compute is attached), so timelines show the phases of a call.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// ------------------------------------------------------------------ launch helpers
inline int div_up(long long a, int b) { return int((a + b - 1) / b); }

// Process-wide count of kernel launches made by this library (porsol_launch_count()).
extern std::atomic<long long> g_launches;
#define PORSOL_COUNT_LAUNCH() ::porsol::g_launches.fetch_add(1, std::memory_order_relaxed)
#define PORSOL_LAUNCH(...)      \
    do {                        \
        __VA_ARGS__;            \
        PORSOL_COUNT_LAUNCH();  \
    } while (0)

// ------------------------------------------------------------------ chained launches
// The kernels of a CG iteration (the SpMV, the vector updates, the preconditioner's cycle) run
// back to back, many of them on small AMG levels and in level-scheduled triangular solves where the
// gap between two kernels costs as much as the work.  Those on grids of fewer than 304 blocks (two
// per SM) are launched with programmatic stream serialisation (programmatic dependent launch, sm_90
// and later): their blocks may be scheduled while the preceding kernel's last blocks still run.
// Every kernel launched through chain() starts with chain_wait(), which returns once the preceding
// kernel has completed and its writes are visible, so the order of all reads and writes is that of
// plain stream launches.  On GB300 this saved 3.5 % of an ILU0-CG solve and 0.1-0.2 ms of an AMG-CG
// solve, while chaining the large grids too cost 0.2-1.3 ms.  Chaining is off while per-kernel event
// timing is on (ChainPause); PORSOL_PDL=0 (never), 1 (every grid) or 2 (small grids, the default)
// in the environment selects it.
bool chain_enabled(long long blocks);
struct ChainPause {   // plain launches in this thread for the scope's duration (nestable)
    explicit ChainPause(bool on = true);
    ~ChainPause();
    ChainPause(const ChainPause&) = delete;
    ChainPause& operator=(const ChainPause&) = delete;

private:
    bool on_;
};

template <class... KA, class... A>
inline void chain(void (*kernel)(KA...), dim3 grid, dim3 block, size_t shm, cudaStream_t s, A&&... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = shm;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = chain_enabled((long long)grid.x * grid.y * grid.z) ? 1 : 0;
    PORSOL_CUDA(cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...));
    PORSOL_COUNT_LAUNCH();
}

#ifdef __CUDACC__
// First statement of every kernel launched by chain(): wait for the preceding kernel (a no-op
// when launched plainly), then let the next chained kernel's blocks be scheduled.  Every block
// runs it before it can return, so completion of a chained kernel implies completion of all
// kernels before it.
__device__ __forceinline__ void chain_wait()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
#endif

}  // namespace porsol
