// plk_sum_sites_noalloc: the compensated sum of per-site log-likelihoods that
// already sit in device memory, with its block partial sums kept in a
// file-scope device array instead of memory from cudaMalloc.
//
// Who needs it: code that cannot allocate device memory at the moment it
// wants the total -- e.g. work being recorded into a CUDA stream capture
// (cudaMalloc is not capturable), a host program whose device memory is owned
// by another allocator (a framework's pool or a fixed arena), or a caller on a
// latency budget that cannot afford cudaMalloc/cudaFree synchronising the
// device.  The caller passes the per-site values and the output location; the
// function allocates nothing.
//
// Limits and sharing: the array holds the partial sums of at most
// kNoallocMaxBlocks blocks of kNoallocThreads sites, so at most 1,048,576
// sites per call (64 KiB of device memory, held by every GPU that loads the
// library until the process exits).  Every call on a device uses the same
// array and leaves its contents behind; each call writes every slot it reads
// before reading it, so nothing needs clearing, but two calls that overlap on
// the GPU (on different streams, or from different host threads without
// ordering) race on the array.  The array's address is looked up once per
// device and context: after a device reset (cudaDeviceReset) the next call
// looks it up again in the new context, so make that call before any stream
// capture as well.
#include <cuda.h>  // CUcontext / CUresult types of the two driver calls below (no -lcuda: entry points)

#include <mutex>
#include <string>

#include "plk_internal.h"

namespace {

constexpr int kNoallocThreads = 256;
constexpr int kNoallocMaxBlocks = 4096;
constexpr int kNoallocMaxSites = kNoallocThreads * kNoallocMaxBlocks;
constexpr int kMaxDevices = 64;

// (sum, compensation) per block
static __device__ __align__(256) double g_noalloc_partials[2 * kNoallocMaxBlocks];

__device__ __forceinline__ void two_sum_na(double a, double b, double& s, double& e) {
    s = __dadd_rn(a, b);
    const double bb = __dsub_rn(s, a);
    e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
}

__device__ __forceinline__ void block_reduce_pair(double& s, double& c) {
    for (int off = 16; off > 0; off >>= 1) {
        const double os = __shfl_down_sync(0xffffffffu, s, off);
        const double oc = __shfl_down_sync(0xffffffffu, c, off);
        double ns, e;
        two_sum_na(s, os, ns, e);
        s = ns;
        c = c + oc + e;
    }
    __shared__ double rs[32], rc[32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { rs[warp] = s; rc[warp] = c; }
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        s = lane < nw ? rs[lane] : 0.0;
        c = lane < nw ? rc[lane] : 0.0;
        for (int off = 16; off > 0; off >>= 1) {
            const double os = __shfl_down_sync(0xffffffffu, s, off);
            const double oc = __shfl_down_sync(0xffffffffu, c, off);
            double ns, e;
            two_sum_na(s, os, ns, e);
            s = ns;
            c = c + oc + e;
        }
    }
}

// one site per thread; block b writes partials[2b], partials[2b+1]
__global__ void __launch_bounds__(kNoallocThreads) noalloc_block_sums(const double* __restrict__ site, int n,
                                                                      double* __restrict__ partials) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double s = i < n ? site[i] : 0.0, c = 0.0;
    block_reduce_pair(s, c);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = s;
        partials[2 * blockIdx.x + 1] = c;
    }
}

__global__ void __launch_bounds__(kNoallocThreads) noalloc_final(const double* __restrict__ partials, int nb,
                                                                 double* __restrict__ out) {
    double s = 0.0, c = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        double ns, e;
        two_sum_na(s, partials[2 * b], ns, e);
        s = ns;
        c = c + partials[2 * b + 1] + e;
    }
    block_reduce_pair(s, c);
    if (threadIdx.x == 0) out[0] = s + c;
}

std::mutex g_setup_mu;
double* g_partials_addr[kMaxDevices] = {nullptr};
unsigned long long g_partials_ctx[kMaxDevices] = {0};  // the context the address belongs to (0: unknown)

}  // namespace

namespace plk {

// Unique id of the current context (cuCtxGetId, fetched through the
// runtime's driver entry points), 0 when it cannot be had.  A device reset
// destroys the primary context and the next runtime call makes a new one
// with a new id, in which device symbols may sit at other addresses and a
// kernel's attributes are back at their defaults.  Thread-safe.
unsigned long long current_ctx_id() {
    typedef CUresult (*GetCurrent)(CUcontext*);
    typedef CUresult (*GetId)(CUcontext, unsigned long long*);
    struct Fns {
        GetCurrent get_current = nullptr;
        GetId get_id = nullptr;
    };
    static const Fns fns = [] {  // looked up once (thread-safe initialisation)
        Fns f;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            f.get_current = reinterpret_cast<GetCurrent>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            f.get_id = reinterpret_cast<GetId>(p);
        return f;
    }();
    if (!fns.get_current || !fns.get_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (fns.get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr) return 0;
    if (fns.get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

}  // namespace plk

extern "C" plk_status plk_sum_sites_noalloc(const double* d_site_lnl, int n_sites, double* d_lnl_out,
                                            void* cuda_stream) {
    if (!d_site_lnl || !d_lnl_out)
        return plk::report_error(PLK_ERR_ARG, "plk_sum_sites_noalloc: NULL device pointer");
    if (n_sites < 1 || n_sites > kNoallocMaxSites)
        return plk::report_error(PLK_ERR_ARG, "plk_sum_sites_noalloc: n_sites must be in 1.." +
                                                  std::to_string(kNoallocMaxSites) + ", got " +
                                                  std::to_string(n_sites));
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return plk::report_error(PLK_ERR_CUDA, std::string("plk_sum_sites_noalloc: cudaGetDevice: ") +
                                                   cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return plk::report_error(PLK_ERR_ARG, "plk_sum_sites_noalloc: device index too large");
    double* partials = nullptr;
    {
        // first call on a device (or in a new context of it, after a device
        // reset): resolve the device address of the array with that device
        // current (host code cannot use the symbol itself)
        std::lock_guard<std::mutex> lock(g_setup_mu);
        const unsigned long long ctx = plk::current_ctx_id();
        if (!g_partials_addr[dev] || (ctx != 0 && ctx != g_partials_ctx[dev])) {
            e = cudaGetSymbolAddress(reinterpret_cast<void**>(&g_partials_addr[dev]), g_noalloc_partials);
            if (e != cudaSuccess) {
                g_partials_addr[dev] = nullptr;
                return plk::report_error(PLK_ERR_CUDA, std::string("plk_sum_sites_noalloc: cudaGetSymbolAddress: ") +
                                                           cudaGetErrorString(e));
            }
            // the id of the context the runtime just used (made, after a reset)
            g_partials_ctx[dev] = ctx != 0 ? ctx : plk::current_ctx_id();
        }
        partials = g_partials_addr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    const int nb = (n_sites + kNoallocThreads - 1) / kNoallocThreads;
    noalloc_block_sums<<<nb, kNoallocThreads, 0, st>>>(d_site_lnl, n_sites, partials);
    noalloc_final<<<1, kNoallocThreads, 0, st>>>(partials, nb, d_lnl_out);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return plk::report_error(PLK_ERR_CUDA, std::string("plk_sum_sites_noalloc: launch: ") + cudaGetErrorString(e));
    return PLK_OK;
}
