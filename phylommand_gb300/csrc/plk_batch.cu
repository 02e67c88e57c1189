// Batch engine kernels: many 4-state alignments, each with its own tree and
// model, scored in one persistent launch.
//
//  batch_pmat_kernel   P(t) = L diag(exp(lambda r t)) R for every (node,
//                      category) of every item, FP64, stored as FP32, plus the
//                      tip tables of tip edges.
//  batch_prune_kernel  persistent: each CTA takes (item, site tile) work units
//                      from an atomic counter (largest trees first) and runs
//                      the staged post-order tile body of plk_prune4s.cuh on
//                      it; one compensated partial sum per unit.
//  batch_reduce_kernel one warp per item sums its units in a fixed order
//                      (TwoSum), so results do not depend on scheduling.
#include "plk_batch.h"
#include "plk_device.cuh"
#include "plk_prune4s.cuh"

namespace plk {
using namespace dev;

namespace {

__global__ void batch_pmat_kernel(BatchDev b) {
    const int C = b.C;
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (long long)b.n_nodes_total * C) return;
    const int g = (int)(gid / C), k = (int)(gid % C);
    const int2 nm = b.node_item[g];
    const BatchItemDev it = b.items[nm.x];
    const double* mdl = b.model + it.model_off;
    const double* lam = mdl;
    const double* L = mdl + 4;
    const double* R = mdl + 20;
    const double* cat_rate = mdl + 40;
    const double t = b.t_eff[g] * cat_rate[k];
    double ex[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) ex[m] = exp(lam[m] * t);
    double P[16];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            double acc = 0.0;
#pragma unroll
            for (int m = 0; m < 4; ++m) acc = fma(L[i * 4 + m] * ex[m], R[m * 4 + j], acc);
            P[i * 4 + j] = acc;
        }
    float* dst = b.P32 + ((size_t)g * C + k) * 16;
#pragma unroll
    for (int q = 0; q < 16; ++q) dst[q] = (float)P[q];
    const int v = nm.y;
    if (v < it.n_tips) {
        float* tt = b.tip32 + (((size_t)(it.tip_off + v) * C + k) * kCodes) * 4;
        for (int code = 0; code < kCodes; ++code)
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                double acc = 0.0;
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if ((code >> j) & 1) acc += P[i * 4 + j];
                tt[code * 4 + i] = (float)acc;
            }
    }
}

template <int CM, int SPT, bool CODES_SMEM>
__global__ void __launch_bounds__(kPruneThreads) batch_prune_kernel(BatchDev b) {
    extern __shared__ __align__(16) unsigned char sm[];
    __shared__ int s_unit;
    constexpr int TILE = kPruneThreads * SPT;
    for (;;) {
        if (threadIdx.x == 0) s_unit = atomicAdd(b.counter, 1);
        __syncthreads();
        const int u = s_unit;
        if (u >= b.n_units) break;
        const int2 unit = b.units[u];
        const BatchItemDev it = b.items[unit.x];
        TileJob j;
        j.ops = b.ops + it.ops_off;
        j.n_ops = it.n_ops;
        j.codes = b.codes + it.codes_off;
        j.site_stride = it.site_stride;
        j.n_sites = it.n_sites;
        j.n_tips = it.n_tips;
        j.P = b.P32 + (size_t)it.node_off * b.C * 16;
        j.tipT = b.tip32 + (size_t)it.tip_off * b.C * kCodes * 4;
        j.root_w = b.model + it.model_off + 36;
        j.cat_w = b.model + it.model_off + 40 + b.C;
        j.C = b.C;
        j.tile_base = unit.y * TILE;
        j.site_lnl = nullptr;
        j.max_depth = b.max_depth;
        double ts = 0.0, tc = 0.0;
        run_tile<CM, SPT, CODES_SMEM>(j, sm, ts, tc);
        block_sum_pair(ts, tc);
        if (threadIdx.x == 0) {
            b.unit_sums[2 * u] = ts;
            b.unit_sums[2 * u + 1] = tc;
        }
        __syncthreads();
    }
}

__global__ void batch_reduce_kernel(BatchDev b) {
    const int item = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (item >= b.n_items) return;
    const int lo = b.item_unit_ptr[item], hi = b.item_unit_ptr[item + 1];
    double s = 0.0, c = 0.0;
    for (int q = lo + lane; q < hi; q += 32) {
        const int u = b.item_units[q];
        double ns, e;
        two_sum(s, b.unit_sums[2 * u], ns, e);
        s = ns;
        c += b.unit_sums[2 * u + 1] + e;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const double os = __shfl_down_sync(0xffffffffu, s, off);
        const double oc = __shfl_down_sync(0xffffffffu, c, off);
        double ns, e;
        two_sum(s, os, ns, e);
        s = ns;
        c = c + oc + e;
    }
    if (lane == 0) b.lnl[item] = s + c;
}

template <int CM, int SPT, bool CODES_SMEM>
cudaError_t launch_batch_prune_t(const BatchDev& b, int grid, size_t smem, cudaStream_t st) {
    auto kern = batch_prune_kernel<CM, SPT, CODES_SMEM>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<grid, kPruneThreads, smem, st>>>(b);
    return cudaGetLastError();
}

template <int CM, int SPT, bool CODES_SMEM>
int occupancy_t(size_t smem) {
    int n = 0;
    auto kern = batch_prune_kernel<CM, SPT, CODES_SMEM>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, kPruneThreads, smem) != cudaSuccess) return 0;
    return n;
}

}  // namespace

size_t batch_smem_bytes(int C, int spt, bool codes_smem, int max_ops, int max_tips, int max_depth) {
    const int cm = C == 1 ? 1 : (C <= 4 ? 4 : 8);
#define PLK_SMEM_CASE(CMV)                                                                                  \
    if (cm == CMV) {                                                                                        \
        if (spt == 1) return codes_smem ? tile_smem_bytes<CMV, 1, true>(max_ops, max_tips, max_depth)      \
                                        : tile_smem_bytes<CMV, 1, false>(max_ops, max_tips, max_depth);    \
        return codes_smem ? tile_smem_bytes<CMV, 2, true>(max_ops, max_tips, max_depth)                    \
                          : tile_smem_bytes<CMV, 2, false>(max_ops, max_tips, max_depth);                  \
    }
    PLK_SMEM_CASE(1)
    PLK_SMEM_CASE(4)
    PLK_SMEM_CASE(8)
#undef PLK_SMEM_CASE
    return 0;
}

int batch_occupancy(int C, int spt, bool codes_smem, size_t smem) {
    const int cm = C == 1 ? 1 : (C <= 4 ? 4 : 8);
#define PLK_OCC_CASE(CMV)                                                                               \
    if (cm == CMV) {                                                                                    \
        if (spt == 1) return codes_smem ? occupancy_t<CMV, 1, true>(smem) : occupancy_t<CMV, 1, false>(smem); \
        return codes_smem ? occupancy_t<CMV, 2, true>(smem) : occupancy_t<CMV, 2, false>(smem);         \
    }
    PLK_OCC_CASE(1)
    PLK_OCC_CASE(4)
    PLK_OCC_CASE(8)
#undef PLK_OCC_CASE
    return 0;
}

cudaError_t launch_batch_pmat(const BatchDev& b, cudaStream_t st) {
    const long long n = (long long)b.n_nodes_total * b.C;
    const int threads = 128;
    const unsigned blocks = (unsigned)((n + threads - 1) / threads);
    if (blocks == 0) return cudaSuccess;
    batch_pmat_kernel<<<blocks, threads, 0, st>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_batch_prune(const BatchDev& b, int spt, bool codes_smem, int grid, size_t smem,
                               cudaStream_t st) {
    const int cm = b.C == 1 ? 1 : (b.C <= 4 ? 4 : 8);
#define PLK_LAUNCH_CASE(CMV)                                                                                   \
    if (cm == CMV) {                                                                                           \
        if (spt == 1) return codes_smem ? launch_batch_prune_t<CMV, 1, true>(b, grid, smem, st)               \
                                        : launch_batch_prune_t<CMV, 1, false>(b, grid, smem, st);             \
        return codes_smem ? launch_batch_prune_t<CMV, 2, true>(b, grid, smem, st)                             \
                          : launch_batch_prune_t<CMV, 2, false>(b, grid, smem, st);                           \
    }
    PLK_LAUNCH_CASE(1)
    PLK_LAUNCH_CASE(4)
    PLK_LAUNCH_CASE(8)
#undef PLK_LAUNCH_CASE
    return cudaErrorInvalidValue;
}

cudaError_t launch_batch_reduce(const BatchDev& b, cudaStream_t st) {
    const int warps_per_block = 8;
    const unsigned blocks = (unsigned)((b.n_items + warps_per_block - 1) / warps_per_block);
    if (blocks == 0) return cudaSuccess;
    batch_reduce_kernel<<<blocks, 32 * warps_per_block, 0, st>>>(b);
    return cudaGetLastError();
}

}  // namespace plk
