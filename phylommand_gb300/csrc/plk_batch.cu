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
//  batch_prune4p_kernel the same over the paired-category tile body of
//                      plk_prune4p.cuh (C = 2, 4, 8; same per-site bits).
//  batch_reduce_kernel one warp per item sums its units in a fixed order
//                      (TwoSum), so results do not depend on scheduling.
#include "plk_batch.h"
#include "plk_device.cuh"
#include "plk_prune4p.cuh"

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
    if (b.write_std) {
        float* dst = b.P32 + ((size_t)g * C + k) * 16;
#pragma unroll
        for (int q = 0; q < 16; ++q) dst[q] = (float)P[q];
    }
    if (b.P32p) {
        float* dst = b.P32p + (size_t)g * C * 16;
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) dst[paired_p_index(k, i, j)] = (float)P[i * 4 + j];
    }
    const int v = nm.y;
    if (v < it.n_tips) {
        float* tt = b.write_std ? b.tip32 + (((size_t)(it.tip_off + v) * C + k) * kCodes) * 4 : nullptr;
        float* tp = b.tip32p ? b.tip32p + (size_t)(it.tip_off + v) * C * kCodes * 4 : nullptr;
        for (int code = 0; code < kCodes; ++code)
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                double acc = 0.0;
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if ((code >> j) & 1) acc += P[i * 4 + j];
                if (tt) tt[code * 4 + i] = (float)acc;
                if (tp) tp[paired_tip_index(k, code, i)] = (float)acc;
            }
    }
}

// The tile job of work unit `unit` (P and tipT in the plain or paired layout).
__device__ __forceinline__ TileJob unit_job(const BatchDev& b, int2 unit, int tile, bool paired) {
    const BatchItemDev it = b.items[unit.x];
    TileJob j;
    j.ops = b.ops + it.ops_off;
    j.n_ops = it.n_ops;
    j.codes = b.codes + it.codes_off;
    j.site_stride = it.site_stride;
    j.n_sites = it.n_sites;
    j.n_tips = it.n_tips;
    j.P = (paired ? b.P32p : b.P32) + (size_t)it.node_off * b.C * 16;
    j.tipT = (paired ? b.tip32p : b.tip32) + (size_t)it.tip_off * b.C * kCodes * 4;
    j.root_w = b.model + it.model_off + 36;
    j.cat_w = b.model + it.model_off + 40 + b.C;
    j.C = b.C;
    j.tile_base = unit.y * tile;
    j.site_lnl = nullptr;
    j.max_depth = b.max_depth;
    return j;
}

// Persistent loop over work units; PAIRED selects the tile body of
// plk_prune4p.cuh (K = pairs) or of plk_prune4s.cuh (K = category bound).
template <bool PAIRED, int K, int SPT, bool CODES_SMEM>
__device__ __forceinline__ void batch_prune_body(const BatchDev& b) {
    extern __shared__ __align__(16) unsigned char sm[];
    __shared__ int s_unit;
    constexpr int TILE = kPruneThreads * SPT;
    for (;;) {
        if (threadIdx.x == 0) s_unit = atomicAdd(b.counter, 1);
        __syncthreads();
        const int u = s_unit;
        if (u >= b.n_units) break;
        const TileJob j = unit_job(b, b.units[u], TILE, PAIRED);
        SiteSum32 sum;
        if constexpr (PAIRED) run_tile4p<K, SPT, CODES_SMEM>(j, sm, sum);
        else run_tile<K, SPT, CODES_SMEM>(j, sm, sum);
        double ts, tc;
        block_sum_site32(sum, ts, tc);
        if (threadIdx.x == 0) {
            b.unit_sums[2 * u] = ts;
            b.unit_sums[2 * u + 1] = tc;
        }
        __syncthreads();
    }
}

template <int CM, int SPT, bool CODES_SMEM>
__global__ void __launch_bounds__(kPruneThreads) batch_prune_kernel(BatchDev b) {
    batch_prune_body<false, CM, SPT, CODES_SMEM>(b);
}

template <int KP, int SPT, bool CODES_SMEM>
__global__ void __launch_bounds__(kPruneThreads) batch_prune4p_kernel(BatchDev b) {
    batch_prune_body<true, KP, SPT, CODES_SMEM>(b);
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

// The kernel of a form, its shared memory for the batch's largest tree.
typedef void (*BatchKernel)(BatchDev);

template <int SPT, bool CODES_SMEM>
BatchKernel kernel_of(int C, bool paired, int max_ops, int max_tips, int max_depth, size_t* smem) {
    if (paired) {
        switch (C) {
            case 2: *smem = tile4p_smem_bytes<1, SPT, CODES_SMEM>(max_ops, max_tips, max_depth);
                    return batch_prune4p_kernel<1, SPT, CODES_SMEM>;
            case 4: *smem = tile4p_smem_bytes<2, SPT, CODES_SMEM>(max_ops, max_tips, max_depth);
                    return batch_prune4p_kernel<2, SPT, CODES_SMEM>;
            case 8: *smem = tile4p_smem_bytes<4, SPT, CODES_SMEM>(max_ops, max_tips, max_depth);
                    return batch_prune4p_kernel<4, SPT, CODES_SMEM>;
            default: return nullptr;
        }
    }
    if (C == 1) {
        *smem = tile_smem_bytes<1, SPT, CODES_SMEM>(max_ops, max_tips, max_depth);
        return batch_prune_kernel<1, SPT, CODES_SMEM>;
    }
    if (C <= 4) {
        *smem = tile_smem_bytes<4, SPT, CODES_SMEM>(max_ops, max_tips, max_depth);
        return batch_prune_kernel<4, SPT, CODES_SMEM>;
    }
    *smem = tile_smem_bytes<8, SPT, CODES_SMEM>(max_ops, max_tips, max_depth);
    return batch_prune_kernel<8, SPT, CODES_SMEM>;
}

BatchKernel form_kernel(int C, const BatchForm& f, int max_ops, int max_tips, int max_depth, size_t* smem) {
    if (!batch_form_valid(C, f)) return nullptr;
    if (f.spt == 1) return f.codes_smem ? kernel_of<1, true>(C, f.paired, max_ops, max_tips, max_depth, smem)
                                        : kernel_of<1, false>(C, f.paired, max_ops, max_tips, max_depth, smem);
    return f.codes_smem ? kernel_of<2, true>(C, f.paired, max_ops, max_tips, max_depth, smem)
                        : kernel_of<2, false>(C, f.paired, max_ops, max_tips, max_depth, smem);
}

}  // namespace

bool batch_form_valid(int C, const BatchForm& f) {
    if (f.spt != 1 && f.spt != 2) return false;
    if (C < 1 || C > 8) return false;
    return !f.paired || C == 2 || C == 4 || C == 8;
}

size_t batch_smem_bytes(int C, const BatchForm& f, int max_ops, int max_tips, int max_depth) {
    size_t smem = 0;
    return form_kernel(C, f, max_ops, max_tips, max_depth, &smem) ? smem : 0;
}

int batch_occupancy(int C, const BatchForm& f, size_t smem) {
    size_t unused = 0;
    const BatchKernel kern = form_kernel(C, f, 0, 0, 0, &unused);
    int n = 0;
    if (!kern) return 0;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, kPruneThreads, smem) != cudaSuccess) return 0;
    return n;
}

cudaError_t launch_batch_pmat(const BatchDev& b, cudaStream_t st) {
    const long long n = (long long)b.n_nodes_total * b.C;
    const int threads = 128;
    const unsigned blocks = (unsigned)((n + threads - 1) / threads);
    if (blocks == 0) return cudaSuccess;
    batch_pmat_kernel<<<blocks, threads, 0, st>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_batch_prune(const BatchDev& b, const BatchForm& f, int grid, size_t smem, cudaStream_t st) {
    size_t unused = 0;
    const BatchKernel kern = form_kernel(b.C, f, 0, 0, 0, &unused);
    if (!kern || (f.paired && (!b.P32p || !b.tip32p))) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<grid, kPruneThreads, smem, st>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_batch_reduce(const BatchDev& b, cudaStream_t st) {
    const int warps_per_block = 8;
    const unsigned blocks = (unsigned)((b.n_items + warps_per_block - 1) / warps_per_block);
    if (blocks == 0) return cudaSuccess;
    batch_reduce_kernel<<<blocks, 32 * warps_per_block, 0, st>>>(b);
    return cudaGetLastError();
}

}  // namespace plk
