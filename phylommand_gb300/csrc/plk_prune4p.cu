// prune4p: the staged 4-state FP32 post-order pass (src/simpleML.cpp:127-197)
// with the rate categories taken in pairs on Blackwell's packed FP32x2 pipe.
//
// Same structure as prune4s (plk_prune4s.cu): a CTA walks the op list over a
// tile of 128 x SPT sites, op o+2's P(t) rows and tip tables travel into a
// three-slot shared-memory ring by cp.async while op o computes, spilled
// vectors sit in a per-thread shared-memory stack.  The tip codes are read
// from global memory at their use, staged for the whole tile, or staged
// with each op in a ring beside the stage slots (CODES 0 / 1 / 2).  The tile body
// (run_tile4p, plk_prune4p.cuh) keeps every value as a pair (category 2q,
// category 2q+1), so each product is one fma.rn.f32x2 / mul.rn.f32x2 for two
// categories, rounding lane by lane exactly as prune4s: the per-site results
// are the same bits.  The number of categories is a compile-time constant
// (2, 4 or 8), so no category loop carries a guard.
//
// relayout4p_kernel writes the paired P(t) and tip layouts from the FP32
// copies of the P(t) kernel.
#include "plk_prune4p.cuh"

namespace plk {
using namespace dev;

namespace {

__global__ void relayout4p_kernel(const float* __restrict__ P, const float* __restrict__ tip, int n_nodes,
                                  int n_tips, int C, float* __restrict__ Pp, float* __restrict__ Tp) {
    const long long n_p = (long long)n_nodes * C * 16;
    const long long n_t = (long long)n_tips * C * kCodes * 4;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n_p + n_t;
         idx += (long long)gridDim.x * blockDim.x) {
        if (idx < n_p) {
            // source P[node][k][i][j]
            const long long node = idx / (C * 16);
            const int w = (int)(idx % (C * 16));
            Pp[node * C * 16 + paired_p_index(w / 16, (w / 4) % 4, w % 4)] = P[idx];
        } else {
            // source tip[tip][k][code][i]
            const long long t = idx - n_p;
            const long long tp = t / (C * kCodes * 4);
            const int w = (int)(t % (C * kCodes * 4));
            Tp[tp * C * kCodes * 4 + paired_tip_index(w / (kCodes * 4), (w / 4) % kCodes, w % 4)] = tip[t];
        }
    }
}

template <int KP, int SPT, int CODES, int TPS>
__global__ void __launch_bounds__(kPruneThreads) prune4p_kernel(PruneArgs a, const float* __restrict__ Pp,
                                                                const float* __restrict__ Tp) {
    extern __shared__ __align__(16) unsigned char sm[];
    TileJob j;
    j.ops = a.ops;
    j.n_ops = a.n_ops;
    j.codes = a.codes;
    j.site_stride = a.site_stride;
    j.n_sites = a.n_sites;
    j.n_tips = a.n_tips;
    j.P = Pp;
    j.tipT = Tp;
    j.root_w = a.root_w;
    j.cat_w = a.cat_w;
    j.C = 2 * KP;
    j.tile_base = blockIdx.x * tile4p_sites<SPT, TPS>();
    j.site_lnl = a.site_lnl;
    j.max_depth = a.max_depth;
    SiteSum32 sum;
    run_tile4p<KP, SPT, CODES, TPS>(j, sm, sum);
    const SiteSum32 bsum = block_sum_site32f(sum);
    if (threadIdx.x == 0) store_site_record(a.block_sum, blockIdx.x, bsum);
    if (a.grid_done) finish_grid_sum32(a.block_sum, a.grid_done, a.lnl_out);
}

// The TMA-fed form (run_tile4p_bulk): one site per thread, codes from global.
template <int KP>
__global__ void __launch_bounds__(kPruneThreads) prune4p_bulk_kernel(PruneArgs a, const float* __restrict__ Pp,
                                                                     const float* __restrict__ Tp) {
    extern __shared__ __align__(16) unsigned char sm[];
    __shared__ __align__(8) uint64_t bars[6];  // full[3], empty[3]
    __shared__ int s_abort;
    if (threadIdx.x == 0) {
        for (int q = 0; q < 3; ++q) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(&bars[q])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(&bars[3 + q])),
                         "r"(kPruneThreads / 32)
                         : "memory");
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        s_abort = 0;
    }
    TileJob j;
    j.ops = a.ops;
    j.n_ops = a.n_ops;
    j.codes = a.codes;
    j.site_stride = a.site_stride;
    j.n_sites = a.n_sites;
    j.n_tips = a.n_tips;
    j.P = Pp;
    j.tipT = Tp;
    j.root_w = a.root_w;
    j.cat_w = a.cat_w;
    j.C = 2 * KP;
    j.tile_base = blockIdx.x * kPruneThreads;
    j.site_lnl = a.site_lnl;
    j.max_depth = a.max_depth;
    SiteSum32 sum;
    run_tile4p_bulk<KP>(j, sm, bars, &s_abort, sum, a.withhold_first_stage != 0);
    const SiteSum32 bsum = block_sum_site32f(sum);
    if (threadIdx.x == 0) store_site_record(a.block_sum, blockIdx.x, bsum);
    if (a.grid_done) finish_grid_sum32(a.block_sum, a.grid_done, a.lnl_out);
}

template <int KP>
cudaError_t launch4p_bulk(const PruneArgs& a, const float* Pp, const float* Tp, int* n_blocks, cudaStream_t st) {
    const size_t smem = tile4p_bulk_smem_bytes<KP>(a.n_ops, a.max_depth);
    if (smem > 227 * 1024) return cudaErrorInvalidConfiguration;
    auto kern = prune4p_bulk_kernel<KP>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int blocks = (a.n_sites + kPruneThreads - 1) / kPruneThreads;
    *n_blocks = blocks;
    kern<<<blocks, kPruneThreads, smem, st>>>(a, Pp, Tp);
    return cudaGetLastError();
}

template <int KP, int SPT, int CODES, int TPS>
cudaError_t launch4p(const PruneArgs& a, const float* Pp, const float* Tp, int* n_blocks, cudaStream_t st) {
    const size_t smem = tile4p_smem_bytes<KP, SPT, CODES, TPS>(a.n_ops, a.n_tips, a.max_depth);
    if (smem > 227 * 1024) return cudaErrorInvalidConfiguration;
    auto kern = prune4p_kernel<KP, SPT, CODES, TPS>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    constexpr int TILE = tile4p_sites<SPT, TPS>();
    const int blocks = (a.n_sites + TILE - 1) / TILE;
    *n_blocks = blocks;
    kern<<<blocks, kPruneThreads, smem, st>>>(a, Pp, Tp);
    return cudaGetLastError();
}

// codes: 0 = stage the tile's codes of every tip in shared memory (global
// memory when they do not fit), 1 = read them from global memory at their use
// (more resident CTAs), 2 = stage each op's codes with its tables (one site
// per thread)
template <int KP, int SPT, int TPS>
cudaError_t launch4p_kp(const PruneArgs& a, const float* Pp, const float* Tp, int codes, int* n_blocks,
                        cudaStream_t st) {
    if constexpr (TPS == 1) {
        if (codes == 2) return launch4p<KP, SPT, 2, TPS>(a, Pp, Tp, n_blocks, st);
    }
    if (codes == 0 && tile4p_smem_bytes<KP, SPT, 1, TPS>(a.n_ops, a.n_tips, a.max_depth) <= 160 * 1024)
        return launch4p<KP, SPT, 1, TPS>(a, Pp, Tp, n_blocks, st);
    return launch4p<KP, SPT, 0, TPS>(a, Pp, Tp, n_blocks, st);
}

}  // namespace

bool prune4p_fits(const PruneArgs& a, int spt, int tps) {
    if (a.C != 2 && a.C != 4 && a.C != 8) return false;
    if (tps == 0) {
        if (spt != 1) return false;
        const size_t smem = a.C == 2   ? tile4p_bulk_smem_bytes<1>(a.n_ops, a.max_depth)
                            : a.C == 4 ? tile4p_bulk_smem_bytes<2>(a.n_ops, a.max_depth)
                                       : tile4p_bulk_smem_bytes<4>(a.n_ops, a.max_depth);
        return smem <= 227 * 1024;
    }
    if (tps == 2) {
        if (spt != 1 || a.C == 2) return false;
        const size_t smem = a.C == 4 ? tile4p_smem_bytes<2, 1, 0, 2>(a.n_ops, a.n_tips, a.max_depth)
                                     : tile4p_smem_bytes<4, 1, 0, 2>(a.n_ops, a.n_tips, a.max_depth);
        return smem <= 227 * 1024;
    }
    if (tps != 1 || (spt != 1 && spt != 2)) return false;
    return tile4p_smem_min(a.C, spt, a.n_ops, a.n_tips, a.max_depth) <= 227 * 1024;
}

size_t prune4p_scratch_bytes(const PruneArgs& a) {
    const size_t p = (size_t)a.n_nodes * a.C * 16 * sizeof(float);
    return ((p + 255) & ~(size_t)255) + (size_t)a.n_tips * a.C * kCodes * 4 * sizeof(float);
}

void prune4p_scratch_parts(void* scratch, int n_nodes, int C, float** Pp, float** Tp) {
    const size_t p = (size_t)n_nodes * C * 16 * sizeof(float);
    *Pp = static_cast<float*>(scratch);
    *Tp = reinterpret_cast<float*>(static_cast<unsigned char*>(scratch) + ((p + 255) & ~(size_t)255));
}

cudaError_t launch_relayout4p(const PruneArgs& a, float* Pp, float* Tp, cudaStream_t st) {
    const long long total = (long long)a.n_nodes * a.C * 16 + (long long)a.n_tips * a.C * kCodes * 4;
    long long blocks = (total + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    relayout4p_kernel<<<(unsigned)blocks, 256, 0, st>>>(static_cast<const float*>(a.P),
                                                         static_cast<const float*>(a.tipT), a.n_nodes, a.n_tips, a.C,
                                                         Pp, Tp);
    return cudaGetLastError();
}

cudaError_t launch_prune4p(const PruneArgs& a, int spt, int codes, int tps, int* n_blocks, cudaStream_t st) {
    // tps 0: the TMA-fed form (one site per thread, codes from global)
    if (!prune4p_fits(a, spt, tps) || a.scratch == nullptr) return cudaErrorInvalidValue;
    float *Pp, *Tp;
    prune4p_scratch_parts(a.scratch, a.n_nodes, a.C, &Pp, &Tp);
    if (!a.paired_ready) {
        cudaError_t e = launch_relayout4p(a, Pp, Tp, st);
        if (e != cudaSuccess) return e;
    }
    if (tps == 2) {
        return a.C == 4 ? launch4p_kp<2, 1, 2>(a, Pp, Tp, codes, n_blocks, st)
                        : launch4p_kp<4, 1, 2>(a, Pp, Tp, codes, n_blocks, st);
    }
    if (tps == 0) {
        switch (a.C / 2) {
            case 1: return launch4p_bulk<1>(a, Pp, Tp, n_blocks, st);
            case 2: return launch4p_bulk<2>(a, Pp, Tp, n_blocks, st);
            default: return launch4p_bulk<4>(a, Pp, Tp, n_blocks, st);
        }
    }
    switch (a.C / 2) {
        case 1: return spt == 1 ? launch4p_kp<1, 1, 1>(a, Pp, Tp, codes, n_blocks, st)
                                : launch4p_kp<1, 2, 1>(a, Pp, Tp, codes, n_blocks, st);
        case 2: return spt == 1 ? launch4p_kp<2, 1, 1>(a, Pp, Tp, codes, n_blocks, st)
                                : launch4p_kp<2, 2, 1>(a, Pp, Tp, codes, n_blocks, st);
        default: return spt == 1 ? launch4p_kp<4, 1, 1>(a, Pp, Tp, codes, n_blocks, st)
                                 : launch4p_kp<4, 2, 1>(a, Pp, Tp, codes, n_blocks, st);
    }
}

}  // namespace plk
