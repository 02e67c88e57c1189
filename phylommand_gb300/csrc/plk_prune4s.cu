// prune4s: the 4-state FP32 post-order pass (src/simpleML.cpp:127-197) with
// everything an op reads staged in shared memory.
//
// A CTA owns a tile of 128 x SPT sites of one tree and walks the host-built op
// list.  Before op o runs, op o+2's inputs -- the P(t) rows of its internal
// children and the tip tables of its tip children -- are already on their way
// into a three-slot shared-memory ring by cp.async; the tile's tip codes were
// copied in once at the start.  So the compute of an op touches only
// registers and shared memory: P rows are broadcast reads, tip vectors are
// 16-byte reads indexed by the site's code, spilled partial vectors sit in a
// per-thread stack.  One barrier per op publishes the staged data and frees
// the slot the next prefetch overwrites.  Per-site power-of-two scaling, the
// root reduction (src/simpleML.h:123-141) and the compensated block sum are
// the same as in prune4_kernel.
//
// run_tile() is the per-tile body; prune4s_kernel runs one tile per CTA of a
// single tree, the batch kernel (plk_batch.cu) runs many trees' tiles from a
// work queue.
#include "plk_device.cuh"
#include "plk_internal.h"
#include "plk_prune4s.cuh"

namespace plk {
using namespace dev;

namespace {

template <int CM, int SPT, bool CODES_SMEM>
__global__ void __launch_bounds__(kPruneThreads) prune4s_kernel(PruneArgs a) {
    extern __shared__ __align__(16) unsigned char sm[];
    TileJob j;
    j.ops = a.ops;
    j.n_ops = a.n_ops;
    j.codes = a.codes;
    j.site_stride = a.site_stride;
    j.n_sites = a.n_sites;
    j.n_tips = a.n_tips;
    j.P = static_cast<const float*>(a.P);
    j.tipT = static_cast<const float*>(a.tipT);
    j.root_w = a.root_w;
    j.cat_w = a.cat_w;
    j.C = a.C;
    j.tile_base = blockIdx.x * kPruneThreads * SPT;
    j.site_lnl = a.site_lnl;
    j.max_depth = a.max_depth;
    SiteSum32 sum;
    run_tile<CM, SPT, CODES_SMEM>(j, sm, sum);
    const SiteSum32 bsum = block_sum_site32f(sum);
    if (threadIdx.x == 0) store_site_record(a.block_sum, blockIdx.x, bsum);
    if (a.grid_done) finish_grid_sum32(a.block_sum, a.grid_done, a.lnl_out);
}

template <int CM, int SPT, bool CODES_SMEM>
cudaError_t launch_one(const PruneArgs& a, int* n_blocks, cudaStream_t st) {
    const size_t smem = tile_smem_bytes<CM, SPT, CODES_SMEM>(a.n_ops, a.n_tips, a.max_depth);
    if (smem > kMaxSmem) return cudaErrorInvalidConfiguration;
    auto kern = prune4s_kernel<CM, SPT, CODES_SMEM>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int blocks = (a.n_sites + kPruneThreads * SPT - 1) / (kPruneThreads * SPT);
    *n_blocks = blocks;
    kern<<<blocks, kPruneThreads, smem, st>>>(a);
    return cudaGetLastError();
}

template <int CM, int SPT>
cudaError_t launch_cm_spt(const PruneArgs& a, int* n_blocks, cudaStream_t st) {
    if (tile_smem_bytes<CM, SPT, true>(a.n_ops, a.n_tips, a.max_depth) <= kCodesSmemBudget)
        return launch_one<CM, SPT, true>(a, n_blocks, st);
    return launch_one<CM, SPT, false>(a, n_blocks, st);
}

}  // namespace

bool prune4s_fits(const PruneArgs& a, int spt) {
    return tile_smem_min(a.C, spt, a.n_ops, a.n_tips, a.max_depth) <= kMaxSmem;
}

cudaError_t launch_prune4s(const PruneArgs& a, int spt, int* n_blocks, cudaStream_t st) {
    const int cm = a.C == 1 ? 1 : (a.C <= 4 ? 4 : 8);
    if (a.C > 8) return cudaErrorInvalidValue;
    if (cm == 1) return spt == 1 ? launch_cm_spt<1, 1>(a, n_blocks, st) : launch_cm_spt<1, 2>(a, n_blocks, st);
    if (cm == 4) return spt == 1 ? launch_cm_spt<4, 1>(a, n_blocks, st) : launch_cm_spt<4, 2>(a, n_blocks, st);
    return spt == 1 ? launch_cm_spt<8, 1>(a, n_blocks, st) : launch_cm_spt<8, 2>(a, n_blocks, st);
}

}  // namespace plk
