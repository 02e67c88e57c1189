// prune4s_kernel: the 4-state FP32 post-order pass (src/simpleML.cpp:127-197)
// with everything an op reads staged in shared memory.
//
// A CTA owns a tile of 128 x SPT sites and walks the host-built op list.
// Before op o runs, op o+2's inputs -- the P(t) rows of its internal
// children and the tip tables of its tip children -- are already on their way
// into a three-slot shared-memory ring by cp.async; the tile's tip codes were
// copied in once at the start.  So the compute of an op touches only
// registers and shared memory: P rows are broadcast reads, tip vectors are
// 16-byte reads indexed by the site's code, spilled partial vectors sit in a
// per-thread stack.  One barrier per op publishes the staged data and frees
// the slot the next prefetch overwrites.  Per-site power-of-two scaling, the
// root reduction (src/simpleML.h:123-141) and the compensated block sum are
// the same as in prune4_kernel.
#include "plk_device.cuh"
#include "plk_internal.h"

namespace plk {
using namespace dev;

namespace {

constexpr int kCodes = 16;  // state sets of a <= 4-state alphabet

template <int CM>
struct alignas(16) Stage {
    float4 p[2][CM][4];          // [child][category][row] of P(t), internal children
    float4 tip[2][CM][kCodes];   // [child][category][code] of the tip table, tip children
};

__host__ __device__ constexpr size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

template <int CM>
__device__ __forceinline__ void stage_op(Stage<CM>* st, const Op& op, int C, const float* __restrict__ P,
                                         const float* __restrict__ tipT) {
    const int n0 = (op.s0 >= 0) ? C * kCodes : C * 4;
    const int n1 = (op.s1 == kSrcNone) ? 0 : ((op.s1 >= 0) ? C * kCodes : C * 4);
    for (int i = threadIdx.x; i < n0 + n1; i += blockDim.x) {
        const int c = i < n0 ? 0 : 1;
        const int j = c ? i - n0 : i;
        const int src = c ? op.s1 : op.s0;
        const int e = c ? op.e1 : op.e0;
        if (src >= 0) {
            const int k = j / kCodes, code = j % kCodes;
            cp_async16(&st->tip[c][k][code], tipT + (((size_t)src * C + k) * kCodes + code) * 4);
        } else {
            const int k = j >> 2, row = j & 3;
            cp_async16(&st->p[c][k][row], P + ((size_t)e * C + k) * 16 + row * 4);
        }
    }
}

__device__ __forceinline__ void mv4(const float4* rows, const float x[4], float out[4]) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float4 r = rows[i];
        float acc = x[0] * r.x;
        acc = fmaf(x[1], r.y, acc);
        acc = fmaf(x[2], r.z, acc);
        acc = fmaf(x[3], r.w, acc);
        out[i] = acc;
    }
}

template <int CM, int SPT, bool CODES_SMEM>
__global__ void __launch_bounds__(kPruneThreads) prune4s_kernel(PruneArgs a) {
    constexpr int TILE = kPruneThreads * SPT;
    extern __shared__ __align__(16) unsigned char sm[];
    Stage<CM>* stages = reinterpret_cast<Stage<CM>*>(sm);
    size_t off = 3 * sizeof(Stage<CM>);
    Op* s_ops = reinterpret_cast<Op*>(sm + off);
    off += align16((size_t)a.n_ops * sizeof(Op));
    uint8_t* s_codes = sm + off;
    if (CODES_SMEM) off += align16((size_t)a.n_tips * TILE);
    float4* s_stack = reinterpret_cast<float4*>(sm + off);

    const int C = a.C;
    const int tid = threadIdx.x;
    const int tile_base = blockIdx.x * TILE;
    const float* __restrict__ P = static_cast<const float*>(a.P);
    const float* __restrict__ tipT = static_cast<const float*>(a.tipT);

    for (int i = tid; i < a.n_ops; i += kPruneThreads) s_ops[i] = a.ops[i];
    if (CODES_SMEM) {
        constexpr int chunks = TILE / 16;
        for (int i = tid; i < a.n_tips * chunks; i += kPruneThreads) {
            const int t = i / chunks, j = i % chunks, col = tile_base + 16 * j;
            uint8_t* dst = s_codes + (size_t)t * TILE + 16 * j;
            if (col < a.site_stride) cp_async16(dst, a.codes + (size_t)t * a.site_stride + col);
            else *reinterpret_cast<uint4*>(dst) = make_uint4(0u, 0u, 0u, 0u);
        }
    }
    __syncthreads();
    stage_op<CM>(&stages[0], s_ops[0], C, P, tipT);
    cp_async_commit();
    if (a.n_ops > 1) stage_op<CM>(&stages[1], s_ops[1], C, P, tipT);
    cp_async_commit();

    float acc[SPT][CM][4];
    int scale_e[SPT];
#pragma unroll
    for (int s = 0; s < SPT; ++s) {
        scale_e[s] = 0;
#pragma unroll
        for (int k = 0; k < CM; ++k)
#pragma unroll
            for (int i = 0; i < 4; ++i) acc[s][k][i] = 1.0f;
    }
    int sp = 0;

    for (int o = 0; o < a.n_ops; ++o) {
        cp_async_wait<1>();
        __syncthreads();
        if (o + 2 < a.n_ops) stage_op<CM>(&stages[(o + 2) % 3], s_ops[o + 2], C, P, tipT);
        cp_async_commit();
        const Op op = s_ops[o];
        const Stage<CM>& stg = stages[o % 3];
        if (op.s0 == kSrcPop) --sp;
#pragma unroll
        for (int s = 0; s < SPT; ++s) {
            const int lsite = tid + s * kPruneThreads;
            float d0[CM][4], d1[CM][4];
            if (op.s0 >= 0) {
                int code;
                if (CODES_SMEM) code = s_codes[(size_t)op.s0 * TILE + lsite];
                else code = a.codes[(size_t)op.s0 * a.site_stride + min(tile_base + lsite, a.site_stride - 1)];
                code &= kCodes - 1;
#pragma unroll
                for (int k = 0; k < CM; ++k)
                    if (k < C) {
                        const float4 t = stg.tip[0][k][code];
                        d0[k][0] = t.x; d0[k][1] = t.y; d0[k][2] = t.z; d0[k][3] = t.w;
                    }
            } else {
#pragma unroll
                for (int k = 0; k < CM; ++k)
                    if (k < C) {
                        float x[4];
                        if (op.s0 == kSrcPop) {
                            const float4 v = s_stack[((size_t)(sp * SPT + s) * CM + k) * kPruneThreads + tid];
                            x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
                        } else {
#pragma unroll
                            for (int i = 0; i < 4; ++i) x[i] = acc[s][k][i];
                        }
                        mv4(stg.p[0][k], x, d0[k]);
                    }
            }
            if (op.s1 >= 0) {
                int code;
                if (CODES_SMEM) code = s_codes[(size_t)op.s1 * TILE + lsite];
                else code = a.codes[(size_t)op.s1 * a.site_stride + min(tile_base + lsite, a.site_stride - 1)];
                code &= kCodes - 1;
#pragma unroll
                for (int k = 0; k < CM; ++k)
                    if (k < C) {
                        const float4 t = stg.tip[1][k][code];
                        d1[k][0] = t.x; d1[k][1] = t.y; d1[k][2] = t.z; d1[k][3] = t.w;
                    }
            } else if (op.s1 == kSrcAcc) {
#pragma unroll
                for (int k = 0; k < CM; ++k)
                    if (k < C) mv4(stg.p[1][k], acc[s][k], d1[k]);
            }
            if (op.s1 == kSrcNone) {
#pragma unroll
                for (int k = 0; k < CM; ++k)
#pragma unroll
                    for (int i = 0; i < 4; ++i) acc[s][k][i] = d0[k][i];
            } else {
#pragma unroll
                for (int k = 0; k < CM; ++k)
#pragma unroll
                    for (int i = 0; i < 4; ++i) acc[s][k][i] = d0[k][i] * d1[k][i];
            }
            float mx = 0.0f;
#pragma unroll
            for (int k = 0; k < CM; ++k)
                if (k < C)
#pragma unroll
                    for (int i = 0; i < 4; ++i) mx = fmaxf(mx, acc[s][k][i]);
            if (mx < scale_threshold<float>() && mx > 0.0f) {
                int e;
                float f1, f2;
                pow2_factors(mx, &e, &f1, &f2);
#pragma unroll
                for (int k = 0; k < CM; ++k)
#pragma unroll
                    for (int i = 0; i < 4; ++i) acc[s][k][i] = (acc[s][k][i] * f1) * f2;
                scale_e[s] += e;
            }
            if (op.push) {
#pragma unroll
                for (int k = 0; k < CM; ++k)
                    if (k < C)
                        s_stack[((size_t)(sp * SPT + s) * CM + k) * kPruneThreads + tid] =
                            make_float4(acc[s][k][0], acc[s][k][1], acc[s][k][2], acc[s][k][3]);
            }
        }
        if (op.push) ++sp;
    }
    cp_async_wait<0>();

    // root: sum_k w_k sum_s L[s] * root_w[s] in FP64, log, scaler exponents
    double tsum = 0.0, tcomp = 0.0;
#pragma unroll
    for (int s = 0; s < SPT; ++s) {
        const int site = tile_base + tid + s * kPruneThreads;
        double lsum = 0.0;
#pragma unroll
        for (int k = 0; k < CM; ++k)
            if (k < C) {
                double lk = (double)acc[s][k][0] * a.root_w[0];
#pragma unroll
                for (int i = 1; i < 4; ++i) lk = fma((double)acc[s][k][i], a.root_w[i], lk);
                lsum = fma(a.cat_w[k], lk, lsum);
            }
        if (site < a.n_sites) {
            const double lnl = log(lsum) + (double)scale_e[s] * 0.69314718055994530942;
            a.site_lnl[site] = lnl;
            double ns, e;
            two_sum(tsum, lnl, ns, e);
            tsum = ns;
            tcomp += e;
        }
    }
    block_sum_pair(tsum, tcomp);
    if (tid == 0) {
        a.block_sum[2 * blockIdx.x] = tsum;
        a.block_sum[2 * blockIdx.x + 1] = tcomp;
    }
}

template <int CM, int SPT, bool CODES_SMEM>
size_t prune4s_smem(const PruneArgs& a) {
    constexpr int TILE = kPruneThreads * SPT;
    size_t s = 3 * sizeof(Stage<CM>) + align16((size_t)a.n_ops * sizeof(Op));
    if (CODES_SMEM) s += align16((size_t)a.n_tips * TILE);
    s += (size_t)(a.max_depth > 0 ? a.max_depth : 1) * SPT * CM * sizeof(float4) * kPruneThreads;
    return s;
}

template <int CM, int SPT, bool CODES_SMEM>
cudaError_t launch_one(const PruneArgs& a, int* n_blocks, cudaStream_t st) {
    const size_t smem = prune4s_smem<CM, SPT, CODES_SMEM>(a);
    if (smem > 227 * 1024) return cudaErrorInvalidConfiguration;
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
    if (prune4s_smem<CM, SPT, true>(a) <= 160 * 1024) return launch_one<CM, SPT, true>(a, n_blocks, st);
    return launch_one<CM, SPT, false>(a, n_blocks, st);
}

}  // namespace

bool prune4s_fits(const PruneArgs& a, int spt) {
    const int cm = a.C == 1 ? 1 : (a.C <= 4 ? 4 : 8);
    size_t s;
    if (cm == 1) s = spt == 1 ? prune4s_smem<1, 1, false>(a) : prune4s_smem<1, 2, false>(a);
    else if (cm == 4) s = spt == 1 ? prune4s_smem<4, 1, false>(a) : prune4s_smem<4, 2, false>(a);
    else s = spt == 1 ? prune4s_smem<8, 1, false>(a) : prune4s_smem<8, 2, false>(a);
    return s <= 227 * 1024;
}

cudaError_t launch_prune4s(const PruneArgs& a, int spt, int* n_blocks, cudaStream_t st) {
    const int cm = a.C == 1 ? 1 : (a.C <= 4 ? 4 : 8);
    if (a.C > 8) return cudaErrorInvalidValue;
    if (cm == 1) return spt == 1 ? launch_cm_spt<1, 1>(a, n_blocks, st) : launch_cm_spt<1, 2>(a, n_blocks, st);
    if (cm == 4) return spt == 1 ? launch_cm_spt<4, 1>(a, n_blocks, st) : launch_cm_spt<4, 2>(a, n_blocks, st);
    return spt == 1 ? launch_cm_spt<8, 1>(a, n_blocks, st) : launch_cm_spt<8, 2>(a, n_blocks, st);
}

}  // namespace plk
