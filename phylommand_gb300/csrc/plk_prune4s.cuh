// Per-tile body of the staged 4-state FP32 post-order pass (see
// plk_prune4s.cu), shared by the single-tree and the batch kernels.
#pragma once

#include "plk_device.cuh"
#include "plk_internal.h"

namespace plk {
namespace dev {

constexpr int kCodes = 16;                      // state sets of a <= 4-state alphabet
constexpr size_t kMaxSmem = 227 * 1024;         // dynamic shared memory per CTA
constexpr size_t kCodesSmemBudget = 160 * 1024; // stage tip codes only below this

template <int CM>
struct alignas(16) Stage {
    float4 p[2][CM][4];          // [child][category][row] of P(t), internal children
    float4 tip[2][CM][kCodes];   // [child][category][code] of the tip table, tip children
};

__host__ __device__ constexpr size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

// One site tile of one tree.
struct TileJob {
    const Op* ops;
    int n_ops;
    const uint8_t* codes;   // [n_tips][site_stride]
    int site_stride;
    int n_sites;
    int n_tips;
    const float* P;         // [n_nodes][C][16]
    const float* tipT;      // [n_tips][C][16][4]
    const double* root_w;   // [4]
    const double* cat_w;    // [C]
    int C;
    int tile_base;          // first site of the tile
    double* site_lnl;       // [n_sites] or null
    int max_depth;          // spill-stack depth (read only with STORE_D)
};

// Where a STORE_D tile leaves the message each internal non-root node sends
// to its parent (D = P(t) x conditional vector, FP32, scaled) and its
// power-of-two exponent: D[(rank * C + k) * TILE + site], ED[rank * TILE + site].
// Requires internal nodes numbered n_tips + post-order rank.
struct DStore {
    float4* D;
    int* ED;
};

// Shared memory: three stage slots | ops | tip codes (optional) | spill stack
// | spill-stack exponents (STORE_D only).
template <int CM, int SPT, bool CODES_SMEM, bool STORE_D = false>
__host__ __device__ inline size_t tile_smem_bytes(int n_ops, int n_tips, int max_depth) {
    constexpr int TILE = kPruneThreads * SPT;
    const size_t depth = (size_t)(max_depth > 0 ? max_depth : 1);
    size_t s = 3 * sizeof(Stage<CM>) + align16((size_t)n_ops * sizeof(Op));
    if (CODES_SMEM) s += align16((size_t)n_tips * TILE);
    s += depth * SPT * CM * 16 * kPruneThreads;
    if (STORE_D) s += depth * SPT * sizeof(int) * kPruneThreads;
    return s;
}

inline size_t tile_smem_min(int C, int spt, int n_ops, int n_tips, int max_depth) {
    const int cm = C == 1 ? 1 : (C <= 4 ? 4 : 8);
    if (cm == 1) return spt == 1 ? tile_smem_bytes<1, 1, false>(n_ops, n_tips, max_depth)
                                 : tile_smem_bytes<1, 2, false>(n_ops, n_tips, max_depth);
    if (cm == 4) return spt == 1 ? tile_smem_bytes<4, 1, false>(n_ops, n_tips, max_depth)
                                 : tile_smem_bytes<4, 2, false>(n_ops, n_tips, max_depth);
    return spt == 1 ? tile_smem_bytes<8, 1, false>(n_ops, n_tips, max_depth)
                    : tile_smem_bytes<8, 2, false>(n_ops, n_tips, max_depth);
}

template <int CM>
__device__ __forceinline__ void stage_op(Stage<CM>* st, const Op& op, int C, const float* __restrict__ P,
                                         const float* __restrict__ tipT) {
    // every child's tip table ([category][code]) or P rows ([category][row])
    // is one contiguous run of 16-byte chunks in global and in the stage slot
    const int n0 = (op.s0 >= 0) ? C * kCodes : C * 4;
    const int n1 = (op.s1 == kSrcNone) ? 0 : ((op.s1 >= 0) ? C * kCodes : C * 4);
    const float4* src0 = reinterpret_cast<const float4*>(op.s0 >= 0 ? tipT + (size_t)op.s0 * C * kCodes * 4
                                                                    : P + (size_t)op.e0 * C * 16);
    float4* dst0 = op.s0 >= 0 ? &st->tip[0][0][0] : &st->p[0][0][0];
    for (int i = threadIdx.x; i < n0; i += blockDim.x) cp_async16(dst0 + i, src0 + i);
    if (n1) {
        const float4* src1 = reinterpret_cast<const float4*>(op.s1 >= 0 ? tipT + (size_t)op.s1 * C * kCodes * 4
                                                                        : P + (size_t)op.e1 * C * 16);
        float4* dst1 = op.s1 >= 0 ? &st->tip[1][0][0] : &st->p[1][0][0];
        for (int i = threadIdx.x; i < n1; i += blockDim.x) cp_async16(dst1 + i, src1 + i);
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

// Tip codes of an op's children at this thread's SPT sites, read from global
// memory (0 where a child is no tip).  The tile bodies load them one op ahead
// of their use, so that the L2 latency hides behind an op's work.
template <int SPT>
__device__ __forceinline__ void load_op_codes(const TileJob& j, const Op& op, int tid, int (&c0)[SPT],
                                              int (&c1)[SPT]) {
#pragma unroll
    for (int s = 0; s < SPT; ++s) {
        const int col = min(j.tile_base + tid + s * kPruneThreads, j.site_stride - 1);
        c0[s] = op.s0 >= 0 ? (int)__ldg(j.codes + (size_t)op.s0 * j.site_stride + col) : 0;
        c1[s] = op.s1 >= 0 ? (int)__ldg(j.codes + (size_t)op.s1 * j.site_stride + col) : 0;
    }
}

// Runs one tile; every thread of the CTA must call it.  Adds this thread's
// site log-likelihoods to sum (site_log32: FP32 root, FP32 TwoSum) and
// writes them to j.site_lnl when it is not null.  Ends with no cp.async in flight; the
// caller must __syncthreads() before reusing the shared memory.  With
// STORE_D, writes instead the message every internal child sends to its
// parent (and its exponent) to *ds, tracking the per-node exponents, and
// skips the root (sum stays untouched).
template <int CM, int SPT, bool CODES_SMEM, bool STORE_D = false>
__device__ void run_tile(const TileJob& j, unsigned char* sm, SiteSum32& sum, const DStore* ds = nullptr) {
    constexpr int TILE = kPruneThreads * SPT;
    Stage<CM>* stages = reinterpret_cast<Stage<CM>*>(sm);
    size_t off = 3 * sizeof(Stage<CM>);
    Op* s_ops = reinterpret_cast<Op*>(sm + off);
    off += align16((size_t)j.n_ops * sizeof(Op));
    uint8_t* s_codes = sm + off;
    if (CODES_SMEM) off += align16((size_t)j.n_tips * TILE);
    float4* s_stack = reinterpret_cast<float4*>(sm + off);
    int* s_stack_e = nullptr;
    if (STORE_D)
        s_stack_e = reinterpret_cast<int*>(sm + off + (size_t)(j.max_depth > 0 ? j.max_depth : 1) * SPT * CM * 16 *
                                                          kPruneThreads);
    int acc_e[SPT];
#pragma unroll
    for (int s = 0; s < SPT; ++s) acc_e[s] = 0;

    const int C = j.C;
    const int tid = threadIdx.x;
    const float* __restrict__ P = j.P;
    const float* __restrict__ tipT = j.tipT;

    for (int i = tid; i < j.n_ops; i += kPruneThreads) s_ops[i] = j.ops[i];
    if (CODES_SMEM) {
        constexpr int chunks = TILE / 16;
        for (int i = tid; i < j.n_tips * chunks; i += kPruneThreads) {
            const int t = i / chunks, q = i % chunks, col = j.tile_base + 16 * q;
            uint8_t* dst = s_codes + (size_t)t * TILE + 16 * q;
            if (col < j.site_stride) cp_async16(dst, j.codes + (size_t)t * j.site_stride + col);
            else *reinterpret_cast<uint4*>(dst) = make_uint4(0u, 0u, 0u, 0u);
        }
    }
    __syncthreads();
    stage_op<CM>(&stages[0], s_ops[0], C, P, tipT);
    cp_async_commit();
    if (j.n_ops > 1) stage_op<CM>(&stages[1], s_ops[1], C, P, tipT);
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
    int pc0[SPT], pc1[SPT];  // tip codes of op o when they are read from global memory
    if constexpr (!CODES_SMEM) load_op_codes<SPT>(j, s_ops[0], tid, pc0, pc1);

    for (int o = 0; o < j.n_ops; ++o) {
        cp_async_wait<1>();
        __syncthreads();
        if (o + 2 < j.n_ops) stage_op<CM>(&stages[(o + 2) % 3], s_ops[o + 2], C, P, tipT);
        cp_async_commit();
        const Op op = s_ops[o];
        int nc0[SPT] = {}, nc1[SPT] = {};
        if constexpr (!CODES_SMEM)
            if (o + 1 < j.n_ops) load_op_codes<SPT>(j, s_ops[o + 1], tid, nc0, nc1);
        const Stage<CM>& stg = stages[o % 3];
        if (op.s0 == kSrcPop) --sp;
#pragma unroll
        for (int s = 0; s < SPT; ++s) {
            const int lsite = tid + s * kPruneThreads;
            float d0[CM][4], d1[CM][4];
            int e_ch0 = 0, e_ch1 = 0;  // exponents of the two child vectors (STORE_D)
            if constexpr (STORE_D) {
                if (op.s0 == kSrcPop) e_ch0 = s_stack_e[(sp * SPT + s) * kPruneThreads + tid];
                else if (op.s0 == kSrcAcc) e_ch0 = acc_e[s];
                if (op.s1 == kSrcAcc) e_ch1 = acc_e[s];
            }
            if (op.s0 >= 0) {
                int code;
                if (CODES_SMEM) code = s_codes[(size_t)op.s0 * TILE + lsite];
                else code = pc0[s];
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
                else code = pc1[s];
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
            if constexpr (STORE_D) {
                // messages of internal children to this node, for the pre-order
                // and NNI phases
                if (op.s0 < 0) {
                    const int r = op.e0 - j.n_tips;
#pragma unroll
                    for (int k = 0; k < CM; ++k)
                        if (k < C) ds->D[((size_t)r * C + k) * TILE + lsite] = make_float4(d0[k][0], d0[k][1], d0[k][2], d0[k][3]);
                    ds->ED[(size_t)r * TILE + lsite] = e_ch0;
                }
                if (op.s1 == kSrcAcc) {
                    const int r = op.e1 - j.n_tips;
#pragma unroll
                    for (int k = 0; k < CM; ++k)
                        if (k < C) ds->D[((size_t)r * C + k) * TILE + lsite] = make_float4(d1[k][0], d1[k][1], d1[k][2], d1[k][3]);
                    ds->ED[(size_t)r * TILE + lsite] = e_ch1;
                }
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
            int e_node = 0;
            if (mx < scale_threshold<float>() && mx > 0.0f) {
                int e;
                float f1, f2;
                pow2_factors(mx, &e, &f1, &f2);
#pragma unroll
                for (int k = 0; k < CM; ++k)
#pragma unroll
                    for (int i = 0; i < 4; ++i) acc[s][k][i] = (acc[s][k][i] * f1) * f2;
                scale_e[s] += e;
                e_node = e;
            }
            if constexpr (STORE_D) acc_e[s] = e_ch0 + e_ch1 + e_node;
            if (op.push) {
#pragma unroll
                for (int k = 0; k < CM; ++k)
                    if (k < C)
                        s_stack[((size_t)(sp * SPT + s) * CM + k) * kPruneThreads + tid] =
                            make_float4(acc[s][k][0], acc[s][k][1], acc[s][k][2], acc[s][k][3]);
                if constexpr (STORE_D) s_stack_e[(sp * SPT + s) * kPruneThreads + tid] = acc_e[s];
            }
        }
        if (op.push) ++sp;
        if constexpr (!CODES_SMEM) {
#pragma unroll
            for (int s = 0; s < SPT; ++s) {
                pc0[s] = nc0[s];
                pc1[s] = nc1[s];
            }
        }
    }
    cp_async_wait<0>();
    if constexpr (STORE_D) return;

    // root: L = sum_k w_k sum_s v_k[s] root_w[s] in FP32, log L = lm + ee ln 2
    float rw[4], cw[CM];
#pragma unroll
    for (int i = 0; i < 4; ++i) rw[i] = (float)j.root_w[i];
#pragma unroll
    for (int k = 0; k < CM; ++k) cw[k] = k < C ? (float)j.cat_w[k] : 0.0f;
#pragma unroll
    for (int s = 0; s < SPT; ++s) {
        const int site = j.tile_base + tid + s * kPruneThreads;
        float lsum = 0.0f;
#pragma unroll
        for (int k = 0; k < CM; ++k)
            if (k < C) {
                float lk = acc[s][k][0] * rw[0];
#pragma unroll
                for (int i = 1; i < 4; ++i) lk = fmaf(acc[s][k][i], rw[i], lk);
                lsum = fmaf(cw[k], lk, lsum);
            }
        if (site < j.n_sites) {
            float lm;
            int ee;
            site_log32(lsum, scale_e[s], lm, ee);
            if (j.site_lnl) j.site_lnl[site] = site_lnl64(lm, ee);
            site_sum_add(sum, lm, ee);
        }
    }
}

}  // namespace dev
}  // namespace plk
