// Per-tile body of the paired-category 4-state FP32 post-order pass (see
// plk_prune4p.cu), shared by the single-tree and the batch kernels.
//
// The tile walks the op list like run_tile (plk_prune4s.cuh), but every value
// is a pair (category 2q, category 2q+1) held in one 64-bit register, so each
// product P(t) x v, child product and rescale is one fma.rn.f32x2 /
// mul.rn.f32x2 for two categories.  Every lane rounds exactly as the scalar
// fmaf / fmul of run_tile in the same order, so per-site results are the
// same bits.
//
// Paired layouts (one block of C x 16 floats per node, C x 64 per tip):
//   P:   [node][pair q][row j][state i][2]      (P_{2q}[i][j], P_{2q+1}[i][j])
//   tip: [tip][pair q][half][code][state i in the half][2]
// Each code's tip row sits in two 16-byte planes (states 0-1 and 2-3): with
// one 32-byte row per code, codes 4 and 8 (C and T) would share banks.
#pragma once

#include "plk_prune4s.cuh"

namespace plk {
namespace dev {

typedef unsigned long long u64;

__device__ __forceinline__ u64 fma2(u64 a, u64 b, u64 c) {
    u64 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;\n" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ u64 mul2(u64 a, u64 b) {
    u64 d;
    asm("mul.rn.f32x2 %0, %1, %2;\n" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ u64 pack2(float lo, float hi) {
    u64 r;
    asm("mov.b64 %0, {%1, %2};\n" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void unpack2(u64 v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;\n" : "=f"(lo), "=f"(hi) : "l"(v));
}

// Offset of P_k[i][j] inside a node's paired block.
__host__ __device__ inline int paired_p_index(int k, int i, int j) {
    return ((k >> 1) * 4 + j) * 8 + i * 2 + (k & 1);
}
// Offset of tip_k[code][i] inside a tip's paired block.
__host__ __device__ inline int paired_tip_index(int k, int code, int i) {
    return (((k >> 1) * 2 + (i >> 1)) * kCodes + code) * 4 + (i & 1) * 2 + (k & 1);
}

template <int KP>
struct alignas(16) StageP {
    u64 p[2][KP][4][4];             // [child][pair][row j][state i]
    u64 tip[2][KP][2][kCodes][2];   // [child][pair][half][code][state in the half]
};

// Sites of one tile: 128 SPT with one thread per site, 64 with two (TPS = 2:
// lanes 2i and 2i+1 take the first and the second half of site i's category
// pairs).
template <int SPT, int TPS>
__host__ __device__ constexpr int tile4p_sites() { return kPruneThreads * SPT / TPS; }

// Where the tip codes come from (CODES): 0 = global memory at their use, 1 =
// the tile's codes of every tip staged in shared memory at the start, 2 = an
// op's codes staged with its tables, two ops ahead, in a ring beside the stage
// slots (2 x TILE bytes per slot).
// Shared memory: three stage slots | ops | tip codes (CODES 1) or the code
// ring (CODES 2) | spill stack.  With CODES 2 and one site per thread the
// ops are read from global memory (L1-cached, the same address in every lane)
// instead of staged, which keeps the ring within the shared memory of the
// other one-site forms (six CTAs per SM on 128 x 100,000; 768 bytes more cost
// one of them); with two sites per thread the ops stay staged (the op loads
// would sit on the critical path of fewer warps).
template <int KP, int SPT, int CODES, int TPS = 1>
__host__ __device__ inline size_t tile4p_smem_bytes(int n_ops, int n_tips, int max_depth) {
    constexpr int TILE = tile4p_sites<SPT, TPS>();
    const size_t depth = (size_t)(max_depth > 0 ? max_depth : 1);
    constexpr bool ops_global = CODES == 2 && SPT == 1;
    size_t s = 3 * sizeof(StageP<KP>) + (ops_global ? 0 : align16((size_t)n_ops * sizeof(Op)));
    if (CODES == 1) s += align16((size_t)n_tips * TILE);
    if (CODES == 2) s += 3 * 2 * TILE;
    s += depth * SPT * (KP / TPS) * 4 * sizeof(u64) * kPruneThreads;
    return s;
}

inline size_t tile4p_smem_min(int C, int spt, int n_ops, int n_tips, int max_depth) {
    switch (C) {
        case 2: return spt == 1 ? tile4p_smem_bytes<1, 1, 0>(n_ops, n_tips, max_depth)
                                : tile4p_smem_bytes<1, 2, 0>(n_ops, n_tips, max_depth);
        case 4: return spt == 1 ? tile4p_smem_bytes<2, 1, 0>(n_ops, n_tips, max_depth)
                                : tile4p_smem_bytes<2, 2, 0>(n_ops, n_tips, max_depth);
        case 8: return spt == 1 ? tile4p_smem_bytes<4, 1, 0>(n_ops, n_tips, max_depth)
                                : tile4p_smem_bytes<4, 2, 0>(n_ops, n_tips, max_depth);
        default: return 0;
    }
}

template <int KP>
__device__ __forceinline__ void stage_op4p(StageP<KP>* st, const Op& op, const float* __restrict__ Pp,
                                           const float* __restrict__ Tp) {
    // 16-byte chunks: internal child KP * 8, tip child KP * 32
    const int n0 = (op.s0 >= 0) ? KP * 32 : KP * 8;
    const int n1 = (op.s1 == kSrcNone) ? 0 : ((op.s1 >= 0) ? KP * 32 : KP * 8);
    for (int i = threadIdx.x; i < n0 + n1; i += blockDim.x) {
        const int c = i < n0 ? 0 : 1;
        const int q = c ? i - n0 : i;
        const int src = c ? op.s1 : op.s0;
        if (src >= 0) {
            cp_async16(reinterpret_cast<float*>(st->tip[c]) + 4 * q, Tp + (size_t)src * KP * 128 + 4 * q);
        } else {
            const int e = c ? op.e1 : op.e0;
            cp_async16(reinterpret_cast<float*>(st->p[c]) + 4 * q, Pp + (size_t)e * KP * 32 + 4 * q);
        }
    }
}

// the op's tip codes of the tile's sites into a ring slot (CODES 2), issued
// by the last 2 TILE / 16 threads of the CTA as 16-byte cp.async; a chunk
// past the end of the code rows reads the rows' last chunk instead (those
// sites are beyond n_sites and never summed)
template <int TILE>
__device__ __forceinline__ void stage_codes4p(uint8_t* dst, const Op& op, const uint8_t* __restrict__ codes,
                                              int site_stride, int tile_base) {
    constexpr int CH = TILE / 16;
    static_assert(2 * CH <= kPruneThreads, "one chunk per thread");
    const int t = (int)threadIdx.x - (kPruneThreads - 2 * CH);
    if (t < 0) return;
    const int c = t / CH, q = t % CH;
    const int src = c ? op.s1 : op.s0;
    if (src < 0) return;
    const int col = min(tile_base + 16 * q, site_stride - 16);
    cp_async16(dst + c * TILE + 16 * q, codes + (size_t)src * site_stride + col);
}

// out[q][i] = sum_j P[q][j][i] x[q][j] for both categories of every pair,
// j ascending with the first term a product (the order of run_tile)
template <int KP>
__device__ __forceinline__ void mv4p(const u64 (*P)[4][4], const u64 x[KP][4], u64 out[KP][4]) {
#pragma unroll
    for (int q = 0; q < KP; ++q) {
        u64 r[4][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const ulonglong2 a = *reinterpret_cast<const ulonglong2*>(&P[q][j][0]);
            const ulonglong2 b = *reinterpret_cast<const ulonglong2*>(&P[q][j][2]);
            r[j][0] = a.x; r[j][1] = a.y; r[j][2] = b.x; r[j][3] = b.y;
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            u64 acc = mul2(x[q][0], r[0][i]);
            acc = fma2(x[q][1], r[1][i], acc);
            acc = fma2(x[q][2], r[2][i], acc);
            acc = fma2(x[q][3], r[3][i], acc);
            out[q][i] = acc;
        }
    }
}

template <int KP>
__device__ __forceinline__ void tip4p(const u64 (*T)[2][kCodes][2], int code, u64 out[KP][4]) {
#pragma unroll
    for (int q = 0; q < KP; ++q) {
        const ulonglong2 a = *reinterpret_cast<const ulonglong2*>(&T[q][0][code][0]);
        const ulonglong2 b = *reinterpret_cast<const ulonglong2*>(&T[q][1][code][0]);
        out[q][0] = a.x; out[q][1] = a.y; out[q][2] = b.x; out[q][3] = b.y;
    }
}

// One tile of sites of one tree with C = 2 KP categories (tile4p_sites);
// j.P and j.tipT are the tree's paired P(t) and tip blocks.  Adds this
// thread's site log-likelihoods to sum (the root and log of run_tile, same
// bits) and writes each site's value to j.site_lnl when it is not null.
// With TPS = 2 a site's pairs are split over two neighbouring lanes: they
// exchange their maxima for the rescale (both scale by the factors of the
// site's maximum, as one thread would) and the even lane adds up the root in
// category order with its partner's category sums, so the per-site results
// are the bits of TPS = 1.  Ends with no cp.async in flight; the caller must
// __syncthreads() before reusing the shared memory.
template <int KP, int SPT, int CODES, int TPS = 1>
__device__ void run_tile4p(const TileJob& j, unsigned char* sm, SiteSum32& sum) {
    static_assert(TPS == 1 || (TPS == 2 && SPT == 1 && KP % 2 == 0), "two threads per site split the pairs");
    constexpr int TILE = tile4p_sites<SPT, TPS>();
    constexpr int KPT = KP / TPS;  // pairs per thread
    StageP<KP>* stages = reinterpret_cast<StageP<KP>*>(sm);
    size_t off = 3 * sizeof(StageP<KP>);
    Op* s_ops = reinterpret_cast<Op*>(sm + off);
    constexpr bool ops_global = CODES == 2 && SPT == 1;
    if (!ops_global) off += align16((size_t)j.n_ops * sizeof(Op));
    const Op* __restrict__ ops = ops_global ? j.ops : s_ops;
    uint8_t* s_codes = sm + off;
    if (CODES == 1) off += align16((size_t)j.n_tips * TILE);
    if (CODES == 2) off += 3 * 2 * TILE;
    ulonglong2* s_stack = reinterpret_cast<ulonglong2*>(sm + off);
    const float* __restrict__ Pp = j.P;
    const float* __restrict__ Tp = j.tipT;

    const int tid = threadIdx.x;
    const int half = TPS == 2 ? (tid & 1) : 0;   // which half of the pairs
    const int q0 = half * KPT;                    // first pair of this thread
    if (!ops_global)
        for (int i = tid; i < j.n_ops; i += kPruneThreads) s_ops[i] = j.ops[i];
    if (CODES == 1) {
        constexpr int chunks = TILE / 16;
        for (int i = tid; i < j.n_tips * chunks; i += kPruneThreads) {
            const int t = i / chunks, q = i % chunks, col = j.tile_base + 16 * q;
            uint8_t* dst = s_codes + (size_t)t * TILE + 16 * q;
            if (col < j.site_stride) cp_async16(dst, j.codes + (size_t)t * j.site_stride + col);
            else *reinterpret_cast<uint4*>(dst) = make_uint4(0u, 0u, 0u, 0u);
        }
    }
    __syncthreads();
    stage_op4p<KP>(&stages[0], ops[0], Pp, Tp);
    if (CODES == 2) stage_codes4p<TILE>(s_codes, ops[0], j.codes, j.site_stride, j.tile_base);
    cp_async_commit();
    if (j.n_ops > 1) {
        stage_op4p<KP>(&stages[1], ops[1], Pp, Tp);
        if (CODES == 2) stage_codes4p<TILE>(s_codes + 2 * TILE, ops[1], j.codes, j.site_stride, j.tile_base);
    }
    cp_async_commit();

    u64 acc[SPT][KPT][4];
    int scale_e[SPT];
    const u64 one2 = pack2(1.0f, 1.0f);
#pragma unroll
    for (int s = 0; s < SPT; ++s) {
        scale_e[s] = 0;
#pragma unroll
        for (int q = 0; q < KPT; ++q)
#pragma unroll
            for (int i = 0; i < 4; ++i) acc[s][q][i] = one2;
    }
    int sp = 0;

    // (with CODES 0 the tip codes are read from global memory at their use:
    // loading them into registers an op ahead, or before the op's barrier,
    // measured slower for this body on the 128 x 100,000 benchmark; CODES 2
    // stages them with the op instead)
    for (int o = 0; o < j.n_ops; ++o) {
        // this op and the one to stage, loaded before the wait and the
        // barrier so that their latency (L1 when the ops are not staged)
        // hides behind them
        const Op op = ops[o];
        Op nx{};
        if (o + 2 < j.n_ops) nx = ops[o + 2];
        cp_async_wait<1>();
        __syncthreads();
        if (o + 2 < j.n_ops) {
            stage_op4p<KP>(&stages[(o + 2) % 3], nx, Pp, Tp);
            if (CODES == 2)
                stage_codes4p<TILE>(s_codes + ((o + 2) % 3) * 2 * TILE, nx, j.codes, j.site_stride,
                                    j.tile_base);
        }
        cp_async_commit();
        const StageP<KP>& stg = stages[o % 3];
        const uint8_t* ring = s_codes + (o % 3) * 2 * TILE;  // CODES 2: this op's codes
        if (op.s0 == kSrcPop) --sp;
#pragma unroll
        for (int s = 0; s < SPT; ++s) {
            const int lsite = TPS == 1 ? tid + s * kPruneThreads : (tid >> 1);
            u64 d0[KPT][4], d1[KPT][4];
            if (op.s0 >= 0) {
                int code;
                if (CODES == 1) code = s_codes[(size_t)op.s0 * TILE + lsite];
                else if (CODES == 2) code = ring[lsite];
                else code = j.codes[(size_t)op.s0 * j.site_stride + min(j.tile_base + lsite, j.site_stride - 1)];
                tip4p<KPT>(stg.tip[0] + q0, code & (kCodes - 1), d0);
            } else if (op.s0 == kSrcPop) {
                u64 x[KPT][4];
#pragma unroll
                for (int q = 0; q < KPT; ++q)
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const ulonglong2 v = s_stack[((size_t)((sp * SPT + s) * KPT + q) * 2 + h) * kPruneThreads + tid];
                        x[q][2 * h] = v.x;
                        x[q][2 * h + 1] = v.y;
                    }
                mv4p<KPT>(stg.p[0] + q0, x, d0);
            } else {
                mv4p<KPT>(stg.p[0] + q0, acc[s], d0);
            }
            if (op.s1 >= 0) {
                int code;
                if (CODES == 1) code = s_codes[(size_t)op.s1 * TILE + lsite];
                else if (CODES == 2) code = ring[TILE + lsite];
                else code = j.codes[(size_t)op.s1 * j.site_stride + min(j.tile_base + lsite, j.site_stride - 1)];
                tip4p<KPT>(stg.tip[1] + q0, code & (kCodes - 1), d1);
            } else if (op.s1 == kSrcAcc) {
                mv4p<KPT>(stg.p[1] + q0, acc[s], d1);
            }
            if (op.s1 == kSrcNone) {
#pragma unroll
                for (int q = 0; q < KPT; ++q)
#pragma unroll
                    for (int i = 0; i < 4; ++i) acc[s][q][i] = d0[q][i];
            } else {
#pragma unroll
                for (int q = 0; q < KPT; ++q)
#pragma unroll
                    for (int i = 0; i < 4; ++i) acc[s][q][i] = mul2(d0[q][i], d1[q][i]);
            }
            float mx = 0.0f;
#pragma unroll
            for (int q = 0; q < KPT; ++q)
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    float lo, hi;
                    unpack2(acc[s][q][i], lo, hi);
                    mx = fmaxf(mx, fmaxf(lo, hi));
                }
            if constexpr (TPS == 2) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
            if (mx < scale_threshold<float>() && mx > 0.0f) {
                int e;
                float f1, f2;
                pow2_factors(mx, &e, &f1, &f2);
                const u64 g1 = pack2(f1, f1), g2 = pack2(f2, f2);
#pragma unroll
                for (int q = 0; q < KPT; ++q)
#pragma unroll
                    for (int i = 0; i < 4; ++i) acc[s][q][i] = mul2(mul2(acc[s][q][i], g1), g2);
                scale_e[s] += e;
            }
            if (op.push) {
#pragma unroll
                for (int q = 0; q < KPT; ++q)
#pragma unroll
                    for (int h = 0; h < 2; ++h)
                        s_stack[((size_t)((sp * SPT + s) * KPT + q) * 2 + h) * kPruneThreads + tid] =
                            make_ulonglong2(acc[s][q][2 * h], acc[s][q][2 * h + 1]);
            }
        }
        if (op.push) ++sp;
    }
    cp_async_wait<0>();

    // root: L = sum_k w_k sum_s v_k[s] root_w[s] in FP32 (categories in
    // order, as run_tile), log L = lm + ee ln 2
    float rw[4], cw[2 * KP];
#pragma unroll
    for (int i = 0; i < 4; ++i) rw[i] = (float)j.root_w[i];
#pragma unroll
    for (int k = 0; k < 2 * KP; ++k) cw[k] = (float)j.cat_w[k];
#pragma unroll
    for (int s = 0; s < SPT; ++s) {
        const int lsite = TPS == 1 ? tid + s * kPruneThreads : (tid >> 1);
        const int site = j.tile_base + lsite;
        float lk[2 * KP];  // sum_s v_k[s] root_w[s] of every category
#pragma unroll
        for (int q = 0; q < KPT; ++q) {
            float v[2][4];
#pragma unroll
            for (int i = 0; i < 4; ++i) unpack2(acc[s][q][i], v[0][i], v[1][i]);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                float x = v[h][0] * rw[0];
#pragma unroll
                for (int i = 1; i < 4; ++i) x = fmaf(v[h][i], rw[i], x);
                lk[2 * q + h] = x;
            }
        }
        if constexpr (TPS == 2) {
            // the even lane holds categories 0 .. 2 KPT - 1, its partner the rest
#pragma unroll
            for (int k = 0; k < 2 * KPT; ++k) lk[2 * KPT + k] = __shfl_xor_sync(0xffffffffu, lk[k], 1);
        }
        float lsum = 0.0f;
#pragma unroll
        for (int k = 0; k < 2 * KP; ++k) lsum = fmaf(cw[k], lk[k], lsum);
        if (site < j.n_sites && half == 0) {
            float lm;
            int ee;
            site_log32(lsum, scale_e[s], lm, ee);
            if (j.site_lnl) j.site_lnl[site] = site_lnl64(lm, ee);
            site_sum_add(sum, lm, ee);
        }
    }
}

// ---------------------------------------------------------------------------
// The same tile body with the stage ring fed by TMA: one thread issues 1-D
// bulk copies (cp.async.bulk, completion counted in bytes on the slot's
// "full" mbarrier) three ops ahead, and every warp releases a slot through
// its "empty" mbarrier once it has read it, so no CTA-wide barrier stands
// between ops.  One site per thread, tip codes from global memory, the
// arithmetic of run_tile4p (same bits).  Every wait is bounded; a wait that
// runs out sets *abort and the tile's sites come out NaN.
// ---------------------------------------------------------------------------
constexpr int kBulkWaitLimit = 1 << 20;  // try_wait rounds (each may suspend briefly); a copy lands in microseconds

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool mbar_try_wait_bounded(uint32_t mbar, uint32_t parity) {
    for (int i = 0; i < kBulkWaitLimit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// bytes one op stages: each child's tip table or P(t) rows
template <int KP>
__device__ __forceinline__ uint32_t bulk_op_bytes(const Op& op) {
    const uint32_t tip = KP * 128 * 4, p = KP * 32 * 4;
    uint32_t b = op.s0 >= 0 ? tip : p;
    if (op.s1 != kSrcNone) b += op.s1 >= 0 ? tip : p;
    return b;
}

// issued by one thread: the op's data into a stage slot, completing on full
template <int KP>
__device__ __forceinline__ void bulk_stage_op(StageP<KP>* st, const Op& op, const float* __restrict__ Pp,
                                              const float* __restrict__ Tp, uint32_t full) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(full), "r"(bulk_op_bytes<KP>(op))
                 : "memory");
    for (int c = 0; c < 2; ++c) {
        const int src = c ? op.s1 : op.s0;
        if (src == kSrcNone) continue;
        const void* from;
        void* to;
        uint32_t bytes;
        if (src >= 0) {
            from = Tp + (size_t)src * KP * 128;
            to = st->tip[c];
            bytes = KP * 128 * 4;
        } else {
            from = Pp + (size_t)(c ? op.e1 : op.e0) * KP * 32;
            to = st->p[c];
            bytes = KP * 32 * 4;
        }
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                smem_addr(to)),
            "l"(from), "r"(bytes), "r"(full)
            : "memory");
    }
}

// Shared memory: three stage slots | ops | spill stack (the mbarriers are
// static shared memory of the kernel).
template <int KP>
__host__ __device__ inline size_t tile4p_bulk_smem_bytes(int n_ops, int max_depth) {
    const size_t depth = (size_t)(max_depth > 0 ? max_depth : 1);
    return 3 * sizeof(StageP<KP>) + align16((size_t)n_ops * sizeof(Op)) + depth * KP * 4 * sizeof(u64) * kPruneThreads;
}

// bars: 6 mbarriers (full[3], empty[3]) initialised by the caller before
// its first __syncthreads: full with 1 arrival, empty with one per warp.
// withhold_first (a test of the failure path): the producer never stages op
// 0, so every wait for it runs out.
template <int KP>
__device__ void run_tile4p_bulk(const TileJob& j, unsigned char* sm, uint64_t* bars, int* abort, SiteSum32& sum,
                                bool withhold_first = false) {
    StageP<KP>* stages = reinterpret_cast<StageP<KP>*>(sm);
    size_t off = 3 * sizeof(StageP<KP>);
    Op* s_ops = reinterpret_cast<Op*>(sm + off);
    off += align16((size_t)j.n_ops * sizeof(Op));
    ulonglong2* s_stack = reinterpret_cast<ulonglong2*>(sm + off);
    const float* __restrict__ Pp = j.P;
    const float* __restrict__ Tp = j.tipT;
    const int tid = threadIdx.x, lane = tid & 31;
    const uint32_t bar0 = smem_addr(bars);  // full[q] at bar0 + 8 q, empty[q] at bar0 + 24 + 8 q
    for (int i = tid; i < j.n_ops; i += kPruneThreads) s_ops[i] = j.ops[i];
    __syncthreads();
    // the producer (thread 0) tracks the staged ops [seen, issued) whose
    // completion it has not observed yet
    int issued = 0, seen = 0;
    if (tid == 0) {
        for (int o = 0; o < 3 && o < j.n_ops; ++o)
            if (!(withhold_first && o == 0)) bulk_stage_op<KP>(&stages[o], s_ops[o], Pp, Tp, bar0 + 8 * o);
        issued = j.n_ops < 3 ? j.n_ops : 3;
    }

    u64 acc[KP][4];
    int scale_e = 0;
    const u64 one2 = pack2(1.0f, 1.0f);
#pragma unroll
    for (int q = 0; q < KP; ++q)
#pragma unroll
        for (int i = 0; i < 4; ++i) acc[q][i] = one2;
    int sp = 0;
    const int lsite = tid;
    for (int o = 0; o < j.n_ops; ++o) {
        const int slot = o % 3;
        const uint32_t parity = (uint32_t)(o / 3) & 1u;
        const uint32_t full = bar0 + 8 * slot, empty = bar0 + 24 + 8 * slot;
        if (*reinterpret_cast<volatile int*>(abort)) break;
        if (!mbar_try_wait_bounded(full, parity)) {
            *reinterpret_cast<volatile int*>(abort) = 1;
            break;
        }
        seen = o + 1;
        const Op op = s_ops[o];
        const StageP<KP>& stg = stages[slot];
        if (op.s0 == kSrcPop) --sp;
        u64 d0[KP][4], d1[KP][4];
        if (op.s0 >= 0) {
            const int code = j.codes[(size_t)op.s0 * j.site_stride + min(j.tile_base + lsite, j.site_stride - 1)];
            tip4p<KP>(stg.tip[0], code & (kCodes - 1), d0);
        } else if (op.s0 == kSrcPop) {
            u64 x[KP][4];
#pragma unroll
            for (int q = 0; q < KP; ++q)
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const ulonglong2 v = s_stack[((size_t)(sp * KP + q) * 2 + h) * kPruneThreads + tid];
                    x[q][2 * h] = v.x;
                    x[q][2 * h + 1] = v.y;
                }
            mv4p<KP>(stg.p[0], x, d0);
        } else {
            mv4p<KP>(stg.p[0], acc, d0);
        }
        if (op.s1 >= 0) {
            const int code = j.codes[(size_t)op.s1 * j.site_stride + min(j.tile_base + lsite, j.site_stride - 1)];
            tip4p<KP>(stg.tip[1], code & (kCodes - 1), d1);
        } else if (op.s1 == kSrcAcc) {
            mv4p<KP>(stg.p[1], acc, d1);
        }
        // the slot is read: release it (one arrival per warp)
        __syncwarp();
        if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(empty) : "memory");
        // the producer refills it with op o + 3 once every warp has let go
        if (tid == 0 && o + 3 < j.n_ops) {
            if (mbar_try_wait_bounded(empty, parity)) {
                bulk_stage_op<KP>(&stages[slot], s_ops[o + 3], Pp, Tp, full);
                issued = o + 4;
            } else {
                *reinterpret_cast<volatile int*>(abort) = 1;
            }
        }
        if (op.s1 == kSrcNone) {
#pragma unroll
            for (int q = 0; q < KP; ++q)
#pragma unroll
                for (int i = 0; i < 4; ++i) acc[q][i] = d0[q][i];
        } else {
#pragma unroll
            for (int q = 0; q < KP; ++q)
#pragma unroll
                for (int i = 0; i < 4; ++i) acc[q][i] = mul2(d0[q][i], d1[q][i]);
        }
        float mx = 0.0f;
#pragma unroll
        for (int q = 0; q < KP; ++q)
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                float lo, hi;
                unpack2(acc[q][i], lo, hi);
                mx = fmaxf(mx, fmaxf(lo, hi));
            }
        if (mx < scale_threshold<float>() && mx > 0.0f) {
            int e;
            float f1, f2;
            pow2_factors(mx, &e, &f1, &f2);
            const u64 g1 = pack2(f1, f1), g2 = pack2(f2, f2);
#pragma unroll
            for (int q = 0; q < KP; ++q)
#pragma unroll
                for (int i = 0; i < 4; ++i) acc[q][i] = mul2(mul2(acc[q][i], g1), g2);
            scale_e += e;
        }
        if (op.push) {
#pragma unroll
            for (int q = 0; q < KP; ++q)
#pragma unroll
                for (int h = 0; h < 2; ++h)
                    s_stack[((size_t)(sp * KP + q) * 2 + h) * kPruneThreads + tid] =
                        make_ulonglong2(acc[q][2 * h], acc[q][2 * h + 1]);
            ++sp;
        }
    }
    // every issued copy was waited for by the consumers unless a wait ran out;
    // then the producer gives the copies it issued and has not seen land a
    // bounded chance to, before the CTA's shared memory goes
    __syncthreads();
    if (*reinterpret_cast<volatile int*>(abort) && tid == 0) {
        for (int o = seen; o < issued; ++o)
            if (!(withhold_first && o == 0))
                if (!mbar_try_wait_bounded(bar0 + 8 * (o % 3), (uint32_t)(o / 3) & 1u)) break;
    }

    // root: as run_tile4p
    float rw[4], cw[2 * KP];
#pragma unroll
    for (int i = 0; i < 4; ++i) rw[i] = (float)j.root_w[i];
#pragma unroll
    for (int k = 0; k < 2 * KP; ++k) cw[k] = (float)j.cat_w[k];
    const int site = j.tile_base + lsite;
    float lk[2 * KP];
#pragma unroll
    for (int q = 0; q < KP; ++q) {
        float v[2][4];
#pragma unroll
        for (int i = 0; i < 4; ++i) unpack2(acc[q][i], v[0][i], v[1][i]);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            float x = v[h][0] * rw[0];
#pragma unroll
            for (int i = 1; i < 4; ++i) x = fmaf(v[h][i], rw[i], x);
            lk[2 * q + h] = x;
        }
    }
    float lsum = 0.0f;
#pragma unroll
    for (int k = 0; k < 2 * KP; ++k) lsum = fmaf(cw[k], lk[k], lsum);
    if (*reinterpret_cast<volatile int*>(abort)) lsum = __int_as_float(0x7fc00000);
    if (site < j.n_sites) {
        float lm;
        int ee;
        site_log32(lsum, scale_e, lm, ee);
        if (j.site_lnl) j.site_lnl[site] = site_lnl64(lm, ee);
        site_sum_add(sum, lm, ee);
    }
}

}  // namespace dev
}  // namespace plk
