// prune4p: the staged 4-state FP32 post-order pass (src/simpleML.cpp:127-197)
// with the rate categories taken in pairs on Blackwell's packed FP32x2 pipe.
//
// Same structure as prune4s (plk_prune4s.cu): a CTA walks the op list over a
// tile of 128 x SPT sites, op o+2's P(t) rows and tip tables travel into a
// three-slot shared-memory ring by cp.async while op o computes, spilled
// vectors sit in a per-thread shared-memory stack.  The difference is the
// register layout: every value is a pair (category 2q, category 2q+1), so
// each product P(t) x v, each child product and each rescale is one
// fma.rn.f32x2 / mul.rn.f32x2 for two categories.  Every lane rounds exactly
// as the scalar fmaf / fmul of prune4s in the same order, so the per-site
// results are the same bits.  The number of categories is a compile-time
// constant (2, 4 or 8), so no category loop carries a guard.
//
// The P(t) and tip tables are read in a paired layout that relayout4p_kernel
// writes from the FP32 copies of the P(t) kernel:
//   P:   [node][pair q][row j][state i][2]      (P_{2q}[i][j], P_{2q+1}[i][j])
//   tip: [tip][pair q][half][code][state i in the half][2]
// (each code's row in two 16-byte planes, states 0-1 and 2-3: a 32-byte
// stride per code would put codes 4 and 8, C and T, on the same banks)
#include "plk_device.cuh"
#include "plk_internal.h"

namespace plk {
using namespace dev;

namespace {

constexpr int kCodes4 = 16;
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

template <int KP>
struct alignas(16) StageP {
    u64 p[2][KP][4][4];          // [child][pair][row j][state i]
    u64 tip[2][KP][2][kCodes4][2];  // [child][pair][half][code][state in the half]
};

template <int KP, int SPT, bool CODES_SMEM>
__host__ __device__ inline size_t smem4p_bytes(int n_ops, int n_tips, int max_depth) {
    constexpr int TILE = kPruneThreads * SPT;
    const size_t depth = (size_t)(max_depth > 0 ? max_depth : 1);
    size_t s = 3 * sizeof(StageP<KP>) + (((size_t)n_ops * sizeof(Op) + 15) & ~(size_t)15);
    if (CODES_SMEM) s += (size_t)n_tips * TILE;
    s += depth * SPT * KP * 4 * sizeof(u64) * kPruneThreads;
    return s;
}

__global__ void relayout4p_kernel(const float* __restrict__ P, const float* __restrict__ tip, int n_nodes,
                                  int n_tips, int C, float* __restrict__ Pp, float* __restrict__ Tp) {
    const int KP = C / 2;
    const long long n_p = (long long)n_nodes * C * 16;
    const long long n_t = (long long)n_tips * C * kCodes4 * 4;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n_p + n_t;
         idx += (long long)gridDim.x * blockDim.x) {
        if (idx < n_p) {
            // Pp[((node*KP + q)*4 + j)*8 + i*2 + h] = P[((node*C + 2q+h)*4 + i)*4 + j]
            const long long node = idx / (C * 16);
            const int w = (int)(idx % (C * 16));
            const int q = w / 32, j = (w / 8) % 4, i = (w / 2) % 4, h = w % 2;
            Pp[idx] = P[((node * C + 2 * q + h) * 4 + i) * 4 + j];
        } else {
            // Tp[(((tip*KP + q)*2 + half)*16 + code)*4 + (i % 2)*2 + h] = tip[((tip*C + 2q+h)*16 + code)*4 + i]
            // with half = i / 2
            const long long t = idx - n_p;
            const long long tp = t / (C * kCodes4 * 4);
            const int w = (int)(t % (C * kCodes4 * 4));
            const int q = w / (kCodes4 * 8), half = (w / (kCodes4 * 4)) % 2, code = (w / 4) % kCodes4;
            const int i = 2 * half + (w / 2) % 2, h = w % 2;
            Tp[t] = tip[((tp * C + 2 * q + h) * kCodes4 + code) * 4 + i];
        }
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

// out[q][i] = sum_j P[q][j][i] x[q][j] for both categories of every pair,
// in the order of prune4s (j ascending, first term a product)
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
__device__ __forceinline__ void tip4p(const u64 (*T)[2][kCodes4][2], int code, u64 out[KP][4]) {
#pragma unroll
    for (int q = 0; q < KP; ++q) {
        const ulonglong2 a = *reinterpret_cast<const ulonglong2*>(&T[q][0][code][0]);
        const ulonglong2 b = *reinterpret_cast<const ulonglong2*>(&T[q][1][code][0]);
        out[q][0] = a.x; out[q][1] = a.y; out[q][2] = b.x; out[q][3] = b.y;
    }
}

template <int KP, int SPT, bool CODES_SMEM>
__global__ void __launch_bounds__(kPruneThreads) prune4p_kernel(PruneArgs a, const float* __restrict__ Pp,
                                                                const float* __restrict__ Tp) {
    extern __shared__ __align__(16) unsigned char sm[];
    constexpr int TILE = kPruneThreads * SPT;
    StageP<KP>* stages = reinterpret_cast<StageP<KP>*>(sm);
    size_t off = 3 * sizeof(StageP<KP>);
    Op* s_ops = reinterpret_cast<Op*>(sm + off);
    off += ((size_t)a.n_ops * sizeof(Op) + 15) & ~(size_t)15;
    uint8_t* s_codes = sm + off;
    if (CODES_SMEM) off += (size_t)a.n_tips * TILE;
    ulonglong2* s_stack = reinterpret_cast<ulonglong2*>(sm + off);

    const int tid = threadIdx.x;
    const int tile_base = blockIdx.x * TILE;
    for (int i = tid; i < a.n_ops; i += kPruneThreads) s_ops[i] = a.ops[i];
    if (CODES_SMEM) {
        constexpr int chunks = TILE / 16;
        for (int i = tid; i < a.n_tips * chunks; i += kPruneThreads) {
            const int t = i / chunks, q = i % chunks, col = tile_base + 16 * q;
            uint8_t* dst = s_codes + (size_t)t * TILE + 16 * q;
            if (col < a.site_stride) cp_async16(dst, a.codes + (size_t)t * a.site_stride + col);
            else *reinterpret_cast<uint4*>(dst) = make_uint4(0u, 0u, 0u, 0u);
        }
    }
    __syncthreads();
    stage_op4p<KP>(&stages[0], s_ops[0], Pp, Tp);
    cp_async_commit();
    if (a.n_ops > 1) stage_op4p<KP>(&stages[1], s_ops[1], Pp, Tp);
    cp_async_commit();

    u64 acc[SPT][KP][4];
    int scale_e[SPT];
    const u64 one2 = pack2(1.0f, 1.0f);
#pragma unroll
    for (int s = 0; s < SPT; ++s) {
        scale_e[s] = 0;
#pragma unroll
        for (int q = 0; q < KP; ++q)
#pragma unroll
            for (int i = 0; i < 4; ++i) acc[s][q][i] = one2;
    }
    int sp = 0;

    for (int o = 0; o < a.n_ops; ++o) {
        cp_async_wait<1>();
        __syncthreads();
        if (o + 2 < a.n_ops) stage_op4p<KP>(&stages[(o + 2) % 3], s_ops[o + 2], Pp, Tp);
        cp_async_commit();
        const Op op = s_ops[o];
        const StageP<KP>& stg = stages[o % 3];
        if (op.s0 == kSrcPop) --sp;
#pragma unroll
        for (int s = 0; s < SPT; ++s) {
            const int lsite = tid + s * kPruneThreads;
            u64 d0[KP][4], d1[KP][4];
            if (op.s0 >= 0) {
                int code;
                if (CODES_SMEM) code = s_codes[(size_t)op.s0 * TILE + lsite];
                else code = a.codes[(size_t)op.s0 * a.site_stride + min(tile_base + lsite, a.site_stride - 1)];
                tip4p<KP>(stg.tip[0], code & (kCodes4 - 1), d0);
            } else if (op.s0 == kSrcPop) {
                u64 x[KP][4];
#pragma unroll
                for (int q = 0; q < KP; ++q)
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const ulonglong2 v = s_stack[((size_t)((sp * SPT + s) * KP + q) * 2 + h) * kPruneThreads + tid];
                        x[q][2 * h] = v.x;
                        x[q][2 * h + 1] = v.y;
                    }
                mv4p<KP>(stg.p[0], x, d0);
            } else {
                mv4p<KP>(stg.p[0], acc[s], d0);
            }
            if (op.s1 >= 0) {
                int code;
                if (CODES_SMEM) code = s_codes[(size_t)op.s1 * TILE + lsite];
                else code = a.codes[(size_t)op.s1 * a.site_stride + min(tile_base + lsite, a.site_stride - 1)];
                tip4p<KP>(stg.tip[1], code & (kCodes4 - 1), d1);
            } else if (op.s1 == kSrcAcc) {
                mv4p<KP>(stg.p[1], acc[s], d1);
            }
            if (op.s1 == kSrcNone) {
#pragma unroll
                for (int q = 0; q < KP; ++q)
#pragma unroll
                    for (int i = 0; i < 4; ++i) acc[s][q][i] = d0[q][i];
            } else {
#pragma unroll
                for (int q = 0; q < KP; ++q)
#pragma unroll
                    for (int i = 0; i < 4; ++i) acc[s][q][i] = mul2(d0[q][i], d1[q][i]);
            }
            float mx = 0.0f;
#pragma unroll
            for (int q = 0; q < KP; ++q)
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    float lo, hi;
                    unpack2(acc[s][q][i], lo, hi);
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
                    for (int i = 0; i < 4; ++i) acc[s][q][i] = mul2(mul2(acc[s][q][i], g1), g2);
                scale_e[s] += e;
            }
            if (op.push) {
#pragma unroll
                for (int q = 0; q < KP; ++q)
#pragma unroll
                    for (int h = 0; h < 2; ++h)
                        s_stack[((size_t)((sp * SPT + s) * KP + q) * 2 + h) * kPruneThreads + tid] =
                            make_ulonglong2(acc[s][q][2 * h], acc[s][q][2 * h + 1]);
            }
        }
        if (op.push) ++sp;
    }
    cp_async_wait<0>();

    // root: sum_k w_k sum_s L[s] root_w[s] in FP64 (categories in order)
    double tsum = 0.0, tcomp = 0.0;
#pragma unroll
    for (int s = 0; s < SPT; ++s) {
        const int site = tile_base + tid + s * kPruneThreads;
        double lsum = 0.0;
#pragma unroll
        for (int q = 0; q < KP; ++q) {
            float v[2][4];
#pragma unroll
            for (int i = 0; i < 4; ++i) unpack2(acc[s][q][i], v[0][i], v[1][i]);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                double lk = (double)v[h][0] * a.root_w[0];
#pragma unroll
                for (int i = 1; i < 4; ++i) lk = fma((double)v[h][i], a.root_w[i], lk);
                lsum = fma(a.cat_w[2 * q + h], lk, lsum);
            }
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
    if (threadIdx.x == 0) {
        a.block_sum[2 * blockIdx.x] = tsum;
        a.block_sum[2 * blockIdx.x + 1] = tcomp;
    }
}

template <int KP, int SPT, bool CODES_SMEM>
cudaError_t launch4p(const PruneArgs& a, const float* Pp, const float* Tp, int* n_blocks, cudaStream_t st) {
    const size_t smem = smem4p_bytes<KP, SPT, CODES_SMEM>(a.n_ops, a.n_tips, a.max_depth);
    if (smem > 227 * 1024) return cudaErrorInvalidConfiguration;
    auto kern = prune4p_kernel<KP, SPT, CODES_SMEM>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int blocks = (a.n_sites + kPruneThreads * SPT - 1) / (kPruneThreads * SPT);
    *n_blocks = blocks;
    kern<<<blocks, kPruneThreads, smem, st>>>(a, Pp, Tp);
    return cudaGetLastError();
}

// codes_global: read the tip codes from global memory (cached) instead of
// staging the tile's codes in shared memory, for more resident CTAs
template <int KP, int SPT>
cudaError_t launch4p_kp(const PruneArgs& a, const float* Pp, const float* Tp, bool codes_global, int* n_blocks,
                        cudaStream_t st) {
    if (!codes_global && smem4p_bytes<KP, SPT, true>(a.n_ops, a.n_tips, a.max_depth) <= 160 * 1024)
        return launch4p<KP, SPT, true>(a, Pp, Tp, n_blocks, st);
    return launch4p<KP, SPT, false>(a, Pp, Tp, n_blocks, st);
}

size_t min_smem4p(const PruneArgs& a, int spt) {
    switch (a.C / 2) {
        case 1: return spt == 1 ? smem4p_bytes<1, 1, false>(a.n_ops, a.n_tips, a.max_depth)
                                : smem4p_bytes<1, 2, false>(a.n_ops, a.n_tips, a.max_depth);
        case 2: return spt == 1 ? smem4p_bytes<2, 1, false>(a.n_ops, a.n_tips, a.max_depth)
                                : smem4p_bytes<2, 2, false>(a.n_ops, a.n_tips, a.max_depth);
        default: return spt == 1 ? smem4p_bytes<4, 1, false>(a.n_ops, a.n_tips, a.max_depth)
                                 : smem4p_bytes<4, 2, false>(a.n_ops, a.n_tips, a.max_depth);
    }
}

}  // namespace

bool prune4p_fits(const PruneArgs& a, int spt) {
    if (a.C != 2 && a.C != 4 && a.C != 8) return false;
    if (spt != 1 && spt != 2) return false;
    return min_smem4p(a, spt) <= 227 * 1024;
}

size_t prune4p_scratch_bytes(const PruneArgs& a) {
    const size_t p = (size_t)a.n_nodes * a.C * 16 * sizeof(float);
    return ((p + 255) & ~(size_t)255) + (size_t)a.n_tips * a.C * kCodes4 * 4 * sizeof(float);
}

cudaError_t launch_prune4p(const PruneArgs& a, int spt, bool codes_global, int* n_blocks, cudaStream_t st) {
    if (!prune4p_fits(a, spt) || a.scratch == nullptr) return cudaErrorInvalidValue;
    float* Pp = static_cast<float*>(a.scratch);
    const size_t p = (size_t)a.n_nodes * a.C * 16 * sizeof(float);
    float* Tp = reinterpret_cast<float*>(static_cast<unsigned char*>(a.scratch) + ((p + 255) & ~(size_t)255));
    const long long total = (long long)a.n_nodes * a.C * 16 + (long long)a.n_tips * a.C * kCodes4 * 4;
    long long blocks = (total + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    relayout4p_kernel<<<(unsigned)blocks, 256, 0, st>>>(static_cast<const float*>(a.P),
                                                         static_cast<const float*>(a.tipT), a.n_nodes, a.n_tips,
                                                         a.C, Pp, Tp);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    switch (a.C / 2) {
        case 1: return spt == 1 ? launch4p_kp<1, 1>(a, Pp, Tp, codes_global, n_blocks, st)
                                : launch4p_kp<1, 2>(a, Pp, Tp, codes_global, n_blocks, st);
        case 2: return spt == 1 ? launch4p_kp<2, 1>(a, Pp, Tp, codes_global, n_blocks, st)
                                : launch4p_kp<2, 2>(a, Pp, Tp, codes_global, n_blocks, st);
        default: return spt == 1 ? launch4p_kp<4, 1>(a, Pp, Tp, codes_global, n_blocks, st)
                                 : launch4p_kp<4, 2>(a, Pp, Tp, codes_global, n_blocks, st);
    }
}

}  // namespace plk
