// Fused post-order pass for 20-state (protein) alignments in FP32 with
// per-site power-of-two scaling: the GPU form of simpleML::calculate_likelihood
// and branch_likelihood (src/simpleML.cpp:127-197) for S = 20.
//
// One CTA takes a tile of 128 sites and one rate category (grid = tiles x C)
// and walks the register-allocated post-order program.  A child message is
// a small matrix product  M[site][i] = sum_j V[site][j] P[i][j]  over the
// tile (128 x 20 x 20); the child vectors V live in shared memory, laid out
// [state][site] so that a warp's sites are contiguous.  Two forms of that
// product, chosen by the autotuner:
//   * CUDA cores: each thread owns 4 sites x 5 states and reads per j one
//     float4 of V and 5 values of P (broadcast to 8 lanes): 20 FMAs per 3
//     shared-memory loads;
//   * tensor cores (mma.sync m16n8k8 TF32, FP32 accumulation) with the
//     three-product split a_hi b_hi + a_hi b_lo + a_lo b_hi, which keeps
//     about FP32 accuracy: per warp 32 sites x 24 states (20 padded) x 24.
// Tip children are look-ups in a per-(tip, category) table P x state set.
// P(t) blocks and tip tables are staged per op through a three-slot cp.async
// ring.  Every node vector gets a fresh slot (slots are allocated uniformly
// across the CTA), so no op reads and writes the same shared memory.
//
// The root sums pi_s L[s] per (site, category) in FP32 and leaves it with
// the category's scaler exponent; combine20_kernel forms
// log(sum_k w_k L_k 2^e_k) per site in FP32 (site_log32) and the compensated
// block sums.
#include "plk_device.cuh"
#include "plk_internal.h"

namespace plk {
using namespace dev;

namespace {

constexpr int kS = 20;
constexpr int kTile = 128;          // sites per CTA
constexpr int kLD = kTile + 8;      // row stride of a node vector (floats)
constexpr int kRows = 24;           // node-vector rows (20 states, 4 zero rows)
constexpr int kThreads = 128;
constexpr int kMaxSlots = 16;       // live node vectors (16-bit mask, 4-bit stack entries)

// staged layouts
//  CUDA cores:   P: [j][group 4][8] (i = 5 group + r, r < 5), 640 floats
//                tip: [code][group 4][8] + 4 padding, 36 floats per code
//  tensor cores: P: hi [j 24][i 24] then lo [j 24][i 24], 1152 floats
//                tip: [code][24] + 4 padding, 28 floats per code
__host__ __device__ inline int p_floats(int mode) { return mode == 1 ? 640 : 2 * kRows * kRows; }
// per-code strides of the tip tables padded past a multiple of 32 floats, so
// that the codes of one warp's sites spread over the shared-memory banks
__host__ __device__ inline int tip_floats_per_code(int mode) { return mode == 1 ? 36 : kRows + 4; }

__host__ __device__ inline int child_floats(int mode, int n_codes) {
    const int p = p_floats(mode), t = n_codes * tip_floats_per_code(mode);
    return ((p > t ? p : t) + 3) & ~3;
}

struct P20Args {
    PruneArgs a;
    int mode;            // 1 = CUDA cores, 2 = tensor cores
    const float* Ps;     // staged P per (node, category)
    const float* Ts;     // staged tip tables per (tip, category)
    float* cat_L;        // [C][n_sites] root sums of each category (FP32)
    int* cat_E;          // [C][n_sites]
    int n_slots;
};

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
    return r;
}

// ---------------------------------------------------------------------------
// relayout of the FP32 P(t) and tip tables into the staged forms
// ---------------------------------------------------------------------------
__global__ void relayout20_kernel(const float* __restrict__ P, const float* __restrict__ tip, int n_nodes,
                                  int n_tips, int C, int n_codes, int mode, float* __restrict__ Ps,
                                  float* __restrict__ Ts) {
    const int pf = p_floats(mode), tf = tip_floats_per_code(mode);
    const long long n_p = (long long)n_nodes * C * pf;
    const long long n_t = (long long)n_tips * C * n_codes * tf;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n_p + n_t;
         idx += (long long)gridDim.x * blockDim.x) {
        if (idx < n_p) {
            const long long nk = idx / pf;  // node * C + k
            const int w = (int)(idx % pf);
            const float* src = P + nk * kS * kS;
            float v = 0.f;
            if (mode == 1) {
                const int j = w / 32, g = (w / 8) % 4, r = w % 8;
                if (r < 5) v = src[(5 * g + r) * kS + j];
            } else {
                const int half = w / (kRows * kRows), q = w % (kRows * kRows);
                const int j = q / kRows, i = q % kRows;
                if (i < kS && j < kS) {
                    const float x = src[i * kS + j];
                    const float hi = __uint_as_float(to_tf32(x));
                    v = half == 0 ? hi : __uint_as_float(to_tf32(x - hi));
                }
            }
            Ps[idx] = v;
        } else {
            const long long t = idx - n_p;
            const long long nkc = t / tf;  // (tip * C + k) * n_codes + code
            const int w = (int)(t % tf);
            const float* src = tip + nkc * kS;
            float v = 0.f;
            if (mode == 1) {
                const int g = w / 8, r = w % 8;
                if (w < 32 && r < 5) v = src[5 * g + r];
            } else if (w < kS) {
                v = src[w];
            }
            Ts[t] = v;
        }
    }
}

// ---------------------------------------------------------------------------
// the pass
// ---------------------------------------------------------------------------
struct Smem20 {
    float* stage[3];     // [child 2][child_floats]
    Op* ops;
    uint8_t* codes;      // [n_tips][kTile]
    float* slots;        // [n_slots][kRows][kLD]
};

__device__ __forceinline__ void stage_op20(float* dst, const Op& op, int k, const P20Args& g, int cf) {
    const PruneArgs& a = g.a;
    const int C = a.C;
    for (int c = 0; c < 2; ++c) {
        const int src = c ? op.s1 : op.s0;
        if (src == kSrcNone) continue;
        const float* from;
        int n;
        if (src >= 0) {
            n = a.n_codes * tip_floats_per_code(g.mode);
            from = g.Ts + ((size_t)src * C + k) * (size_t)n;
        } else {
            n = p_floats(g.mode);
            from = g.Ps + ((size_t)(c ? op.e1 : op.e0) * C + k) * (size_t)n;
        }
        float* to = dst + c * cf;
        for (int q = threadIdx.x; q < n / 4; q += blockDim.x) cp_async16(to + 4 * q, from + 4 * q);
    }
}

// CUDA-core child message: m[s][r] for sites sbase + s (s < SPS), states
// 5 grp + r
template <int SPS>
__device__ __forceinline__ void child_cc(const float* __restrict__ V, const float* __restrict__ Pst, int sbase,
                                         int grp, float m[SPS][5]) {
#pragma unroll
    for (int s = 0; s < SPS; ++s)
#pragma unroll
        for (int r = 0; r < 5; ++r) m[s][r] = 0.f;
#pragma unroll 4
    for (int j = 0; j < kS; ++j) {
        float vs[SPS];
        if constexpr (SPS == 4) {
            const float4 v = *reinterpret_cast<const float4*>(V + j * kLD + sbase);
            vs[0] = v.x; vs[1] = v.y; vs[2] = v.z; vs[3] = v.w;
        } else {
            const float2 v = *reinterpret_cast<const float2*>(V + j * kLD + sbase);
            vs[0] = v.x; vs[1] = v.y;
        }
        const float4 p = *reinterpret_cast<const float4*>(Pst + (j * 4 + grp) * 8);
        const float p4 = Pst[(j * 4 + grp) * 8 + 4];
        const float ps[5] = {p.x, p.y, p.z, p.w, p4};
#pragma unroll
        for (int s = 0; s < SPS; ++s)
#pragma unroll
            for (int r = 0; r < 5; ++r) m[s][r] = fmaf(ps[r], vs[s], m[s][r]);
    }
}

template <int SPS>
__device__ __forceinline__ void tip_cc(const float* __restrict__ T, const uint8_t* __restrict__ codes, int sbase,
                                       int grp, int n_codes, float m[SPS][5]) {
#pragma unroll
    for (int s = 0; s < SPS; ++s) {
        int code = codes[sbase + s];
        code = code < n_codes ? code : 0;
        const float* row = T + code * tip_floats_per_code(1) + grp * 8;
        const float4 p = *reinterpret_cast<const float4*>(row);
        m[s][0] = p.x; m[s][1] = p.y; m[s][2] = p.z; m[s][3] = p.w;
        m[s][4] = row[4];
    }
}

// tensor-core child message for a warp's MT x 16 sites: acc[mt][nt][4] in
// the m16n8 accumulator layout (rows = sites mt*16 + g (+8), cols = states
// nt*8 + 2t (+1))
template <int MT>
__device__ __forceinline__ void child_tc(const float* __restrict__ V, const float* __restrict__ Pst, int wbase,
                                         int lane, float acc[MT][3][4]) {
    const int g = lane >> 2, t = lane & 3;
    const float* Phi = Pst;
    const float* Plo = Pst + kRows * kRows;
#pragma unroll
    for (int mt = 0; mt < MT; ++mt)
#pragma unroll
        for (int nt = 0; nt < 3; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[mt][nt][q] = 0.f;
#pragma unroll
    for (int ks = 0; ks < 3; ++ks) {
        const int j0 = ks * 8 + t, j1 = j0 + 4;
        uint32_t bh[3][2], bl[3][2];
#pragma unroll
        for (int nt = 0; nt < 3; ++nt) {
            const int i = nt * 8 + g;
            bh[nt][0] = __float_as_uint(Phi[j0 * kRows + i]);
            bh[nt][1] = __float_as_uint(Phi[j1 * kRows + i]);
            bl[nt][0] = __float_as_uint(Plo[j0 * kRows + i]);
            bl[nt][1] = __float_as_uint(Plo[j1 * kRows + i]);
        }
#pragma unroll
        for (int mt = 0; mt < MT; ++mt) {
            const int r0 = wbase + mt * 16 + g, r1 = r0 + 8;
            const float x[4] = {V[j0 * kLD + r0], V[j0 * kLD + r1], V[j1 * kLD + r0], V[j1 * kLD + r1]};
            uint32_t ah[4], al[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                ah[q] = to_tf32(x[q]);
                al[q] = to_tf32(x[q] - __uint_as_float(ah[q]));
            }
#pragma unroll
            for (int nt = 0; nt < 3; ++nt) {
                float* d = acc[mt][nt];
                // small products first
                asm volatile(
                    "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                    "{%0,%1,%2,%3};\n"
                    : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                    : "r"(al[0]), "r"(al[1]), "r"(al[2]), "r"(al[3]), "r"(bh[nt][0]), "r"(bh[nt][1]));
                asm volatile(
                    "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                    "{%0,%1,%2,%3};\n"
                    : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                    : "r"(ah[0]), "r"(ah[1]), "r"(ah[2]), "r"(ah[3]), "r"(bl[nt][0]), "r"(bl[nt][1]));
                asm volatile(
                    "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                    "{%0,%1,%2,%3};\n"
                    : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                    : "r"(ah[0]), "r"(ah[1]), "r"(ah[2]), "r"(ah[3]), "r"(bh[nt][0]), "r"(bh[nt][1]));
            }
        }
    }
}

template <int MT>
__device__ __forceinline__ void tip_tc(const float* __restrict__ T, const uint8_t* __restrict__ codes, int wbase,
                                       int lane, int n_codes, float acc[MT][3][4]) {
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int mt = 0; mt < MT; ++mt)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            int code = codes[wbase + mt * 16 + g + 8 * h];
            code = code < n_codes ? code : 0;
#pragma unroll
            for (int nt = 0; nt < 3; ++nt) {
                const float2 v = *reinterpret_cast<const float2*>(T + code * tip_floats_per_code(2) + nt * 8 + 2 * t);
                acc[mt][nt][2 * h] = v.x;
                acc[mt][nt][2 * h + 1] = v.y;
            }
        }
}

// MODE 1 = CUDA cores, 2 = tensor cores; WARPS = 4 or 8 warps per 128-site
// tile (a warp takes 128 / WARPS sites: CUDA cores 8 site groups of SPS
// sites x 4 state groups, tensor cores MT m16 tiles)
template <int MODE, int WARPS>
__global__ void __launch_bounds__(32 * WARPS) prune20_kernel(P20Args g) {
    constexpr int NT = 32 * WARPS;
    constexpr int SW = kTile / WARPS;  // sites per warp
    constexpr int SPS = SW / 8;        // CUDA cores: sites per thread
    constexpr int MT = SW / 16;        // tensor cores: m16 tiles per warp
    extern __shared__ __align__(16) unsigned char smem[];
    const PruneArgs& a = g.a;
    const int k = blockIdx.y;
    const int tile0 = blockIdx.x * kTile;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int cf = child_floats(MODE, a.n_codes);

    Smem20 sm;
    size_t off = 0;
    for (int q = 0; q < 3; ++q) {
        sm.stage[q] = reinterpret_cast<float*>(smem + off);
        off += (size_t)2 * cf * sizeof(float);
    }
    sm.ops = reinterpret_cast<Op*>(smem + off);
    off += ((size_t)a.n_ops * sizeof(Op) + 15) & ~(size_t)15;
    sm.codes = smem + off;
    off += (size_t)a.n_tips * kTile;
    sm.slots = reinterpret_cast<float*>(smem + off);
    const size_t slot_floats = (size_t)kRows * kLD;

    __shared__ float s_rw[kS];  // root weights in FP32
    if (tid < kS) s_rw[tid] = (float)a.root_w[tid];
    for (int i = tid; i < a.n_ops; i += NT) sm.ops[i] = a.ops[i];
    {
        constexpr int chunks = kTile / 16;
        for (int i = tid; i < a.n_tips * chunks; i += NT) {
            const int t = i / chunks, q = i % chunks, col = tile0 + 16 * q;
            uint8_t* dst = sm.codes + (size_t)t * kTile + 16 * q;
            if (col < a.site_stride) cp_async16(dst, a.codes + (size_t)t * a.site_stride + col);
            else *reinterpret_cast<uint4*>(dst) = make_uint4(0u, 0u, 0u, 0u);
        }
    }
    // rows 20..23 of every slot stay zero (the padded K rows of the tensor form)
    for (int i = tid; i < g.n_slots * (kRows - kS) * kLD; i += NT) {
        const int sl = i / ((kRows - kS) * kLD), q = i % ((kRows - kS) * kLD);
        sm.slots[sl * slot_floats + kS * kLD + q] = 0.f;
    }
    __syncthreads();
    stage_op20(sm.stage[0], sm.ops[0], k, g, cf);
    cp_async_commit();
    if (a.n_ops > 1) stage_op20(sm.stage[1], sm.ops[1], k, g, cf);
    cp_async_commit();

    // uniform slot bookkeeping: the spill stack packs 4-bit slot numbers
    uint64_t stack = 0;
    int sp = 0, cur = -1;
    uint32_t live = 0;

    // per-thread sites: CUDA cores: SPS sites (sbase..), state group grp;
    // tensor cores: rows g, g+8 of the warp's MT m16 tiles
    const int sbase = warp * SW + (lane >> 2) * SPS;
    const int grp = lane & 3;
    int e_site[4] = {0, 0, 0, 0};

    for (int o = 0; o < a.n_ops; ++o) {
        cp_async_wait<1>();
        __syncthreads();
        if (o + 2 < a.n_ops) stage_op20(sm.stage[(o + 2) % 3], sm.ops[o + 2], k, g, cf);
        cp_async_commit();
        const Op op = sm.ops[o];
        const float* st = sm.stage[o % 3];
        int src0 = -1, src1 = -1;
        if (op.s0 == kSrcPop) src0 = (int)((stack >> (4 * --sp)) & 15u);
        else if (op.s0 == kSrcAcc) src0 = cur;
        if (op.s1 == kSrcAcc) src1 = cur;
        const int dst = __ffs(~live) - 1;  // a slot no live vector uses
        float* D = sm.slots + (size_t)dst * slot_floats;

        if constexpr (MODE == 1) {
            float m0[SPS][5], m1[SPS][5];
            if (op.s0 >= 0) tip_cc<SPS>(st, sm.codes + (size_t)op.s0 * kTile, sbase, grp, a.n_codes, m0);
            else child_cc<SPS>(sm.slots + (size_t)src0 * slot_floats, st, sbase, grp, m0);
            if (op.s1 != kSrcNone) {
                if (op.s1 >= 0) tip_cc<SPS>(st + cf, sm.codes + (size_t)op.s1 * kTile, sbase, grp, a.n_codes, m1);
                else child_cc<SPS>(sm.slots + (size_t)src1 * slot_floats, st + cf, sbase, grp, m1);
#pragma unroll
                for (int s = 0; s < SPS; ++s)
#pragma unroll
                    for (int r = 0; r < 5; ++r) m0[s][r] *= m1[s][r];
            }
#pragma unroll
            for (int s = 0; s < SPS; ++s) {
                float mx = m0[s][0];
#pragma unroll
                for (int r = 1; r < 5; ++r) mx = fmaxf(mx, m0[s][r]);
                mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
                mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 2));
                if (mx < scale_threshold<float>() && mx > 0.f) {
                    int e;
                    float f1, f2;
                    pow2_factors(mx, &e, &f1, &f2);
#pragma unroll
                    for (int r = 0; r < 5; ++r) m0[s][r] = (m0[s][r] * f1) * f2;
                    e_site[s] += e;
                }
            }
#pragma unroll
            for (int r = 0; r < 5; ++r) {
                float* row = D + (5 * grp + r) * kLD + sbase;
                if constexpr (SPS == 4) *reinterpret_cast<float4*>(row) = make_float4(m0[0][r], m0[1][r], m0[2][r], m0[3][r]);
                else *reinterpret_cast<float2*>(row) = make_float2(m0[0][r], m0[1][r]);
            }
        } else {
            const int wbase = warp * SW;
            float m0[MT][3][4], m1[MT][3][4];
            if (op.s0 >= 0) tip_tc<MT>(st, sm.codes + (size_t)op.s0 * kTile, wbase, lane, a.n_codes, m0);
            else child_tc<MT>(sm.slots + (size_t)src0 * slot_floats, st, wbase, lane, m0);
            if (op.s1 != kSrcNone) {
                if (op.s1 >= 0) tip_tc<MT>(st + cf, sm.codes + (size_t)op.s1 * kTile, wbase, lane, a.n_codes, m1);
                else child_tc<MT>(sm.slots + (size_t)src1 * slot_floats, st + cf, wbase, lane, m1);
#pragma unroll
                for (int mt = 0; mt < MT; ++mt)
#pragma unroll
                    for (int nt = 0; nt < 3; ++nt)
#pragma unroll
                        for (int q = 0; q < 4; ++q) m0[mt][nt][q] *= m1[mt][nt][q];
            }
            // per-site maxima: this thread's rows are (mt, h) -> site wbase + mt*16 + g + 8h
#pragma unroll
            for (int mt = 0; mt < MT; ++mt)
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    float mx = 0.f;
#pragma unroll
                    for (int nt = 0; nt < 3; ++nt) mx = fmaxf(mx, fmaxf(m0[mt][nt][2 * h], m0[mt][nt][2 * h + 1]));
                    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
                    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 2));
                    if (mx < scale_threshold<float>() && mx > 0.f) {
                        int e;
                        float f1, f2;
                        pow2_factors(mx, &e, &f1, &f2);
#pragma unroll
                        for (int nt = 0; nt < 3; ++nt) {
                            m0[mt][nt][2 * h] = (m0[mt][nt][2 * h] * f1) * f2;
                            m0[mt][nt][2 * h + 1] = (m0[mt][nt][2 * h + 1] * f1) * f2;
                        }
                        e_site[mt * 2 + h] += e;
                    }
                }
            const int gg = lane >> 2, t = lane & 3;
#pragma unroll
            for (int mt = 0; mt < MT; ++mt)
#pragma unroll
                for (int nt = 0; nt < 3; ++nt) {
                    const int i = nt * 8 + 2 * t;
                    if (i < kS) {
                        const int r0 = wbase + mt * 16 + gg;
                        D[i * kLD + r0] = m0[mt][nt][0];
                        D[(i + 1) * kLD + r0] = m0[mt][nt][1];
                        D[i * kLD + r0 + 8] = m0[mt][nt][2];
                        D[(i + 1) * kLD + r0 + 8] = m0[mt][nt][3];
                    }
                }
        }
        // retire the sources, place the result
        if (src0 >= 0) live &= ~(1u << src0);
        if (src1 >= 0) live &= ~(1u << src1);
        live |= 1u << dst;
        if (op.push) {
            stack = (stack & ~(15ull << (4 * sp))) | ((uint64_t)dst << (4 * sp));
            ++sp;
            cur = -1;
        } else {
            cur = dst;
        }
    }
    cp_async_wait<0>();
    __syncthreads();

    // root: L = sum_s pi_s R[s] per site in FP32 (this category)
    const float* R = sm.slots + (size_t)cur * slot_floats;
    if constexpr (MODE == 1) {
#pragma unroll
        for (int s = 0; s < SPS; ++s) {
            float l = 0.0f;
#pragma unroll
            for (int r = 0; r < 5; ++r) l = fmaf(R[(5 * grp + r) * kLD + sbase + s], s_rw[5 * grp + r], l);
            l += __shfl_xor_sync(0xffffffffu, l, 1);
            l += __shfl_xor_sync(0xffffffffu, l, 2);
            const int site = tile0 + sbase + s;
            if (grp == 0 && site < a.n_sites) {
                g.cat_L[(size_t)k * a.n_sites + site] = l;
                g.cat_E[(size_t)k * a.n_sites + site] = e_site[s];
            }
        }
    } else {
        const int gg = lane >> 2, t = lane & 3;
#pragma unroll
        for (int mt = 0; mt < MT; ++mt)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int ls = warp * SW + mt * 16 + gg + 8 * h;
                float l = 0.0f;
                for (int i = t; i < kS; i += 4) l = fmaf(R[i * kLD + ls], s_rw[i], l);
                l += __shfl_xor_sync(0xffffffffu, l, 1);
                l += __shfl_xor_sync(0xffffffffu, l, 2);
                const int site = tile0 + ls;
                if (t == 0 && site < a.n_sites) {
                    g.cat_L[(size_t)k * a.n_sites + site] = l;
                    g.cat_E[(size_t)k * a.n_sites + site] = e_site[mt * 2 + h];
                }
            }
    }
}

// per site: log(sum_k w_k L_k 2^e_k) with the largest exponent factored out,
// in FP32 (site_log32), then the compensated block sums (added up by the
// last CTA when grid_done is set)
__global__ void __launch_bounds__(kThreads) combine20_kernel(const float* __restrict__ cat_L,
                                                             const int* __restrict__ cat_E, const double* cat_w,
                                                             int C, int n_sites, double* site_lnl,
                                                             double* block_sum, unsigned* grid_done,
                                                             double* lnl_out) {
    const int site = blockIdx.x * blockDim.x + threadIdx.x;
    SiteSum32 sum;
    if (site < n_sites) {
        int E = cat_E[site];
        for (int k = 1; k < C; ++k) E = max(E, cat_E[(size_t)k * n_sites + site]);
        float l = 0.0f;
        for (int k = 0; k < C; ++k)
            l = fmaf((float)cat_w[k], ldexpf(cat_L[(size_t)k * n_sites + site], cat_E[(size_t)k * n_sites + site] - E),
                     l);
        float lm;
        int ee;
        site_log32(l, E, lm, ee);
        site_lnl[site] = site_lnl64(lm, ee);
        site_sum_add(sum, lm, ee);
    }
    const SiteSum32 bsum = block_sum_site32f(sum);
    if (threadIdx.x == 0) store_site_record(block_sum, blockIdx.x, bsum);
    if (grid_done) finish_grid_sum32(block_sum, grid_done, lnl_out);
}

size_t smem20_bytes(const PruneArgs& a, int mode) {
    const int n_slots = a.max_depth + 2;
    return (size_t)3 * 2 * child_floats(mode, a.n_codes) * sizeof(float) +
           (((size_t)a.n_ops * sizeof(Op) + 15) & ~(size_t)15) + (size_t)a.n_tips * kTile +
           (size_t)n_slots * kRows * kLD * sizeof(float);
}

}  // namespace

// variant 1 / 2: CUDA cores / tensor cores with 4 warps per tile; 3 / 4: the
// same with 8 warps per tile
bool prune20_fits(const PruneArgs& a, int variant) {
    if (a.C < 1 || a.n_codes < 1 || a.n_ops < 1 || a.max_depth + 2 > kMaxSlots) return false;
    if (variant < 1 || variant > 4) return false;
    return smem20_bytes(a, (variant - 1) % 2 + 1) <= 227 * 1024;
}

size_t prune20_scratch_bytes(const PruneArgs& a, int n_nodes) {
    const size_t pf = (size_t)p_floats(2) > (size_t)p_floats(1) ? p_floats(2) : p_floats(1);
    const size_t tf = (size_t)(tip_floats_per_code(1) > tip_floats_per_code(2) ? tip_floats_per_code(1)
                                                                                : tip_floats_per_code(2));
    const size_t ps = (size_t)n_nodes * a.C * pf * sizeof(float);
    const size_t ts = (size_t)a.n_tips * a.C * a.n_codes * tf * sizeof(float);
    const size_t cl = (((size_t)a.C * a.n_sites * sizeof(float) + 255) & ~(size_t)255) +
                      (size_t)a.C * a.n_sites * sizeof(int);
    return ((ps + 255) & ~(size_t)255) + ((ts + 255) & ~(size_t)255) + cl;
}

cudaError_t launch_prune20(const PruneArgs& a, int n_nodes, int variant, void* scratch, int* n_blocks,
                           cudaStream_t st) {
    if (!prune20_fits(a, variant) || scratch == nullptr) return cudaErrorInvalidValue;
    const int mode = (variant - 1) % 2 + 1;
    const int warps = variant <= 2 ? 4 : 8;
    const size_t pf = p_floats(mode);
    const size_t ps = (size_t)n_nodes * a.C * pf * sizeof(float);
    const size_t pf_max = (size_t)p_floats(2);
    const size_t ts_max = (size_t)a.n_tips * a.C * a.n_codes *
                          std::max(tip_floats_per_code(1), tip_floats_per_code(2)) * sizeof(float);
    unsigned char* base = static_cast<unsigned char*>(scratch);
    P20Args g{};
    g.a = a;
    g.mode = mode;
    g.Ps = reinterpret_cast<float*>(base);
    size_t off = (((size_t)n_nodes * a.C * pf_max * sizeof(float)) + 255) & ~(size_t)255;
    g.Ts = reinterpret_cast<float*>(base + off);
    off += (ts_max + 255) & ~(size_t)255;
    g.cat_L = reinterpret_cast<float*>(base + off);
    off += (((size_t)a.C * a.n_sites * sizeof(float)) + 255) & ~(size_t)255;
    g.cat_E = reinterpret_cast<int*>(base + off);
    g.n_slots = a.max_depth + 2;
    (void)ps;
    {
        const long long total = (long long)n_nodes * a.C * pf + (long long)a.n_tips * a.C * a.n_codes *
                                                                    tip_floats_per_code(mode);
        long long blocks = (total + 255) / 256;
        if (blocks > 152 * 8) blocks = 152 * 8;
        relayout20_kernel<<<(unsigned)blocks, 256, 0, st>>>(static_cast<const float*>(a.P),
                                                             static_cast<const float*>(a.tipT), n_nodes, a.n_tips,
                                                             a.C, a.n_codes, mode, const_cast<float*>(g.Ps),
                                                             const_cast<float*>(g.Ts));
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    const size_t smem = smem20_bytes(a, mode);
    dim3 grid((a.n_sites + kTile - 1) / kTile, a.C);
    cudaError_t e;
    auto run = [&](auto kern) -> cudaError_t {
        cudaError_t r = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (r != cudaSuccess) return r;
        kern<<<grid, 32 * warps, smem, st>>>(g);
        return cudaGetLastError();
    };
    if (mode == 1) e = warps == 4 ? run(prune20_kernel<1, 4>) : run(prune20_kernel<1, 8>);
    else e = warps == 4 ? run(prune20_kernel<2, 4>) : run(prune20_kernel<2, 8>);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_combine20(g.cat_L, g.cat_E, a, n_blocks, st);
}

cudaError_t launch_combine20(const float* cat_L, const int* cat_E, const PruneArgs& a, int* n_blocks,
                             cudaStream_t st) {
    const int blocks = (a.n_sites + kThreads - 1) / kThreads;
    combine20_kernel<<<blocks, kThreads, 0, st>>>(cat_L, cat_E, a.cat_w, a.C, a.n_sites, a.site_lnl, a.block_sum,
                                                  a.grid_done, a.lnl_out);
    *n_blocks = blocks;
    return cudaGetLastError();
}

}  // namespace plk
