// NNI-neighbour scoring of a batch: the likelihood of every tree one nearest
// neighbour interchange away from each batch tree (the rearrangements
// treebender --nni writes out, src/tree.cpp:2482-2548, which treeator then
// re-parses and scores from scratch, src/treeator.cpp:705-990), with branch
// lengths kept on their edges.
//
// Per work unit (one site tile of one tree) a CTA runs three phases:
//  A  the staged post-order pass (plk_prune4s.cuh, STORE_D): every internal
//     non-root node's message to its parent, D = P(t) x conditional vector,
//     goes to the CTA's scratch slice with its power-of-two exponent;
//  B  pre-order: outside vectors Out(v) = P_v^T (Out(u) x D_sibling),
//     Out(root) = frequencies, into the scratch slice;
//  C  every move of the tree: for an interchange across edge (u, v) the new
//     pair v' = (x, y) and u' = (v', z) give
//       L = sum_k w_k sum_s Out_u[s] D_z[s] (P_v (D_x x D_y))[s],
//     and across the root edge (v, c): v' = (x, y), c' = (p, q),
//       L = sum_k w_k sum_s pi_s (P_v (D_x x D_y))[s] (P_c (D_p x D_q))[s];
//     in FP32 per site (the FP64 pipe of this part is a small fraction of
//     its FP32 rate): a site's log-likelihood is logf of the mantissa of L
//     plus its power-of-two exponent times ln 2, the mantissa logs summed per
//     warp with FP32 TwoSum, the exponents as integers, then per CTA in warp
//     order in FP64.
// A last kernel sums each (tree, move) over its tiles in site order.
#include "plk_batch.h"
#include "plk_device.cuh"
#include "plk_prune4s.cuh"

namespace plk {
using namespace dev;

namespace {

constexpr int TILE = kPruneThreads;  // one site per thread

struct ItemView {
    const BatchItemDev* it;
    const float* P;        // item's P32
    const float* tipT;     // item's tip32
    const uint8_t* codes;  // item's codes
    const int2* child;     // item's child table
    const double* root_w;
    const double* cat_w;
};

// FP32 copies of an item's root and category weights (converted once per unit)
template <int CM>
struct Weights32 {
    float4 root;
    float cat[CM];
};

template <int CM>
__device__ __forceinline__ Weights32<CM> weights32(const ItemView& iv, int C) {
    Weights32<CM> w;
    w.root = make_float4((float)iv.root_w[0], (float)iv.root_w[1], (float)iv.root_w[2], (float)iv.root_w[3]);
#pragma unroll
    for (int k = 0; k < CM; ++k) w.cat[k] = k < C ? (float)iv.cat_w[k] : 0.0f;
    return w;
}

// Message of node `node` to its parent at this thread's site, category k,
// and its exponent: tip -> tip-table row of the site's code, internal ->
// scratch written by phase A.
__device__ __forceinline__ float4 message(const ItemView& iv, const BatchDev& b, int node, int k, int site_c, int tid,
                                          const float4* sD, const int* sED, int* e) {
    const BatchItemDev& it = *iv.it;
    if (node < it.n_tips) {
        const int code = iv.codes[(size_t)node * it.site_stride + site_c] & (kCodes - 1);
        *e = 0;
        return *reinterpret_cast<const float4*>(iv.tipT + (((size_t)node * b.C + k) * kCodes + code) * 4);
    }
    const int r = node - it.n_tips;
    *e = sED[(size_t)r * TILE + tid];
    return sD[((size_t)r * b.C + k) * TILE + tid];
}

__device__ __forceinline__ float4 mul4(float4 a, float4 c) { return make_float4(a.x * c.x, a.y * c.y, a.z * c.z, a.w * c.w); }

__device__ __forceinline__ float4 pmv(const float* Pk, float4 x) {
    const float4 r0 = *reinterpret_cast<const float4*>(Pk);
    const float4 r1 = *reinterpret_cast<const float4*>(Pk + 4);
    const float4 r2 = *reinterpret_cast<const float4*>(Pk + 8);
    const float4 r3 = *reinterpret_cast<const float4*>(Pk + 12);
    float4 o;
    o.x = fmaf(x.w, r0.w, fmaf(x.z, r0.z, fmaf(x.y, r0.y, x.x * r0.x)));
    o.y = fmaf(x.w, r1.w, fmaf(x.z, r1.z, fmaf(x.y, r1.y, x.x * r1.x)));
    o.z = fmaf(x.w, r2.w, fmaf(x.z, r2.z, fmaf(x.y, r2.y, x.x * r2.x)));
    o.w = fmaf(x.w, r3.w, fmaf(x.z, r3.z, fmaf(x.y, r3.y, x.x * r3.x)));
    return o;
}

// y = P^T x (outside propagation): y[b] = sum_a x[a] P[a][b]
__device__ __forceinline__ float4 pmv_t(const float* Pk, float4 x) {
    const float4 r0 = *reinterpret_cast<const float4*>(Pk);
    const float4 r1 = *reinterpret_cast<const float4*>(Pk + 4);
    const float4 r2 = *reinterpret_cast<const float4*>(Pk + 8);
    const float4 r3 = *reinterpret_cast<const float4*>(Pk + 12);
    float4 o;
    o.x = fmaf(x.w, r3.x, fmaf(x.z, r2.x, fmaf(x.y, r1.x, x.x * r0.x)));
    o.y = fmaf(x.w, r3.y, fmaf(x.z, r2.y, fmaf(x.y, r1.y, x.x * r0.y)));
    o.z = fmaf(x.w, r3.z, fmaf(x.z, r2.z, fmaf(x.y, r1.z, x.x * r0.z)));
    o.w = fmaf(x.w, r3.w, fmaf(x.z, r2.w, fmaf(x.y, r1.w, x.x * r0.w)));
    return o;
}

__device__ __forceinline__ float max4(float4 a) { return fmaxf(fmaxf(a.x, a.y), fmaxf(a.z, a.w)); }

__device__ __forceinline__ float4 scale4(float4 a, float f1, float f2) {
    return make_float4((a.x * f1) * f2, (a.y * f1) * f2, (a.z * f1) * f2, (a.w * f1) * f2);
}

template <int CM>
__device__ void phase_b(const ItemView& iv, const BatchDev& b, int site_c, int tid, const float4* sD, const int* sED,
                        float4* sO, int* sEO) {
    const BatchItemDev& it = *iv.it;
    const int C = b.C;
    for (int r = it.n_int - 1; r >= 0; --r) {
        const int u = it.n_tips + r;
        const bool is_root = r == it.n_int - 1;
        float4 ou[CM];
        int eu = 0;
#pragma unroll
        for (int k = 0; k < CM; ++k)
            if (k < C) {
                if (is_root) ou[k] = make_float4((float)iv.root_w[0], (float)iv.root_w[1], (float)iv.root_w[2], (float)iv.root_w[3]);
                else ou[k] = sO[((size_t)r * C + k) * TILE + tid];
            }
        if (!is_root) eu = sEO[(size_t)r * TILE + tid];
        const int2 ch = iv.child[u];
        const int kids[2] = {ch.x, ch.y};
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const int v = kids[c], w = kids[1 - c];
            if (v < it.n_tips) continue;  // tips (and absent children) need no outside vector
            float4 ov[CM];
            int ew = 0;
            float mx = 0.0f;
#pragma unroll
            for (int k = 0; k < CM; ++k)
                if (k < C) {
                    float4 t = ou[k];
                    if (w >= 0) t = mul4(t, message(iv, b, w, k, site_c, tid, sD, sED, &ew));
                    ov[k] = pmv_t(iv.P + ((size_t)v * C + k) * 16, t);
                    mx = fmaxf(mx, max4(ov[k]));
                }
            int e = 0;
            if (mx < scale_threshold<float>() && mx > 0.0f) {
                float f1, f2;
                pow2_factors(mx, &e, &f1, &f2);
#pragma unroll
                for (int k = 0; k < CM; ++k) ov[k] = scale4(ov[k], f1, f2);
            }
            const int rv = v - it.n_tips;
#pragma unroll
            for (int k = 0; k < CM; ++k)
                if (k < C) sO[((size_t)rv * C + k) * TILE + tid] = ov[k];
            sEO[(size_t)rv * TILE + tid] = eu + ew + e;
        }
    }
}

// Likelihood of one move at this thread's site in FP32:  L = lsum 2^etot,
// lsum = sum_k w_k sum_s Out[s] (P_v (D_x x D_y))[s] D_z[s]  (kind 0) or
// sum_k w_k sum_s pi_s (P_v (D_x x D_y))[s] (P_c (D_p x D_q))[s]  (kind 1).
// SCALE multiplies lsum by 2^64 (the outside / root weights scaled, exact)
// for the rare site whose FP32 lsum would fall below the normal range.
template <int CM>
__device__ float move_site_l(const ItemView& iv, const BatchDev& b, const NniMoveDev& mv, int site_c, int tid,
                             const float4* sD, const int* sED, const float4* sO, const int* sEO,
                             const Weights32<CM>& w, float scale, int* etot_out) {
    const BatchItemDev& it = *iv.it;
    const int C = b.C;
    float4 t1[CM];
    int ex = 0, ey = 0, ez = 0, ep = 0, eq = 0;
    float mx = 0.0f;
#pragma unroll
    for (int k = 0; k < CM; ++k)
        if (k < C) {
            t1[k] = mul4(message(iv, b, mv.x, k, site_c, tid, sD, sED, &ex),
                         message(iv, b, mv.y, k, site_c, tid, sD, sED, &ey));
            mx = fmaxf(mx, max4(t1[k]));
        }
    int e1 = 0;
    if (mx < scale_threshold<float>() && mx > 0.0f) {
        float f1, f2;
        pow2_factors(mx, &e1, &f1, &f2);
#pragma unroll
        for (int k = 0; k < CM; ++k) t1[k] = scale4(t1[k], f1, f2);
    }
    float lsum = 0.0f;
    int etot = ex + ey + e1;
    if (mv.kind == 0) {
        const int ru = mv.u - it.n_tips;
        const bool u_root = ru == it.n_int - 1;
        etot += u_root ? 0 : sEO[(size_t)ru * TILE + tid];
#pragma unroll
        for (int k = 0; k < CM; ++k)
            if (k < C) {
                const float4 a = pmv(iv.P + ((size_t)mv.v * C + k) * 16, t1[k]);
                const float4 z = message(iv, b, mv.z, k, site_c, tid, sD, sED, &ez);
                float4 o = u_root ? w.root : sO[((size_t)ru * C + k) * TILE + tid];
                o = make_float4(o.x * scale, o.y * scale, o.z * scale, o.w * scale);
                float lk = o.x * (a.x * z.x);
                lk = fmaf(o.y, a.y * z.y, lk);
                lk = fmaf(o.z, a.z * z.z, lk);
                lk = fmaf(o.w, a.w * z.w, lk);
                lsum = fmaf(w.cat[k], lk, lsum);
            }
        etot += ez;
    } else {
        const float4 pi = make_float4(w.root.x * scale, w.root.y * scale, w.root.z * scale, w.root.w * scale);
#pragma unroll
        for (int k = 0; k < CM; ++k)
            if (k < C) {
                const float4 a = pmv(iv.P + ((size_t)mv.v * C + k) * 16, t1[k]);
                const float4 t4 = mul4(message(iv, b, mv.p, k, site_c, tid, sD, sED, &ep),
                                       message(iv, b, mv.q, k, site_c, tid, sD, sED, &eq));
                const float4 c = pmv(iv.P + ((size_t)mv.c * C + k) * 16, t4);
                float lk = pi.x * (a.x * c.x);
                lk = fmaf(pi.y, a.y * c.y, lk);
                lk = fmaf(pi.z, a.z * c.z, lk);
                lk = fmaf(pi.w, a.w * c.w, lk);
                lsum = fmaf(w.cat[k], lk, lsum);
            }
        etot += ep + eq;
    }
    *etot_out = etot;
    return lsum;
}

// log L of one move at this thread's site as lm + ee ln 2, lm = log of the
// mantissa of L in [0, ln 2)
template <int CM>
__device__ __forceinline__ void move_site_log(const ItemView& iv, const BatchDev& b, const NniMoveDev& mv, int site_c,
                                              int tid, const float4* sD, const int* sED, const float4* sO,
                                              const int* sEO, const Weights32<CM>& w, float* lm, int* ee) {
    int etot;
    float l = move_site_l<CM>(iv, b, mv, site_c, tid, sD, sED, sO, sEO, w, 1.0f, &etot);
    if (!(l >= 1.17549435e-38f)) {  // below the normal range (or zero): again with 2^64 on the weights
        l = move_site_l<CM>(iv, b, mv, site_c, tid, sD, sED, sO, sEO, w, 1.8446744073709552e19f, &etot);
        etot -= 64;
    }
    const int bits = __float_as_int(l);
    *ee = etot + ((bits >> 23) & 255) - 127;
    *lm = logf(__int_as_float((bits & 0x007fffff) | 0x3f800000));
}

// registers capped for three CTAs per SM (168; a few bytes spill): with the
// tip codes read from global memory three CTAs fit beside each other
template <int CM, bool CODES_SMEM>
__global__ void __launch_bounds__(kPruneThreads, 3) batch_nni_kernel(BatchDev b) {
    extern __shared__ __align__(16) unsigned char sm[];
    __shared__ int s_unit;
    // per warp and move of a round: the warp's mantissa-log sum (FP32 TwoSum
    // pair) and exponent sum
    __shared__ float s_rh[kPruneThreads / 32][32], s_rl[kPruneThreads / 32][32];
    __shared__ int s_re[kPruneThreads / 32][32];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const size_t vec_slice = (size_t)b.scratch_int * b.C * TILE;
    const size_t int_slice = (size_t)b.scratch_int * TILE;
    float4* sD = b.scr_D + blockIdx.x * vec_slice;
    int* sED = b.scr_ED + blockIdx.x * int_slice;
    float4* sO = b.scr_O + blockIdx.x * vec_slice;
    int* sEO = b.scr_EO + blockIdx.x * int_slice;
    for (;;) {
        if (tid == 0) s_unit = atomicAdd(b.counter, 1);
        __syncthreads();
        const int u = s_unit;
        if (u >= b.n_units) break;
        const int2 unit = b.units[u];
        const BatchItemDev* itp = b.items + unit.x;
        const BatchItemDev it = *itp;
        ItemView iv;
        iv.it = &it;
        iv.P = b.P32 + (size_t)it.node_off * b.C * 16;
        iv.tipT = b.tip32 + (size_t)it.tip_off * b.C * kCodes * 4;
        iv.codes = b.codes + it.codes_off;
        iv.child = b.child + it.node_off;
        iv.root_w = b.model + it.model_off + 36;
        iv.cat_w = b.model + it.model_off + 40 + b.C;
        // phase A
        TileJob j;
        j.ops = b.ops + it.ops_off;
        j.n_ops = it.n_ops;
        j.codes = iv.codes;
        j.site_stride = it.site_stride;
        j.n_sites = it.n_sites;
        j.n_tips = it.n_tips;
        j.P = iv.P;
        j.tipT = iv.tipT;
        j.root_w = iv.root_w;
        j.cat_w = iv.cat_w;
        j.C = b.C;
        j.tile_base = unit.y * TILE;
        j.site_lnl = nullptr;
        j.max_depth = b.max_depth;
        DStore ds{sD, sED};
        SiteSum32 unused;  // untouched with STORE_D (no root)
        run_tile<CM, 1, CODES_SMEM, true>(j, sm, unused, &ds);
        // phases B and C touch only this thread's site column of the scratch
        const int site = j.tile_base + tid;
        const bool valid = site < it.n_sites;
        const int site_c = min(site, it.site_stride - 1);
        phase_b<CM>(iv, b, site_c, tid, sD, sED, sO, sEO);
        const long long out_off = b.unit_move_off[u];
        const Weights32<CM> w32 = weights32<CM>(iv, b.C);
        for (int m0 = 0; m0 < it.n_moves; m0 += 32) {
            const int mcount = min(32, it.n_moves - m0);
            for (int mi = 0; mi < mcount; ++mi) {
                const NniMoveDev mv = b.moves[it.moves_off + m0 + mi];
                float lm = 0.0f;
                int ee = 0;
                if (valid) move_site_log<CM>(iv, b, mv, site_c, tid, sD, sED, sO, sEO, w32, &lm, &ee);
                // the warp's mantissa logs with FP32 TwoSum, exponents exactly
                float hi = lm, lo = 0.0f;
                warp_two_sum_f(hi, lo);
                const int esum = __reduce_add_sync(0xffffffffu, ee);
                if (lane == 0) {
                    s_rh[warp][mi] = hi;
                    s_rl[warp][mi] = lo;
                    s_re[warp][mi] = esum;
                }
            }
            __syncthreads();
            if (tid < mcount) {
                // the warps in order, FP32 TwoSum and integer sums (FP64
                // chains here cost GB300 tens of cycles per instruction),
                // stored as the move's 16-byte record of this tile
                SiteSum32 t;
                for (int w = 0; w < kPruneThreads / 32; ++w) {
                    float ns, e;
                    two_sum_f(t.hi, s_rh[w][tid], ns, e);
                    t.hi = ns;
                    t.lo = __fadd_rn(t.lo, __fadd_rn(s_rl[w][tid], e));
                    t.ee += s_re[w][tid];
                }
                store_site_record(b.unit_move_sums, (size_t)(out_off + m0 + tid), t);
            }
            __syncthreads();
        }
    }
}

// one thread per (item, move): fold its tiles' records in site order (FP32
// TwoSum, integer exponents), lnL = ee ln 2 + hi + lo in FP64 at the end
__global__ void batch_nni_reduce_kernel(BatchDev b) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= b.total_moves) return;
    const int item = b.move_item[g];
    const BatchItemDev it = b.items[item];
    const int m = g - it.move_out_off;
    const float4* rec = reinterpret_cast<const float4*>(b.unit_move_sums);
    SiteSum32 t;
    for (int q = b.item_unit_ptr[item]; q < b.item_unit_ptr[item + 1]; ++q) {
        const int u = b.item_units[q];
        const float4 v = rec[b.unit_move_off[u] + m];
        float ns, e;
        two_sum_f(t.hi, v.x, ns, e);
        t.hi = ns;
        t.lo = __fadd_rn(t.lo, __fadd_rn(v.y, e));
        t.ee += __float_as_int(v.z);
    }
    b.nni_out[g] = fma((double)t.ee, 0.69314718055994530942, (double)t.hi + (double)t.lo);
}

// ---------------------------------------------------------------------------
// Branch-length derivatives (no counterpart in the reference, whose branch
// lengths are fixed inputs, src/tree.cpp:136, 176).  For the edge above v
// (parent u, sibling w) the site likelihood as a function of its length t is
//   L(t) = sum_k w_k A_k^T P(r_k t) c_k,   A_k = Out(u) x D_w,  c_k = cond(v),
// and with P(t) = L diag(exp(lambda t)) R (the model's eigen form)
//   L(t) = sum_k w_k sum_m a_km b_km exp(rho_km t),  rho_km = lambda_m r_k,
//   a_k = L^T A_k,  b_k = R c_k,
// so L' and L'' only weight the same terms by rho and rho^2.  Every site adds
// d1 = L'/L and d2 = L''/L - (L'/L)^2 (the first and second derivatives of its
// log likelihood; the power-of-two exponents cancel in the ratios).  Edge
// slot i of an item is child i % 2 of internal node n_tips + i / 2.
//
// All per-site arithmetic is FP32: the model's eigenvectors and rates are
// converted once per work unit and the factors exp(rho_km t) once per edge
// (shared memory), the ratios are IEEE FP32 divisions, and a warp's 32 site
// terms are summed with FP32 TwoSum before the FP64 sums across warps.
// ---------------------------------------------------------------------------
template <int CM>
struct BlenModel32 {
    float L[16], R[16];
    float rho[CM][4];
};
constexpr int kBlenSlots = 32;  // edge slots per pass over the tile

template <int CM>
__device__ void edge_site_derivs(const ItemView& iv, const BatchDev& b, int u, int v, int w, int site_c, int tid,
                                 const float4* sD, const int* sED, const float4* sO, const BlenModel32<CM>& mf,
                                 const float* ex, const float4& root32, const float* cat32, float* d1, float* d2) {
    const BatchItemDev& it = *iv.it;
    const int C = b.C;
    const bool u_root = (u - it.n_tips) == it.n_int - 1;
    // cond(v): a tip's state set, or the product of v's children's messages
    float4 cv[CM];
    int e = 0;
    if (v < it.n_tips) {
        const int code = iv.codes[(size_t)v * it.site_stride + site_c] & (kCodes - 1);
        const float4 m = make_float4((float)(code & 1), (float)((code >> 1) & 1), (float)((code >> 2) & 1),
                                     (float)((code >> 3) & 1));
#pragma unroll
        for (int k = 0; k < CM; ++k) cv[k] = m;
    } else {
        const int2 ch = iv.child[v];
#pragma unroll
        for (int k = 0; k < CM; ++k)
            if (k < C) {
                cv[k] = message(iv, b, ch.x, k, site_c, tid, sD, sED, &e);
                if (ch.y >= 0) cv[k] = mul4(cv[k], message(iv, b, ch.y, k, site_c, tid, sD, sED, &e));
            }
    }
    float l0 = 0.f, l1 = 0.f, l2 = 0.f;
#pragma unroll
    for (int k = 0; k < CM; ++k)
        if (k < C) {
            float4 A = u_root ? root32 : sO[((size_t)(u - it.n_tips) * C + k) * TILE + tid];
            if (w >= 0) A = mul4(A, message(iv, b, w, k, site_c, tid, sD, sED, &e));
            const float Av[4] = {A.x, A.y, A.z, A.w};
            const float cvv[4] = {cv[k].x, cv[k].y, cv[k].z, cv[k].w};
            float s0 = 0.f, s1 = 0.f, s2 = 0.f;
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                float a = 0.f, bb = 0.f;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    a = fmaf(Av[i], mf.L[i * 4 + m], a);
                    bb = fmaf(mf.R[m * 4 + i], cvv[i], bb);
                }
                const float rho = mf.rho[k][m];
                const float term = a * bb * ex[k * 4 + m];
                s0 += term;
                s1 = fmaf(rho, term, s1);
                s2 = fmaf(rho * rho, term, s2);
            }
            const float wk = cat32[k];
            l0 = fmaf(wk, s0, l0);
            l1 = fmaf(wk, s1, l1);
            l2 = fmaf(wk, s2, l2);
        }
    const float g = __fdiv_rn(l1, l0);
    *d1 = g;
    *d2 = __fsub_rn(__fdiv_rn(l2, l0), __fmul_rn(g, g));
}

// registers capped for three CTAs per SM, as batch_nni_kernel
template <int CM, bool CODES_SMEM>
__global__ void __launch_bounds__(kPruneThreads, 3) batch_blen_kernel(BatchDev b, BlenDev bd) {
    extern __shared__ __align__(16) unsigned char sm[];
    __shared__ int s_unit;
    __shared__ double s_red[kPruneThreads / 32][kBlenSlots][2];
    __shared__ BlenModel32<CM> s_mf;
    __shared__ float s_ex[kBlenSlots][CM * 4];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const size_t vec_slice = (size_t)b.scratch_int * b.C * TILE;
    const size_t int_slice = (size_t)b.scratch_int * TILE;
    float4* sD = b.scr_D + blockIdx.x * vec_slice;
    int* sED = b.scr_ED + blockIdx.x * int_slice;
    float4* sO = b.scr_O + blockIdx.x * vec_slice;
    int* sEO = b.scr_EO + blockIdx.x * int_slice;
    for (;;) {
        if (tid == 0) s_unit = atomicAdd(b.counter, 1);
        __syncthreads();
        const int u_idx = s_unit;
        if (u_idx >= b.n_units) break;
        const int2 unit = b.units[u_idx];
        const BatchItemDev it = b.items[unit.x];
        ItemView iv;
        iv.it = &it;
        iv.P = b.P32 + (size_t)it.node_off * b.C * 16;
        iv.tipT = b.tip32 + (size_t)it.tip_off * b.C * kCodes * 4;
        iv.codes = b.codes + it.codes_off;
        iv.child = b.child + it.node_off;
        iv.root_w = b.model + it.model_off + 36;
        iv.cat_w = b.model + it.model_off + 40 + b.C;
        const double* mdl = b.model + it.model_off;
        // the item's model in FP32: eigenvectors, rates rho_km = lambda_m r_k
        if (tid < 16) {
            s_mf.L[tid] = (float)mdl[4 + tid];
            s_mf.R[tid] = (float)mdl[20 + tid];
        } else if (tid < 16 + CM * 4) {
            const int k = (tid - 16) / 4, m = (tid - 16) % 4;
            s_mf.rho[k][m] = k < b.C ? (float)(mdl[m] * mdl[40 + k]) : 0.0f;
        }
        TileJob j;
        j.ops = b.ops + it.ops_off;
        j.n_ops = it.n_ops;
        j.codes = iv.codes;
        j.site_stride = it.site_stride;
        j.n_sites = it.n_sites;
        j.n_tips = it.n_tips;
        j.P = iv.P;
        j.tipT = iv.tipT;
        j.root_w = iv.root_w;
        j.cat_w = iv.cat_w;
        j.C = b.C;
        j.tile_base = unit.y * TILE;
        j.site_lnl = nullptr;
        j.max_depth = b.max_depth;
        DStore ds{sD, sED};
        SiteSum32 unused;  // untouched with STORE_D (no root)
        run_tile<CM, 1, CODES_SMEM, true>(j, sm, unused, &ds);
        const int site = j.tile_base + tid;
        const bool valid = site < it.n_sites;
        const int site_c = min(site, it.site_stride - 1);
        phase_b<CM>(iv, b, site_c, tid, sD, sED, sO, sEO);
        const Weights32<CM> w32 = weights32<CM>(iv, b.C);
        const BlenModel32<CM>& mf = s_mf;
        const long long out_off = bd.unit_edge_off[u_idx];
        const int n_slots = 2 * it.n_int;
        for (int s0 = 0; s0 < n_slots; s0 += kBlenSlots) {
            const int count = min(kBlenSlots, n_slots - s0);
            // exp(rho_km t) of every edge of this pass
            for (int q = tid; q < count * CM * 4; q += kPruneThreads) {
                const int si = q / (CM * 4), km = q % (CM * 4);
                const int slot = s0 + si;
                const int2 ch = iv.child[it.n_tips + slot / 2];
                const int v = (slot % 2 == 0) ? ch.x : ch.y;
                const float t = v >= 0 ? (float)b.t_eff[it.node_off + v] : 0.0f;
                s_ex[si][km] = expf(mf.rho[km / 4][km % 4] * t);
            }
            __syncthreads();
            for (int si = 0; si < count; ++si) {
                const int slot = s0 + si;
                const int u = it.n_tips + slot / 2;
                const int2 ch = iv.child[u];
                const int v = (slot % 2 == 0) ? ch.x : ch.y;
                const int w = (slot % 2 == 0) ? ch.y : ch.x;
                float d1 = 0.0f, d2 = 0.0f;
                if (valid && v >= 0)
                    edge_site_derivs<CM>(iv, b, u, v, w, site_c, tid, sD, sED, sO, mf, s_ex[si], w32.root, w32.cat,
                                         &d1, &d2);
                float c1 = 0.0f, c2 = 0.0f;
                warp_two_sum_f(d1, c1);
                warp_two_sum_f(d2, c2);
                if (lane == 0) {
                    s_red[warp][si][0] = (double)d1 + (double)c1;
                    s_red[warp][si][1] = (double)d2 + (double)c2;
                }
            }
            __syncthreads();
            if (tid < count) {
                double a = 0.0, c = 0.0;
                for (int q = 0; q < kPruneThreads / 32; ++q) {
                    a += s_red[q][tid][0];
                    c += s_red[q][tid][1];
                }
                bd.unit_edge_sums[2 * (out_off + s0 + tid)] = a;
                bd.unit_edge_sums[2 * (out_off + s0 + tid) + 1] = c;
            }
            __syncthreads();
        }
    }
}

// one thread per (item, edge slot): the item's units in site order
__global__ void batch_blen_reduce_kernel(BatchDev b, BlenDev bd) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= bd.total_slots) return;
    const int item = bd.edge_item[g];
    const int slot = g - bd.item_edge_off[item];
    double a = 0.0, c = 0.0;
    for (int q = b.item_unit_ptr[item]; q < b.item_unit_ptr[item + 1]; ++q) {
        const int u = b.item_units[q];
        const double* p = bd.unit_edge_sums + 2 * (bd.unit_edge_off[u] + slot);
        a += p[0];
        c += p[1];
    }
    bd.edge_out[2 * g] = a;
    bd.edge_out[2 * g + 1] = c;
}

template <int CM, bool CODES_SMEM>
cudaError_t launch_blen_t(const BatchDev& b, const BlenDev& bd, int grid, size_t smem, cudaStream_t st) {
    auto kern = batch_blen_kernel<CM, CODES_SMEM>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<grid, kPruneThreads, smem, st>>>(b, bd);
    return cudaGetLastError();
}

template <int CM, bool CODES_SMEM>
cudaError_t launch_nni_t(const BatchDev& b, int grid, size_t smem, cudaStream_t st) {
    auto kern = batch_nni_kernel<CM, CODES_SMEM>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<grid, kPruneThreads, smem, st>>>(b);
    return cudaGetLastError();
}

}  // namespace

size_t nni_smem_bytes(int C, bool codes_smem, int max_ops, int max_tips, int max_depth) {
    const int cm = C == 1 ? 1 : (C <= 4 ? 4 : 8);
    if (cm == 1) return codes_smem ? tile_smem_bytes<1, 1, true, true>(max_ops, max_tips, max_depth)
                                   : tile_smem_bytes<1, 1, false, true>(max_ops, max_tips, max_depth);
    if (cm == 4) return codes_smem ? tile_smem_bytes<4, 1, true, true>(max_ops, max_tips, max_depth)
                                   : tile_smem_bytes<4, 1, false, true>(max_ops, max_tips, max_depth);
    return codes_smem ? tile_smem_bytes<8, 1, true, true>(max_ops, max_tips, max_depth)
                      : tile_smem_bytes<8, 1, false, true>(max_ops, max_tips, max_depth);
}

template <typename K>
int occupancy_of(K kern, size_t smem) {
    int n = 0;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, kPruneThreads, smem) != cudaSuccess) return 0;
    return n;
}

int nni_occupancy(int C, bool codes_smem, size_t smem, bool blen) {
    const int cm = C == 1 ? 1 : (C <= 4 ? 4 : 8);
    if (blen) {
        if (cm == 1) return codes_smem ? occupancy_of(batch_blen_kernel<1, true>, smem) : occupancy_of(batch_blen_kernel<1, false>, smem);
        if (cm == 4) return codes_smem ? occupancy_of(batch_blen_kernel<4, true>, smem) : occupancy_of(batch_blen_kernel<4, false>, smem);
        return codes_smem ? occupancy_of(batch_blen_kernel<8, true>, smem) : occupancy_of(batch_blen_kernel<8, false>, smem);
    }
    if (cm == 1) return codes_smem ? occupancy_of(batch_nni_kernel<1, true>, smem) : occupancy_of(batch_nni_kernel<1, false>, smem);
    if (cm == 4) return codes_smem ? occupancy_of(batch_nni_kernel<4, true>, smem) : occupancy_of(batch_nni_kernel<4, false>, smem);
    return codes_smem ? occupancy_of(batch_nni_kernel<8, true>, smem) : occupancy_of(batch_nni_kernel<8, false>, smem);
}

cudaError_t launch_batch_nni(const BatchDev& b, bool codes_smem, int grid, size_t smem, cudaStream_t st) {
    const int cm = b.C == 1 ? 1 : (b.C <= 4 ? 4 : 8);
    if (cm == 1) return codes_smem ? launch_nni_t<1, true>(b, grid, smem, st) : launch_nni_t<1, false>(b, grid, smem, st);
    if (cm == 4) return codes_smem ? launch_nni_t<4, true>(b, grid, smem, st) : launch_nni_t<4, false>(b, grid, smem, st);
    return codes_smem ? launch_nni_t<8, true>(b, grid, smem, st) : launch_nni_t<8, false>(b, grid, smem, st);
}

cudaError_t launch_batch_blen(const BatchDev& b, const BlenDev& bd, bool codes_smem, int grid, size_t smem,
                              cudaStream_t st) {
    const int cm = b.C == 1 ? 1 : (b.C <= 4 ? 4 : 8);
    if (cm == 1) return codes_smem ? launch_blen_t<1, true>(b, bd, grid, smem, st) : launch_blen_t<1, false>(b, bd, grid, smem, st);
    if (cm == 4) return codes_smem ? launch_blen_t<4, true>(b, bd, grid, smem, st) : launch_blen_t<4, false>(b, bd, grid, smem, st);
    return codes_smem ? launch_blen_t<8, true>(b, bd, grid, smem, st) : launch_blen_t<8, false>(b, bd, grid, smem, st);
}

cudaError_t launch_batch_blen_reduce(const BatchDev& b, const BlenDev& bd, cudaStream_t st) {
    if (bd.total_slots == 0) return cudaSuccess;
    const int threads = 128;
    batch_blen_reduce_kernel<<<(bd.total_slots + threads - 1) / threads, threads, 0, st>>>(b, bd);
    return cudaGetLastError();
}

cudaError_t launch_batch_nni_reduce(const BatchDev& b, cudaStream_t st) {
    if (b.total_moves == 0) return cudaSuccess;
    const int threads = 128;
    batch_nni_reduce_kernel<<<(b.total_moves + threads - 1) / threads, threads, 0, st>>>(b);
    return cudaGetLastError();
}

}  // namespace plk
