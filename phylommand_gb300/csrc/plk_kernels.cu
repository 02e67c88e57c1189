// Device code of libplk (sm_103a).
//
//  pmat_kernel      P(t) for every (edge, category): the reference's
//                   Taylor-plus-20-squarings (src/marth/marth.cpp:129-140),
//                   an eigen form for reversible Q, or scaling-and-squaring
//                   for non-reversible Q; FP64, plus FP32 copies and the
//                   per-tip-edge lookup tables (P times each tip state set).
//  prune4_kernel    post-order pass for 4 states (src/simpleML.cpp:127-197):
//                   one thread per site walks the whole register-allocated
//                   op list; partial vectors live in registers, spills in a
//                   per-thread shared-memory stack; per-site power-of-two
//                   scaling; root reduction (src/simpleML.h:123-141) fused;
//                   compensated block sums of the per-site lnL, added up by
//                   the grid's last CTA (finish_grid_sum).
//  prune_generic    the same pass for any state count (<= 24), vectors in a
//                   global work buffer.
//  preorder_kernel  outside vectors from the root down and normalised
//                   marginal posteriors (absent in the reference).
#include <cstdio>
#include <type_traits>

#include "plk_device.cuh"
#include "plk_internal.h"
#include "plk_prune4p.cuh"

namespace plk {

using namespace dev;

// =========================================================================
// P(t)
// =========================================================================
constexpr int kPmatOut = 4;  // P(t) entries per thread at most (see launch_pmat)

// FP32 to TF32, round to nearest with ties away from zero (the tcgen05 B images)
__device__ __forceinline__ float tf32_rna_dev(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__global__ void pmat_kernel(DeviceModel m, int p_kind) {
    // a pass launched after it with programmatic stream serialization may be
    // scheduled now (it waits for this kernel's completion before reading)
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
    const int v = blockIdx.x / m.C, k = blockIdx.x % m.C;
    const int S = m.S, SS = S * S;
    extern __shared__ double pm_smem[];
    double* A = pm_smem;
    double* B = pm_smem + SS;
    double* X = pm_smem + 2 * SS;  // eigen exponentials / series term
    const double t = __dmul_rn(m.t_eff[v], m.cat_rate[k]);
    if (p_kind == 0) {
        // A = I + (Q t) / 2^20, then 20 squarings with prod[i][j] summed
        // over k ascending from 0, every operation rounded on its own.
        for (int idx = threadIdx.x; idx < SS; idx += blockDim.x) {
            const int i = idx / S, j = idx % S;
            const double q = __ddiv_rn(__dmul_rn(m.Q[idx], t), 1048576.0);
            A[idx] = (i == j) ? __dadd_rn(1.0, q) : q;
        }
        __syncthreads();
        for (int it = 0; it < 20; ++it) {
            for (int idx = threadIdx.x; idx < SS; idx += blockDim.x) {
                const int i = idx / S, j = idx % S;
                double acc = __dmul_rn(A[i * S], A[j]);
                for (int kk = 1; kk < S; ++kk) acc = __dadd_rn(acc, __dmul_rn(A[i * S + kk], A[kk * S + j]));
                B[idx] = acc;
            }
            __syncthreads();
            double* tmp = A; A = B; B = tmp;
        }
    } else if (p_kind == 1) {
        // P = L diag(exp(lambda t)) R with L diag(.) and R staged in shared
        // memory (B: the exponentials, X: L diag(.), A: R, then P); each
        // product rounded before its FMA, as in the oracle
        for (int i = threadIdx.x; i < S; i += blockDim.x) B[i] = exp(m.eig_lam[i] * t);
        for (int idx = threadIdx.x; idx < SS; idx += blockDim.x) A[idx] = m.eig_R[idx];
        __syncthreads();
        for (int idx = threadIdx.x; idx < SS; idx += blockDim.x) X[idx] = m.eig_L[idx] * B[idx % S];
        __syncthreads();
        // launch_pmat gives every thread at most kPmatOut entries (S <= 24:
        // 576 entries over 256 threads, < 256 over 64, < 64 over 32)
        double out[kPmatOut];
#pragma unroll
        for (int r = 0; r < kPmatOut; ++r) {
            const int idx = threadIdx.x + r * blockDim.x;
            if (idx < SS) {
                const int i = idx / S, j = idx % S;
                double acc = 0.0;
                for (int mm = 0; mm < S; ++mm) acc = fma(X[i * S + mm], A[mm * S + j], acc);
                out[r] = acc;
            }
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kPmatOut; ++r) {
            const int idx = threadIdx.x + r * blockDim.x;
            if (idx < SS) A[idx] = out[r];
        }
        __syncthreads();
    } else {
        // scaling and squaring: A0 = Q t 2^-s with ||A0|| <= 1/8, Taylor to 18
        __shared__ int s_sq;
        if (threadIdx.x == 0) {
            double norm = 0.0;
            for (int i = 0; i < S; ++i) {
                double r = 0.0;
                for (int j = 0; j < S; ++j) r += fabs(m.Q[i * S + j] * t);
                norm = fmax(norm, r);
            }
            int s = 0;
            while (norm > 0.125 && s < 1000) { norm *= 0.5; ++s; }
            s_sq = s;
        }
        __syncthreads();
        const int s = s_sq;
        const double f = ldexp(t, -s);
        double* term = X;   // needs SS doubles
        for (int idx = threadIdx.x; idx < SS; idx += blockDim.x) {
            const int i = idx / S, j = idx % S;
            term[idx] = (i == j) ? 1.0 : 0.0;
            A[idx] = term[idx];
        }
        __syncthreads();
        for (int mm = 1; mm <= 18; ++mm) {
            for (int idx = threadIdx.x; idx < SS; idx += blockDim.x) {
                const int i = idx / S, j = idx % S;
                double acc = 0.0;
                for (int kk = 0; kk < S; ++kk) acc = fma(term[i * S + kk], m.Q[kk * S + j] * f, acc);
                B[idx] = acc / mm;
            }
            __syncthreads();
            for (int idx = threadIdx.x; idx < SS; idx += blockDim.x) {
                term[idx] = B[idx];
                A[idx] += B[idx];
            }
            __syncthreads();
        }
        for (int it = 0; it < s; ++it) {
            for (int idx = threadIdx.x; idx < SS; idx += blockDim.x) {
                const int i = idx / S, j = idx % S;
                double acc = 0.0;
                for (int kk = 0; kk < S; ++kk) acc = fma(A[i * S + kk], A[kk * S + j], acc);
                B[idx] = acc;
            }
            __syncthreads();
            double* tmp = A; A = B; B = tmp;
        }
    }
    const size_t base = ((size_t)v * m.C + k) * SS;
    for (int idx = threadIdx.x; idx < SS; idx += blockDim.x) {
        m.P64[base + idx] = A[idx];
        m.P32[base + idx] = (float)A[idx];
        if (m.P32p) m.P32p[(size_t)v * m.C * 16 + paired_p_index(k, idx / 4, idx % 4)] = (float)A[idx];
    }
    if (m.B20 && S == 20 && m.b20_bf16) {
        // the split-BF16 image (bf16_image_index), in the first 4 KB of the slot
        uint32_t* Bw = reinterpret_cast<uint32_t*>(m.B20 + ((size_t)v * m.C + k) * 1536);
        for (int w = threadIdx.x; w < kB16Bytes / 4; w += blockDim.x) {
            int part, i, j0;
            bf16_image_index(w, part, i, j0);
            const float x0 = (i < 20 && j0 < 20) ? (float)A[i * 20 + j0] : 0.0f;
            const float x1 = (i < 20 && j0 + 1 < 20) ? (float)A[i * 20 + j0 + 1] : 0.0f;
            uint32_t hi, lo;
            bf16_split2(x0, x1, hi, lo);
            Bw[w] = part == 0 ? hi : lo;
        }
    } else if (m.B20 && S == 20) {
        // the tcgen05 B-operand image of this (node, category): [part][4-column
        // group g][8-row block nb][row r][column c], state i = 8 nb + r, j =
        // 4 g + c, TF32 hi and lo parts of the FP32 P (zero outside 20 x 20),
        // as relayout20u_kernel writes it
        float* Bv = m.B20 + ((size_t)v * m.C + k) * 1536;
        for (int w = threadIdx.x; w < 1536; w += blockDim.x) {
            const int part = w / 768, q = w % 768;
            const int g = q / 128, nb = (q / 32) % 4, r = (q / 4) % 8, c = q % 4;
            const int i = 8 * nb + r, j = 4 * g + c;
            float val = 0.0f;
            if (i < 20 && j < 20) {
                const float x = (float)A[i * 20 + j];
                const float hi = tf32_rna_dev(x);
                val = part == 0 ? hi : tf32_rna_dev(x - hi);
            }
            Bv[w] = val;
        }
    }
    if (v < m.n_tips) {
        // table[code][i] = sum over allowed j (ascending) of P[i][j]: what
        // branch_likelihood gives for a 0/1 tip vector (0 * P adds nothing).
        const size_t tb = ((size_t)v * m.C + k) * m.n_codes * S;
        for (int idx = threadIdx.x; idx < m.n_codes * S; idx += blockDim.x) {
            const int c = idx / S, i = idx % S;
            const uint32_t mask = m.code_mask ? m.code_mask[c] : (uint32_t)c;
            double acc = 0.0;
            bool first = true;
            for (int j = 0; j < S; ++j)
                if ((mask >> j) & 1u) {
                    acc = first ? A[i * S + j] : __dadd_rn(acc, A[i * S + j]);
                    first = false;
                }
            m.tip64[tb + idx] = acc;
            m.tip32[tb + idx] = (float)acc;
            if (m.tip32p) m.tip32p[(size_t)v * m.C * kCodes * 4 + paired_tip_index(k, c, i)] = (float)acc;
            if (m.T20) m.T20[((size_t)v * m.C + k) * (20 * m.ncs20) + (size_t)i * m.ncs20 + c] = (float)acc;
        }
        if (m.T20) {  // the padding codes of every state row
            const int pad = m.ncs20 - m.n_codes;
            for (int idx = threadIdx.x; idx < 20 * pad; idx += blockDim.x)
                m.T20[((size_t)v * m.C + k) * (20 * m.ncs20) + (size_t)(idx / pad) * m.ncs20 + m.n_codes + idx % pad] =
                    0.0f;
        }
    }
}

// P(t) of the eigen form for 4 states, eight (node, category) matrices per
// warp: lane 4 w + r of a warp holds row r of matrix w.  GB300 retires a
// warp-wide FP64 instruction at a small fraction of the FP32 rate whatever
// the number of active lanes, so the one-matrix-per-CTA kernel spent most
// of its time in FP64 instructions with 4 or 16 of 32 lanes busy.  Here
// every FP64 instruction works on 32 lanes, with the operations and their
// order of pmat_kernel (p_kind 1), so P(t) and the tip tables keep their
// bits: e_m = exp(lambda_m t) (lane m of the matrix), X[r][m] = L[r][m] e_m,
// P[r][j] = fma over m ascending from 0, tips summed over the allowed
// states j ascending.
__global__ void __launch_bounds__(128) pmat4_eigen_kernel(DeviceModel m) {
    // the post-order pass after it may be scheduled now (it waits for this
    // kernel's completion before reading the tables)
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
    const int lane = threadIdx.x & 31;
    const int item = (blockIdx.x * blockDim.x + threadIdx.x) >> 2;  // (node, category)
    const int r = lane & 3;
    const int n_items = m.n_nodes * m.C;
    const bool live = item < n_items;
    const int it = live ? item : n_items - 1;  // lanes past the end repeat the last item, store nothing
    const int v = it / m.C, k = it % m.C;
    const double t = __dmul_rn(m.t_eff[v], m.cat_rate[k]);
    const double e_own = exp(m.eig_lam[r] * t);
    double e[4];
#pragma unroll
    for (int mm = 0; mm < 4; ++mm) e[mm] = __shfl_sync(0xffffffffu, e_own, (lane & ~3) | mm);
    double x[4], p[4];
#pragma unroll
    for (int mm = 0; mm < 4; ++mm) x[mm] = m.eig_L[r * 4 + mm] * e[mm];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        double acc = 0.0;
#pragma unroll
        for (int mm = 0; mm < 4; ++mm) acc = fma(x[mm], m.eig_R[mm * 4 + j], acc);
        p[j] = acc;
    }
    if (!live) return;
    const size_t base = (size_t)it * 16 + r * 4;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        m.P64[base + j] = p[j];
        m.P32[base + j] = (float)p[j];
        if (m.P32p) m.P32p[(size_t)v * m.C * 16 + paired_p_index(k, r, j)] = (float)p[j];
    }
    if (v < m.n_tips && m.code_mask == nullptr && m.n_codes == kCodes) {
        // the 16 state sets themselves as codes: every mask known at compile
        // time, so the 16 sums are straight-line and independent
        const size_t tb = (size_t)it * kCodes * 4;
#pragma unroll
        for (int c = 0; c < kCodes; ++c) {
            double acc = 0.0;
            bool first = true;
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if ((c >> j) & 1) {
                    acc = first ? p[j] : __dadd_rn(acc, p[j]);
                    first = false;
                }
            m.tip64[tb + (size_t)c * 4 + r] = acc;
            m.tip32[tb + (size_t)c * 4 + r] = (float)acc;
            if (m.tip32p) m.tip32p[(size_t)v * m.C * kCodes * 4 + paired_tip_index(k, c, r)] = (float)acc;
        }
    } else if (v < m.n_tips) {
        const size_t tb = (size_t)it * m.n_codes * 4;
        for (int c = 0; c < m.n_codes; ++c) {
            const uint32_t mask = m.code_mask ? m.code_mask[c] : (uint32_t)c;
            double acc = 0.0;
            bool first = true;
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if ((mask >> j) & 1u) {
                    acc = first ? p[j] : __dadd_rn(acc, p[j]);
                    first = false;
                }
            m.tip64[tb + (size_t)c * 4 + r] = acc;
            m.tip32[tb + (size_t)c * 4 + r] = (float)acc;
            if (m.tip32p) m.tip32p[(size_t)v * m.C * kCodes * 4 + paired_tip_index(k, c, r)] = (float)acc;
        }
    }
}

cudaError_t launch_pmat(const DeviceModel& m, int p_kind, cudaStream_t st) {
    if (m.S == 4 && p_kind == 1 && m.B20 == nullptr) {
        const int lanes = m.n_nodes * m.C * 4;
        pmat4_eigen_kernel<<<(lanes + 127) / 128, 128, 0, st>>>(m);
        return cudaGetLastError();
    }
    const int SS = m.S * m.S;
    const size_t smem = sizeof(double) * (size_t)(3 * SS);
    const int threads = SS >= 256 ? 256 : (SS >= 64 ? 64 : 32);
    if ((SS + threads - 1) / threads > kPmatOut) return cudaErrorInvalidConfiguration;
    pmat_kernel<<<m.n_nodes * m.C, threads, smem, st>>>(m, p_kind);
    return cudaGetLastError();
}

// =========================================================================
// Post-order pass, 4 states
// =========================================================================
namespace {

template <typename T, bool EXACT>
__device__ __forceinline__ void matvec4(const T* __restrict__ Pm, const T x[4], T out[4]) {
    const V4<T>* rows = reinterpret_cast<const V4<T>*>(Pm);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const V4<T> r = rows[i];
        if (EXACT) {
            T acc = mul_rn(x[0], r.v[0]);
            acc = add_rn(acc, mul_rn(x[1], r.v[1]));
            acc = add_rn(acc, mul_rn(x[2], r.v[2]));
            acc = add_rn(acc, mul_rn(x[3], r.v[3]));
            out[i] = acc;
        } else {
            T acc = x[0] * r.v[0];
            acc = fma(x[1], r.v[1], acc);
            acc = fma(x[2], r.v[2], acc);
            acc = fma(x[3], r.v[3], acc);
            out[i] = acc;
        }
    }
}

template <typename T, int CM, bool EXACT, bool STORE>
__global__ void __launch_bounds__(kPruneThreads) prune4_kernel(PruneArgs a) {
    extern __shared__ __align__(32) unsigned char pr_smem[];
    Op* s_ops = reinterpret_cast<Op*>(pr_smem);
    V4<T>* s_stack = reinterpret_cast<V4<T>*>(pr_smem + (((size_t)a.n_ops * sizeof(Op) + 31) & ~(size_t)31));
    for (int i = threadIdx.x; i < a.n_ops; i += blockDim.x) s_ops[i] = a.ops[i];
    __syncthreads();

    const int C = a.C;
    const int site = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = site < a.n_sites;
    const int cs = site;
    const T* __restrict__ P = static_cast<const T*>(a.P);
    const T* __restrict__ tipT = static_cast<const T*>(a.tipT);
    const uint8_t* __restrict__ codes = a.codes;
    T acc[CM][4];
#pragma unroll
    for (int k = 0; k < CM; ++k)
#pragma unroll
        for (int i = 0; i < 4; ++i) acc[k][i] = T(1);
    int scale_e = 0;
    int sp = 0;
    const int nthr = blockDim.x;

    for (int o = 0; valid && o < a.n_ops; ++o) {
        const Op op = s_ops[o];
        T d0[CM][4], d1[CM][4];
        // ---- first child vector
        if (op.s0 >= 0) {
            const int code = codes[(size_t)op.s0 * a.site_stride + cs] & (kCodes - 1);  // streamed codes: raw bytes
#pragma unroll
            for (int k = 0; k < CM; ++k)
                if (k < C) {
                    const V4<T> tv = *reinterpret_cast<const V4<T>*>(
                        tipT + (((size_t)op.s0 * C + k) * a.n_codes + code) * 4);
#pragma unroll
                    for (int i = 0; i < 4; ++i) d0[k][i] = tv.v[i];
                }
        } else {
            if (op.s0 == kSrcPop) --sp;
#pragma unroll
            for (int k = 0; k < CM; ++k)
                if (k < C) {
                    T x[4];
                    if (op.s0 == kSrcPop) {
                        const V4<T> sv = s_stack[((size_t)sp * CM + k) * nthr + threadIdx.x];
#pragma unroll
                        for (int i = 0; i < 4; ++i) x[i] = sv.v[i];
                    } else {
#pragma unroll
                        for (int i = 0; i < 4; ++i) x[i] = acc[k][i];
                    }
                    matvec4<T, EXACT>(P + ((size_t)op.e0 * C + k) * 16, x, d0[k]);
                }
        }
        // ---- second child vector
        if (op.s1 >= 0) {
            const int code = codes[(size_t)op.s1 * a.site_stride + cs] & (kCodes - 1);
#pragma unroll
            for (int k = 0; k < CM; ++k)
                if (k < C) {
                    const V4<T> tv = *reinterpret_cast<const V4<T>*>(
                        tipT + (((size_t)op.s1 * C + k) * a.n_codes + code) * 4);
#pragma unroll
                    for (int i = 0; i < 4; ++i) d1[k][i] = tv.v[i];
                }
        } else if (op.s1 == kSrcAcc) {
#pragma unroll
            for (int k = 0; k < CM; ++k)
                if (k < C) matvec4<T, EXACT>(P + ((size_t)op.e1 * C + k) * 16, acc[k], d1[k]);
        }
        // ---- combine: left assigns, right multiplies (commutative)
        if (op.s1 == kSrcNone) {
#pragma unroll
            for (int k = 0; k < CM; ++k)
#pragma unroll
                for (int i = 0; i < 4; ++i) acc[k][i] = d0[k][i];
        } else {
#pragma unroll
            for (int k = 0; k < CM; ++k)
#pragma unroll
                for (int i = 0; i < 4; ++i) acc[k][i] = EXACT ? mul_rn(d0[k][i], d1[k][i]) : d0[k][i] * d1[k][i];
        }
        // ---- per-site power-of-two scaling (exact)
        T mx = T(0);
#pragma unroll
        for (int k = 0; k < CM; ++k)
            if (k < C)
#pragma unroll
                for (int i = 0; i < 4; ++i) mx = fmax(mx, acc[k][i]);
        if (mx < scale_threshold<T>() && mx > T(0)) {
            int e;
            T f1, f2;
            pow2_factors(mx, &e, &f1, &f2);
#pragma unroll
            for (int k = 0; k < CM; ++k)
#pragma unroll
                for (int i = 0; i < 4; ++i) acc[k][i] = (acc[k][i] * f1) * f2;
            scale_e += e;
        }
        if (STORE) {
            T* cond = static_cast<T*>(a.cond);
#pragma unroll
            for (int k = 0; k < CM; ++k)
                if (k < C) {
                    V4<T> w;
#pragma unroll
                    for (int i = 0; i < 4; ++i) w.v[i] = acc[k][i];
                    *reinterpret_cast<V4<T>*>(cond + (((size_t)op.rank * C + k) * a.n_sites + site) * 4) = w;
                }
        }
        if (op.push) {
#pragma unroll
            for (int k = 0; k < CM; ++k)
                if (k < C) {
                    V4<T> w;
#pragma unroll
                    for (int i = 0; i < 4; ++i) w.v[i] = acc[k][i];
                    s_stack[((size_t)sp * CM + k) * nthr + threadIdx.x] = w;
                }
            ++sp;
        }
    }
    if constexpr (std::is_same<T, float>::value) {
        // ---- root in FP32 and its log as lm + ee ln 2 (site_log32), in the
        // operation order of run_tile: the same per-site bits as the staged
        // kernels
        float lsum = 0.0f;
#pragma unroll
        for (int k = 0; k < CM; ++k)
            if (k < C) {
                float lk = acc[k][0] * (float)a.root_w[0];
#pragma unroll
                for (int s = 1; s < 4; ++s) lk = fmaf(acc[k][s], (float)a.root_w[s], lk);
                lsum = fmaf((float)a.cat_w[k], lk, lsum);
            }
        SiteSum32 sum;
        if (valid) {
            float lm;
            int ee;
            site_log32(lsum, scale_e, lm, ee);
            a.site_lnl[site] = site_lnl64(lm, ee);
            site_sum_add(sum, lm, ee);
        }
        const SiteSum32 bsum = block_sum_site32f(sum);
        if (threadIdx.x == 0) store_site_record(a.block_sum, blockIdx.x, bsum);
    } else {
        // ---- root: sum_k w_k sum_s L[s] * root_w[s]
        double lsum = 0.0;
#pragma unroll
        for (int k = 0; k < CM; ++k)
            if (k < C) {
                double lk;
                if (EXACT) {
                    lk = __dmul_rn((double)acc[k][0], a.root_w[0]);
#pragma unroll
                    for (int s = 1; s < 4; ++s) lk = __dadd_rn(lk, __dmul_rn((double)acc[k][s], a.root_w[s]));
                    lsum = (k == 0) ? __dmul_rn(a.cat_w[0], lk) : __dadd_rn(lsum, __dmul_rn(a.cat_w[k], lk));
                } else {
                    lk = (double)acc[k][0] * a.root_w[0];
#pragma unroll
                    for (int s = 1; s < 4; ++s) lk = fma((double)acc[k][s], a.root_w[s], lk);
                    lsum = fma(a.cat_w[k], lk, lsum);
                }
            }
        const double lnl = valid ? log(lsum) + (double)scale_e * 0.69314718055994530942 : 0.0;
        if (valid) a.site_lnl[site] = lnl;
        // ---- compensated block reduction
        double s = valid ? lnl : 0.0, c = 0.0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const double os = __shfl_down_sync(0xffffffffu, s, off);
            const double oc = __shfl_down_sync(0xffffffffu, c, off);
            double ns, e;
            two_sum(s, os, ns, e);
            s = ns;
            c = c + oc + e;
        }
        __shared__ double red_s[32], red_c[32];
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        if (lane == 0) { red_s[warp] = s; red_c[warp] = c; }
        __syncthreads();
        if (warp == 0) {
            const int nw = blockDim.x >> 5;
            s = lane < nw ? red_s[lane] : 0.0;
            c = lane < nw ? red_c[lane] : 0.0;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const double os = __shfl_down_sync(0xffffffffu, s, off);
                const double oc = __shfl_down_sync(0xffffffffu, c, off);
                double ns, e;
                two_sum(s, os, ns, e);
                s = ns;
                c = c + oc + e;
            }
            if (lane == 0) {
                a.block_sum[2 * blockIdx.x] = s;
                a.block_sum[2 * blockIdx.x + 1] = c;
            }
        }
    }
    if (a.grid_done) {  // FP32: SiteSum32 records; FP64: compensated pairs
        if constexpr (std::is_same<T, float>::value) finish_grid_sum32(a.block_sum, a.grid_done, a.lnl_out);
        else finish_grid_sum(a.block_sum, a.grid_done, a.lnl_out);
    }
}

}  // namespace

// =========================================================================
// Post-order pass, any state count: vectors in a global work buffer laid
// out [rank][k][site][S]; one thread per site.
// =========================================================================
namespace {

struct GenericArgs {
    PruneArgs a;
    const int* order;
    const int* left;
    const int* right;
    const int* rank;
    int n_int, n_tips, S;
};

template <typename T, bool EXACT>
__device__ __forceinline__ void child_vec_generic(const GenericArgs& g, int v, int k, int site,
                                                  int cs, const T* work, const T* P, T* out) {
    const PruneArgs& a = g.a;
    const int S = g.S, C = a.C;
    if (v < g.n_tips) {
        int code = a.codes[(size_t)v * a.site_stride + cs];
        if (S <= 4) code &= (1 << S) - 1;  // state sets (a streamed alignment's codes are the caller's bytes)
        const T* tv = static_cast<const T*>(a.tipT) + (((size_t)v * C + k) * a.n_codes + code) * S;
        for (int i = 0; i < S; ++i) out[i] = tv[i];
        return;
    }
    const T* x = work + (((size_t)g.rank[v] * C + k) * a.n_sites + site) * S;
    const T* Pm = P + ((size_t)v * C + k) * S * S;
    for (int i = 0; i < S; ++i) {
        T acc;
        if (EXACT) {
            acc = mul_rn(x[0], Pm[i * S]);
            for (int j = 1; j < S; ++j) acc = add_rn(acc, mul_rn(x[j], Pm[i * S + j]));
        } else {
            acc = x[0] * Pm[i * S];
            for (int j = 1; j < S; ++j) acc = fma(x[j], Pm[i * S + j], acc);
        }
        out[i] = acc;
    }
}

template <typename T, bool EXACT>
__global__ void __launch_bounds__(kPruneThreads) prune_generic_kernel(GenericArgs g) {
    const PruneArgs& a = g.a;
    const int S = g.S, C = a.C;
    const int site = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = site < a.n_sites;
    const int cs = valid ? site : a.n_sites - 1;
    T* work = static_cast<T*>(a.work);
    const T* P = static_cast<const T*>(a.P);
    int scale_e = 0;
    T d0[kMaxStates], d1[kMaxStates];
    for (int r = 0; valid && r < g.n_int; ++r) {
        const int u = g.order[r];
        const int l = g.left[u], rr = g.right[u];
        T mx = T(0);
        for (int k = 0; k < C; ++k) {
            T* dst = work + (((size_t)r * C + k) * a.n_sites + cs) * S;
            const int c0 = l >= 0 ? l : rr;
            const int c1 = l >= 0 ? rr : -1;
            child_vec_generic<T, EXACT>(g, c0, k, cs, cs, work, P, d0);
            if (c1 >= 0) {
                child_vec_generic<T, EXACT>(g, c1, k, cs, cs, work, P, d1);
                for (int i = 0; i < S; ++i) d0[i] = EXACT ? mul_rn(d0[i], d1[i]) : d0[i] * d1[i];
            }
            for (int i = 0; i < S; ++i) mx = fmax(mx, d0[i]);
            for (int i = 0; i < S; ++i) dst[i] = d0[i];
        }
        if (mx < scale_threshold<T>() && mx > T(0)) {
            int e;
            T f1, f2;
            pow2_factors(mx, &e, &f1, &f2);
            for (int k = 0; k < C; ++k) {
                T* dst = work + (((size_t)r * C + k) * a.n_sites + cs) * S;
                for (int i = 0; i < S; ++i) dst[i] = (dst[i] * f1) * f2;
            }
            scale_e += e;
        }
    }
    double lnl = 0.0;
    if (valid) {
        const int r = g.n_int - 1;
        double lsum = 0.0;
        for (int k = 0; k < C; ++k) {
            const T* R = work + (((size_t)r * C + k) * a.n_sites + site) * S;
            double lk;
            if (EXACT) {
                lk = __dmul_rn((double)R[0], a.root_w[0]);
                for (int s = 1; s < S; ++s) lk = __dadd_rn(lk, __dmul_rn((double)R[s], a.root_w[s]));
                lsum = (k == 0) ? __dmul_rn(a.cat_w[0], lk) : __dadd_rn(lsum, __dmul_rn(a.cat_w[k], lk));
            } else {
                lk = (double)R[0] * a.root_w[0];
                for (int s = 1; s < S; ++s) lk = fma((double)R[s], a.root_w[s], lk);
                lsum = fma(a.cat_w[k], lk, lsum);
            }
        }
        lnl = log(lsum) + (double)scale_e * 0.69314718055994530942;
        a.site_lnl[site] = lnl;
    }
    double s = lnl, c = 0.0;
    for (int off = 16; off > 0; off >>= 1) {
        const double os = __shfl_down_sync(0xffffffffu, s, off);
        const double oc = __shfl_down_sync(0xffffffffu, c, off);
        double ns, e;
        two_sum(s, os, ns, e);
        s = ns;
        c = c + oc + e;
    }
    __shared__ double red_s[32], red_c[32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { red_s[warp] = s; red_c[warp] = c; }
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        s = lane < nw ? red_s[lane] : 0.0;
        c = lane < nw ? red_c[lane] : 0.0;
        for (int off = 16; off > 0; off >>= 1) {
            const double os = __shfl_down_sync(0xffffffffu, s, off);
            const double oc = __shfl_down_sync(0xffffffffu, c, off);
            double ns, e;
            two_sum(s, os, ns, e);
            s = ns;
            c = c + oc + e;
        }
        if (lane == 0) {
            a.block_sum[2 * blockIdx.x] = s;
            a.block_sum[2 * blockIdx.x + 1] = c;
        }
    }
    if (a.grid_done) finish_grid_sum(a.block_sum, a.grid_done, a.lnl_out);
}

}  // namespace

template <typename T, int CM, bool EXACT>
static cudaError_t launch_prune4(const PruneArgs& a, bool store, int blocks, cudaStream_t st) {
    const size_t ops_bytes = ((size_t)a.n_ops * sizeof(Op) + 31) & ~(size_t)31;
    const size_t stack_bytes = (size_t)(a.max_depth > 0 ? a.max_depth : 1) * CM * sizeof(V4<T>) * kPruneThreads;
    const size_t smem = ops_bytes + stack_bytes;
    if (smem > 227 * 1024) return cudaErrorInvalidConfiguration;
    cudaError_t err;
    if (store) {
        auto kern = prune4_kernel<T, CM, EXACT, true>;
        err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return err;
        kern<<<blocks, kPruneThreads, smem, st>>>(a);
    } else {
        auto kern = prune4_kernel<T, CM, EXACT, false>;
        err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return err;
        kern<<<blocks, kPruneThreads, smem, st>>>(a);
    }
    return cudaGetLastError();
}

cudaError_t launch_prune(const PruneArgs& a, int S, int precision, bool store, int* n_blocks,
                         cudaStream_t st) {
    const int blocks = (a.n_sites + kPruneThreads - 1) / kPruneThreads;
    *n_blocks = blocks;
    const bool fp64 = precision == PLK_FP64;
    if (!fp64 && !store && S == 4 && a.C <= 8 && (a.variant == 1 || a.variant == 2) && prune4s_fits(a, a.variant))
        return launch_prune4s(a, a.variant, n_blocks, st);
    if (!fp64 && !store && S == 4 && a.variant >= 3 && a.variant <= 6 && prune4p_fits(a, (a.variant + 1) % 2 + 1))
        return launch_prune4p(a, (a.variant + 1) % 2 + 1, a.variant >= 5 ? 1 : 0, 1, n_blocks, st);
    if (!fp64 && !store && S == 4 && (a.variant == 7 || a.variant == 8) && prune4p_fits(a, 1, 2))
        return launch_prune4p(a, 1, a.variant == 7 ? 1 : 0, 2, n_blocks, st);
    if (!fp64 && !store && S == 4 && a.variant == 9 && prune4p_fits(a, 1, 0))
        return launch_prune4p(a, 1, 1, 0, n_blocks, st);
    if (!fp64 && !store && S == 4 && (a.variant == 10 || a.variant == 11) && prune4p_fits(a, a.variant - 9))
        return launch_prune4p(a, a.variant - 9, 2, 1, n_blocks, st);
    if (!fp64 && !store && S == 4 && a.variant >= 12 && a.variant <= 18) {
        const int spt = (a.variant == 12 || a.variant == 15) ? 1 : ((a.variant == 14 || a.variant == 17) ? 4 : 2);
        const int ts = a.variant >= 15 ? 1 : 0, tps = a.variant == 18 ? 2 : 1;
        if (prune4w_fits(a, spt, ts, tps)) return launch_prune4w(a, spt, ts, tps, n_blocks, st);
    }
    if (!fp64 && !store && S == 20 && a.variant >= 5 && a.variant <= 7 && prune20u_fits(a, a.variant - 5))
        return launch_prune20u(a, a.n_nodes, a.scratch, a.variant - 5, n_blocks, st);
    if (!fp64 && !store && S == 20 && a.variant > 0 && a.variant < 5 && prune20_fits(a, a.variant))
        return launch_prune20(a, a.n_nodes, a.variant, a.scratch, n_blocks, st);
    if (S == 4 && a.C <= 8) {
        const size_t ops_bytes = ((size_t)a.n_ops * sizeof(Op) + 31) & ~(size_t)31;
        const int cm = a.C == 1 ? 1 : (a.C <= 4 ? 4 : 8);
        const size_t stack_bytes = (size_t)(a.max_depth > 0 ? a.max_depth : 1) * cm *
                                   (fp64 ? 32 : 16) * kPruneThreads;
        if (ops_bytes + stack_bytes <= 227 * 1024) {
            if (fp64) {
                if (cm == 1) return launch_prune4<double, 1, true>(a, store, blocks, st);
                if (cm == 4) return launch_prune4<double, 4, true>(a, store, blocks, st);
                return launch_prune4<double, 8, true>(a, store, blocks, st);
            }
            if (cm == 1) return launch_prune4<float, 1, false>(a, store, blocks, st);
            if (cm == 4) return launch_prune4<float, 4, false>(a, store, blocks, st);
            return launch_prune4<float, 8, false>(a, store, blocks, st);
        }
    }
    if (a.work == nullptr) return cudaErrorInvalidValue;
    GenericArgs g{a, a.order, a.left, a.right, a.rank, a.n_int, a.n_tips, S};
    if (fp64) prune_generic_kernel<double, true><<<blocks, kPruneThreads, 0, st>>>(g);
    else prune_generic_kernel<float, false><<<blocks, kPruneThreads, 0, st>>>(g);
    return cudaGetLastError();
}

// =========================================================================
// Tip encoding for alphabets of <= 4 states: the code is the state set
// itself; a cell with no allowed state sets the flag to the alignment's
// generation number gen (check_nodes), so the flag needs no clearing between
// alignments.
// =========================================================================
template <typename M>
__global__ void encode_small_kernel(const M* __restrict__ masks, int n_tips, int n_sites, int stride, uint32_t all,
                                    uint8_t* __restrict__ codes, int* __restrict__ bad, int gen) {
    // one thread per 4 consecutive sites of a row; rows of `codes` are padded
    // to `stride` (a multiple of 16) and the padding is written as 0
    const int chunks = stride / 4;
    const size_t total = (size_t)n_tips * chunks;
    const size_t step = (size_t)gridDim.x * blockDim.x;
    int any_bad = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += step) {
        const int t = (int)(i / chunks), s0 = (int)(i % chunks) * 4;
        const M* row = masks + (size_t)t * n_sites;
        uint8_t c[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int s = s0 + j;
            if (s < n_sites) {
                const uint32_t m = (uint32_t)row[s] & all;
                any_bad |= (m == 0);
                c[j] = (uint8_t)m;
            } else {
                c[j] = 0;
            }
        }
        reinterpret_cast<uchar4*>(codes + (size_t)t * stride)[s0 / 4] = make_uchar4(c[0], c[1], c[2], c[3]);
    }
    if (__any_sync(0xffffffffu, any_bad) && (threadIdx.x & 31) == 0) *reinterpret_cast<volatile int*>(bad) = gen;
}

// Byte masks whose rows are a multiple of 16 sites (so the code rows carry
// no padding and both row starts are 16-byte aligned): 16 cells per thread
// in one 16-byte load and store; an empty cell is a zero byte after the AND
// (the "has a zero byte" test of each 32-bit word).
__global__ void encode_bytes16_kernel(const uint4* __restrict__ masks, size_t n_vec, uint32_t all4,
                                      uint4* __restrict__ codes, int* __restrict__ bad, int gen) {
    int any_bad = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_vec; i += (size_t)gridDim.x * blockDim.x) {
        uint4 v = masks[i];
        v.x &= all4;
        v.y &= all4;
        v.z &= all4;
        v.w &= all4;
        const uint32_t z = ((v.x - 0x01010101u) & ~v.x) | ((v.y - 0x01010101u) & ~v.y) |
                           ((v.z - 0x01010101u) & ~v.z) | ((v.w - 0x01010101u) & ~v.w);
        any_bad |= (z & 0x80808080u) != 0;
        codes[i] = v;
    }
    if (__any_sync(0xffffffffu, any_bad) && (threadIdx.x & 31) == 0) *reinterpret_cast<volatile int*>(bad) = gen;
}

cudaError_t launch_encode_small(const void* masks, int elem_bytes, int n_tips, int n_sites, int stride, uint32_t all,
                                uint8_t* codes, int* bad, int gen, cudaStream_t st) {
    if (elem_bytes == 1 && n_sites % 16 == 0 && stride == n_sites &&
        (reinterpret_cast<uintptr_t>(masks) & 15) == 0 && (reinterpret_cast<uintptr_t>(codes) & 15) == 0) {
        const size_t n_vec = (size_t)n_tips * n_sites / 16;
        size_t blocks = (n_vec + 255) / 256;
        if (blocks < 1) blocks = 1;
        if (blocks > 152 * 8) blocks = 152 * 8;
        const uint32_t all4 = (all & 0xffu) * 0x01010101u;
        encode_bytes16_kernel<<<(unsigned)blocks, 256, 0, st>>>(static_cast<const uint4*>(masks), n_vec, all4,
                                                                reinterpret_cast<uint4*>(codes), bad, gen);
        return cudaGetLastError();
    }
    const int threads = 256;
    const size_t total = (size_t)n_tips * (stride / 4);
    size_t blocks = (total + threads - 1) / threads;
    if (blocks < 1) blocks = 1;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (elem_bytes == 1)
        encode_small_kernel<uint8_t><<<(unsigned)blocks, threads, 0, st>>>(static_cast<const uint8_t*>(masks), n_tips,
                                                                          n_sites, stride, all, codes, bad, gen);
    else
        encode_small_kernel<uint32_t><<<(unsigned)blocks, threads, 0, st>>>(static_cast<const uint32_t*>(masks),
                                                                           n_tips, n_sites, stride, all, codes, bad, gen);
    return cudaGetLastError();
}

// Copies bytes from mapped pinned host memory (the handle's upload arena)
// into device memory with loads over the host link, not a DMA copy: a small
// upload then never queues behind a large host-to-device copy (a streamed
// alignment's chunks) on the copy engines.
__global__ void arena_copy_kernel(unsigned char* __restrict__ dst, const unsigned char* __restrict__ src,
                                  size_t bytes) {
    const size_t n16 = bytes / 16;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x, step = (size_t)gridDim.x * blockDim.x;
    for (size_t i = t; i < n16; i += step)
        reinterpret_cast<uint4*>(dst)[i] = reinterpret_cast<const uint4*>(src)[i];
    for (size_t i = n16 * 16 + t; i < bytes; i += step) dst[i] = src[i];
}

cudaError_t launch_arena_copy(void* dst, const void* src, size_t bytes, cudaStream_t st) {
    if (bytes == 0) return cudaSuccess;
    if ((reinterpret_cast<uintptr_t>(dst) & 15) != 0 || (reinterpret_cast<uintptr_t>(src) & 15) != 0)
        return cudaErrorInvalidValue;
    size_t blocks = (bytes / 16 + 255) / 256;
    if (blocks < 1) blocks = 1;
    if (blocks > 64) blocks = 64;
    arena_copy_kernel<<<(unsigned)blocks, 256, 0, st>>>(static_cast<unsigned char*>(dst),
                                                        static_cast<const unsigned char*>(src), bytes);
    return cudaGetLastError();
}

// The empty-cell check of the streamed alignment: 16 codes of a row per
// thread (rows are code_stride bytes, 16-byte aligned), sites past n_sites
// ignored.
__global__ void check_codes_kernel(const uint4* __restrict__ codes, int n_tips, int n_sites, int vec_per_row,
                                   uint32_t all4, int* __restrict__ bad, int gen) {
    int any_bad = 0;
    const size_t n_vec = (size_t)n_tips * vec_per_row;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_vec; i += (size_t)gridDim.x * blockDim.x) {
        const int first = (int)(i % vec_per_row) * 16;  // the vector's first site
        uint4 v = codes[i];
        v.x &= all4;
        v.y &= all4;
        v.z &= all4;
        v.w &= all4;
        uint32_t z[4] = {(v.x - 0x01010101u) & ~v.x, (v.y - 0x01010101u) & ~v.y, (v.z - 0x01010101u) & ~v.z,
                         (v.w - 0x01010101u) & ~v.w};
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            const int valid = min(max(n_sites - (first + 4 * w), 0), 4);  // bytes of this word within the row
            const uint32_t keep = valid >= 4 ? 0xffffffffu : ((1u << (8 * valid)) - 1u);
            any_bad |= (z[w] & keep & 0x80808080u) != 0;
        }
    }
    if (__any_sync(0xffffffffu, any_bad) && (threadIdx.x & 31) == 0) *reinterpret_cast<volatile int*>(bad) = gen;
}

cudaError_t launch_check_codes(const uint8_t* codes, int n_tips, int n_sites, int stride, uint32_t all, int* bad,
                               int gen, cudaStream_t st) {
    if (stride % 16 != 0 || (reinterpret_cast<uintptr_t>(codes) & 15) != 0) return cudaErrorInvalidValue;
    const size_t n_vec = (size_t)n_tips * (stride / 16);
    size_t blocks = (n_vec + 255) / 256;
    if (blocks < 1) blocks = 1;
    if (blocks > 152 * 4) blocks = 152 * 4;
    const uint32_t all4 = (all & 0xffu) * 0x01010101u;
    check_codes_kernel<<<(unsigned)blocks, 256, 0, st>>>(reinterpret_cast<const uint4*>(codes), n_tips, n_sites,
                                                         stride / 16, all4, bad, gen);
    return cudaGetLastError();
}

// sum_i w_i x_i with TwoSum compensation in one CTA (site patterns: x = the
// pattern lnL, w = its number of sites)
__global__ void __launch_bounds__(1024) weighted_sum_kernel(const double* __restrict__ x,
                                                            const double* __restrict__ w, int n, double* out) {
    double s = 0.0, c = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double p = w[i] * x[i];
        const double pe = fma(w[i], x[i], -p);  // exact rounding error of the product
        double ns, e;
        two_sum(s, p, ns, e);
        s = ns;
        c = c + e + pe;
    }
    block_sum_pair(s, c);
    if (threadIdx.x == 0) *out = s + c;
}

cudaError_t launch_weighted_sum(const double* x, const double* w, int n, double* out, cudaStream_t st) {
    weighted_sum_kernel<<<1, 1024, 0, st>>>(x, w, n, out);
    return cudaGetLastError();
}

// =========================================================================
// Node-state outputs
// =========================================================================
template <typename T>
__global__ void cond_normalise_kernel(const T* __restrict__ cond, const double* __restrict__ cat_w,
                                      int n_int, int C, int n_sites, int S, double* __restrict__ out) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)n_int * n_sites) return;
    const int r = (int)(idx / n_sites), site = (int)(idx % n_sites);
    double v[kMaxStates];
    double tot = 0.0;
    for (int s = 0; s < S; ++s) {
        double acc = 0.0;
        for (int k = 0; k < C; ++k) acc += cat_w[k] * (double)cond[(((size_t)r * C + k) * n_sites + site) * S + s];
        v[s] = acc;
        tot += acc;
    }
    for (int s = 0; s < S; ++s) out[idx * S + s] = v[s] / tot;
}

cudaError_t launch_cond_normalise(const void* cond, const double* cat_w, int n_int, int C,
                                  int n_sites, int S, int precision, double* out,
                                  cudaStream_t st) {
    const size_t n = (size_t)n_int * n_sites;
    const int threads = 256;
    const unsigned blocks = (unsigned)((n + threads - 1) / threads);
    if (precision == PLK_FP64)
        cond_normalise_kernel<double><<<blocks, threads, 0, st>>>(static_cast<const double*>(cond), cat_w, n_int, C, n_sites, S, out);
    else
        cond_normalise_kernel<float><<<blocks, threads, 0, st>>>(static_cast<const float*>(cond), cat_w, n_int, C, n_sites, S, out);
    return cudaGetLastError();
}

// Pre-order pass: Out(root) = root weights; for an internal child v of u with
// sibling w, Out(v)[b] = sum_a Out(u)[a] * D_w[a] * P_v[a][b], D_w = P_w x_w.
// Marginal(u)[s] ∝ sum_k w_k Out(u)[k][s] Cond(u)[k][s].  Vectors are
// rescaled by powers of two (a common factor per node and site cancels in
// the normalisation).
template <typename T>
__global__ void __launch_bounds__(128) preorder_kernel(PreorderArgs a) {
    const int site = blockIdx.x * blockDim.x + threadIdx.x;
    if (site >= a.n_sites) return;
    const int S = a.S, C = a.C;
    const T* cond = static_cast<const T*>(a.cond);
    T* outside = static_cast<T*>(a.outside);
    const T* P = static_cast<const T*>(a.P);
    const T* tipT = static_cast<const T*>(a.tipT);
    T o[kMaxStates], dw[kMaxStates], tmp[kMaxStates];
    double marg[kMaxStates];
    for (int r = a.n_int - 1; r >= 0; --r) {
        const int u = a.order[r];
        for (int s = 0; s < S; ++s) marg[s] = 0.0;
        for (int k = 0; k < C; ++k) {
            const T* cu = cond + (((size_t)r * C + k) * a.n_sites + site) * S;
            const T* ou = outside + (((size_t)r * C + k) * a.n_sites + site) * S;
            for (int s = 0; s < S; ++s) {
                const T os = (r == a.n_int - 1) ? (T)a.root_w[s] : ou[s];
                marg[s] += a.cat_w[k] * (double)os * (double)cu[s];
            }
        }
        double tot = 0.0;
        for (int s = 0; s < S; ++s) tot += marg[s];
        for (int s = 0; s < S; ++s) a.out[((size_t)r * a.n_sites + site) * S + s] = marg[s] / tot;
        const int kids[2] = {a.left[u], a.right[u]};
        for (int c = 0; c < 2; ++c) {
            const int v = kids[c], w = kids[1 - c];
            if (v < 0 || v < a.n_tips) continue;
            const int rv = a.rank[v];
            T mx = T(0);
            for (int k = 0; k < C; ++k) {
                const T* ou = outside + (((size_t)r * C + k) * a.n_sites + site) * S;
                for (int s = 0; s < S; ++s) o[s] = (r == a.n_int - 1) ? (T)a.root_w[s] : ou[s];
                if (w >= 0) {
                    if (w < a.n_tips) {
                        int code = a.codes[(size_t)w * a.site_stride + site];
                        if (S <= 4) code &= (1 << S) - 1;  // state sets (streamed codes are the caller's bytes)
                        const T* tv = tipT + (((size_t)w * C + k) * a.n_codes + code) * S;
                        for (int i = 0; i < S; ++i) dw[i] = tv[i];
                    } else {
                        const T* x = cond + (((size_t)a.rank[w] * C + k) * a.n_sites + site) * S;
                        const T* Pw = P + ((size_t)w * C + k) * S * S;
                        for (int i = 0; i < S; ++i) {
                            T acc = T(0);
                            for (int j = 0; j < S; ++j) acc = fma(x[j], Pw[i * S + j], acc);
                            dw[i] = acc;
                        }
                    }
                    for (int i = 0; i < S; ++i) tmp[i] = o[i] * dw[i];
                } else {
                    for (int i = 0; i < S; ++i) tmp[i] = o[i];
                }
                const T* Pv = P + ((size_t)v * C + k) * S * S;
                T* ov = outside + (((size_t)rv * C + k) * a.n_sites + site) * S;
                for (int b = 0; b < S; ++b) {
                    T acc = T(0);
                    for (int i = 0; i < S; ++i) acc = fma(tmp[i], Pv[i * S + b], acc);
                    ov[b] = acc;
                    mx = fmax(mx, acc);
                }
            }
            if (mx < scale_threshold<T>() && mx > T(0)) {
                int e;
                T f1, f2;
                pow2_factors(mx, &e, &f1, &f2);
                for (int k = 0; k < C; ++k) {
                    T* ov = outside + (((size_t)rv * C + k) * a.n_sites + site) * S;
                    for (int b = 0; b < S; ++b) ov[b] = (ov[b] * f1) * f2;
                }
            }
        }
    }
}

cudaError_t launch_preorder(const PreorderArgs& a, int precision, cudaStream_t st) {
    const int threads = 128;
    const int blocks = (a.n_sites + threads - 1) / threads;
    if (precision == PLK_FP64) preorder_kernel<double><<<blocks, threads, 0, st>>>(a);
    else preorder_kernel<float><<<blocks, threads, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace plk
