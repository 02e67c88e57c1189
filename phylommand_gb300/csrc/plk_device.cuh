// Device helpers shared by the kernels of libplk.
#pragma once

#include <cuda_bf16.h>

#include <cstdint>

#include "plk_internal.h"

namespace plk {
namespace dev {

constexpr int kPruneThreads = 128;

template <typename T>
struct alignas(4 * sizeof(T)) V4 {
    T v[4];
};

// EXACT arithmetic keeps every multiply and add separately rounded in the
// reference's order; the fast forms use FMA chains.
template <typename T>
__device__ __forceinline__ T mul_rn(T a, T b);
template <>
__device__ __forceinline__ double mul_rn<double>(double a, double b) { return __dmul_rn(a, b); }
template <>
__device__ __forceinline__ float mul_rn<float>(float a, float b) { return __fmul_rn(a, b); }
template <typename T>
__device__ __forceinline__ T add_rn(T a, T b);
template <>
__device__ __forceinline__ double add_rn<double>(double a, double b) { return __dadd_rn(a, b); }
template <>
__device__ __forceinline__ float add_rn<float>(float a, float b) { return __fadd_rn(a, b); }

__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
    s = __dadd_rn(a, b);
    const double bb = __dsub_rn(s, a);
    e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
}

template <typename T>
__device__ __forceinline__ T scale_threshold();
template <>
__device__ __forceinline__ float scale_threshold<float>() { return 2.3283064365386963e-10f; }  // 2^-32
template <>
__device__ __forceinline__ double scale_threshold<double>() { return 8.636168555094445e-78; }  // 2^-256

// Rescale a vector whose maximum mx lies below the threshold so that the
// maximum lands in [0.5, 1): multiply by 2^-e (mx = f 2^e) in two exact
// power-of-two steps, each finite in T even when mx is subnormal.
template <typename T>
__device__ __forceinline__ void pow2_factors(T mx, int* e, T* f1, T* f2) {
    frexp(mx, e);
    const int k = -*e, half = k / 2;
    *f1 = ldexp(T(1), half);
    *f2 = ldexp(T(1), k - half);
}

// Compensated (TwoSum) reduction of (s, c) over the block; thread 0 of the
// block ends with the block's pair.  All threads of the block must call it.
__device__ __forceinline__ void block_sum_pair(double& s, double& c) {
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
    __syncthreads();
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
    }
}

__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// FP32 TwoSum reduction of (hi, lo) over a warp; lane 0 ends with the pair
__device__ __forceinline__ void warp_two_sum_f(float& hi, float& lo) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const float oh = __shfl_down_sync(0xffffffffu, hi, off);
        const float ol = __shfl_down_sync(0xffffffffu, lo, off);
        float ns, e;
        two_sum_f(hi, oh, ns, e);
        hi = ns;
        lo = __fadd_rn(lo, __fadd_rn(ol, e));
    }
}

// FP32 site log-likelihoods.  GB300's FP64 pipe retires a small fraction of
// its FP32 rate, so the per-site root stays in FP32: a site's likelihood is
// L = lsum 2^e (lsum the FP32 root sum, e the scaler exponent), and
//   log L = lm + ee ln 2,   lm = log of the mantissa of lsum, in [0, ln 2),
// so logf's error is absolute (about 6e-8), not relative to log L.
__device__ __forceinline__ void site_log32(float lsum, int e, float& lm, int& ee) {
    if (lsum > 0.0f && lsum < 1.17549435e-38f) {  // subnormal: exact rescale by 2^64
        lsum *= 1.8446744073709552e19f;
        e -= 64;
    }
    const int bits = __float_as_int(lsum);
    ee = e + ((bits >> 23) & 255) - 127;
    // zero, infinity and NaN keep logf's own result (-inf, inf, NaN)
    lm = (lsum > 0.0f && lsum <= 3.40282347e38f) ? logf(__int_as_float((bits & 0x007fffff) | 0x3f800000))
                                                 : logf(lsum);
}

__device__ __forceinline__ double site_lnl64(float lm, int ee) {
    return fma((double)ee, 0.69314718055994530942, (double)lm);
}

// A thread's running sum of site log-likelihoods: the mantissa logs in FP32
// TwoSum (hi, lo), the exponents as an integer.
struct SiteSum32 {
    float hi = 0.0f, lo = 0.0f;
    int ee = 0;
};

__device__ __forceinline__ void site_sum_add(SiteSum32& a, float lm, int ee) {
    float s, e;
    two_sum_f(a.hi, lm, s, e);
    a.hi = s;
    a.lo = __fadd_rn(a.lo, e);
    a.ee += ee;
}

// Block total of the threads' SiteSum32, valid in thread 0: FP32 TwoSum and
// integer sums only, within each warp and then across the warps (GB300's
// FP64 pipe would make a chain of FP64 shuffle steps the longest part of a
// short pass).  All threads of the block must call it.
__device__ inline SiteSum32 block_sum_site32f(SiteSum32 a) {
    warp_two_sum_f(a.hi, a.lo);
    a.ee = __reduce_add_sync(0xffffffffu, a.ee);
    __shared__ float r_h[32], r_l[32];
    __shared__ int r_e[32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();  // an earlier call may still be reading r_h / r_l / r_e
    if (lane == 0) {
        r_h[warp] = a.hi;
        r_l[warp] = a.lo;
        r_e[warp] = a.ee;
    }
    __syncthreads();
    SiteSum32 t;
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        t.hi = lane < nw ? r_h[lane] : 0.0f;
        t.lo = lane < nw ? r_l[lane] : 0.0f;
        t.ee = lane < nw ? r_e[lane] : 0;
        warp_two_sum_f(t.hi, t.lo);
        t.ee = __reduce_add_sync(0xffffffffu, t.ee);
    }
    return t;
}

// The same total as a compensated FP64 pair (s, c) in thread 0 (0 elsewhere):
// sum = ee ln 2 + hi + lo.
__device__ inline void block_sum_site32(SiteSum32 a, double& s, double& c) {
    const SiteSum32 t = block_sum_site32f(a);
    s = 0.0;
    c = 0.0;
    if (threadIdx.x == 0) {
        two_sum((double)t.ee * 0.69314718055994530942, (double)t.hi, s, c);
        c += (double)t.lo;
    }
}

// A block's SiteSum32 record in the 16 bytes of its block-sum pair:
// (hi, lo, ee, 0) as one 16-byte store by thread 0.
__device__ __forceinline__ void store_site_record(double* bs, size_t slot, const SiteSum32& t) {
    reinterpret_cast<float4*>(bs)[slot] = make_float4(t.hi, t.lo, __int_as_float(t.ee), 0.0f);
}

// Compensated sum of the n (sum, compensation) pairs of bs by one CTA:
// thread i folds pairs i, i + blockDim.x, ... (TwoSum), then the block
// reduction of block_sum_pair; the result is valid in thread 0.  Loads go
// through L2 so that pairs other CTAs of the same grid stored are seen.
__device__ inline double cta_sum_pairs(const double* bs, int n) {
    constexpr int U = 8;  // a thread's loads of one round, all in flight before the sums
    double s = 0.0, c = 0.0;
    for (int base = 0; base < n; base += U * (int)blockDim.x) {
        double2 v[U];
#pragma unroll
        for (int q = 0; q < U; ++q) {
            const int i = base + q * (int)blockDim.x + (int)threadIdx.x;
            v[q] = i < n ? __ldcg(reinterpret_cast<const double2*>(bs) + i) : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int q = 0; q < U; ++q) {
            if (base + q * (int)blockDim.x + (int)threadIdx.x >= n) break;  // past the end: nothing to fold
            double ns, e;
            two_sum(s, v[q].x, ns, e);
            s = ns;
            c = c + v[q].y + e;
        }
    }
    block_sum_pair(s, c);
    return s + c;
}

// Epilogue of a 1-D grid whose CTAs each stored one pair at bs[2 blockIdx.x]
// from thread 0: every CTA counts itself in with one atomicAdd after a fence,
// and the CTA that arrives last sums all pairs in index order into *out and
// re-arms the counter (zero between launches).  Nothing waits on another CTA.
// Every thread of the CTA must call it, after thread 0's store.
__device__ inline void finish_grid_sum(const double* bs, unsigned* counter, double* out) {
    __shared__ int s_last;
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const double t = cta_sum_pairs(bs, (int)gridDim.x);
    if (threadIdx.x == 0) {
        *out = t;
        *counter = 0u;
    }
}

// The same epilogue for grids whose CTAs each stored a SiteSum32 record
// (store_site_record): the last CTA folds the records in index order with
// FP32 TwoSum and integer sums and writes ee ln 2 + hi + lo as one FP64 value.
__device__ inline void finish_grid_sum32(const double* bs, unsigned* counter, double* out) {
    __shared__ int s_last;
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const float4* rec = reinterpret_cast<const float4*>(bs);
    SiteSum32 a;
    for (int i = (int)threadIdx.x; i < (int)gridDim.x; i += (int)blockDim.x) {
        const float4 v = __ldcg(rec + i);
        float ns, e;
        two_sum_f(a.hi, v.x, ns, e);
        a.hi = ns;
        a.lo = __fadd_rn(a.lo, __fadd_rn(v.y, e));
        a.ee += __float_as_int(v.z);
    }
    const SiteSum32 t = block_sum_site32f(a);
    if (threadIdx.x == 0) {
        *out = fma((double)t.ee, 0.69314718055994530942, (double)t.hi + (double)t.lo);
        *counter = 0u;
    }
}

// Split-BF16 B-operand image of a 20-state P(t) for the tcgen05 kind::f16
// form (plk_prune20u.cu): two parts (hi = bf16(x), lo = bf16(x - hi)), each
// [8-column group g (4)][8-row block nb (4)][row r (8)][8 BF16 columns], the
// N index (output state) i = 8 nb + r, the K index (input state) j = 8 g + c,
// zero outside 20 x 20.
constexpr int kB16PartBytes = 2048;
constexpr int kB16Bytes = 2 * kB16PartBytes;

// the elements of 32-bit word w of the image: its part, i and the first j
__host__ __device__ inline void bf16_image_index(int w, int& part, int& i, int& j0) {
    const int e = 2 * w;
    part = e / (kB16PartBytes / 2);
    const int q = e % (kB16PartBytes / 2);
    const int g = q / 256, nb = (q / 64) % 4, r = (q / 8) % 8, c = q % 8;
    i = 8 * nb + r;
    j0 = 8 * g + c;
}

// BF16 hi and lo parts of two values, packed as the operands store them
// (element 2k in the low half of a 32-bit word); x - hi is exact in FP32
__device__ __forceinline__ void bf16_split2(float x0, float x1, uint32_t& hi, uint32_t& lo) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
    const float2 hf = __bfloat1622float2(h);
    const __nv_bfloat162 l = __floats2bfloat162_rn(x0 - hf.x, x1 - hf.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
}

// 16-byte asynchronous global-to-shared copies (sm_80+ cp.async).
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

}  // namespace dev
}  // namespace plk
