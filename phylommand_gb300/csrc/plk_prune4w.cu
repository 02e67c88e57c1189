// prune4w: the 4-state FP32 post-order pass (src/simpleML.cpp:127-197) with
// every warp on its own sites, SPT sites per thread, and nothing staged.
//
// The staged forms (prune4s, prune4p) copy each op's P(t) rows and tip
// tables into shared memory and hold the CTA at a barrier per op; on the
// 128-taxon x 100,000-site benchmark that staging, the barrier and the
// generic op decoding cost more instructions than the arithmetic itself.
// Here a warp walks the op list alone, over 32 x SPT sites:
//  * a thread carries SPT adjacent sites (SPT lane + s of the warp's tile),
//    so every P(t) row it loads feeds the products of SPT sites, the SPT
//    sites' independent products hide the latency of the next loads, and one
//    load of SPT bytes brings a child's tip codes for all of them;
//  * TS = 0: P(t) pairs and tip tables are read where the P(t) kernel wrote
//    them (the paired layouts of plk_prune4p.cuh), through the read-only L1
//    path: a P(t) row of an op is the same address in every lane (one
//    broadcast load of 32 bytes feeds two packed FMAs per site), a tip-table
//    load gathers each lane's code row;
//  * spilled vectors sit in tensor memory (tcgen05.st / tcgen05.ld, one
//    instruction per category pair and op), not in shared memory;
//  * the tip codes of op o + 2 are loaded while op o computes (a register
//    ring, not allocated in L1), so their L2 / DRAM latency hides behind two
//    ops of arithmetic;
//  * TS = 1 (trees whose tables fit): the CTA first brings the paired tables
//    and the op list into shared memory with bulk copies (cp.async.bulk on
//    one mbarrier, a bounded wait) and reads them there;
//  * every branch on the op's shape is uniform across the warp, and no CTA
//    barrier stands between ops; one CTA per SM, its warp count chosen per
//    launch so that every warp has a tile;
//  * the rescale test first takes the maximum of one category pair; only when
//    a lane of the warp falls below the threshold does the warp take the full
//    maximum (the same decision and factors);
//  * a streamed alignment's codes land while the pass runs: a warp waits
//    (bounded) for its tile's chunk flag before its walk;
//  * the launch overlaps the P(t) kernel before it (programmatic stream
//    serialization; griddepcontrol.wait before any read of its tables).
// The arithmetic is run_tile4p's (plk_prune4p.cuh) in the same order -- every
// product, rescale and root sum on fma.rn.f32x2 / mul.rn.f32x2 lanes -- so the
// per-site results are the bits of prune4s and prune4p; the sites' sum is the
// FP32 record epilogue of every FP32 form (block_sum_site32f).
#include "plk_prune4p.cuh"

#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <tuple>

namespace plk {
using namespace dev;

namespace {

constexpr int kWMinWarps = 4;
constexpr int kWMaxWarps = 24;
constexpr uint32_t kWChunk = 16384;  // bytes per bulk copy of the TS = 1 prologue

// FP32 lane pairs as float2, multiplied on the packed FP32x2 path
// (fma.rn.f32x2 / mul.rn.f32x2 through __ffma2_rn / __fmul2_rn)
typedef float2 f2;
__device__ __forceinline__ f2 mul2(f2 a, f2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ f2 pk2(float lo, float hi) { return make_float2(lo, hi); }
__device__ __forceinline__ void unpack2(f2 v, float& lo, float& hi) {
    lo = v.x;
    hi = v.y;
}
__device__ __forceinline__ void ldg_v4(const f2* p, f2& a, f2& b, f2& c, f2& d) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
        : "=f"(a.x), "=f"(a.y), "=f"(b.x), "=f"(b.y), "=f"(c.x), "=f"(c.y), "=f"(d.x), "=f"(d.y)
        : "l"(p));
}
__device__ __forceinline__ void ldg_v2(const f2* p, f2& a, f2& b) {
    asm("ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%4];\n" : "=f"(a.x), "=f"(a.y), "=f"(b.x), "=f"(b.y) : "l"(p));
}
// three-input maximum (PTX ISA 8.8+, sm_100+): the same value as two fmaxf
__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;\n" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

__device__ __forceinline__ void lds_v2(uint32_t addr, f2& a, f2& b) {
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];\n" : "=f"(a.x), "=f"(a.y), "=f"(b.x), "=f"(b.y) : "r"(addr));
}
__device__ __forceinline__ int4 lds_int4(uint32_t addr) {
    int4 v;
    asm volatile("ld.shared.v4.s32 {%0, %1, %2, %3}, [%4];\n" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "r"(addr));
    return v;
}
__device__ __forceinline__ int2 lds_int2(uint32_t addr) {
    int2 v;
    asm volatile("ld.shared.v2.s32 {%0, %1}, [%2];\n" : "=r"(v.x), "=r"(v.y) : "r"(addr));
    return v;
}

// Where the paired tables and the ops are read: TS = 0 global memory through
// the read-only L1 path, TS = 1 shared memory (32-bit addresses).
//   p_pair(node, q, r): one category pair of a node's paired P(t) block, rows
//     j = 0..3, each the pairs of states i = 0..3;
//   tip(tip, q, code, out): pair q of the tip table row of a code
//     ([pair][half][code][state in the half][2]);
//   op(o): the op's e0, e1 and s0, s1, push.
template <int KP, int TS>
struct Tables;

template <int KP>
struct Tables<KP, 0> {
    const f2* P;
    const f2* T;
    const Op* ops;
    __device__ __forceinline__ void p_pair(int node, int q, f2 (&r)[4][4]) const {
        const f2* b = P + (size_t)node * KP * 16 + q * 16;
#pragma unroll
        for (int j = 0; j < 4; ++j) ldg_v4(b + j * 4, r[j][0], r[j][1], r[j][2], r[j][3]);
    }
    __device__ __forceinline__ void tip(int t, int q, int code, f2 (&out)[4]) const {
        const f2* b = T + (size_t)t * KP * 64 + (q * 2 * kCodes + code) * 2;
        ldg_v2(b, out[0], out[1]);
        ldg_v2(b + kCodes * 2, out[2], out[3]);
    }
    __device__ __forceinline__ void op(int o, int4& ea, int4& sb) const {
        ea = __ldg(reinterpret_cast<const int4*>(ops + o));
        sb = __ldg(reinterpret_cast<const int4*>(ops + o) + 1);
    }
    __device__ __forceinline__ int2 sources(int o) const { return __ldg(reinterpret_cast<const int2*>(&ops[o].s0)); }
};

template <int KP>
struct Tables<KP, 1> {
    uint32_t P, T, ops;  // shared-memory addresses
    __device__ __forceinline__ void p_pair(int node, int q, f2 (&r)[4][4]) const {
        const uint32_t b = P + (uint32_t)node * (KP * 128) + q * 128;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            lds_v2(b + j * 32, r[j][0], r[j][1]);
            lds_v2(b + j * 32 + 16, r[j][2], r[j][3]);
        }
    }
    __device__ __forceinline__ void tip(int t, int q, int code, f2 (&out)[4]) const {
        const uint32_t b = T + (uint32_t)t * (KP * 512) + q * 512 + (uint32_t)code * 16;
        lds_v2(b, out[0], out[1]);
        lds_v2(b + 256, out[2], out[3]);
    }
    __device__ __forceinline__ void op(int o, int4& ea, int4& sb) const {
        ea = lds_int4(ops + (uint32_t)o * 32);
        sb = lds_int4(ops + (uint32_t)o * 32 + 16);
    }
    __device__ __forceinline__ int2 sources(int o) const { return lds_int2(ops + (uint32_t)o * 32 + 16); }
};

// out[i] = sum_j r[j][i] x[j], j ascending, the first term a product (the
// order of mv4p)
__device__ __forceinline__ void mv_pair(const f2 (&r)[4][4], const f2 (&x)[4], f2 (&out)[4]) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        f2 acc = mul2(x[0], r[0][i]);
        acc = fma2(x[1], r[1][i], acc);
        acc = fma2(x[2], r[2][i], acc);
        acc = fma2(x[3], r[3][i], acc);
        out[i] = acc;
    }
}

// ---- the spill stack in tensor memory ------------------------------------
// A spilled slot holds, for every category pair q and every site s of the
// thread, the 4 pairs = 8 32-bit values: 8 x SPT TMEM columns per pair,
// [q][s][8].  Warp w owns TMEM lanes 32 (w % 4) .. + 31 (the lanes a warp may
// access) and, among the warps sharing those lanes, the column range
// (w / 4) x depth x KP x SPT x 8.  N = 8 SPT columns move in one instruction.
template <int N>
__device__ __forceinline__ void tmem_st(uint32_t taddr, const uint32_t (&r)[N]) {
    static_assert(N == 8 || N == 16 || N == 32, "8, 16 or 32 columns");
    if constexpr (N == 8) {
        asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};\n" ::"r"(taddr),
                     "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7])
                     : "memory");
    } else if constexpr (N == 16) {
        asm volatile(
            "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};\n" ::
                "r"(taddr),
            "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]),
            "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
            : "memory");
    } else {
        asm volatile(
            "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
            "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};\n" ::"r"(taddr),
            "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]),
            "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(r[16]),
            "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]), "r"(r[24]),
            "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31])
            : "memory");
    }
}
template <int N>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, uint32_t (&r)[N]) {
    static_assert(N == 8 || N == 16 || N == 32, "8, 16 or 32 columns");
    if constexpr (N == 8) {
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                     : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                     : "r"(taddr)
                     : "memory");
    } else if constexpr (N == 16) {
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(taddr)
            : "memory");
    } else {
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,"
            "%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
              "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
              "=r"(r[30]), "=r"(r[31])
            : "r"(taddr)
            : "memory");
    }
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory"); }
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

// this thread's tip codes (SPT adjacent sites, one load of SPT bytes),
// loaded without allocating in L1 (which holds the tables).  Plain (coherent)
// loads, not the read-only path: a streamed alignment's codes land while the
// pass runs (a warp reads its tile's codes only after their arrival flag).
template <int SPT>
__device__ __forceinline__ int ldg_codes_na(const uint8_t* p) {
    if constexpr (SPT == 1) {
        unsigned short v;
        asm volatile("ld.global.L1::no_allocate.u8 %0, [%1];\n" : "=h"(v) : "l"(p));
        return (int)v;
    } else if constexpr (SPT == 2) {
        unsigned short v;
        asm volatile("ld.global.L1::no_allocate.u16 %0, [%1];\n" : "=h"(v) : "l"(p));
        return (int)v;
    } else {
        int v;
        asm volatile("ld.global.L1::no_allocate.u32 %0, [%1];\n" : "=r"(v) : "l"(p));
        return v;
    }
}

// The arrival of a streamed tile's codes: arrive[c] reaching gen (written by a
// copy after the chunk's copy on the alignment's copy stream).  Every lane
// reads the flag with acquire semantics, so its code loads that follow see
// the chunk.  Bounded: false after kArriveLimitNs of waiting.
constexpr unsigned long long kArriveLimitNs = 2000000000ull;  // 2 s: far above any chunk's copy time
__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    return t;
}
__device__ __forceinline__ bool wait_arrival(const int* flag, int gen) {
    if (ld_acquire_gpu(flag) == gen) return true;
    const unsigned long long t0 = global_ns();
    for (;;) {
        __nanosleep(256);
        if (ld_acquire_gpu(flag) == gen) return true;
        if (global_ns() - t0 > kArriveLimitNs) return false;
    }
}

template <int SPT, class Tab>
__device__ __forceinline__ void op_codes(const Tab& tab, int o, const uint8_t* colp, int stride, int& c0, int& c1) {
    const int2 sv = tab.sources(o);
    c0 = sv.x >= 0 ? ldg_codes_na<SPT>(colp + (size_t)sv.x * stride) : 0;
    c1 = sv.y >= 0 ? ldg_codes_na<SPT>(colp + (size_t)sv.y * stride) : 0;
}

// The register budget of a thread: one CTA of 32 x warps threads per SM.
__host__ __device__ constexpr int prune4w_maxnreg(int KP, int SPT, int TPS) {
    return TPS == 2 ? (KP == 4 ? 168 : 124)
                    : (SPT == 1 ? (KP == 4 ? 128 : 96)
                                : (SPT == 2 ? (KP == 4 ? 232 : (KP == 2 ? 168 : 128)) : (KP == 1 ? 192 : 255)));
}

// One CTA per SM (the launch keeps the occupancy at one), blockDim.x / 32
// warps, each walking warp tiles of 32 SPT sites g, g + T, ... with g = warp
// x gridDim.x + blockIdx.x and T the grid's warps, so that the tiles of a
// last, partial round fall on every SM alike.  tmem_cols: the CTA's TMEM
// allocation (a power of two >= 32 holding every warp's stack).
// TS = 1: the CTA first copies the tree's paired P(t) and tip tables into
// shared memory and reads them there (trees whose tables fit).
// TPS = 2: the two lanes 2i, 2i + 1 share sites, each holding half of the
// category pairs (they exchange their maxima for the rescale, and the even
// lane adds up the root in category order, so the bits are those of TPS = 1);
// a warp tile is 16 x SPT sites.
template <int KP, int SPT, int TS, int TPS>
__global__ void __maxnreg__(prune4w_maxnreg(KP, SPT, TPS)) prune4w_kernel(PruneArgs a, const float* __restrict__ Pp,
                                                                          const float* __restrict__ Tp, int tmem_cols) {
    // the kernel before this one in the stream (P(t), which writes the
    // tables) has completed and its writes are visible
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
    constexpr int NC = 8 * SPT;     // TMEM columns of one category pair of a slot
    constexpr int KPT = KP / TPS;   // category pairs per thread
    constexpr int WS = 32 / TPS;    // sites per warp and site index s
    __shared__ uint32_t s_tmem;
    const int nthr = blockDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int half = TPS == 2 ? (lane & 1) : 0;
    const int q0 = half * KPT;      // this thread's first pair
    const int n_wtiles = (a.n_sites + WS * SPT - 1) / (WS * SPT);
    const int total_warps = (nthr >> 5) * gridDim.x;
    extern __shared__ __align__(16) unsigned char wtab[];
    __shared__ __align__(8) uint64_t s_bar;
    Tables<KP, TS> tab;
    if constexpr (TS) {
        // [P(t) of every node][tip tables of every tip][ops] by bulk copies
        // (cp.async.bulk, 16-byte aligned, sizes multiples of 16) that one
        // thread issues in chunks, completing on one mbarrier; the TMEM
        // allocation below overlaps them
        const uint32_t pb = (uint32_t)a.n_nodes * KP * 128, tb = (uint32_t)a.n_tips * KP * 512;
        const uint32_t ob = (uint32_t)a.n_ops * (uint32_t)sizeof(Op);
        const uint32_t base = static_cast<uint32_t>(__cvta_generic_to_shared(wtab));
        const uint32_t bar = static_cast<uint32_t>(__cvta_generic_to_shared(&s_bar));
        if (tid == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(pb + tb + ob)
                         : "memory");
            if (!a.withhold_first_stage) {
                const unsigned char* src[3] = {reinterpret_cast<const unsigned char*>(Pp),
                                               reinterpret_cast<const unsigned char*>(Tp),
                                               reinterpret_cast<const unsigned char*>(a.ops)};
                const uint32_t len[3] = {pb, tb, ob};
                uint32_t dst = base;
                for (int k = 0; k < 3; ++k) {
                    for (uint32_t off = 0; off < len[k]; off += kWChunk) {
                        const uint32_t n = min(kWChunk, len[k] - off);
                        asm volatile(
                            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                                dst + off),
                            "l"(src[k] + off), "r"(n), "r"(bar)
                            : "memory");
                    }
                    dst += len[k];
                }
            }
        }
        tab.P = base;
        tab.T = base + pb;
        tab.ops = base + pb + tb;
    } else {
        tab.P = reinterpret_cast<const f2*>(Pp);
        tab.T = reinterpret_cast<const f2*>(Tp);
        tab.ops = a.ops;
    }
    const int n_ops = a.n_ops;
    const int depth = a.max_depth > 0 ? a.max_depth : 1;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         static_cast<uint32_t>(__cvta_generic_to_shared(&s_tmem))),
                     "r"(tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    // TS = 1: the tables have landed (a bounded wait; one that runs out
    // leaves this thread's sum NaN, so the evaluation reports a non-finite
    // value, after a second bounded wait for copies still in flight)
    bool tables_ok = true;
    if constexpr (TS) {
        const uint32_t bar = static_cast<uint32_t>(__cvta_generic_to_shared(&s_bar));
        if (!mbar_try_wait_bounded(bar, 0)) {
            tables_ok = false;
            if (!a.withhold_first_stage) mbar_try_wait_bounded(bar, 0);
        }
    }
    // this warp's stack: its lanes, its column range
    const uint32_t tstack =
        s_tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)((warp >> 2) * depth * KPT * NC);
    SiteSum32 sum;
    const int stride = a.site_stride;
    const f2 one2 = pk2(1.0f, 1.0f);
    if (!tables_ok) site_sum_add(sum, __int_as_float(0x7fc00000), 0);
    for (int wtile = warp * gridDim.x + blockIdx.x; tables_ok && wtile < n_wtiles; wtile += total_warps) {
        if (a.arrive) {  // a streamed alignment: this tile's chunk of codes first (the test hook withholds it)
            const int want = a.withhold_first_stage ? (a.arrive_gen ^ 0x40000000) : a.arrive_gen;
            if (!wait_arrival(a.arrive + (wtile * WS * SPT) / a.chunk_sites, want)) {
                site_sum_add(sum, __int_as_float(0x7fc00000), 0);  // NaN: the evaluation reports a numeric error
                continue;
            }
        }
        const int base = wtile * WS * SPT + (TPS == 2 ? lane >> 1 : lane) * SPT;  // site s: base + s
        const uint8_t* colp = a.codes + min(base, stride - SPT);
        f2 acc[SPT][KPT][4];
        int scale_e[SPT];
#pragma unroll
        for (int s = 0; s < SPT; ++s) {
            scale_e[s] = 0;
#pragma unroll
            for (int q = 0; q < KPT; ++q)
#pragma unroll
                for (int i = 0; i < 4; ++i) acc[s][q][i] = one2;
        }
        int sp = 0;
        // codes of ops o (c0, c1) and o + 1 (n0, n1)
        int c0 = 0, c1 = 0, n0 = 0, n1 = 0;
        if (n_ops > 0) op_codes<SPT>(tab, 0, colp, stride, c0, c1);
        if (n_ops > 1) op_codes<SPT>(tab, 1, colp, stride, n0, n1);
        for (int o = 0; o < n_ops; ++o) {
            int m0 = 0, m1 = 0;
            if (o + 2 < n_ops) op_codes<SPT>(tab, o + 2, colp, stride, m0, m1);
            // the op (32 bytes, 32-byte aligned): node, rank, e0, e1 | s0, s1, push, pad
            int4 oa, ob;
            tab.op(o, oa, ob);
            const int e0 = oa.z, e1 = oa.w, s0 = ob.x, s1 = ob.y, push = ob.z;
            // the three shapes the op program has (build_program) with their
            // branches taken once per op; anything else (one child) below
            if (s0 >= 0 && s1 >= 0) {  // two tips
#pragma unroll
                for (int q = 0; q < KPT; ++q)
#pragma unroll
                    for (int s = 0; s < SPT; ++s) {
                        f2 d0[4], d1[4];
                        tab.tip(s1, q0 + q, (c1 >> (8 * s)) & (kCodes - 1), d1);
                        tab.tip(s0, q0 + q, (c0 >> (8 * s)) & (kCodes - 1), d0);
#pragma unroll
                        for (int i = 0; i < 4; ++i) acc[s][q][i] = mul2(d0[i], d1[i]);
                    }
            } else if (s0 == kSrcAcc && s1 >= 0) {  // the running vector and a tip
#pragma unroll
                for (int q = 0; q < KPT; ++q) {
                    f2 r[4][4];
                    tab.p_pair(e0, q0 + q, r);
#pragma unroll
                    for (int s = 0; s < SPT; ++s) {
                        f2 d0[4], d1[4];
                        tab.tip(s1, q0 + q, (c1 >> (8 * s)) & (kCodes - 1), d1);
                        mv_pair(r, acc[s][q], d0);
#pragma unroll
                        for (int i = 0; i < 4; ++i) acc[s][q][i] = mul2(d0[i], d1[i]);
                    }
                }
            } else if (s0 == kSrcPop && s1 == kSrcAcc) {  // the popped vector and the running one
                --sp;
                // the popped slot's loads go out first (after the stores of
                // earlier pushes), the running vector's messages cover them
                tmem_wait_st();
                uint32_t w[KPT][NC];
#pragma unroll
                for (int q = 0; q < KPT; ++q) tmem_ld<NC>(tstack + (uint32_t)((sp * KPT + q) * NC), w[q]);
                f2 d1[SPT][KPT][4];
#pragma unroll
                for (int q = 0; q < KPT; ++q) {
                    f2 r[4][4];
                    tab.p_pair(e1, q0 + q, r);
#pragma unroll
                    for (int s = 0; s < SPT; ++s) mv_pair(r, acc[s][q], d1[s][q]);
                }
                tmem_wait_ld();
#pragma unroll
                for (int q = 0; q < KPT; ++q)
#pragma unroll
                    for (int k = 0; k < NC; ++k) asm volatile("" : "+r"(w[q][k]));  // no use ahead of the wait
#pragma unroll
                for (int q = 0; q < KPT; ++q) {
                    f2 r[4][4];
                    tab.p_pair(e0, q0 + q, r);
#pragma unroll
                    for (int s = 0; s < SPT; ++s) {
                        f2 x[4], d0[4];
#pragma unroll
                        for (int i = 0; i < 4; ++i)
                            x[i] = pk2(__uint_as_float(w[q][8 * s + 2 * i]), __uint_as_float(w[q][8 * s + 2 * i + 1]));
                        mv_pair(r, x, d0);
#pragma unroll
                        for (int i = 0; i < 4; ++i) acc[s][q][i] = mul2(d0[i], d1[s][q][i]);
                    }
                }
            } else {
                if (s0 == kSrcPop) --sp;
#pragma unroll
                for (int q = 0; q < KPT; ++q) {
                    const int qg = q0 + q;  // the pair in the tables
                    // the second child's messages first: they read the running
                    // vector, which the products then overwrite
                    f2 d1[SPT][4];
                    if (s1 >= 0) {
#pragma unroll
                        for (int s = 0; s < SPT; ++s) tab.tip(s1, qg, (c1 >> (8 * s)) & (kCodes - 1), d1[s]);
                    } else if (s1 == kSrcAcc) {
                        f2 r[4][4];
                        tab.p_pair(e1, qg, r);
#pragma unroll
                        for (int s = 0; s < SPT; ++s) mv_pair(r, acc[s][q], d1[s]);
                    } else {
#pragma unroll
                        for (int s = 0; s < SPT; ++s)
#pragma unroll
                            for (int i = 0; i < 4; ++i) d1[s][i] = one2;
                    }
                    if (s0 >= 0) {
#pragma unroll
                        for (int s = 0; s < SPT; ++s) {
                            f2 d0[4];
                            tab.tip(s0, qg, (c0 >> (8 * s)) & (kCodes - 1), d0);
#pragma unroll
                            for (int i = 0; i < 4; ++i) acc[s][q][i] = mul2(d0[i], d1[s][i]);
                        }
                    } else {
                        f2 r[4][4];
                        tab.p_pair(e0, qg, r);
                        if (s0 == kSrcPop) {
                            uint32_t w[NC];
                            tmem_wait_st();
                            tmem_ld<NC>(tstack + (uint32_t)((sp * KPT + q) * NC), w);
                            tmem_wait_ld();
#pragma unroll
                            for (int s = 0; s < SPT; ++s) {
                                f2 x[4], d0[4];
#pragma unroll
                                for (int i = 0; i < 4; ++i)
                                    x[i] = pk2(__uint_as_float(w[8 * s + 2 * i]), __uint_as_float(w[8 * s + 2 * i + 1]));
                                mv_pair(r, x, d0);
#pragma unroll
                                for (int i = 0; i < 4; ++i) acc[s][q][i] = mul2(d0[i], d1[s][i]);
                            }
                        } else {
#pragma unroll
                            for (int s = 0; s < SPT; ++s) {
                                f2 d0[4];
                                mv_pair(r, acc[s][q], d0);
#pragma unroll
                                for (int i = 0; i < 4; ++i) acc[s][q][i] = mul2(d0[i], d1[s][i]);
                            }
                        }
                    }
                }
            }
            // a quick exact test first (TPS = 1, two or more pairs): when the
            // maximum of the first pair's eight values reaches the threshold
            // so does the node maximum, and no rescale follows; only when
            // some lane of the warp falls short does the warp take the full
            // maximum below, with the decision and factors it always had
            bool full_test = true;
            if constexpr (TPS == 1 && KPT >= 2) {
                bool near = false;
#pragma unroll
                for (int s = 0; s < SPT; ++s) {
                    const f2* a0 = acc[s][0];
                    const float pm = fmax3(fmax3(a0[0].x, a0[0].y, a0[1].x), fmax3(a0[1].y, a0[2].x, a0[2].y),
                                           fmaxf(a0[3].x, a0[3].y));
                    near |= !(pm >= scale_threshold<float>());
                }
                full_test = __any_sync(0xffffffffu, near);
            }
            if (full_test) {
#pragma unroll
                for (int s = 0; s < SPT; ++s) {
                    // the node maximum (three-input max: the same value as the
                    // fmaxf chain of run_tile4p; TPS = 2: with the partner's)
                    float v[KPT * 8];
#pragma unroll
                    for (int q = 0; q < KPT; ++q)
#pragma unroll
                        for (int i = 0; i < 4; ++i) unpack2(acc[s][q][i], v[q * 8 + 2 * i], v[q * 8 + 2 * i + 1]);
                    float mx;
                    if constexpr (KPT == 1) {
                        mx = fmax3(fmax3(v[0], v[1], v[2]), fmax3(v[3], v[4], v[5]), fmaxf(v[6], v[7]));
                    } else if constexpr (KPT == 2) {
                        const float m0x = fmax3(v[0], v[1], v[2]), m1x = fmax3(v[3], v[4], v[5]);
                        const float m2x = fmax3(v[6], v[7], v[8]), m3x = fmax3(v[9], v[10], v[11]);
                        const float m4x = fmax3(v[12], v[13], v[14]);
                        mx = fmax3(fmax3(m0x, m1x, m2x), fmax3(m3x, m4x, v[15]), 0.0f);
                    } else {
                        float m[11];
#pragma unroll
                        for (int k = 0; k < 10; ++k) m[k] = fmax3(v[3 * k], v[3 * k + 1], v[3 * k + 2]);
                        m[10] = fmaxf(v[30], v[31]);
                        const float g0 = fmax3(m[0], m[1], m[2]), g1 = fmax3(m[3], m[4], m[5]);
                        const float g2 = fmax3(m[6], m[7], m[8]), g3 = fmaxf(m[9], m[10]);
                        mx = fmax3(fmax3(g0, g1, g2), g3, 0.0f);
                    }
                    if constexpr (TPS == 2) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
                    if (mx < scale_threshold<float>() && mx > 0.0f) {
                        int e;
                        float g1, g2;
                        pow2_factors(mx, &e, &g1, &g2);
                        const f2 h1 = pk2(g1, g1), h2 = pk2(g2, g2);
#pragma unroll
                        for (int q = 0; q < KPT; ++q)
#pragma unroll
                            for (int i = 0; i < 4; ++i) acc[s][q][i] = mul2(mul2(acc[s][q][i], h1), h2);
                        scale_e[s] += e;
                    }
                }
            }
            if (push) {
                // the slot's columns, all pairs (KPT x NC), leave in as few
                // instructions as fit; the wait for them stands before the
                // next pop's loads
                uint32_t w[KPT * NC];
#pragma unroll
                for (int q = 0; q < KPT; ++q)
#pragma unroll
                    for (int s = 0; s < SPT; ++s)
#pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            float lo, hi;
                            unpack2(acc[s][q][i], lo, hi);
                            w[q * NC + 8 * s + 2 * i] = __float_as_uint(lo);
                            w[q * NC + 8 * s + 2 * i + 1] = __float_as_uint(hi);
                        }
                const uint32_t ta = tstack + (uint32_t)(sp * KPT * NC);
                if constexpr (KPT * NC <= 32) {
                    tmem_st<KPT * NC>(ta, w);
                } else {
#pragma unroll
                    for (int q = 0; q < KPT; ++q) {
                        uint32_t wq[NC];
#pragma unroll
                        for (int k = 0; k < NC; ++k) wq[k] = w[q * NC + k];
                        tmem_st<NC>(ta + (uint32_t)(q * NC), wq);
                    }
                }
                ++sp;
            }
            c0 = n0;
            c1 = n1;
            n0 = m0;
            n1 = m1;
        }

        // root: L = sum_k w_k sum_s v_k[s] root_w[s] in FP32, categories in
        // order (run_tile4p), log L = lm + ee ln 2
        float rw[4], cw[2 * KP];
#pragma unroll
        for (int i = 0; i < 4; ++i) rw[i] = (float)a.root_w[i];
#pragma unroll
        for (int k = 0; k < 2 * KP; ++k) cw[k] = (float)a.cat_w[k];
#pragma unroll
        for (int s = 0; s < SPT; ++s) {
            float lk[2 * KP];  // this thread's categories first (the even lane's are 0 .. 2 KPT - 1)
#pragma unroll
            for (int q = 0; q < KPT; ++q) {
                float vv[2][4];
#pragma unroll
                for (int i = 0; i < 4; ++i) unpack2(acc[s][q][i], vv[0][i], vv[1][i]);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    float x = vv[h][0] * rw[0];
#pragma unroll
                    for (int i = 1; i < 4; ++i) x = fmaf(vv[h][i], rw[i], x);
                    lk[2 * q + h] = x;
                }
            }
            if constexpr (TPS == 2) {
#pragma unroll
                for (int k = 0; k < 2 * KPT; ++k) lk[2 * KPT + k] = __shfl_xor_sync(0xffffffffu, lk[k], 1);
            }
            float lsum = 0.0f;
#pragma unroll
            for (int k = 0; k < 2 * KP; ++k) lsum = fmaf(cw[k], lk[k], lsum);
            const int site = base + s;
            if (site < a.n_sites && half == 0) {
                float lm;
                int ee;
                site_log32(lsum, scale_e[s], lm, ee);
                if (a.site_lnl) a.site_lnl[site] = site_lnl64(lm, ee);
                site_sum_add(sum, lm, ee);
            }
        }
    }
    // every warp is done with its stack (its stores complete): free the TMEM
    tmem_wait_st();
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(s_tmem), "r"(tmem_cols)
                     : "memory");
    }
    const SiteSum32 bsum = block_sum_site32f(sum);
    if (tid == 0) store_site_record(a.block_sum, blockIdx.x, bsum);
    if (a.grid_done) finish_grid_sum32(a.block_sum, a.grid_done, a.lnl_out);
}

template <int KP, int SPT, int TS, int TPS = 1>
const void* prune4w_fn() {
    return reinterpret_cast<const void*>(prune4w_kernel<KP, SPT, TS, TPS>);
}

const void* prune4w_fn_of(int KP, int SPT, int TS, int TPS = 1) {
    if (TPS == 2) return KP == 2 ? prune4w_fn<2, 2, 1, 2>() : prune4w_fn<4, 2, 1, 2>();
    if (TS) {
        switch (KP * 10 + SPT) {
            case 11: return prune4w_fn<1, 1, 1>();
            case 12: return prune4w_fn<1, 2, 1>();
            case 14: return prune4w_fn<1, 4, 1>();
            case 21: return prune4w_fn<2, 1, 1>();
            case 22: return prune4w_fn<2, 2, 1>();
            case 24: return prune4w_fn<2, 4, 1>();
            case 41: return prune4w_fn<4, 1, 1>();
            default: return prune4w_fn<4, 2, 1>();
        }
    }
    switch (KP * 10 + SPT) {
        case 11: return prune4w_fn<1, 1, 0>();
        case 12: return prune4w_fn<1, 2, 0>();
        case 14: return prune4w_fn<1, 4, 0>();
        case 21: return prune4w_fn<2, 1, 0>();
        case 22: return prune4w_fn<2, 2, 0>();
        case 24: return prune4w_fn<2, 4, 0>();
        case 41: return prune4w_fn<4, 1, 0>();
        default: return prune4w_fn<4, 2, 0>();
    }
}

// shared memory of the TS = 1 form: the tree's paired tables
size_t prune4w_table_bytes(const PruneArgs& a) {
    return (size_t)a.n_nodes * (a.C / 2) * 128 + (size_t)a.n_tips * (a.C / 2) * 512 + (size_t)a.n_ops * sizeof(Op);
}
constexpr size_t kWMaxTable = kMaxSmem - 8 * 1024;

// TMEM columns a CTA of `warps` warps needs for stacks of `depth` slots: the
// warps sharing a lane quarter stack their column ranges; a power of two of
// at least 32 (0: more than the 512 an SM has)
int prune4w_tmem_cols(int KP, int SPT, int warps, int depth, int TPS = 1) {
    const int need = ((warps + 3) / 4) * (depth > 0 ? depth : 1) * (KP / TPS) * 8 * SPT;
    int cols = 32;
    while (cols < need) cols *= 2;
    return cols <= 512 ? cols : 0;
}

// resident CTAs per SM with `warps` warps (occupancy calculator, cached: the
// launch runs every evaluation); the carveout gives the L1 cache all the
// shared memory the kernel does not use
int prune4w_ctas_per_sm(int KP, int SPT, int TS, int warps, size_t smem, int TPS = 1) {
    if (TS) {  // sized per launch (the tables): cached per device, context, kernel, warps and bytes
        const void* fn = prune4w_fn_of(KP, SPT, 1, TPS);
        int dev = 0;
        cudaGetDevice(&dev);
        const unsigned long long ctx = current_ctx_id();  // a device reset starts the caches over
        static std::mutex mu;
        static std::map<std::tuple<int, unsigned long long, const void*, int, size_t>, int> occ;
        static std::map<std::tuple<int, unsigned long long, const void*>, size_t> attr;  // the largest size allowed
        std::lock_guard<std::mutex> lock(mu);
        size_t& allowed = attr[std::make_tuple(dev, ctx, fn)];
        if (smem > allowed) {
            if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
            allowed = smem;
        }
        const auto key = std::make_tuple(dev, ctx, fn, warps, smem);
        const auto it = occ.find(key);
        if (it != occ.end()) return it->second;
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, warps * 32, smem) != cudaSuccess) n = 0;
        occ[key] = n;
        return n;
    }
    static std::atomic<int> cache[3][3][kWMaxWarps + 1];
    static std::atomic<bool> init{false};
    if (!init.load()) {
        for (auto& a : cache)
            for (auto& b : a)
                for (auto& c : b) c.store(-1);
        init.store(true);
    }
    const int ki = KP == 1 ? 0 : (KP == 2 ? 1 : 2), si = SPT == 1 ? 0 : (SPT == 2 ? 1 : 2);
    int v = cache[ki][si][warps].load();
    if (v >= 0) return v;
    const void* fn = prune4w_fn_of(KP, SPT, 0);
    cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, warps * 32, 0) != cudaSuccess) n = 0;
    cache[ki][si][warps].store(n);
    return n;
}

int sm_count() {
    static std::atomic<int> n{0};
    int v = n.load();
    if (v > 0) return v;
    int dev = 0, c = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || c <= 0) c = 1;
    n.store(c);
    return c;
}

// warps per CTA: enough that every SM's CTA has a tile per warp where the
// tiles allow, at most what keeps the stacks within the TMEM and the
// registers (and, for TS = 1, the tables) within one CTA per SM (0: no size
// works)
int prune4w_warps(int KP, int SPT, int TS, int TPS, size_t smem, int depth, int tiles, int sms) {
    int hi = 0;
    for (int w = kWMaxWarps; w >= kWMinWarps; --w)
        if (prune4w_tmem_cols(KP, SPT, w, depth, TPS) > 0 && prune4w_ctas_per_sm(KP, SPT, TS, w, smem, TPS) >= 1) {
            hi = w;
            break;
        }
    if (hi == 0) return 0;
    const int want = (tiles + sms - 1) / sms;
    return std::max(kWMinWarps, std::min(hi, want));
}

}  // namespace

bool prune4w_fits(const PruneArgs& a, int spt, int ts, int tps) {
    if (a.C != 2 && a.C != 4 && a.C != 8) return false;
    if (spt != 1 && spt != 2 && spt != 4) return false;
    if (tps == 2 && (a.C == 2 || spt != 2 || !ts)) return false;  // instantiated: two sites, shared tables
    if (tps == 2)
        return prune4w_table_bytes(a) <= kWMaxTable && prune4w_tmem_cols(a.C / 2, spt, kWMinWarps, a.max_depth, 2) > 0;
    if (spt == 4 && a.C == 8) return false;  // four sites of 8 categories exceed the registers
    if (ts && prune4w_table_bytes(a) > kWMaxTable) return false;
    return prune4w_tmem_cols(a.C / 2, spt, kWMinWarps, a.max_depth) > 0;
}

cudaError_t launch_prune4w(const PruneArgs& a, int spt, int ts, int tps, int* n_blocks, cudaStream_t st) {
    if (!prune4w_fits(a, spt, ts, tps) || a.scratch == nullptr) return cudaErrorInvalidValue;
    const int KP = a.C / 2;
    float *Pp, *Tp;
    prune4p_scratch_parts(a.scratch, a.n_nodes, a.C, &Pp, &Tp);
    if (!a.paired_ready) {
        cudaError_t e = launch_relayout4p(a, Pp, Tp, st);
        if (e != cudaSuccess) return e;
    }
    const size_t smem = ts ? prune4w_table_bytes(a) : 0;
    const int ws = 32 / tps * spt;  // sites per warp tile
    const int tiles = (a.n_sites + ws - 1) / ws;
    const int sms = sm_count();
    const int warps = prune4w_warps(KP, spt, ts, tps, smem, a.max_depth, tiles, sms);
    if (warps == 0) return cudaErrorInvalidConfiguration;
    const int tmem_cols = prune4w_tmem_cols(KP, spt, warps, a.max_depth, tps);
    const int blocks = std::max(1, std::min(sms, (tiles + warps - 1) / warps));
    *n_blocks = blocks;
    // launched with programmatic stream serialization: the CTAs may be
    // scheduled while the P(t) kernel before them finishes (it lets its
    // dependents launch at its start); the kernel waits for it
    // (griddepcontrol.wait) before reading anything it wrote
    const void* fn = prune4w_fn_of(KP, spt, ts, tps);
    PruneArgs args_a = a;
    const float* args_p = Pp;
    const float* args_t = Tp;
    int args_cols = tmem_cols;
    void* args[] = {&args_a, &args_p, &args_t, &args_cols};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(warps * 32);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelExC(&cfg, fn, args);
}

}  // namespace plk
