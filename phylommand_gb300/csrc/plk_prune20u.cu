// prune20u: the 20-state FP32 post-order pass (src/simpleML.cpp:127-197 for
// S = 20) with the child messages on Blackwell's fifth-generation tensor
// cores: tcgen05.mma kind::tf32 with the accumulators in tensor memory (TMEM).
//
// A CTA takes 128 sites of one rate category (grid = tiles x C); thread t
// owns site t, which is lane t of the TMEM accumulators.  For an internal
// child the message M[site][i] = sum_j V[site][j] P[i][j] is one
// M = 128 x N = 32 x K = 24 product (20 states, padded), split in TF32 hi and
// lo parts, V_lo P_hi + V_hi P_lo + V_hi P_hi (about FP32 accuracy): nine
// tcgen05.mma of K = 8 issued by one thread into a TMEM accumulator and
// completed through an mbarrier.  Operands sit in shared memory in the
// K-major canonical layout without swizzle (8-row x 16-byte core matrices,
// 128 bytes between row blocks (SBO), the 4-column groups LBO apart):
//   * the running vector and a vector popped from the spill stack are written
//     row by row by their threads as A operands (hi and lo parts);
//   * P(t) arrives as a B operand image prepared by relayout20u_kernel and is
//     staged through a three-slot cp.async ring, two ops ahead;
//   * spilled vectors are thread-private rows in TMEM (tcgen05.st / ld).
// Tip children are look-ups in the staged tip table, laid out [state][code]
// so that the lanes of a warp, whose sites carry different codes, read
// different banks.  The root forms
// sum_s pi_s L[s] per site in FP32 for combine20_kernel.
//
// Every mbarrier wait is bounded: a wait that runs out sets the tile's sites
// to NaN (the evaluation then fails with a numeric error) and the CTA still
// frees its TMEM.  TMEM per CTA: 64 columns for the two accumulators plus 32
// per spill slot, rounded up to a power of two; the dynamic shared memory is
// padded so that no more CTAs fit on an SM than its 512 columns serve, so an
// allocation never waits.
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>

#include "plk_device.cuh"
#include "plk_internal.h"

namespace plk {
using namespace dev;

namespace {

constexpr int kS = 20;
constexpr int kTile = 128;
constexpr int kThreads = 128;
constexpr int kN = 32;                   // MMA N: output states, padded
constexpr int kAGroup = 16 * 128;        // bytes of a 4-column group of an A operand (LBO of A)
constexpr int kAPart = 6 * kAGroup;      // one TF32 part of an A operand (K = 24)
constexpr int kAOperand = 2 * kAPart;    // hi and lo
constexpr int kAPart5 = 5 * kAGroup;      // one TF32 part without its zero group (compact form)
constexpr int kAOperand5 = 2 * kAPart5;
constexpr int kBGroup = 4 * 128;         // bytes of a 4-column group of a B operand (LBO of B)
constexpr int kBPart = 6 * kBGroup;
constexpr int kBFloats = 2 * kBPart / 4;  // staged B image per (node, category): 1,536 floats
constexpr int kAccCols = 64;              // TMEM columns of the two accumulators
constexpr int kSlotCols = 32;             // TMEM columns per spill slot (20 used)
constexpr uint32_t kIdesc = (1u << 4)          // D: F32
                            | (2u << 7)        // A: TF32
                            | (2u << 10)       // B: TF32
                            | ((kN >> 3) << 17)    // N
                            | ((128 >> 4) << 24);  // M
constexpr int kWaitLimit = 1 << 20;       // try_wait rounds before a wait gives up (MMAs land in microseconds)

struct P20UArgs {
    PruneArgs a;
    const float* Ps;   // B images [node][category][kBFloats]
    const float* Ts;   // tip tables [tip][category][state][code (n_codes padded to 4)]
    float* cat_L;      // [C][n_sites]
    int* cat_E;        // [C][n_sites]
    float* spill;      // compact form: spilled vectors [CTA][slot][state][site of the tile]
    int child_bytes;   // bytes of one child's slot in a stage
    int tmem_cols;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// the same rounding in integer arithmetic (round to nearest, ties away from
// zero, at TF32's 10-bit mantissa: half of the last kept bit added to the
// magnitude, the 13 dropped bits cleared); equal to cvt.rna.tf32.f32 for
// every finite value that does not round past the largest float
__device__ __forceinline__ float tf32_round_int(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// shared-memory matrix descriptor: K-major, no swizzle (layout type 0),
// descriptor version 1
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ void umma_tf32(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase) {
    for (int i = 0; i < kWaitLimit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// 20 columns of this thread's TMEM lane, the wait for the load inside the
// same statement so that no use of x can move ahead of it (warp-collective:
// the warp reconverges first)
__device__ __forceinline__ void tmem_ld20(uint32_t taddr, float x[kS]) {
    uint32_t r[kS];
    __syncwarp();
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%20];\n"
        "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%16,%17,%18,%19}, [%21];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19])
        : "r"(taddr), "r"(taddr + 16)
        : "memory");
#pragma unroll
    for (int i = 0; i < kS; ++i) x[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_st20(uint32_t taddr, const float x[kS]) {
    __syncwarp();
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17};\n"
        "tcgen05.st.sync.aligned.32x32b.x4.b32 [%1], {%18,%19,%20,%21};\n"
        "tcgen05.wait::st.sync.aligned;\n" ::"r"(taddr),
        "r"(taddr + 16), "r"(__float_as_uint(x[0])), "r"(__float_as_uint(x[1])), "r"(__float_as_uint(x[2])),
        "r"(__float_as_uint(x[3])), "r"(__float_as_uint(x[4])), "r"(__float_as_uint(x[5])),
        "r"(__float_as_uint(x[6])), "r"(__float_as_uint(x[7])), "r"(__float_as_uint(x[8])),
        "r"(__float_as_uint(x[9])), "r"(__float_as_uint(x[10])), "r"(__float_as_uint(x[11])),
        "r"(__float_as_uint(x[12])), "r"(__float_as_uint(x[13])), "r"(__float_as_uint(x[14])),
        "r"(__float_as_uint(x[15])), "r"(__float_as_uint(x[16])), "r"(__float_as_uint(x[17])),
        "r"(__float_as_uint(x[18])), "r"(__float_as_uint(x[19]))
        : "memory");
}

// row t of an A operand: TF32 hi and lo parts of the 20 values, the lo part
// APART bytes after the hi part.  With APART = kAPart the columns 20-23 of
// each part are a group of their own that stays zero; with APART = kAPart5
// the K step over columns 16-23 reads the next part's first group (or the
// zero pad after the last operand) as columns 20-23: finite values that meet
// the zero rows 20-23 of every B image, so they add exact zeros.
template <int APART>
__device__ __forceinline__ void write_operand(unsigned char* area, int t, const float x[kS]) {
    const int row = (t >> 3) * 128 + (t & 7) * 16;
#pragma unroll
    for (int g = 0; g < 5; ++g) {
        float4 h, l;
        h.x = tf32_round_int(x[4 * g]);
        h.y = tf32_round_int(x[4 * g + 1]);
        h.z = tf32_round_int(x[4 * g + 2]);
        h.w = tf32_round_int(x[4 * g + 3]);
        l.x = tf32_round_int(x[4 * g] - h.x);
        l.y = tf32_round_int(x[4 * g + 1] - h.y);
        l.z = tf32_round_int(x[4 * g + 2] - h.z);
        l.w = tf32_round_int(x[4 * g + 3] - h.w);
        *reinterpret_cast<float4*>(area + g * kAGroup + row) = h;
        *reinterpret_cast<float4*>(area + APART + g * kAGroup + row) = l;
    }
}

// nine MMAs of one child message into the accumulator at d_tmem (A's lo
// part APART bytes after its hi part)
template <int APART>
__device__ __forceinline__ void issue_child(uint32_t d_tmem, uint32_t a_addr, uint32_t b_addr) {
#pragma unroll
    for (int ks = 0; ks < 3; ++ks) {
        const uint64_t a_hi = smem_desc(a_addr + ks * 2 * kAGroup, kAGroup, 128);
        const uint64_t a_lo = smem_desc(a_addr + APART + ks * 2 * kAGroup, kAGroup, 128);
        const uint64_t b_hi = smem_desc(b_addr + ks * 2 * kBGroup, kBGroup, 128);
        const uint64_t b_lo = smem_desc(b_addr + kBPart + ks * 2 * kBGroup, kBGroup, 128);
        umma_tf32(d_tmem, a_lo, b_hi, ks > 0 ? 1u : 0u);  // small products first
        umma_tf32(d_tmem, a_hi, b_lo, 1u);
        umma_tf32(d_tmem, a_hi, b_hi, 1u);
    }
}

// The same nine MMAs from precomputed descriptor low words: a descriptor's
// high word (SBO 128 B, version bit) is the same for every operand here, and
// its low word is (address >> 4) | (LBO >> 4) << 16, so an operand at base +
// off has the low word of base plus off >> 4 (shared-memory addresses stay
// below 2^18: no carry into the LBO field).
constexpr uint32_t kDescHi = (128u >> 4) | (1u << 14);

__device__ __forceinline__ uint32_t desc_lo(uint32_t addr, uint32_t lbo) {
    return ((addr >> 4) & 0x3FFFu) | (((lbo >> 4) & 0x3FFFu) << 16);
}

__device__ __forceinline__ uint64_t desc_of(uint32_t lo) { return ((uint64_t)kDescHi << 32) | lo; }

template <int APART>
__device__ __forceinline__ void issue_child_lo(uint32_t d_tmem, uint32_t a_lo, uint32_t b_lo) {
#pragma unroll
    for (int ks = 0; ks < 3; ++ks) {
        const uint64_t a_hi = desc_of(a_lo + ks * 2 * kAGroup / 16);
        const uint64_t a_l = desc_of(a_lo + (APART + ks * 2 * kAGroup) / 16);
        const uint64_t b_hi = desc_of(b_lo + ks * 2 * kBGroup / 16);
        const uint64_t b_l = desc_of(b_lo + (kBPart + ks * 2 * kBGroup) / 16);
        umma_tf32(d_tmem, a_l, b_hi, ks > 0 ? 1u : 0u);  // small products first
        umma_tf32(d_tmem, a_hi, b_l, 1u);
        umma_tf32(d_tmem, a_hi, b_hi, 1u);
    }
}

// ---- the split-BF16 form (kind::f16, both operands BF16, FP32 accumulate) --
// A value x is split into hi = bf16(x) and lo = bf16(x - hi) (x - hi is exact
// in FP32); a child message is lo*hi + hi*lo + hi*hi over K = 32 (20 states,
// padded), two K steps of 16 each: six MMAs instead of the split TF32's nine.
// The dropped lo*lo term and the rounding of lo leave about 2^-16 relative
// per product.  An A operand part holds K columns 0-23 as three 8-column
// groups (16 bytes of BF16 per row); the second K step reads columns 16-31,
// whose last group is the next part's first group (or the zero group after
// the last operand): finite values that meet the zero rows 24-31 of every B
// image.  A B image part holds K = 32 as four 8-column groups of 32 rows.
constexpr int kAPartB = 3 * kAGroup;      // one BF16 part of an A operand
constexpr int kAOperandB = 2 * kAPartB;
constexpr int kBPartB = kB16PartBytes;    // one BF16 part of a B image: 4 groups of 32 rows x 16 bytes
constexpr int kBBytesB = kB16Bytes;       // hi and lo: 4 KB, within the 6 KB slot of a TF32 image
static_assert(kBPartB == 4 * kBGroup, "BF16 image part");
constexpr uint32_t kIdescB = (1u << 4)          // D: F32
                             | (1u << 7)        // A: BF16
                             | (1u << 10)       // B: BF16
                             | ((kN >> 3) << 17)    // N
                             | ((128 >> 4) << 24);  // M

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(kIdescB), "r"(accumulate));
}

// row t of a BF16 A operand: hi part, then the lo part kAPartB bytes later;
// columns 20-23 of the third group are zero
__device__ __forceinline__ void write_operand_bf16(unsigned char* area, int t, const float x[kS]) {
    const int row = (t >> 3) * 128 + (t & 7) * 16;
#pragma unroll
    for (int g = 0; g < 3; ++g) {
        uint4 h, l;
        bf16_split2(x[8 * g], x[8 * g + 1], h.x, l.x);
        bf16_split2(x[8 * g + 2], x[8 * g + 3], h.y, l.y);
        if (g < 2) {
            bf16_split2(x[8 * g + 4], x[8 * g + 5], h.z, l.z);
            bf16_split2(x[8 * g + 6], x[8 * g + 7], h.w, l.w);
        } else {
            h.z = h.w = l.z = l.w = 0u;
        }
        *reinterpret_cast<uint4*>(area + g * kAGroup + row) = h;
        *reinterpret_cast<uint4*>(area + kAPartB + g * kAGroup + row) = l;
    }
}

// the six MMAs of one child message, from descriptor low words
__device__ __forceinline__ void issue_child_bf16(uint32_t d_tmem, uint32_t a_lo, uint32_t b_lo) {
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
        const uint64_t a_hi = desc_of(a_lo + ks * 2 * kAGroup / 16);
        const uint64_t a_l = desc_of(a_lo + (kAPartB + ks * 2 * kAGroup) / 16);
        const uint64_t b_hi = desc_of(b_lo + ks * 2 * kBGroup / 16);
        const uint64_t b_l = desc_of(b_lo + (kBPartB + ks * 2 * kBGroup) / 16);
        umma_bf16(d_tmem, a_l, b_hi, ks > 0 ? 1u : 0u);  // small products first
        umma_bf16(d_tmem, a_hi, b_l, 1u);
        umma_bf16(d_tmem, a_hi, b_hi, 1u);
    }
}

__host__ __device__ inline int codes_padded(int n_codes) { return (n_codes + 3) & ~3; }

// P(t) as B operand images and the tip tables transposed to [state][code]
__global__ void relayout20u_kernel(const float* __restrict__ P, const float* __restrict__ tip, int n_nodes,
                                   int n_tips, int C, int n_codes, float* __restrict__ Ps, float* __restrict__ Ts,
                                   int bf16) {
    const int ncs = codes_padded(n_codes);
    const long long n_p = (long long)n_nodes * C * kBFloats;
    const long long n_t = (long long)n_tips * C * kS * ncs;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n_p + n_t;
         idx += (long long)gridDim.x * blockDim.x) {
        if (idx < n_p && bf16) {
            // the BF16 image in the first kBBytesB bytes of the slot, one
            // 32-bit word (two elements) per index; the rest of the slot unused
            const long long nk = idx / kBFloats;
            const int w = (int)(idx % kBFloats);
            if (w >= kBBytesB / 4) continue;
            int part, i, j0;
            bf16_image_index(w, part, i, j0);
            float x0 = 0.0f, x1 = 0.0f;
            if (i < kS && j0 < kS) x0 = P[nk * kS * kS + i * kS + j0];
            if (i < kS && j0 + 1 < kS) x1 = P[nk * kS * kS + i * kS + j0 + 1];
            uint32_t hi, lo;
            bf16_split2(x0, x1, hi, lo);
            reinterpret_cast<uint32_t*>(Ps)[idx] = part == 0 ? hi : lo;
        } else if (idx < n_p) {
            // [part][group g][row block nb][row r][column c]: state i = 8 nb + r, j = 4 g + c
            const long long nk = idx / kBFloats;
            const int w = (int)(idx % kBFloats);
            const int part = w / (kBPart / 4), q = w % (kBPart / 4);
            const int g = q / 128, nb = (q / 32) % 4, r = (q / 4) % 8, c = q % 4;
            const int i = 8 * nb + r, j = 4 * g + c;
            float v = 0.0f;
            if (i < kS && j < kS) {
                const float x = P[nk * kS * kS + i * kS + j];
                const float hi = tf32_rna(x);
                v = part == 0 ? hi : tf32_rna(x - hi);
            }
            Ps[idx] = v;
        } else {
            const long long t = idx - n_p;
            const long long nk = t / (kS * ncs);  // tip * C + k
            const int w = (int)(t % (kS * ncs));
            const int i = w / ncs, code = w % ncs;
            Ts[t] = code < n_codes ? tip[(nk * n_codes + code) * kS + i] : 0.0f;
        }
    }
}

__device__ __forceinline__ void stage_op20u(unsigned char* dst, const Op& op, int k, const P20UArgs& g) {
    const PruneArgs& a = g.a;
    for (int c = 0; c < 2; ++c) {
        const int src = c ? op.s1 : op.s0;
        if (src == kSrcNone) continue;
        const float* from;
        int n;
        if (src >= 0) {
            n = kS * codes_padded(a.n_codes);
            from = g.Ts + ((size_t)src * a.C + k) * (size_t)n;
        } else {
            n = kBFloats;
            from = g.Ps + ((size_t)(c ? op.e1 : op.e0) * a.C + k) * (size_t)kBFloats;
        }
        float* to = reinterpret_cast<float*>(dst + c * g.child_bytes);
        for (int q = threadIdx.x; q < n / 4; q += kThreads) cp_async16(to + 4 * q, from + 4 * q);
    }
}

// the same with the table's code stride NCS known at compile time (NCS = 0:
// read it from n_codes)
template <int NCS>
__device__ __forceinline__ void tip_row_n(const unsigned char* stage_child, int code, int n_codes, float m[kS]) {
    code = code < n_codes ? code : 0;
    const int ncs = NCS > 0 ? NCS : codes_padded(n_codes);
    const float* col = reinterpret_cast<const float*>(stage_child) + code;
#pragma unroll
    for (int i = 0; i < kS; ++i) m[i] = col[i * ncs];
}

__device__ __forceinline__ void tip_row(const unsigned char* stage_child, int code, int n_codes, float m[kS]) {
    code = code < n_codes ? code : 0;
    const int ncs = codes_padded(n_codes);
    const float* col = reinterpret_cast<const float*>(stage_child) + code;
#pragma unroll
    for (int i = 0; i < kS; ++i) m[i] = col[i * ncs];
}

// issued by one thread: an op's children (B images or tip tables) into a
// stage slot as 1-D bulk copies, completing in bytes on the slot's mbarrier
template <bool BF>
__device__ __forceinline__ void bulk_stage20(unsigned char* dst, const Op& op, int k, const P20UArgs& g,
                                             uint32_t full) {
    const PruneArgs& a = g.a;
    const uint32_t tip_bytes = kS * codes_padded(a.n_codes) * 4, b_bytes = BF ? kBBytesB : kBFloats * 4;
    uint32_t total = op.s0 >= 0 ? tip_bytes : b_bytes;
    if (op.s1 != kSrcNone) total += op.s1 >= 0 ? tip_bytes : b_bytes;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(full), "r"(total) : "memory");
    for (int c = 0; c < 2; ++c) {
        const int src = c ? op.s1 : op.s0;
        if (src == kSrcNone) continue;
        const float* from;
        uint32_t bytes;
        if (src >= 0) {
            bytes = tip_bytes;
            from = g.Ts + ((size_t)src * a.C + k) * (size_t)(tip_bytes / 4);
        } else {
            bytes = b_bytes;
            from = g.Ps + ((size_t)(c ? op.e1 : op.e0) * a.C + k) * (size_t)kBFloats;
        }
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                smem_u32(dst + c * g.child_bytes)),
            "l"(from), "r"(bytes), "r"(full)
            : "memory");
    }
}

__global__ void __launch_bounds__(kThreads, 1) prune20u_kernel(P20UArgs g) {
    asm volatile("griddepcontrol.wait;\n" ::: "memory");  // the kernel before it (P(t)) has completed
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t s_mbar;
    __shared__ uint32_t s_tmem;
    __shared__ float s_rw[kS];
    __shared__ int s_abort;
    const PruneArgs& a = g.a;
    const int k = blockIdx.y;
    const int tile0 = blockIdx.x * kTile;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int cb = g.child_bytes;
    unsigned char* acc_op = smem;               // A operand of the running vector
    unsigned char* pop_op = smem + kAOperand;   // A operand of a vector popped from the stack
    unsigned char* stages = smem + 2 * kAOperand;
    Op* s_ops = reinterpret_cast<Op*>(stages + 3 * 2 * cb);
    uint8_t* s_codes = reinterpret_cast<uint8_t*>(s_ops) + (((size_t)a.n_ops * sizeof(Op) + 15) & ~(size_t)15);
    const uint32_t mbar = smem_u32(&s_mbar);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&s_tmem)),
                     "r"(g.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        s_abort = 0;
    }
    if (tid < kS) s_rw[tid] = (float)a.root_w[tid];
    for (int i = tid; i < a.n_ops; i += kThreads) s_ops[i] = a.ops[i];
    {
        constexpr int chunks = kTile / 16;
        for (int i = tid; i < a.n_tips * chunks; i += kThreads) {
            const int t = i / chunks, q = i % chunks, col = tile0 + 16 * q;
            uint8_t* dst = s_codes + (size_t)t * kTile + 16 * q;
            if (col < a.site_stride) cp_async16(dst, a.codes + (size_t)t * a.site_stride + col);
            else *reinterpret_cast<uint4*>(dst) = make_uint4(0u, 0u, 0u, 0u);
        }
    }
    // columns 20-23 (group 5) of both parts of both A operands stay zero
    for (int i = tid; i < 4 * (kAGroup / 16); i += kThreads) {
        const int part = i / (kAGroup / 16), q = i % (kAGroup / 16);
        unsigned char* base = (part < 2 ? acc_op : pop_op) + (part % 2) * kAPart + 5 * kAGroup;
        reinterpret_cast<uint4*>(base)[q] = make_uint4(0u, 0u, 0u, 0u);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s_tmem;
    const uint32_t lane = tmem + ((uint32_t)(warp * 32) << 16);  // this warp's TMEM lanes
    stage_op20u(stages, s_ops[0], k, g);
    cp_async_commit();
    if (a.n_ops > 1) stage_op20u(stages + 2 * cb, s_ops[1], k, g);
    cp_async_commit();

    float m0[kS], m1[kS];
    int e_site = 0, sp = 0;
    uint32_t phase = 0;
    bool pending = false;  // an MMA commit whose completion was not observed
    bool withheld = false;  // the failure-path test withholds the first commit
    for (int o = 0; o < a.n_ops; ++o) {
        cp_async_wait<1>();
        const Op op = s_ops[o];
        if (op.s0 == kSrcPop) {
            --sp;
            tmem_ld20(lane + kAccCols + kSlotCols * sp, m0);
            write_operand<kAPart>(pop_op, tid, m0);
        }
        fence_proxy_async();  // cp.async data and operand rows -> the tensor cores
        tc_fence_before();
        __syncthreads();
        if (s_abort) break;
        if (o + 2 < a.n_ops) stage_op20u(stages + ((o + 2) % 3) * 2 * cb, s_ops[o + 2], k, g);
        cp_async_commit();
        const unsigned char* st = stages + (o % 3) * 2 * cb;
        const bool mma0 = op.s0 < 0, mma1 = op.s1 == kSrcAcc;
        if (tid == 0 && (mma0 || mma1)) {
            tc_fence_after();
            if (mma0) issue_child<kAPart>(tmem, smem_u32(op.s0 == kSrcPop ? pop_op : acc_op), smem_u32(st));
            if (mma1) issue_child<kAPart>(tmem + 32, smem_u32(acc_op), smem_u32(st + cb));
            if (!(a.withhold_first_stage && !withheld)) umma_commit(mbar);
        }
        if ((mma0 || mma1) && a.withhold_first_stage) withheld = true;
        if (op.s0 >= 0) tip_row(st, s_codes[(size_t)op.s0 * kTile + tid], a.n_codes, m0);
        if (op.s1 >= 0) tip_row(st + cb, s_codes[(size_t)op.s1 * kTile + tid], a.n_codes, m1);
        if (mma0 || mma1) {
            pending = true;
            if (!mbar_wait(mbar, phase)) s_abort = 1;
            else pending = false;
            phase ^= 1u;
            tc_fence_after();
            if (mma0) tmem_ld20(lane, m0);
            if (mma1) tmem_ld20(lane + 32, m1);
        }
        if (op.s1 != kSrcNone) {
#pragma unroll
            for (int i = 0; i < kS; ++i) m0[i] *= m1[i];
        }
        float mx = 0.0f;
#pragma unroll
        for (int i = 0; i < kS; ++i) mx = fmaxf(mx, m0[i]);
        if (mx < scale_threshold<float>() && mx > 0.0f) {
            int e;
            float f1, f2;
            pow2_factors(mx, &e, &f1, &f2);
#pragma unroll
            for (int i = 0; i < kS; ++i) m0[i] = (m0[i] * f1) * f2;
            e_site += e;
        }
        if (o == a.n_ops - 1) break;  // the root vector stays in m0
        if (op.push) {
            tmem_st20(lane + kAccCols + kSlotCols * sp, m0);
            ++sp;
        } else {
            write_operand<kAPart>(acc_op, tid, m0);
        }
    }
    cp_async_wait<0>();
    // a commit still in flight after a timed-out wait.  In the failure-path
    // test the withheld commit is issued now and waited for, so that every
    // MMA this CTA issued is seen to complete before its TMEM and shared
    // memory are given up.
    if (a.withhold_first_stage && withheld) {
        if (tid == 0) umma_commit(mbar);
        mbar_wait(mbar, phase ^ 1u);
    } else if (pending) {
        mbar_wait(mbar, phase ^ 1u);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(g.tmem_cols)
                     : "memory");
    }
    // root: L = sum_s pi_s R[s] in FP32 (this category)
    float l = 0.0f;
#pragma unroll
    for (int i = 0; i < kS; ++i) l = fmaf(m0[i], s_rw[i], l);
    if (s_abort) l = __int_as_float(0x7fc00000);  // NaN: the evaluation reports a numeric error
    const int site = tile0 + tid;
    if (site < a.n_sites) {
        g.cat_L[(size_t)k * a.n_sites + site] = l;
        g.cat_E[(size_t)k * a.n_sites + site] = e_site;
    }
}

// The compact form of prune20u_kernel: the same MMAs and scaling with less
// shared memory and TMEM per CTA, so that three CTAs share an SM instead of
// two (a 128-site tile's op chain is latency-bound, and the grid is
// tiles x categories of such chains):
//   * A operands without their zero column group (20 KB instead of 24 KB,
//     one zero group after the last operand);
//   * a two-slot stage ring, one op ahead (24 KB instead of 36 KB), fed by
//     1-D bulk copies that one thread issues (completion counted in bytes
//     on the slot's mbarrier) instead of every thread's cp.async;
//   * spilled vectors in global memory (an L2-resident scratch written at a
//     push and read back one op before the pop, by the thread that wrote
//     them), so that TMEM holds only the two accumulators (64 columns);
//   * tip codes read from global memory one op ahead instead of staged.
// BF: the split-BF16 products (kind::f16) instead of split TF32: smaller A
// operands and B images (four CTAs per SM), six MMAs per child message.
// the op record o (32 bytes, 32-byte aligned) through the read-only path: the
// same address in every thread
__device__ __forceinline__ Op ldg_op(const Op* ops, int o) {
    const int4 x = __ldg(reinterpret_cast<const int4*>(ops + o));
    const int4 y = __ldg(reinterpret_cast<const int4*>(ops + o) + 1);
    Op op;
    op.node = x.x;
    op.rank = x.y;
    op.e0 = x.z;
    op.e1 = x.w;
    op.s0 = y.x;
    op.s1 = y.y;
    op.push = y.z;
    op.pad = y.w;
    return op;
}

template <int NCS, bool BF>
__global__ void __launch_bounds__(kThreads, BF ? 5 : 3) prune20v_kernel(P20UArgs g) {
    asm volatile("griddepcontrol.wait;\n" ::: "memory");  // the kernel before it (P(t)) has completed
    constexpr int APART = BF ? kAPartB : kAPart5;
    constexpr int AOPER = 2 * APART;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t s_mbar;
    __shared__ __align__(8) uint64_t s_full[2];  // stage slots: bulk copies landed
    __shared__ uint32_t s_tmem;
    __shared__ float s_rw[kS];
    __shared__ int s_abort;
    const PruneArgs& a = g.a;
    const int k = blockIdx.y;
    const int tile0 = blockIdx.x * kTile;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int cb = g.child_bytes;
    unsigned char* acc_op = smem;                // A operand of the running vector
    unsigned char* pop_op = smem + AOPER;        // A operand of a vector popped from the stack
    unsigned char* stages = smem + 2 * AOPER + kAGroup;  // after the zero group
    // the op list: in shared memory (split TF32), or read through L1 (split
    // BF16, whose CTAs fit five to an SM only without it)
    Op* s_ops = reinterpret_cast<Op*>(stages + 2 * 2 * cb);
    auto load_op = [&](int o) -> Op {
        if constexpr (BF) return ldg_op(a.ops, o);
        else return s_ops[o];
    };
    const uint32_t mbar = smem_u32(&s_mbar);
    const uint32_t full0 = smem_u32(&s_full[0]);  // slot j's barrier: full0 + 8 j
    const int site = tile0 + tid;
    const bool has_code = site < a.site_stride;
    float* spill = g.spill + (size_t)(blockIdx.y * gridDim.x + blockIdx.x) * (size_t)(a.max_depth > 1 ? a.max_depth : 1) *
                                 (kS * kTile) + tid;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&s_tmem)),
                     "r"(g.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mbar) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(full0) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(full0 + 8) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        s_abort = 0;
    }
    if (tid < kS) s_rw[tid] = (float)a.root_w[tid];
    if constexpr (!BF)
        for (int i = tid; i < a.n_ops; i += kThreads) s_ops[i] = a.ops[i];
    // both A operands and the zero group after them: every column an MMA
    // reads is finite from the start
    for (int i = tid; i < (2 * AOPER + kAGroup) / 16; i += kThreads)
        reinterpret_cast<uint4*>(smem)[i] = make_uint4(0u, 0u, 0u, 0u);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s_tmem;
    const uint32_t lane = tmem + ((uint32_t)(warp * 32) << 16);  // this warp's TMEM lanes
    if (tid == 0) bulk_stage20<BF>(stages, load_op(0), k, g, full0);
    const uint32_t acc_lo = desc_lo(smem_u32(acc_op), kAGroup), pop_lo = desc_lo(smem_u32(pop_op), kAGroup);
    const uint32_t stage_lo = desc_lo(smem_u32(stages), kBGroup);  // slot j, child c: + (2 j + c) cb / 16

    auto code_of = [&](int src) -> int {
        if (src < 0 || !has_code) return 0;
        unsigned short v;  // not allocated in L1, which keeps the op list
        asm volatile("ld.global.nc.L1::no_allocate.u8 %0, [%1];\n"
                     : "=h"(v)
                     : "l"(a.codes + (size_t)src * a.site_stride + site));
        return (int)v;
    };
    // the op records of ops o, o + 1 and o + 2: each is read two ops before
    // its own, so no decision of an op waits on a load
    Op op = load_op(0);
    Op nx = a.n_ops > 1 ? load_op(1) : op;
    int c0 = code_of(op.s0), c1 = code_of(op.s1);
    float m0[kS], m1[kS], pre[kS];
    int e_site = 0, sp = 0;
    uint32_t phase = 0;
    bool pending = false;   // an MMA commit whose completion was not observed
    bool withheld = false;  // the failure-path test withholds the first commit
    int lost = -1;  // the op whose stage wait ran out: its copy may still land
    for (int o = 0; o < a.n_ops; ++o) {
        if (!mbar_wait(full0 + 8 * (o & 1), (uint32_t)(o >> 1) & 1u)) {
            lost = o;
            s_abort = 1;
        }
        const bool has_next = o + 1 < a.n_ops;
        const Op nn = o + 2 < a.n_ops ? load_op(o + 2) : nx;
        int n0 = 0, n1 = 0;
        bool next_pops = false;
        if (has_next) {
            n0 = code_of(nx.s0);
            n1 = code_of(nx.s1);
            next_pops = nx.s0 == kSrcPop;
        }
        if (op.s0 == kSrcPop) {
            --sp;
            if constexpr (BF) write_operand_bf16(pop_op, tid, pre);
            else write_operand<kAPart5>(pop_op, tid, pre);
        }
        fence_proxy_async();  // operand rows written by the threads -> the tensor cores
        tc_fence_before();
        __syncthreads();
        if (s_abort) break;
        // the slot op o-1 used: its MMAs completed and its tip rows were read
        // before the barrier
        if (tid == 0 && has_next)
            bulk_stage20<BF>(stages + ((o + 1) & 1) * 2 * cb, nx, k, g, full0 + 8 * ((o + 1) & 1));
        // the vector the next op pops (this op does not push when the next pops)
        if (next_pops) {
#pragma unroll
            for (int i = 0; i < kS; ++i) pre[i] = spill[(size_t)((sp - 1) * kS + i) * kTile];
        }
        const unsigned char* st = stages + (o & 1) * 2 * cb;
        const bool mma0 = op.s0 < 0, mma1 = op.s1 == kSrcAcc;
        if (tid == 0 && (mma0 || mma1)) {
            tc_fence_after();
            const uint32_t b0 = stage_lo + (uint32_t)((o & 1) * 2 * cb) / 16;
            if constexpr (BF) {
                if (mma0) issue_child_bf16(tmem, op.s0 == kSrcPop ? pop_lo : acc_lo, b0);
                if (mma1) issue_child_bf16(tmem + 32, acc_lo, b0 + (uint32_t)cb / 16);
            } else {
                if (mma0) issue_child_lo<kAPart5>(tmem, op.s0 == kSrcPop ? pop_lo : acc_lo, b0);
                if (mma1) issue_child_lo<kAPart5>(tmem + 32, acc_lo, b0 + (uint32_t)cb / 16);
            }
            if (!(a.withhold_first_stage && !withheld)) umma_commit(mbar);
        }
        if ((mma0 || mma1) && a.withhold_first_stage) withheld = true;
        if (op.s0 >= 0) tip_row_n<NCS>(st, c0, a.n_codes, m0);
        if (op.s1 >= 0) tip_row_n<NCS>(st + cb, c1, a.n_codes, m1);
        if (mma0 || mma1) {
            pending = true;
            if (!mbar_wait(mbar, phase)) s_abort = 1;
            else pending = false;
            phase ^= 1u;
            tc_fence_after();
            if (mma0) tmem_ld20(lane, m0);
            if (mma1) tmem_ld20(lane + 32, m1);
        }
        if (op.s1 != kSrcNone) {
#pragma unroll
            for (int i = 0; i < kS; ++i) m0[i] *= m1[i];
        }
        float mx;
        {  // a tree of maxima instead of a chain of twenty
            float t[10];
#pragma unroll
            for (int i = 0; i < 10; ++i) t[i] = fmaxf(m0[i], m0[i + 10]);
#pragma unroll
            for (int i = 0; i < 5; ++i) t[i] = fmaxf(t[i], t[i + 5]);
            mx = fmaxf(fmaxf(fmaxf(t[0], t[1]), fmaxf(t[2], t[3])), t[4]);
        }
        if (mx < scale_threshold<float>() && mx > 0.0f) {
            int e;
            float f1, f2;
            pow2_factors(mx, &e, &f1, &f2);
#pragma unroll
            for (int i = 0; i < kS; ++i) m0[i] = (m0[i] * f1) * f2;
            e_site += e;
        }
        if (o == a.n_ops - 1) break;  // the root vector stays in m0
        if (op.push) {
#pragma unroll
            for (int i = 0; i < kS; ++i) spill[(size_t)(sp * kS + i) * kTile] = m0[i];
            ++sp;
        } else {
            if constexpr (BF) write_operand_bf16(acc_op, tid, m0);
            else write_operand<kAPart5>(acc_op, tid, m0);
        }
        c0 = n0;
        c1 = n1;
        op = nx;
        nx = nn;
    }
    // every issued stage was waited for, unless a wait ran out: give that
    // copy one more bounded wait before the shared memory is given up
    if (lost >= 0) mbar_wait(full0 + 8 * (lost & 1), (uint32_t)(lost >> 1) & 1u);
    // a commit still in flight after a timed-out wait.  In the failure-path
    // test the withheld commit is issued now and waited for, so that every
    // MMA this CTA issued is seen to complete before its TMEM and shared
    // memory are given up.
    if (a.withhold_first_stage && withheld) {
        if (tid == 0) umma_commit(mbar);
        mbar_wait(mbar, phase ^ 1u);
    } else if (pending) {
        mbar_wait(mbar, phase ^ 1u);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(g.tmem_cols)
                     : "memory");
    }
    float l = 0.0f;
#pragma unroll
    for (int i = 0; i < kS; ++i) l = fmaf(m0[i], s_rw[i], l);
    if (s_abort) l = __int_as_float(0x7fc00000);
    if (site < a.n_sites) {
        g.cat_L[(size_t)k * a.n_sites + site] = l;
        g.cat_E[(size_t)k * a.n_sites + site] = e_site;
    }
    if (!a.tile_done) return;
    // the last of the tile's category CTAs combines them per site (the
    // arithmetic and block grouping of combine20_kernel: the same bits) and,
    // as the last tile, adds up the block sums
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(a.tile_done + blockIdx.x, 1u) == gridDim.y - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    SiteSum32 sum;
    if (site < a.n_sites) {
        int E = __ldcg(g.cat_E + site);
        for (int kk = 1; kk < a.C; ++kk) E = max(E, __ldcg(g.cat_E + (size_t)kk * a.n_sites + site));
        float lsum = 0.0f;
        for (int kk = 0; kk < a.C; ++kk)
            lsum = fmaf((float)a.cat_w[kk],
                        ldexpf(__ldcg(g.cat_L + (size_t)kk * a.n_sites + site),
                               __ldcg(g.cat_E + (size_t)kk * a.n_sites + site) - E),
                        lsum);
        float lm;
        int ee;
        site_log32(lsum, E, lm, ee);
        if (a.site_lnl) a.site_lnl[site] = site_lnl64(lm, ee);
        site_sum_add(sum, lm, ee);
    }
    const SiteSum32 bsum = block_sum_site32f(sum);
    if (tid == 0) {
        store_site_record(a.block_sum, blockIdx.x, bsum);
        a.tile_done[blockIdx.x] = 0u;  // re-armed for the next launch
    }
    if (a.grid_done) finish_grid_sum32(a.block_sum, a.grid_done, a.lnl_out);
}

int tmem_cols_for(const PruneArgs& a, int form) {
    if (form >= 1) return kAccCols;
    const int need = kAccCols + kSlotCols * std::max(a.max_depth, 1);
    int cols = 32;
    while (cols < need) cols *= 2;
    return cols;
}

int child_bytes_for(const PruneArgs& a, int form) {
    const int tip = kS * codes_padded(a.n_codes) * 4;
    return (std::max(form == 2 ? kBBytesB : 2 * kBPart, tip) + 127) & ~127;
}

size_t smem20u_bytes(const PruneArgs& a, int form) {
    const size_t ops = ((size_t)a.n_ops * sizeof(Op) + 15) & ~(size_t)15;
    // the split-BF16 compact form reads the op list through L1
    if (form == 1) return (size_t)2 * kAOperand5 + kAGroup + (size_t)2 * 2 * child_bytes_for(a, form) + ops;
    if (form == 2) return (size_t)2 * kAOperandB + kAGroup + (size_t)2 * 2 * child_bytes_for(a, form);
    return (size_t)2 * kAOperand + (size_t)3 * 2 * child_bytes_for(a, form) + ops + (size_t)a.n_tips * kTile;
}

size_t spill_bytes(const PruneArgs& a) {
    const size_t tiles = (size_t)(a.n_sites + kTile - 1) / kTile;
    return tiles * a.C * (size_t)std::max(a.max_depth, 1) * kS * kTile * sizeof(float);
}

}  // namespace

bool prune20u_fits(const PruneArgs& a, int form) {
    if (a.C < 1 || a.n_codes < 1 || a.n_ops < 1 || form < 0 || form > 2) return false;
    if (tmem_cols_for(a, form) > 512) return false;
    return smem20u_bytes(a, form) <= 200 * 1024;
}

void prune20u_scratch_parts(void* scratch, const PruneArgs& a, int n_nodes, float** B, float** T) {
    unsigned char* base = static_cast<unsigned char*>(scratch);
    *B = reinterpret_cast<float*>(base);
    *T = reinterpret_cast<float*>(base + ((((size_t)n_nodes * a.C * kBFloats * sizeof(float)) + 255) & ~(size_t)255));
}

int prune20u_codes_padded(int n_codes) { return codes_padded(n_codes); }

size_t prune20u_scratch_bytes(const PruneArgs& a, int n_nodes) {
    const size_t ps = (size_t)n_nodes * a.C * kBFloats * sizeof(float);
    const size_t ts = (size_t)a.n_tips * a.C * kS * codes_padded(a.n_codes) * sizeof(float);
    const size_t cl = (((size_t)a.C * a.n_sites * sizeof(float) + 255) & ~(size_t)255) +
                      (((size_t)a.C * a.n_sites * sizeof(int) + 255) & ~(size_t)255);
    return ((ps + 255) & ~(size_t)255) + ((ts + 255) & ~(size_t)255) + cl + spill_bytes(a);
}

// The dynamic shared memory of a launch of `ctas` chains: its own bytes,
// padded until an SM holds no more CTAs than (1) its TMEM serves (max_ctas)
// and (2) the fewest that still run the grid in the fewest rounds.  Every
// chain of a round takes about as long, so 628 chains at 4 per SM (608 in a
// first round, 20 in a second) take twice as long as at 5 per SM in one, and
// at 3 per SM (456 and 172) the two rounds are shorter than at 4.  Cached per
// device, context, kernel, bytes and grid: the attribute and occupancy calls cost
// microseconds of host time per launch.
static cudaError_t pick_ctas_per_sm(void (*kern)(P20UArgs), size_t base, int max_ctas, int ctas, size_t* smem_out) {
    static std::mutex mu;
    static std::map<std::tuple<int, unsigned long long, const void*, size_t, int, int>, size_t> cache;
    static std::map<std::tuple<int, unsigned long long, const void*>, size_t> allowed;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 1;
    const unsigned long long ctx = current_ctx_id();  // a device reset starts the caches over
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_tuple(dev, ctx, reinterpret_cast<const void*>(kern), base, max_ctas, ctas);
    const auto hit = cache.find(key);
    size_t& allow = allowed[std::make_tuple(dev, ctx, reinterpret_cast<const void*>(kern))];
    auto set_attr = [&](size_t bytes) -> cudaError_t {
        if (bytes <= allow) return cudaSuccess;
        const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        if (e == cudaSuccess) allow = bytes;
        return e;
    };
    if (hit != cache.end()) {
        *smem_out = hit->second;
        return set_attr(hit->second);
    }
    auto occupancy = [&](size_t bytes, int* occ) -> cudaError_t {
        const cudaError_t e = set_attr(bytes);
        if (e != cudaSuccess) return e;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, kern, kThreads, bytes);
    };
    int occ = 0;
    cudaError_t e = occupancy(base, &occ);
    if (e != cudaSuccess) return e;
    if (occ < 1) return cudaErrorInvalidConfiguration;
    const int most = std::min(occ, max_ctas);
    const int rounds = (ctas + sms * most - 1) / (sms * most);
    const int target = std::max(1, std::min(most, (ctas + sms * rounds - 1) / (sms * rounds)));
    size_t smem = base;
    while (occ > target) {
        smem += 1024;
        if (smem > 227 * 1024) return cudaErrorInvalidConfiguration;
        if ((e = occupancy(smem, &occ)) != cudaSuccess) return e;
    }
    if (occ < 1) return cudaErrorInvalidConfiguration;
    cache[key] = smem;
    *smem_out = smem;
    return cudaSuccess;
}

cudaError_t launch_prune20u(const PruneArgs& a, int n_nodes, void* scratch, int form, int* n_blocks,
                            cudaStream_t st) {
    if (!prune20u_fits(a, form) || scratch == nullptr) return cudaErrorInvalidValue;
    unsigned char* base = static_cast<unsigned char*>(scratch);
    P20UArgs g{};
    g.a = a;
    g.Ps = reinterpret_cast<float*>(base);
    size_t off = (((size_t)n_nodes * a.C * kBFloats * sizeof(float)) + 255) & ~(size_t)255;
    g.Ts = reinterpret_cast<float*>(base + off);
    off += (((size_t)a.n_tips * a.C * kS * codes_padded(a.n_codes) * sizeof(float)) + 255) & ~(size_t)255;
    g.cat_L = reinterpret_cast<float*>(base + off);
    off += (((size_t)a.C * a.n_sites * sizeof(float)) + 255) & ~(size_t)255;
    g.cat_E = reinterpret_cast<int*>(base + off);
    off += (((size_t)a.C * a.n_sites * sizeof(int)) + 255) & ~(size_t)255;
    g.spill = reinterpret_cast<float*>(base + off);
    g.child_bytes = child_bytes_for(a, form);
    g.tmem_cols = tmem_cols_for(a, form);
    if (!a.paired_ready) {  // else the P(t) kernel wrote both layouts
        const long long total =
            (long long)n_nodes * a.C * kBFloats + (long long)a.n_tips * a.C * kS * codes_padded(a.n_codes);
        long long blocks = (total + 255) / 256;
        if (blocks > 152 * 8) blocks = 152 * 8;
        relayout20u_kernel<<<(unsigned)blocks, 256, 0, st>>>(static_cast<const float*>(a.P),
                                                              static_cast<const float*>(a.tipT), n_nodes, a.n_tips,
                                                              a.C, a.n_codes, const_cast<float*>(g.Ps),
                                                              const_cast<float*>(g.Ts), form == 2 ? 1 : 0);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    void (*kern)(P20UArgs) = prune20u_kernel;
    if (form == 1) {
        const int ncs = codes_padded(a.n_codes);
        kern = ncs == 20 ? prune20v_kernel<20, false> : ncs == 24 ? prune20v_kernel<24, false>
                                                                  : prune20v_kernel<0, false>;
    } else if (form == 2) {
        const int ncs = codes_padded(a.n_codes);
        kern = ncs == 20 ? prune20v_kernel<20, true> : ncs == 24 ? prune20v_kernel<24, true>
                                                                 : prune20v_kernel<0, true>;
    }
    dim3 grid((a.n_sites + kTile - 1) / kTile, a.C);
    size_t smem = 0;
    const cudaError_t pe = pick_ctas_per_sm(kern, smem20u_bytes(a, form), 512 / g.tmem_cols, (int)(grid.x * grid.y), &smem);
    if (pe != cudaSuccess) return pe;
    // programmatic stream serialization: the CTAs may be scheduled while the
    // P(t) kernel before them finishes; the kernels wait for it
    // (griddepcontrol.wait) before reading anything it wrote
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, kern, g);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (form >= 1 && a.tile_done) {  // combined in the kernel
        *n_blocks = (int)grid.x;
        return cudaSuccess;
    }
    return launch_combine20(g.cat_L, g.cat_E, a, n_blocks, st);
}

}  // namespace plk
