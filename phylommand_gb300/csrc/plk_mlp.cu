// The warm-start network: a fully connected ReLU MLP trained and run with
// hand-written kernels (absent in the reference, whose optimiser always starts
// from fixed values, src/treeator.cpp:612-615).
//
//  gemm_tc_kernel    C[M x N] = sum_k A(m, k) B(n, k) with BF16 operands read
//                    through arbitrary strides (so one kernel serves X W^T,
//                    dZ W and dZ^T A), FP32 accumulation in tensor memory
//                    (tcgen05.mma kind::f16), fused epilogue: + bias, ReLU,
//                    ReLU mask of the backward pass, FP32 and/or BF16 stores.
//  loss_kernel       mean squared error over the real outputs and its
//                    gradient (BF16) for the backward GEMMs.
//  colsum_kernel     bias gradients.
//  adam_kernel       Adam (Kingma & Ba 2015) on the FP32 master weights, then
//                    the BF16 copies the GEMMs read.
// Weights are BF16 in every GEMM (the network's storage precision), master
// weights and optimiser moments FP32.  Feature dimensions are padded to 16
// and the batch to 64 with zeros.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_bf16.h>

#include "plk_internal.h"

namespace plk {

namespace {

inline int pad16(int x) { return (x + 15) & ~15; }
inline int pad64(int x) { return (x + 63) & ~63; }

struct GemmArgs {
    const __nv_bfloat16* A;
    long long sa_m, sa_k;
    const __nv_bfloat16* B;
    long long sb_n, sb_k;
    int M, N, K;
    const float* bias;           // [N] or null
    const __nv_bfloat16* mask;   // ReLU mask source (mask(m, n) > 0 keeps), or null
    long long smask_m;           // row stride of mask
    int relu;
    float* Cf;                   // fp32 out or null
    __nv_bfloat16* Cb;           // bf16 out or null
    long long ldc;
};

// loss = mean over rows < n_rows and columns < n_out of (y - t)^2;
// dY = 2 (y - t) / (n_rows n_out) as BF16, zero in the padding
__global__ void loss_kernel(const float* y, int ldy, const float* t, int n_rows, int rows_pad, int n_out, int cols_pad,
                            __nv_bfloat16* dy, float* loss) {
    __shared__ float red[256];
    float s = 0.f;
    const float scale = 2.f / ((float)n_rows * n_out);
    for (int i = threadIdx.x; i < rows_pad * cols_pad; i += blockDim.x) {
        const int r = i / cols_pad, c = i % cols_pad;
        float g = 0.f;
        if (r < n_rows && c < n_out) {
            const float d = y[r * ldy + c] - t[r * n_out + c];
            s += d * d;
            g = scale * d;
        }
        dy[r * cols_pad + c] = __float2bfloat16(g);
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) *loss = red[0] / ((float)n_rows * n_out);
}

__global__ void colsum_kernel(const __nv_bfloat16* d, int rows, int cols, int ld, float* out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float s = 0.f;
    for (int r = 0; r < rows; ++r) s += __bfloat162float(d[r * ld + c]);
    out[c] = s;
}

__global__ void adam_kernel(float* p, const float* g, float* m, float* v, int n, float lr, float b1, float b2, float eps,
                            float c1, float c2, __nv_bfloat16* pb, int rows, int cols, int ldb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    m[i] = b1 * m[i] + (1.f - b1) * gi;
    v[i] = b2 * v[i] + (1.f - b2) * gi * gi;
    p[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + eps);
    if (pb) {
        const int r = i / cols, c = i % cols;
        if (r < rows) pb[r * ldb + c] = __float2bfloat16(p[i]);
    }
}

__global__ void to_bf16_padded(const float* x, int rows, int cols, __nv_bfloat16* out, int rows_pad, int cols_pad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows_pad * cols_pad) return;
    const int r = i / cols_pad, c = i % cols_pad;
    out[i] = __float2bfloat16((r < rows && c < cols) ? x[r * cols + c] : 0.f);
}

// ---------------------------------------------------------------------------
// The same GEMM on Blackwell's fifth-generation tensor cores: a CTA computes a
// 128 x 64 tile of C with tcgen05.mma.kind::f16 (BF16 operands, FP32
// accumulator in TMEM), K in chunks of 64 staged in shared memory in the
// K-major canonical layout without swizzle (8-row x 16-byte core matrices:
// 16 bytes = 8 BF16 along K; A: 128 rows, 2 KB between K-adjacent core
// matrices; B: 32 rows, 512 bytes), four MMAs of K = 16 per chunk issued by one
// thread and completed through an mbarrier (a bounded wait: one that runs
// out turns the tile's outputs NaN, so the loss shows it).  The operands are
// gathered through the same arbitrary strides as gemm_bf16_kernel (rows and
// K beyond the matrix read as zero); the epilogue reads each thread's TMEM
// lane (its row) and applies the same bias / ReLU / mask.
// ---------------------------------------------------------------------------
constexpr int kGM = 128, kGN = 32, kGK = 64;  // N = 32: more CTAs for the network's small GEMMs
constexpr uint32_t kGIdesc = (1u << 4)            // D: F32
                             | (1u << 7)          // A: BF16
                             | (1u << 10)         // B: BF16
                             | ((kGN >> 3) << 17)  // N
                             | ((kGM >> 4) << 24); // M
constexpr int kGWaitLimit = 1 << 20;

__device__ __forceinline__ uint64_t g_smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__global__ void __launch_bounds__(128, 1) gemm_tc_kernel(GemmArgs g) {
    __shared__ __align__(128) __nv_bfloat16 As[kGM * kGK];  // [K group 8][row 128][8]
    __shared__ __align__(128) __nv_bfloat16 Bs[kGN * kGK];  // [K group 8][row 32][8]
    __shared__ __align__(8) uint64_t s_mbar;
    __shared__ uint32_t s_tmem;
    __shared__ int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * kGM, n0 = blockIdx.x * kGN;
    const uint32_t mbar = static_cast<uint32_t>(__cvta_generic_to_shared(&s_mbar));
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         static_cast<uint32_t>(__cvta_generic_to_shared(&s_tmem))),
                     "r"(kGN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        s_fail = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = s_tmem;
    const uint32_t a_base = static_cast<uint32_t>(__cvta_generic_to_shared(As));
    const uint32_t b_base = static_cast<uint32_t>(__cvta_generic_to_shared(Bs));
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    uint32_t phase = 0;
    for (int k0 = 0; k0 < g.K; k0 += kGK) {
        // element (row r, column c) of a chunk at [c / 8][r][c % 8]
        for (int i = tid; i < kGM * kGK; i += 128) {
            const int r = i / kGK, c = i % kGK, m = m0 + r, k = k0 + c;
            As[((c >> 3) * kGM + r) * 8 + (c & 7)] = (m < g.M && k < g.K) ? g.A[m * g.sa_m + k * g.sa_k] : zero;
        }
        for (int i = tid; i < kGN * kGK; i += 128) {
            const int r = i / kGK, c = i % kGK, n = n0 + r, k = k0 + c;
            Bs[((c >> 3) * kGN + r) * 8 + (c & 7)] = (n < g.N && k < g.K) ? g.B[n * g.sb_n + k * g.sb_k] : zero;
        }
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // the rows -> the tensor cores
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
            for (int ks = 0; ks < kGK / 16; ++ks) {
                const uint64_t ad = g_smem_desc(a_base + ks * 2 * (kGM * 16), kGM * 16, 128);
                const uint64_t bd = g_smem_desc(b_base + ks * 2 * (kGN * 16), kGN * 16, 128);
                const uint32_t accum = (k0 > 0 || ks > 0) ? 1u : 0u;
                asm volatile(
                    "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(kGIdesc), "r"(accum));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
                         : "memory");
        }
        // the chunk's MMAs done: the accumulator is current and the staged
        // operands may be overwritten (bounded wait)
        bool done = false;
        for (int it = 0; it < kGWaitLimit && !done; ++it) {
            uint32_t ok;
            asm volatile(
                "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                "selp.u32 %0, 1, 0, p;\n}\n"
                : "=r"(ok)
                : "r"(mbar), "r"(phase)
                : "memory");
            done = ok != 0;
        }
        if (!done) s_fail = 1;
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        __syncthreads();
        if (s_fail) {
            // the MMAs whose completion was not seen get one more bounded
            // wait before the CTA gives up their TMEM and operands
            for (int it = 0; it < kGWaitLimit; ++it) {
                uint32_t ok;
                asm volatile(
                    "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                    "selp.u32 %0, 1, 0, p;\n}\n"
                    : "=r"(ok)
                    : "r"(mbar), "r"(phase ^ 1u)
                    : "memory");
                if (ok) break;
            }
            break;
        }
    }
    // epilogue: this thread's row m0 + 32 warp + lane is its TMEM lane
    uint32_t r[kGN];
    const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16);
#pragma unroll
    for (int c = 0; c < kGN / 16; ++c)
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
            : "=r"(r[16 * c + 0]), "=r"(r[16 * c + 1]), "=r"(r[16 * c + 2]), "=r"(r[16 * c + 3]),
              "=r"(r[16 * c + 4]), "=r"(r[16 * c + 5]), "=r"(r[16 * c + 6]), "=r"(r[16 * c + 7]),
              "=r"(r[16 * c + 8]), "=r"(r[16 * c + 9]), "=r"(r[16 * c + 10]), "=r"(r[16 * c + 11]),
              "=r"(r[16 * c + 12]), "=r"(r[16 * c + 13]), "=r"(r[16 * c + 14]), "=r"(r[16 * c + 15])
            : "r"(taddr + 16 * c)
            : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
    const int m = m0 + 32 * warp + lane;
    const bool fail = s_fail != 0;
    if (m < g.M) {
#pragma unroll
        for (int c = 0; c < kGN; ++c) {
            const int n = n0 + c;
            if (n >= g.N) break;
            float v = fail ? __int_as_float(0x7fc00000) : __uint_as_float(r[c]);
            if (g.bias) v += g.bias[n];
            if (g.relu) v = fmaxf(v, 0.f);
            if (g.mask && !(__bfloat162float(g.mask[m * g.smask_m + n]) > 0.f)) v = 0.f;
            if (g.Cf) g.Cf[m * g.ldc + n] = v;
            if (g.Cb) g.Cb[m * g.ldc + n] = __float2bfloat16(v);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kGN) : "memory");
    }
}

cudaError_t gemm(const GemmArgs& g, cudaStream_t st) {
    dim3 grid((g.N + kGN - 1) / kGN, (g.M + kGM - 1) / kGM);
    gemm_tc_kernel<<<grid, 128, 0, st>>>(g);
    return cudaGetLastError();
}

}  // namespace
}  // namespace plk

using namespace plk;

struct plk_mlp {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    std::vector<int> dims;      // real sizes: n_in, hidden..., n_out
    std::vector<int> pdims;     // padded to 16
    std::vector<size_t> w_off, b_off;  // offsets of each layer's W [out x in] and b [out] in the flat vector
    size_t n_params = 0;
    float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;  // FP32 master, gradient, Adam moments
    std::vector<__nv_bfloat16*> wb;   // BF16 weight copies [pout x pin]
    int batch_cap = 0;
    std::vector<__nv_bfloat16*> act;  // BF16 activations [batch_pad x pdims[l]]
    std::vector<float*> pre;          // FP32 layer outputs [batch_pad x pdims[l]]
    __nv_bfloat16 *dz = nullptr, *dz2 = nullptr;
    float *xin = nullptr, *tin = nullptr, *loss = nullptr;
    long long step = 0;
    ~plk_mlp() {
        cudaFree(p); cudaFree(g); cudaFree(m); cudaFree(v);
        for (auto* q : wb) cudaFree(q);
        for (auto* q : act) cudaFree(q);
        for (auto* q : pre) cudaFree(q);
        cudaFree(dz); cudaFree(dz2); cudaFree(xin); cudaFree(tin); cudaFree(loss);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

plk_status mfail(plk_mlp* m, plk_status s, const std::string& msg) {
    if (m) m->err = msg;
    else report_error(s, msg);
    return s;
}

#define PLK_MCUDA(m, expr, what)                                                                        \
    do {                                                                                                \
        cudaError_t _e = (expr);                                                                        \
        if (_e != cudaSuccess)                                                                          \
            return mfail(m, _e == cudaErrorMemoryAllocation ? PLK_ERR_ALLOC : PLK_ERR_CUDA,              \
                         std::string(what) + ": " + cudaGetErrorString(_e));                            \
    } while (0)

int n_layers(const plk_mlp* m) { return (int)m->dims.size() - 1; }

plk_status ensure_batch(plk_mlp* m, int batch) {
    const int bp = pad64(batch);
    if (bp <= m->batch_cap) return PLK_OK;
    for (auto* q : m->act) cudaFree(q);
    for (auto* q : m->pre) cudaFree(q);
    m->act.assign(m->dims.size(), nullptr);
    m->pre.assign(m->dims.size(), nullptr);
    cudaFree(m->dz); cudaFree(m->dz2); cudaFree(m->xin); cudaFree(m->tin);
    int widest = 0;
    for (size_t l = 0; l < m->dims.size(); ++l) {
        widest = std::max(widest, m->pdims[l]);
        PLK_MCUDA(m, cudaMalloc(&m->act[l], (size_t)bp * m->pdims[l] * sizeof(__nv_bfloat16)), "allocate activations");
        PLK_MCUDA(m, cudaMalloc(&m->pre[l], (size_t)bp * m->pdims[l] * sizeof(float)), "allocate activations");
    }
    PLK_MCUDA(m, cudaMalloc(&m->dz, (size_t)bp * widest * sizeof(__nv_bfloat16)), "allocate gradients");
    PLK_MCUDA(m, cudaMalloc(&m->dz2, (size_t)bp * widest * sizeof(__nv_bfloat16)), "allocate gradients");
    PLK_MCUDA(m, cudaMalloc(&m->xin, (size_t)bp * m->dims.front() * sizeof(float)), "allocate inputs");
    PLK_MCUDA(m, cudaMalloc(&m->tin, (size_t)bp * m->dims.back() * sizeof(float)), "allocate targets");
    m->batch_cap = bp;
    return PLK_OK;
}

plk_status refresh_bf16(plk_mlp* m) {
    // BF16 copies of every layer's weights from the FP32 master
    std::vector<float> host(m->n_params);
    PLK_MCUDA(m, cudaMemcpy(host.data(), m->p, m->n_params * sizeof(float), cudaMemcpyDeviceToHost), "read weights");
    for (int l = 0; l < n_layers(m); ++l) {
        const int in = m->dims[l], out = m->dims[l + 1], pin = m->pdims[l], pout = m->pdims[l + 1];
        std::vector<__nv_bfloat16> w((size_t)pout * pin, __float2bfloat16(0.f));
        for (int r = 0; r < out; ++r)
            for (int c = 0; c < in; ++c) w[(size_t)r * pin + c] = __float2bfloat16(host[m->w_off[l] + (size_t)r * in + c]);
        PLK_MCUDA(m, cudaMemcpy(m->wb[l], w.data(), w.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice),
                  "upload weights");
    }
    return PLK_OK;
}

// forward of `batch` rows already in m->xin; leaves layer outputs in pre/act
plk_status forward(plk_mlp* m, int batch) {
    const int bp = pad64(batch);
    const int L = n_layers(m);
    const int total = bp * m->pdims[0];
    to_bf16_padded<<<(total + 255) / 256, 256, 0, m->stream>>>(m->xin, batch, m->dims[0], m->act[0], bp, m->pdims[0]);
    PLK_MCUDA(m, cudaGetLastError(), "input conversion");
    for (int l = 0; l < L; ++l) {
        GemmArgs ga{};
        ga.A = m->act[l]; ga.sa_m = m->pdims[l]; ga.sa_k = 1;
        ga.B = m->wb[l]; ga.sb_n = m->pdims[l]; ga.sb_k = 1;
        ga.M = bp; ga.N = m->pdims[l + 1]; ga.K = m->pdims[l];
        ga.bias = m->p + m->b_off[l];
        ga.relu = l < L - 1;
        ga.Cf = m->pre[l + 1];
        ga.Cb = m->act[l + 1];
        ga.ldc = m->pdims[l + 1];
        // the padded output columns beyond the real width carry bias reads;
        // restrict N to the real width and keep the padding zero
        ga.N = m->dims[l + 1];
        PLK_MCUDA(m, cudaMemsetAsync(m->act[l + 1], 0, (size_t)bp * m->pdims[l + 1] * sizeof(__nv_bfloat16), m->stream),
                  "clear activations");
        PLK_MCUDA(m, cudaMemsetAsync(m->pre[l + 1], 0, (size_t)bp * m->pdims[l + 1] * sizeof(float), m->stream),
                  "clear activations");
        PLK_MCUDA(m, gemm(ga, m->stream), "forward GEMM");
    }
    return PLK_OK;
}

// gradients of the mean squared error into m->g; loss into m->loss
plk_status backward(plk_mlp* m, int batch) {
    const int bp = pad64(batch);
    const int L = n_layers(m);
    loss_kernel<<<1, 256, 0, m->stream>>>(m->pre[L], m->pdims[L], m->tin, batch, bp, m->dims[L], m->pdims[L], m->dz,
                                          m->loss);
    PLK_MCUDA(m, cudaGetLastError(), "loss kernel");
    __nv_bfloat16* dz = m->dz;
    __nv_bfloat16* dn = m->dz2;
    for (int l = L - 1; l >= 0; --l) {
        const int in = m->dims[l], out = m->dims[l + 1], pin = m->pdims[l], pout = m->pdims[l + 1];
        // dW[out x in] = dZ^T A_prev
        GemmArgs gw{};
        gw.A = dz; gw.sa_m = 1; gw.sa_k = pout;
        gw.B = m->act[l]; gw.sb_n = 1; gw.sb_k = pin;
        gw.M = out; gw.N = in; gw.K = batch;
        gw.Cf = m->g + m->w_off[l];
        gw.ldc = in;
        PLK_MCUDA(m, gemm(gw, m->stream), "weight-gradient GEMM");
        colsum_kernel<<<(out + 127) / 128, 128, 0, m->stream>>>(dz, batch, out, pout, m->g + m->b_off[l]);
        PLK_MCUDA(m, cudaGetLastError(), "bias gradient");
        if (l > 0) {
            // dA_prev[B x in] = dZ W, masked by ReLU of layer l's input
            GemmArgs gd{};
            gd.A = dz; gd.sa_m = pout; gd.sa_k = 1;
            gd.B = m->wb[l]; gd.sb_n = 1; gd.sb_k = pin;
            gd.M = bp; gd.N = in; gd.K = out;
            gd.mask = m->act[l]; gd.smask_m = pin;
            gd.Cb = dn;
            gd.ldc = pin;
            PLK_MCUDA(m, cudaMemsetAsync(dn, 0, (size_t)bp * pin * sizeof(__nv_bfloat16), m->stream), "clear gradients");
            PLK_MCUDA(m, gemm(gd, m->stream), "activation-gradient GEMM");
            std::swap(dz, dn);
        }
    }
    return PLK_OK;
}

// SplitMix64 stream for the initial weights
uint64_t sm64(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

}  // namespace

extern "C" {

plk_status plk_mlp_create(plk_mlp** out, int device, int n_in, int n_hidden, int n_hidden_layers, int n_out,
                          uint64_t seed) {
    if (!out) return report_error(PLK_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (n_in < 1 || n_hidden < 1 || n_hidden_layers < 0 || n_out < 1)
        return report_error(PLK_ERR_ARG, "bad network sizes");
    int nd = 0;
    if (cudaGetDeviceCount(&nd) != cudaSuccess || nd == 0) return report_error(PLK_ERR_NODEV, "no CUDA device");
    if (device < 0 || device >= nd) return report_error(PLK_ERR_ARG, "device index out of range");
    cudaSetDevice(device);
    plk_mlp* m = new (std::nothrow) plk_mlp();
    if (!m) return report_error(PLK_ERR_ALLOC, "host allocation failed");
    m->device = device;
    m->dims.push_back(n_in);
    for (int i = 0; i < n_hidden_layers; ++i) m->dims.push_back(n_hidden);
    m->dims.push_back(n_out);
    for (int d : m->dims) m->pdims.push_back(pad16(d));
    size_t off = 0;
    for (int l = 0; l + 1 < (int)m->dims.size(); ++l) {
        m->w_off.push_back(off);
        off += (size_t)m->dims[l + 1] * m->dims[l];
        m->b_off.push_back(off);
        off += m->dims[l + 1];
    }
    m->n_params = off;
    cudaError_t e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&m->p, off * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&m->g, off * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&m->m, off * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&m->v, off * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&m->loss, sizeof(float));
    for (int l = 0; e == cudaSuccess && l + 1 < (int)m->dims.size(); ++l) {
        __nv_bfloat16* w = nullptr;
        e = cudaMalloc(&w, (size_t)m->pdims[l + 1] * m->pdims[l] * sizeof(__nv_bfloat16));
        m->wb.push_back(w);
    }
    if (e != cudaSuccess) {
        delete m;
        return report_error(PLK_ERR_ALLOC, cudaGetErrorString(e));
    }
    // He-normal weights (Box-Muller on a SplitMix64 stream), zero biases
    std::vector<float> host(off, 0.f);
    uint64_t s = seed;
    for (int l = 0; l + 1 < (int)m->dims.size(); ++l) {
        const double sd = std::sqrt(2.0 / m->dims[l]);
        for (size_t i = 0; i < (size_t)m->dims[l + 1] * m->dims[l]; ++i) {
            const double u1 = ((sm64(s) >> 11) + 1.0) / 9007199254740993.0, u2 = (sm64(s) >> 11) / 9007199254740992.0;
            host[m->w_off[l] + i] = (float)(sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
        }
    }
    cudaMemcpy(m->p, host.data(), off * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemset(m->m, 0, off * sizeof(float));
    cudaMemset(m->v, 0, off * sizeof(float));
    plk_status st = refresh_bf16(m);
    if (st != PLK_OK) {
        report_error(st, m->err);
        delete m;
        return st;
    }
    *out = m;
    return PLK_OK;
}

void plk_mlp_destroy(plk_mlp* m) {
    if (!m) return;
    cudaSetDevice(m->device);
    delete m;
}

const char* plk_mlp_last_error(const plk_mlp* m) { return m ? m->err.c_str() : plk_last_error(nullptr); }

int plk_mlp_n_params(const plk_mlp* m) { return m ? (int)m->n_params : 0; }

plk_status plk_mlp_get_params(const plk_mlp* m, float* out) {
    if (!m || !out) return PLK_ERR_ARG;
    cudaSetDevice(m->device);
    if (cudaMemcpy(out, m->p, m->n_params * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) return PLK_ERR_CUDA;
    return PLK_OK;
}

plk_status plk_mlp_set_params(plk_mlp* m, const float* in) {
    if (!m || !in) return PLK_ERR_ARG;
    PLK_MCUDA(m, cudaSetDevice(m->device), "cudaSetDevice");
    PLK_MCUDA(m, cudaMemcpy(m->p, in, m->n_params * sizeof(float), cudaMemcpyHostToDevice), "upload weights");
    return refresh_bf16(m);
}

plk_status plk_mlp_forward(plk_mlp* m, int batch, const float* x, float* y) {
    if (!m || batch < 1 || !x || !y) return m ? mfail(m, PLK_ERR_ARG, "bad arguments to plk_mlp_forward") : PLK_ERR_ARG;
    PLK_MCUDA(m, cudaSetDevice(m->device), "cudaSetDevice");
    plk_status s = ensure_batch(m, batch);
    if (s != PLK_OK) return s;
    PLK_MCUDA(m, cudaMemcpyAsync(m->xin, x, (size_t)batch * m->dims.front() * sizeof(float), cudaMemcpyHostToDevice,
                                 m->stream), "upload inputs");
    if ((s = forward(m, batch)) != PLK_OK) return s;
    const int L = n_layers(m), out = m->dims[L];
    PLK_MCUDA(m, cudaMemcpy2DAsync(y, out * sizeof(float), m->pre[L], m->pdims[L] * sizeof(float), out * sizeof(float),
                                   batch, cudaMemcpyDeviceToHost, m->stream), "download outputs");
    PLK_MCUDA(m, cudaStreamSynchronize(m->stream), "forward");
    return PLK_OK;
}

plk_status plk_mlp_gradients(plk_mlp* m, int batch, const float* x, const float* t, float* grad, float* loss) {
    if (!m || batch < 1 || !x || !t) return m ? mfail(m, PLK_ERR_ARG, "bad arguments to plk_mlp_gradients") : PLK_ERR_ARG;
    PLK_MCUDA(m, cudaSetDevice(m->device), "cudaSetDevice");
    plk_status s = ensure_batch(m, batch);
    if (s != PLK_OK) return s;
    PLK_MCUDA(m, cudaMemcpyAsync(m->xin, x, (size_t)batch * m->dims.front() * sizeof(float), cudaMemcpyHostToDevice,
                                 m->stream), "upload inputs");
    PLK_MCUDA(m, cudaMemcpyAsync(m->tin, t, (size_t)batch * m->dims.back() * sizeof(float), cudaMemcpyHostToDevice,
                                 m->stream), "upload targets");
    if ((s = forward(m, batch)) != PLK_OK) return s;
    if ((s = backward(m, batch)) != PLK_OK) return s;
    if (grad)
        PLK_MCUDA(m, cudaMemcpyAsync(grad, m->g, m->n_params * sizeof(float), cudaMemcpyDeviceToHost, m->stream),
                  "download gradients");
    if (loss) PLK_MCUDA(m, cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream), "download loss");
    PLK_MCUDA(m, cudaStreamSynchronize(m->stream), "gradients");
    return PLK_OK;
}

plk_status plk_mlp_train_step(plk_mlp* m, int batch, const float* x, const float* t, float lr, float* loss) {
    plk_status s = plk_mlp_gradients(m, batch, x, t, nullptr, nullptr);
    if (s != PLK_OK) return s;
    ++m->step;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)m->step), c2 = 1.f - std::pow(b2, (float)m->step);
    for (int l = 0; l < n_layers(m); ++l) {
        const int in = m->dims[l], out = m->dims[l + 1];
        const int nw = in * out;
        adam_kernel<<<(nw + 255) / 256, 256, 0, m->stream>>>(m->p + m->w_off[l], m->g + m->w_off[l], m->m + m->w_off[l],
                                                            m->v + m->w_off[l], nw, lr, b1, b2, 1e-8f, c1, c2, m->wb[l],
                                                            out, in, m->pdims[l]);
        adam_kernel<<<(out + 255) / 256, 256, 0, m->stream>>>(m->p + m->b_off[l], m->g + m->b_off[l], m->m + m->b_off[l],
                                                             m->v + m->b_off[l], out, lr, b1, b2, 1e-8f, c1, c2,
                                                             nullptr, 0, 1, 0);
    }
    PLK_MCUDA(m, cudaGetLastError(), "Adam update");
    if (loss) PLK_MCUDA(m, cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream), "download loss");
    PLK_MCUDA(m, cudaStreamSynchronize(m->stream), "train step");
    return PLK_OK;
}

}  // extern "C"
