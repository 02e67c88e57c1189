// The warm-start network: a fully connected ReLU MLP trained and run with
// hand-written kernels (absent in the reference, whose optimiser always starts
// from fixed values, src/treeator.cpp:612-615).
//
//  gemm_bf16_kernel  C[M x N] = sum_k A(m, k) B(n, k) with BF16 operands read
//                    through arbitrary strides (so one kernel serves X W^T,
//                    dZ W and dZ^T A), FP32 accumulation on the tensor cores
//                    (mma.sync m16n8k16), fused epilogue: + bias, ReLU, ReLU
//                    mask of the backward pass, FP32 and/or BF16 stores.
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

constexpr int kTM = 64, kTN = 32, kTK = 16;  // block tile; 4 warps of 16 x 32

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

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    const uint32_t l = (uint32_t)__bfloat16_as_ushort(lo), h = (uint32_t)__bfloat16_as_ushort(hi);
    return l | (h << 16);
}

__global__ void __launch_bounds__(128) gemm_bf16_kernel(GemmArgs g) {
    __shared__ __nv_bfloat16 As[kTM][kTK + 8];
    __shared__ __nv_bfloat16 Bs[kTN][kTK + 8];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int gid = lane >> 2, tq = lane & 3;
    const int m0 = blockIdx.y * kTM, n0 = blockIdx.x * kTN;
    float acc[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[j][q] = 0.f;
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    for (int k0 = 0; k0 < g.K; k0 += kTK) {
        for (int i = tid; i < kTM * kTK; i += 128) {
            const int r = i / kTK, c = i % kTK, m = m0 + r, k = k0 + c;
            As[r][c] = (m < g.M && k < g.K) ? g.A[m * g.sa_m + k * g.sa_k] : zero;
        }
        for (int i = tid; i < kTN * kTK; i += 128) {
            const int r = i / kTK, c = i % kTK, n = n0 + r, k = k0 + c;
            Bs[r][c] = (n < g.N && k < g.K) ? g.B[n * g.sb_n + k * g.sb_k] : zero;
        }
        __syncthreads();
        const int r0 = warp * 16;
        uint32_t a[4];
        a[0] = pack2(As[r0 + gid][2 * tq], As[r0 + gid][2 * tq + 1]);
        a[1] = pack2(As[r0 + gid + 8][2 * tq], As[r0 + gid + 8][2 * tq + 1]);
        a[2] = pack2(As[r0 + gid][2 * tq + 8], As[r0 + gid][2 * tq + 9]);
        a[3] = pack2(As[r0 + gid + 8][2 * tq + 8], As[r0 + gid + 8][2 * tq + 9]);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int nn = j * 8 + gid;
            const uint32_t b0 = pack2(Bs[nn][2 * tq], Bs[nn][2 * tq + 1]);
            const uint32_t b1 = pack2(Bs[nn][2 * tq + 8], Bs[nn][2 * tq + 9]);
            asm volatile(
                "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                "{%0,%1,%2,%3};\n"
                : "+f"(acc[j][0]), "+f"(acc[j][1]), "+f"(acc[j][2]), "+f"(acc[j][3])
                : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
        }
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int m = m0 + warp * 16 + gid + (q >= 2 ? 8 : 0);
            const int n = n0 + j * 8 + 2 * tq + (q & 1);
            if (m >= g.M || n >= g.N) continue;
            float v = acc[j][q];
            if (g.bias) v += g.bias[n];
            if (g.relu) v = fmaxf(v, 0.f);
            if (g.mask && !(__bfloat162float(g.mask[m * g.smask_m + n]) > 0.f)) v = 0.f;
            if (g.Cf) g.Cf[m * g.ldc + n] = v;
            if (g.Cb) g.Cb[m * g.ldc + n] = __float2bfloat16(v);
        }
}

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

cudaError_t gemm(const GemmArgs& g, cudaStream_t st) {
    dim3 grid((g.N + kTN - 1) / kTN, (g.M + kTM - 1) / kTM);
    gemm_bf16_kernel<<<grid, 128, 0, st>>>(g);
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
