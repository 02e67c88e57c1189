// Alignment summary statistics of every batch item, the inputs of the
// warm-start network (43 values per item):
//   [0, 4)    base frequencies of the unambiguous cells
//   [4, 10)   mean pairwise proportions of the six substitution types
//             A<->G, A<->C, A<->T, G<->C, G<->T, C<->T among all tip pairs
//             that carry unambiguous states at a site
//   [10, 42)  histogram of per-site collision (order-2 Renyi) entropy in 32
//             bins over [0, ln 4]
//   42        mean pairwise p-distance
// Statistics are taken over at most 32 taxa, rows floor(q n / 32) for
// q < 32, so that a network trained on 32-taxon alignments sees the same
// sampling spread on larger ones.
// Per site only the four state counts c_s of the unambiguous tips matter:
// pairs of type (a, b) number c_a c_b and identical pairs c_a (c_a - 1) / 2,
// so no pair loop is needed.  One CTA per item, sums in FP64.  No counterpart
// in the reference.
#include "plk_batch.h"
#include "plk_device.cuh"

namespace plk {
using namespace dev;

namespace {

constexpr int kFeatThreads = 256;
constexpr int kFeatureTaxa = 32;  // taxa the statistics are taken over

__global__ void __launch_bounds__(kFeatThreads) features_kernel(BatchDev b, float* out) {
    const int item = blockIdx.x;
    const BatchItemDev it = b.items[item];
    const uint8_t* codes = b.codes + it.codes_off;
    // per thread: base counts (4), type pairs (6), same pairs, all pairs, hist (32), sites
    double acc[4 + 6 + 2 + 32];
    for (int q = 0; q < 44; ++q) acc[q] = 0.0;
    // a fixed number of taxa, evenly spread over the rows, so that alignments
    // of any size present statistics with the same sampling spread
    const int m_taxa = it.n_tips < kFeatureTaxa ? it.n_tips : kFeatureTaxa;
    for (int site = threadIdx.x; site < it.n_sites; site += blockDim.x) {
        int c[4] = {0, 0, 0, 0};
        for (int q = 0; q < m_taxa; ++q) {
            const int t = (int)(((long long)q * it.n_tips) / m_taxa);
            const int code = codes[(size_t)t * it.site_stride + site];
            // unambiguous: exactly one of the four bits
            if (code == 1) ++c[0];
            else if (code == 2) ++c[1];
            else if (code == 4) ++c[2];
            else if (code == 8) ++c[3];
        }
        const int m = c[0] + c[1] + c[2] + c[3];
        for (int s = 0; s < 4; ++s) acc[s] += c[s];
        acc[4] += (double)c[0] * c[1];  // A-G
        acc[5] += (double)c[0] * c[2];  // A-C
        acc[6] += (double)c[0] * c[3];  // A-T
        acc[7] += (double)c[1] * c[2];  // G-C
        acc[8] += (double)c[1] * c[3];  // G-T
        acc[9] += (double)c[2] * c[3];  // C-T
        double same = 0.0;
        for (int s = 0; s < 4; ++s) same += 0.5 * c[s] * (c[s] - 1);
        acc[10] += same;
        acc[11] += 0.5 * (double)m * (m - 1);
        // collision entropy -ln(sum_s c_s (c_s - 1) / (m (m - 1))): the pair
        // estimate is unbiased for any number of observed taxa m, so the
        // histogram does not drift with the taxon count; sites with fewer
        // than two observed taxa or no identical pair go to the last bin
        int bin = 31;
        if (m >= 2 && same > 0.0) {
            const double h = -log(same / (0.5 * (double)m * (m - 1)));
            // entropies exactly on a bin edge go up whatever the last bit of
            // log(); 1e-9 is far below the spacing integer counts can give
            bin = (int)(h / 1.3862943611198906 * 32.0 + 1e-9);
        }
        bin = bin < 0 ? 0 : (bin > 31 ? 31 : bin);
        acc[12 + bin] += 1.0;
    }
    // block sums, deterministic order: warp shuffles then warps in order
    __shared__ double red[kFeatThreads / 32][44];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int q = 0; q < 44; ++q) {
        double v = acc[q];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) red[warp][q] = v;
    }
    __syncthreads();
    if (threadIdx.x < 44) {
        double v = 0.0;
        for (int w = 0; w < kFeatThreads / 32; ++w) v += red[w][threadIdx.x];
        red[0][threadIdx.x] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const double* r = red[0];
        float* o = out + (size_t)item * 43;
        const double nb = r[0] + r[1] + r[2] + r[3];
        for (int s = 0; s < 4; ++s) o[s] = nb > 0 ? (float)(r[s] / nb) : 0.25f;
        const double pairs = r[11];
        for (int q = 0; q < 6; ++q) o[4 + q] = pairs > 0 ? (float)(r[4 + q] / pairs) : 0.0f;
        for (int q = 0; q < 32; ++q) o[10 + q] = (float)(r[12 + q] / it.n_sites);
        o[42] = pairs > 0 ? (float)(1.0 - r[10] / pairs) : 0.0f;
    }
}

}  // namespace

cudaError_t launch_features(const BatchDev& b, float* out, cudaStream_t st) {
    if (b.n_items == 0) return cudaSuccess;
    features_kernel<<<b.n_items, kFeatThreads, 0, st>>>(b, out);
    return cudaGetLastError();
}

}  // namespace plk
