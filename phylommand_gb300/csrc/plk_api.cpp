// C ABI of libplk (include/plk.h): argument checks, host-side preparation,
// device buffers and kernel sequencing.  Host code only; kernels live in
// plk_kernels.cu.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "plk_internal.h"

using namespace plk;

namespace {

thread_local std::string g_create_error;

// Owning device allocation that only grows.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    cudaError_t ensure(size_t n) {
        if (n <= bytes && p) return cudaSuccess;
        release();
        if (n == 0) n = 16;
        cudaError_t e = cudaMalloc(&p, n);
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        bytes = n;
        return cudaSuccess;
    }
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
};

// A device array inside a DevBuf block that holds a group of arrays uploaded
// together (upload_group); not owned.
struct DevView {
    void* p = nullptr;
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
};

}  // namespace

plk_status plk::report_error(plk_status s, const std::string& msg) {
    g_create_error = msg;
    return s;
}

struct plk_handle {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    // alignment
    bool have_aln = false;
    int n_tips = 0, n_sites = 0, S = 0;
    bool bad_tip = false;
    int n_codes = 0;
    std::vector<uint32_t> code_mask;
    DevBuf d_codes, d_code_mask;
    // site patterns (plk_set_patterns): the kernels see n_sites = the number
    // of distinct columns; site_pattern maps every input site to its column
    bool patterns = false;
    int n_sites_full = 0;
    std::vector<int> site_pattern;
    std::vector<double> pattern_w;
    DevBuf d_pattern_w;
    // tree
    bool have_tree = false;
    int n_nodes = 0, tree_tips = 0, root = -1;
    std::vector<int> left, right, post, rank;
    std::vector<double> bl;
    Program prog;
    DevBuf d_tree_block;  // the tree's arrays, one upload (upload_group)
    DevView d_ops, d_order, d_left, d_right, d_rank;
    // rate model
    bool root_quirk = true;
    std::vector<float> cut_off, cut_rate, clade_rate;
    std::vector<int> clade_of_node;
    std::vector<double> t_eff;
    bool teff_dirty = true;
    DevBuf d_teff;
    // substitution model
    bool have_model = false;
    int C = 1, p_kind = 0, reversible = 1;
    std::vector<double> Q, root_w, cat_rate, cat_w, lam, L, R;
    DevBuf d_model_block;  // the model's arrays, one upload (upload_group)
    DevView d_Q, d_rootw, d_catr, d_catw, d_lam, d_L, d_R;
    // P(t) and tip tables
    DevBuf d_P64, d_P32, d_tip64, d_tip32;
    // results and scratch
    DevBuf d_site_lnl, d_block, d_lnl, d_work, d_cond, d_outside, d_nodes_out;
    DevBuf d_done;  // arrival counters (finish_grid_sum, then one per 128-site tile), zero between launches
    bool paired_written = false;  // this evaluation's P(t) kernel also wrote prune4p's layouts
    bool withhold_stage = false;  // plk_test_withhold_stage: armed for the next FP32 pass
    DevBuf d_mask_raw, d_flag;
    bool have_lnl = false;
    bool lnl_pending = false;
    int fit_method = PLK_FIT_NELDER_MEAD;
    // autotuned 4-state FP32 kernel (-1: not tuned for the current inputs)
    int variant = -1;
    float tune_ms[3] = {0.f, 0.f, 0.f};
    std::map<std::array<int, 6>, int> tune_cache;  // (sites, tips, ops, depth, cats, states) -> variant
    // streams: own_stream is created with the handle; stream is the active one
    cudaStream_t own_stream = nullptr;
    // kernel timing (plk_set_profiling)
    bool profiling = false;
    struct EvSet { cudaEvent_t e[4]; };
    std::vector<EvSet> evs;
    size_t ev_used = 0;
    // pinned arena of small host-to-device uploads, and the event after the
    // last copy out of it; a pinned word for the tip-check flag
    char* arena = nullptr;
    char* arena_dev = nullptr;  // the arena's device address (mapped)
    size_t arena_off = 0;
    cudaEvent_t arena_done = nullptr;
    int* h_flag = nullptr;
    bool flag_pending = false;
    int flag_gen = 0;  // value the encode kernel stores for an empty cell of the current alignment
    // the tip masks' copy and encode run on copy_stream, so that the tree and
    // model uploads and the P(t) kernel on the main stream overlap them; the
    // main stream waits for codes_ready just before the post-order pass
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t main_done = nullptr, codes_ready = nullptr;
    bool codes_pending = false;
    // a streamed alignment (byte masks, 4 states): the masks are copied in
    // place as codes in chunks of chunk_sites sites, each chunk followed by a
    // 4-byte copy of the alignment's generation (flag_gen, from the pinned
    // ring h_gen) into d_arrive[chunk]; a warp-independent pass starts
    // before the last chunk lands and waits per tile
    bool codes_streamed = false;
    int chunk_sites = 0;
    DevBuf d_arrive;
    int* h_gen = nullptr;
    ~plk_handle() {
        for (auto& s : evs)
            for (auto& e : s.e) cudaEventDestroy(e);
        if (arena) cudaFreeHost(arena);
        if (arena_done) cudaEventDestroy(arena_done);
        if (h_flag) cudaFreeHost(h_flag);
        if (h_gen) cudaFreeHost(h_gen);
        if (main_done) cudaEventDestroy(main_done);
        if (codes_ready) cudaEventDestroy(codes_ready);
    }
};

namespace {

plk_status fail(plk_handle* h, plk_status s, const std::string& msg) {
    if (h) h->err = msg;
    else g_create_error = msg;
    return s;
}

plk_status cuda_fail(plk_handle* h, cudaError_t e, const char* what) {
    const plk_status s = (e == cudaErrorMemoryAllocation) ? PLK_ERR_ALLOC : PLK_ERR_CUDA;
    return fail(h, s, std::string(what) + ": " + cudaGetErrorString(e));
}

#define PLK_CUDA(h, expr, what)                          \
    do {                                                 \
        cudaError_t _e = (expr);                         \
        if (_e != cudaSuccess) return cuda_fail(h, _e, what); \
    } while (0)

constexpr size_t kArenaBytes = 1 << 20;
// streamed alignments (plk_set_alignment8, 4 states): from this many sites
// on, in this many chunks; the pinned ring of generations the arrival flags
// are copied from
constexpr int kStreamMinSites = 16384;
constexpr int kStreamChunks = 16;  // at most; 2 by default (PLK_STREAM_CHUNKS)
constexpr int kGenRing = 256;

// The handle's pinned upload arena, mapped into the device's address space.
cudaError_t ensure_arena(plk_handle* h) {
    if (h->arena) return cudaSuccess;
    cudaError_t e = cudaHostAlloc(&h->arena, kArenaBytes, cudaHostAllocMapped);
    if (e != cudaSuccess) return e;
    void* dev = nullptr;
    if ((e = cudaHostGetDevicePointer(&dev, h->arena, 0)) != cudaSuccess) return e;
    h->arena_dev = static_cast<char*>(dev);
    if ((e = cudaEventCreateWithFlags(&h->arena_done, cudaEventDisableTiming)) != cudaSuccess) return e;
    h->arena_off = 0;
    return cudaSuccess;
}

// Host-to-device upload of v into b on the handle's stream.  Small arrays go
// through the handle's pinned arena and are copied by a kernel that reads
// the mapped arena (asynchronous, and never queued behind a large DMA copy);
// the arena starts over once the event after its last copy has completed.
// Larger arrays are copied from pageable memory.
template <typename T>
cudaError_t upload(plk_handle* h, DevBuf& b, const std::vector<T>& v) {
    cudaError_t e = b.ensure(sizeof(T) * std::max<size_t>(v.size(), 1));
    if (e != cudaSuccess) return e;
    if (v.empty()) return cudaSuccess;
    const size_t bytes = sizeof(T) * v.size();
    if (bytes > kArenaBytes) return cudaMemcpyAsync(b.p, v.data(), bytes, cudaMemcpyHostToDevice, h->stream);
    if ((e = ensure_arena(h)) != cudaSuccess) return e;
    if (h->arena_off + bytes > kArenaBytes) {
        if ((e = cudaEventSynchronize(h->arena_done)) != cudaSuccess) return e;
        h->arena_off = 0;
    }
    char* src = h->arena + h->arena_off;
    std::memcpy(src, v.data(), bytes);
    h->arena_off = (h->arena_off + bytes + 15) & ~(size_t)15;
    if ((e = launch_arena_copy(b.p, h->arena_dev + (src - h->arena), bytes, h->stream)) != cudaSuccess) return e;
    return cudaEventRecord(h->arena_done, h->stream);
}

// One part of a group upload: host data and the view that will point at its
// device copy.
struct UploadPart {
    DevView* dst;
    const void* src;
    size_t bytes;
};

template <typename T>
UploadPart part(DevView& dst, const std::vector<T>& v) {
    return UploadPart{&dst, v.data(), sizeof(T) * v.size()};
}

// Uploads a group of arrays into one device block at 256-byte aligned
// offsets with one host-to-device copy from the pinned arena (one API call
// instead of one per array; each cudaMemcpyAsync costs microseconds of host
// time), and points the views at their parts.  A group larger than the arena
// is copied part by part from pageable memory.
cudaError_t upload_group(plk_handle* h, DevBuf& block, std::initializer_list<UploadPart> parts) {
    size_t total = 0;
    for (const UploadPart& q : parts) total += (q.bytes + 255) & ~(size_t)255;
    cudaError_t e = block.ensure(std::max<size_t>(total, 256));
    if (e != cudaSuccess) return e;
    size_t off = 0;
    for (const UploadPart& q : parts) {
        q.dst->p = static_cast<char*>(block.p) + off;
        off += (q.bytes + 255) & ~(size_t)255;
    }
    if (total > kArenaBytes) {
        for (const UploadPart& q : parts)
            if (q.bytes && (e = cudaMemcpyAsync(q.dst->p, q.src, q.bytes, cudaMemcpyHostToDevice, h->stream)) !=
                               cudaSuccess)
                return e;
        return cudaSuccess;
    }
    if (total == 0) return cudaSuccess;
    if ((e = ensure_arena(h)) != cudaSuccess) return e;
    h->arena_off = (h->arena_off + 255) & ~(size_t)255;
    if (h->arena_off + total > kArenaBytes) {
        if ((e = cudaEventSynchronize(h->arena_done)) != cudaSuccess) return e;
        h->arena_off = 0;
    }
    char* src = h->arena + h->arena_off;
    off = 0;
    for (const UploadPart& q : parts) {
        if (q.bytes) std::memcpy(src + off, q.src, q.bytes);
        off += (q.bytes + 255) & ~(size_t)255;
    }
    h->arena_off += total;
    if ((e = launch_arena_copy(block.p, h->arena_dev + (src - h->arena), total, h->stream)) != cudaSuccess) return e;
    return cudaEventRecord(h->arena_done, h->stream);
}

plk_status ready(plk_handle* h) {
    if (!h) return PLK_ERR_ARG;
    if (!h->have_aln) return fail(h, PLK_ERR_STATE, "no alignment set (plk_set_alignment)");
    if (!h->have_tree) return fail(h, PLK_ERR_STATE, "no tree set (plk_set_tree)");
    if (!h->have_model) return fail(h, PLK_ERR_STATE, "no model set (plk_set_model)");
    if (h->tree_tips != h->n_tips)
        return fail(h, PLK_ERR_ARG, "tree has " + std::to_string(h->tree_tips) + " tips, alignment has " +
                                        std::to_string(h->n_tips) + " rows");
    if (h->S != (int)std::lround(std::sqrt((double)h->Q.size())))
        return fail(h, PLK_ERR_ARG, "model and alignment state counts differ");
    PLK_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
    return PLK_OK;
}

plk_status refresh_teff(plk_handle* h) {
    if (!h->teff_dirty) return PLK_OK;
    h->t_eff.assign(h->n_nodes, 0.0);
    effective_lengths(h->n_nodes, h->left.data(), h->right.data(), h->root, h->bl.data(), h->root_quirk,
                      h->cut_off, h->cut_rate, h->clade_of_node, h->clade_rate, h->t_eff.data());
    PLK_CUDA(h, upload(h, h->d_teff, h->t_eff), "upload effective lengths");
    h->teff_dirty = false;
    return PLK_OK;
}

// P(t) of every edge and category; with paired, also the layouts prune4p
// reads, into its scratch (so no relayout launch follows).
PruneArgs prune_args(plk_handle* h, int precision);

// The post-order form the next FP32 evaluation will run: forced by
// PLK_PRUNE_VARIANT, tuned on this handle, or cached for the shape (-1: not
// tuned yet).
int tuned_variant(const plk_handle* h) {
    int v = h->variant;
    if (const char* f = getenv("PLK_PRUNE_VARIANT")) v = atoi(f);
    if (v < 0) {
        const std::array<int, 6> key = {h->n_sites, h->n_tips, (int)h->prog.ops.size(), h->prog.max_depth, h->C, h->S};
        auto hit = h->tune_cache.find(key);
        if (hit != h->tune_cache.end()) v = hit->second;
    }
    return v;
}

// 20 states: whether the tuned post-order form is one of the tcgen05 forms
// (5, 6), whose B-operand images and transposed tip tables the P(t) kernel
// then writes itself (no relayout launch)
bool tuned_tc20(const plk_handle* h) {
    if (h->S != 20) return false;
    const int v = tuned_variant(h);
    return v == 5 || v == 6 || v == 7;
}

plk_status build_pmats(plk_handle* h, bool paired = false, bool tc20 = false) {
    plk_status s = refresh_teff(h);
    if (s != PLK_OK) return s;
    const size_t SS = (size_t)h->S * h->S;
    const size_t np = (size_t)h->n_nodes * h->C * SS;
    const size_t nt = (size_t)h->n_tips * h->C * h->n_codes * h->S;
    PLK_CUDA(h, h->d_P64.ensure(np * sizeof(double)), "allocate P");
    PLK_CUDA(h, h->d_P32.ensure(np * sizeof(float)), "allocate P");
    PLK_CUDA(h, h->d_tip64.ensure(nt * sizeof(double)), "allocate tip tables");
    PLK_CUDA(h, h->d_tip32.ensure(nt * sizeof(float)), "allocate tip tables");
    DeviceModel m{};
    m.S = h->S; m.C = h->C; m.n_nodes = h->n_nodes; m.n_tips = h->n_tips; m.n_codes = h->n_codes;
    m.t_eff = h->d_teff.as<double>(); m.cat_rate = h->d_catr.as<double>(); m.Q = h->d_Q.as<double>();
    m.eig_lam = h->d_lam.as<double>(); m.eig_L = h->d_L.as<double>(); m.eig_R = h->d_R.as<double>();
    m.code_mask = h->S <= 4 ? nullptr : h->d_code_mask.as<uint32_t>();  // <= 4 states: code = state set
    m.P64 = h->d_P64.as<double>(); m.P32 = h->d_P32.as<float>();
    m.tip64 = h->d_tip64.as<double>(); m.tip32 = h->d_tip32.as<float>();
    m.P32p = nullptr;
    m.tip32p = nullptr;
    if (paired) {
        PruneArgs a{};
        a.n_nodes = h->n_nodes;
        a.n_tips = h->n_tips;
        a.C = h->C;
        PLK_CUDA(h, h->d_work.ensure(prune4p_scratch_bytes(a)), "allocate scratch");
        prune4p_scratch_parts(h->d_work.p, h->n_nodes, h->C, &m.P32p, &m.tip32p);
    }
    m.B20 = nullptr;
    m.T20 = nullptr;
    m.ncs20 = 0;
    m.b20_bf16 = 0;
    if (tc20) {
        // the scratch as the post-order launch sizes it, so that it does not
        // move between this kernel and the pass
        const PruneArgs a = prune_args(h, PLK_FP32S);
        PLK_CUDA(h, h->d_work.ensure(std::max(prune20_scratch_bytes(a, h->n_nodes),
                                               prune20u_scratch_bytes(a, h->n_nodes))),
                 "allocate scratch");
        prune20u_scratch_parts(h->d_work.p, a, h->n_nodes, &m.B20, &m.T20);
        m.ncs20 = prune20u_codes_padded(h->n_codes);
        m.b20_bf16 = tuned_variant(h) == 7 ? 1 : 0;
    }
    h->paired_written = paired || tc20;
    PLK_CUDA(h, launch_pmat(m, h->p_kind, h->stream), "P(t) kernel launch");
    return PLK_OK;
}

PruneArgs prune_args(plk_handle* h, int precision) {
    PruneArgs a{};
    const bool fp64 = precision == PLK_FP64;
    a.ops = h->d_ops.as<Op>();
    a.n_ops = (int)h->prog.ops.size();
    a.max_depth = h->prog.max_depth;
    a.codes = h->d_codes.as<uint8_t>();
    a.site_stride = code_stride(h->n_sites);
    a.n_sites = h->n_sites;
    a.n_codes = h->n_codes;
    a.C = h->C;
    a.P = fp64 ? (const void*)h->d_P64.p : (const void*)h->d_P32.p;
    a.tipT = fp64 ? (const void*)h->d_tip64.p : (const void*)h->d_tip32.p;
    a.root_w = h->d_rootw.as<double>();
    a.cat_w = h->d_catw.as<double>();
    a.site_lnl = h->d_site_lnl.as<double>();
    a.block_sum = h->d_block.as<double>();
    a.order = h->d_order.as<int>();
    a.left = h->d_left.as<int>();
    a.right = h->d_right.as<int>();
    a.rank = h->d_rank.as<int>();
    a.n_int = (int)h->post.size();
    a.n_tips = h->n_tips;
    a.n_nodes = h->n_nodes;
    return a;
}

bool fused_kernel_applies(const plk_handle* h, int precision) {
    if (h->S != 4 || h->C > 8) return false;
    const int cm = h->C == 1 ? 1 : (h->C <= 4 ? 4 : 8);
    const size_t ops_bytes = (h->prog.ops.size() * sizeof(Op) + 31) & ~(size_t)31;
    const size_t stack = (size_t)std::max(h->prog.max_depth, 1) * cm * (precision == PLK_FP64 ? 32 : 16) * 128;
    return ops_bytes + stack <= 227 * 1024;
}

// Autotuner of the FP32 post-order kernels: times every candidate on this
// handle's tree and sites -- one warm-up and three timed launches each, CUDA
// events on the handle's stream -- and keeps the fastest until the tree,
// alignment or model changes.  4 states: prune4_kernel and prune4s_kernel
// with 1 and 2 sites per thread; 20 states: prune20_kernel on CUDA cores and
// on tensor cores.  PLK_PRUNE_VARIANT=<n> forces candidate n where it applies.
plk_status autotune_prune(plk_handle* h, PruneArgs a, const std::vector<int>& cands) {
    if (cands.empty()) return fail(h, PLK_ERR_STATE, "no post-order kernel applies");
    if (const char* f = getenv("PLK_PRUNE_VARIANT")) {
        const int v = atoi(f);
        if (std::find(cands.begin(), cands.end(), v) != cands.end()) {
            h->variant = v;
            return PLK_OK;
        }
    }
    // same sizes as an earlier tuning on this handle: reuse its choice
    const std::array<int, 6> key = {a.n_sites, a.n_tips, a.n_ops, a.max_depth, a.C, h->S};
    auto hit = h->tune_cache.find(key);
    if (hit != h->tune_cache.end()) {
        h->variant = hit->second;
        return PLK_OK;
    }
    if (cands.size() == 1) {
        h->variant = cands[0];
        h->tune_cache[key] = cands[0];
        return PLK_OK;
    }
    cudaEvent_t e0, e1;
    PLK_CUDA(h, cudaEventCreate(&e0), "cudaEventCreate");
    PLK_CUDA(h, cudaEventCreate(&e1), "cudaEventCreate");
    // two passes over the candidates, each candidate's best pass counts (an
    // early candidate may run before the clocks and caches settle)
    std::vector<float> cand_ms(cands.size(), 1e30f);
    cudaError_t err = cudaSuccess;
    for (int pass = 0; pass < 2 && err == cudaSuccess; ++pass) {
        for (size_t i = 0; i < cands.size(); ++i) {
            const int v = cands[i];
            if (err != cudaSuccess) break;
            a.variant = v;
            int nb = 0;
            err = launch_prune(a, h->S, PLK_FP32S, false, &nb, h->stream);
            if (err != cudaSuccess) break;
            err = cudaEventRecord(e0, h->stream);
            for (int r = 0; r < 3 && err == cudaSuccess; ++r)
                err = launch_prune(a, h->S, PLK_FP32S, false, &nb, h->stream);
            if (err == cudaSuccess) err = cudaEventRecord(e1, h->stream);
            if (err == cudaSuccess) err = cudaEventSynchronize(e1);
            float ms = 0.f;
            if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
            if (err == cudaSuccess) cand_ms[i] = std::min(cand_ms[i], ms);
        }
    }
    float best = 1e30f;
    int best_v = cands[0];
    float best_staged = 1e30f;  // the fastest form that stages each op's tip codes
    int best_staged_v = -1;
    for (size_t i = 0; i < cands.size(); ++i) {
        const int v = cands[i];
        if (v >= 0 && v < 3) h->tune_ms[v] = cand_ms[i] / 3.0f;
        if (cand_ms[i] < best) { best = cand_ms[i]; best_v = v; }
        if (h->S == 4 && v >= 10 && v <= 18 && cand_ms[i] < best_staged) {
            best_staged = cand_ms[i];
            best_staged_v = v;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (err != cudaSuccess) return cuda_fail(h, err, "autotune post-order kernel");
    // The timed launches run back to back with the tip codes warm in L2.  A
    // form that stages each op's codes with its tables, or loads them two ops
    // ahead (prune4w), does not depend on that: within 3 % of the fastest it is
    // taken, since other work between evaluations (other partitions, other
    // alignments) evicts the codes that the faster form reads at use.  On
    // 128 x 100,000 the two are level warm (0.155 ms), and with the codes
    // evicted the staged form takes 0.148 against 0.159 ms.
    if (best_staged_v >= 0 && best_staged <= best * 1.03f) best_v = best_staged_v;
    h->variant = best_v;
    h->tune_cache[key] = best_v;
    return PLK_OK;
}

// Whether the FP32 pass of this handle's current shape will run a paired
// form (prune4p): the tuning already chose one for the shape, or
// PLK_PRUNE_VARIANT forces one.  Before the first tuning this is false and
// prune4p relays the layouts out itself.
bool tuned_paired(const plk_handle* h) {
    if (h->S != 4 || (h->C != 2 && h->C != 4 && h->C != 8) || !fused_kernel_applies(h, PLK_FP32S)) return false;
    const int v = tuned_variant(h);
    return v >= 3 && v <= 18;
}

// Re-arms the arrival counters of the passes' in-kernel totals (zero between
// launches; every CTA of a completed launch leaves them so) after a launch
// that may have stopped part-way; errors here are ignored, the caller
// reports the first one.
void clear_counters(plk_handle* h) {
    if (h->d_done.p && h->d_done.bytes) cudaMemsetAsync(h->d_done.p, 0, h->d_done.bytes, h->stream);
}

// Runs the post-order pass (P(t) already built); store != null asks for the
// conditional vectors of every internal node in *store.
plk_status run_prune(plk_handle* h, int precision, void** store, cudaEvent_t* after_prune = nullptr) {
    // a streamed alignment's codes: a tuned warp-independent FP32 pass starts
    // while they land and waits per tile; every other pass after all of them
    bool streamed = false;
    if (h->codes_pending) {  // the tip codes come from the copy stream
        const int v = tuned_variant(h);
        streamed = h->codes_streamed && precision == PLK_FP32S && store == nullptr && v >= 12 && v <= 18;
        if (!streamed) {
            PLK_CUDA(h, cudaStreamWaitEvent(h->stream, h->codes_ready, 0), "cudaStreamWaitEvent");
            h->codes_pending = false;
        }
    }
    const size_t tsz = precision == PLK_FP64 ? sizeof(double) : sizeof(float);
    const size_t vec_bytes = (size_t)h->post.size() * h->C * h->n_sites * h->S * tsz;
    const int blocks = (h->n_sites + 63) / 64;  // the smallest tile: 64 sites (prune4p, two threads per site)
    PLK_CUDA(h, h->d_site_lnl.ensure(sizeof(double) * h->n_sites), "allocate site lnL");
    PLK_CUDA(h, h->d_block.ensure(sizeof(double) * 2 * blocks), "allocate block sums");
    PLK_CUDA(h, h->d_lnl.ensure(sizeof(double)), "allocate lnL");
    // arrival counters, zero between launches: the grid's, then one per
    // 128-site tile (the 20-state compact form's in-kernel combine)
    const size_t counters = (1 + (size_t)(h->n_sites + 127) / 128) * sizeof(unsigned);
    if (h->d_done.bytes < counters) {
        PLK_CUDA(h, h->d_done.ensure(counters), "allocate counters");
        PLK_CUDA(h, cudaMemsetAsync(h->d_done.p, 0, counters, h->stream), "clear counters");
    }
    PruneArgs a = prune_args(h, precision);
    // the last CTA of the post-order pass (or of its per-site combine) adds
    // up the block sums into d_lnl: no separate reduction launch
    a.grid_done = h->d_done.as<unsigned>();
    a.tile_done = h->d_done.as<unsigned>() + 1;
    a.lnl_out = h->d_lnl.as<double>();
    a.paired_ready = (precision == PLK_FP32S && h->paired_written) ? 1 : 0;
    a.withhold_first_stage = (precision == PLK_FP32S && h->withhold_stage) ? 1 : 0;
    if (precision == PLK_FP32S) h->withhold_stage = false;
    const bool fused = fused_kernel_applies(h, precision);
    std::vector<int> cands20;
    if (!store && precision == PLK_FP32S && h->S == 20)
        for (int v = 1; v <= 4; ++v)
            if (prune20_fits(a, v)) cands20.push_back(v);
    if (!store && precision == PLK_FP32S && h->S == 20)
        for (int form = 0; form < 3; ++form)  // split TF32, its compact form, split BF16 (compact)
            if (prune20u_fits(a, form)) cands20.push_back(5 + form);
    if (!cands20.empty()) {
        PLK_CUDA(h, h->d_work.ensure(std::max(prune20_scratch_bytes(a, h->n_nodes), prune20u_scratch_bytes(a, h->n_nodes))),
                 "allocate scratch");
        a.scratch = h->d_work.p;
        if (h->variant < 0) {
            plk_status s = autotune_prune(h, a, cands20);
            if (s != PLK_OK) return s;
        }
        a.variant = h->variant;
    } else if (!fused) {
        PLK_CUDA(h, h->d_work.ensure(vec_bytes), "allocate work vectors");
        a.work = h->d_work.p;
        a.cond = h->d_work.p;
    } else if (store) {
        PLK_CUDA(h, h->d_cond.ensure(vec_bytes), "allocate node vectors");
        a.cond = h->d_cond.p;
    }
    if (fused && !store && precision == PLK_FP32S) {
        // the paired kernels read P(t) and tip tables re-laid out in scratch
        const bool paired = prune4p_fits(a, 1) || prune4p_fits(a, 2) || prune4w_fits(a, 1);
        if (paired) {
            PLK_CUDA(h, h->d_work.ensure(prune4p_scratch_bytes(a)), "allocate scratch");
            a.scratch = h->d_work.p;
        }
        if (h->variant < 0) {
            std::vector<int> cands = {0};
            for (int v = 1; v <= 2; ++v)
                if (prune4s_fits(a, v)) cands.push_back(v);
            for (int v = 3; v <= 6; ++v)
                if (prune4p_fits(a, (v + 1) % 2 + 1)) cands.push_back(v);
            if (prune4p_fits(a, 1, 2)) {  // two threads per site
                cands.push_back(7);
                cands.push_back(8);
            }
            if (prune4p_fits(a, 1, 0)) cands.push_back(9);  // TMA-fed stage ring
            for (int v = 10; v <= 11; ++v)  // codes staged with each op
                if (prune4p_fits(a, v - 9)) cands.push_back(v);
            for (int v = 12; v <= 18; ++v)  // warp-independent: 1/2/4 sites per thread, tables via L1 or smem
                if (prune4w_fits(a, (v == 12 || v == 15) ? 1 : ((v == 14 || v == 17) ? 4 : 2), v >= 15 ? 1 : 0,
                                 v == 18 ? 2 : 1))
                    cands.push_back(v);
            plk_status s = autotune_prune(h, a, cands);
            if (s != PLK_OK) return s;
        }
        a.variant = h->variant;
    }
    if (streamed && a.variant >= 12 && a.variant <= 18) {
        a.arrive = h->d_arrive.as<int>();
        a.arrive_gen = h->flag_gen;
        a.chunk_sites = h->chunk_sites;
    }
    int nb = 0;
    const cudaError_t le = launch_prune(a, h->S, precision, store != nullptr, &nb, h->stream);
    if (streamed) {  // the rest of the copy stream (the empty-cell check) before anything after the pass
        PLK_CUDA(h, cudaStreamWaitEvent(h->stream, h->codes_ready, 0), "cudaStreamWaitEvent");
        h->codes_pending = false;
    }
    if (le != cudaSuccess) {
        clear_counters(h);  // a launch that failed part-way may leave arrivals counted
        return cuda_fail(h, le, "post-order kernel launch");
    }
    if (after_prune) PLK_CUDA(h, cudaEventRecord(*after_prune, h->stream), "cudaEventRecord");
    if (store) *store = a.cond;
    return PLK_OK;
}

bool finite_masks(uint32_t m, int S) {
    const uint32_t all = S >= 32 ? 0xffffffffu : ((1u << S) - 1u);
    return (m & all) != 0;
}

}  // namespace

extern "C" {

int plk_api_version(void) { return PLK_API_VERSION; }

const char* plk_status_string(plk_status s) {
    switch (s) {
        case PLK_OK: return "ok";
        case PLK_ERR_ARG: return "bad argument";
        case PLK_ERR_ALLOC: return "allocation failed";
        case PLK_ERR_CUDA: return "CUDA error";
        case PLK_ERR_STATE: return "call order (missing input)";
        case PLK_ERR_TIMEOUT: return "bounded device wait gave up";
        case PLK_ERR_NUMERIC: return "non-finite likelihood";
        case PLK_ERR_TIP: return "a tip cell allows no state";
        case PLK_ERR_NODEV: return "no CUDA device";
        case PLK_ERR_UNSUPPORTED: return "unsupported configuration";
        default: return "unknown status";
    }
}

const char* plk_last_error(const plk_handle* h) {
    return h ? h->err.c_str() : g_create_error.c_str();
}

plk_status plk_create(plk_handle** out, int device) {
    if (!out) return fail(nullptr, PLK_ERR_ARG, "out is NULL");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        return fail(nullptr, PLK_ERR_NODEV, std::string("no CUDA device: ") + cudaGetErrorString(e));
    if (device < 0 || device >= n) return fail(nullptr, PLK_ERR_ARG, "device index out of range");
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail(nullptr, PLK_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    plk_handle* h = new (std::nothrow) plk_handle();
    if (!h) return fail(nullptr, PLK_ERR_ALLOC, "host allocation failed");
    h->device = device;
    e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete h;
        return fail(nullptr, PLK_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
    }
    h->stream = h->own_stream;
    *out = h;
    return PLK_OK;
}

void plk_destroy(plk_handle* h) {
    if (!h) return;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->copy_stream) {
        cudaStreamSynchronize(h->copy_stream);
        cudaStreamDestroy(h->copy_stream);
    }
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    delete h;
}

plk_status plk_set_patterns(plk_handle* h, int on) {
    if (!h) return PLK_ERR_ARG;
    if ((on != 0) != h->patterns) {
        h->patterns = on != 0;
        h->have_aln = false;  // the next plk_set_alignment applies the choice
        h->have_lnl = false;
    }
    return PLK_OK;
}

int plk_n_patterns(const plk_handle* h) { return h && h->have_aln ? h->n_sites : 0; }

}  // extern "C"

namespace {

// plk_set_alignment with the state sets as 32-bit masks, or (masks8, only for
// n_states <= 4 without site patterns) as bytes
plk_status set_alignment_impl(plk_handle* h, int n_tips, int n_sites, int n_states, const uint32_t* masks,
                              const uint8_t* masks8) {
    if (!h) return PLK_ERR_ARG;
    if (n_tips < 1 || n_sites < 1 || n_states < 1 || n_states > kMaxStates || (!masks && !masks8))
        return fail(h, PLK_ERR_ARG, "alignment needs n_tips >= 1, n_sites >= 1, 1 <= n_states <= 24");
    PLK_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
    if (h->codes_pending) {  // an earlier alignment's copy and encode are still on the copy stream
        PLK_CUDA(h, cudaStreamWaitEvent(h->stream, h->codes_ready, 0), "cudaStreamWaitEvent");
        h->codes_pending = false;
    }
    h->codes_streamed = false;
    h->n_sites_full = n_sites;
    h->site_pattern.clear();
    h->pattern_w.clear();
    h->flag_pending = false;
    std::vector<uint32_t> pmasks;
    if (h->patterns) {
        // distinct columns in order of first appearance, with their counts
        const uint32_t keep = (n_states >= 32) ? 0xffffffffu : ((1u << n_states) - 1u);
        std::unordered_map<uint64_t, std::vector<int>> buckets;
        std::vector<int> first;  // first site of every pattern
        h->site_pattern.resize(n_sites);
        for (int s = 0; s < n_sites; ++s) {
            uint64_t hash = 1469598103934665603ull;  // FNV-1a over the column
            for (int t = 0; t < n_tips; ++t) {
                hash ^= (uint64_t)(masks[(size_t)t * n_sites + s] & keep);
                hash *= 1099511628211ull;
            }
            std::vector<int>& cand = buckets[hash];
            int found = -1;
            for (int p : cand) {
                const int f = first[p];
                int t = 0;
                while (t < n_tips && (masks[(size_t)t * n_sites + f] & keep) == (masks[(size_t)t * n_sites + s] & keep)) ++t;
                if (t == n_tips) { found = p; break; }
            }
            if (found < 0) {
                found = (int)first.size();
                first.push_back(s);
                cand.push_back(found);
                h->pattern_w.push_back(0.0);
            }
            h->site_pattern[s] = found;
            h->pattern_w[found] += 1.0;
        }
        const int n_pat = (int)first.size();
        pmasks.resize((size_t)n_tips * n_pat);
        for (int t = 0; t < n_tips; ++t)
            for (int p = 0; p < n_pat; ++p) pmasks[(size_t)t * n_pat + p] = masks[(size_t)t * n_sites + first[p]];
        PLK_CUDA(h, upload(h, h->d_pattern_w, h->pattern_w), "upload pattern weights");
        masks = pmasks.data();
        n_sites = n_pat;
    }
    const uint32_t all = (n_states >= 32) ? 0xffffffffu : ((1u << n_states) - 1u);
    const size_t n_cells = (size_t)n_tips * n_sites;
    std::vector<uint32_t> table;
    bool bad = false;
    if (n_states <= 4) {
        // small alphabets: the code is the state set itself, encoded on the
        // device straight from the caller's masks
        for (uint32_t c = 0; c < (1u << n_states); ++c) table.push_back(c);
        const int eb = masks8 ? 1 : (int)sizeof(uint32_t);
        PLK_CUDA(h, h->d_mask_raw.ensure(n_cells * eb), "allocate mask staging");
        PLK_CUDA(h, h->d_codes.ensure((size_t)n_tips * code_stride(n_sites)), "allocate tip codes");
        if (!h->copy_stream) {
            PLK_CUDA(h, cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking), "create copy stream");
            PLK_CUDA(h, cudaEventCreateWithFlags(&h->main_done, cudaEventDisableTiming), "cudaEventCreate");
            PLK_CUDA(h, cudaEventCreateWithFlags(&h->codes_ready, cudaEventDisableTiming), "cudaEventCreate");
        }
        if (!h->d_flag.p) {  // zero once; every alignment then marks with its own generation
            PLK_CUDA(h, h->d_flag.ensure(sizeof(int)), "allocate flag");
            PLK_CUDA(h, cudaMemsetAsync(h->d_flag.p, 0, sizeof(int), h->stream), "clear flag");
        }
        if (!h->h_flag) PLK_CUDA(h, cudaMallocHost(&h->h_flag, sizeof(int)), "allocate flag");
        h->flag_gen = h->flag_gen == 0x7fffffff ? 1 : h->flag_gen + 1;
        // byte masks of 4 states are the codes themselves (the passes mask a
        // code to its low four bits): copied in place in chunks, with an
        // arrival flag per chunk, once the alignment is large enough for the
        // pass to overlap the copy
        // PLK_STREAM_CHUNKS: the number of chunks (0: no streaming).  Two
        // measured best on 128 x 100,000 end to end (164 us a step against
        // 178 unstreamed, 172 with three chunks or four, 187 with eight: each
        // chunk costs two API calls of host time before the pass is launched)
        int chunks = 2;
        if (const char* e = getenv("PLK_STREAM_CHUNKS")) chunks = std::max(0, std::min(kStreamChunks, atoi(e)));
        const bool stream_codes = masks8 != nullptr && n_states == 4 && n_sites >= kStreamMinSites && chunks > 0;
        int n_chunks = 0;
        if (stream_codes) {
            const int want = std::min(chunks, (n_sites + 127) / 128);
            h->chunk_sites = ((n_sites + want - 1) / want + 127) / 128 * 128;  // whole 128-site tiles
            n_chunks = (n_sites + h->chunk_sites - 1) / h->chunk_sites;
            if (h->d_arrive.bytes < sizeof(int) * kStreamChunks) {  // zero once: generations count from 1
                PLK_CUDA(h, h->d_arrive.ensure(sizeof(int) * kStreamChunks), "allocate arrival flags");
                PLK_CUDA(h, cudaMemsetAsync(h->d_arrive.p, 0, sizeof(int) * kStreamChunks, h->stream),
                         "clear arrival flags");
            }
            if (!h->h_gen) PLK_CUDA(h, cudaMallocHost(&h->h_gen, sizeof(int) * kGenRing), "allocate generations");
        }
        // the copy stream starts after all work already on the main stream
        // (earlier passes still reading the masks or codes, the flag clear)
        PLK_CUDA(h, cudaEventRecord(h->main_done, h->stream), "cudaEventRecord");
        PLK_CUDA(h, cudaStreamWaitEvent(h->copy_stream, h->main_done, 0), "cudaStreamWaitEvent");
        if (stream_codes) {
            // a ring slot of the pinned generations: its last reader (the
            // copy kGenRing alignments ago) is done once the copy stream has
            // drained, which is waited for when the ring wraps
            const int slot = h->flag_gen % kGenRing;
            if (slot == 0) PLK_CUDA(h, cudaStreamSynchronize(h->copy_stream), "drain copy stream");
            h->h_gen[slot] = h->flag_gen;
            const size_t stride = (size_t)code_stride(n_sites);
            for (int c = 0; c < n_chunks; ++c) {
                const size_t s0 = (size_t)c * h->chunk_sites;
                const size_t w = std::min((size_t)h->chunk_sites, (size_t)n_sites - s0);
                PLK_CUDA(h, cudaMemcpy2DAsync(h->d_codes.as<uint8_t>() + s0, stride, masks8 + s0, (size_t)n_sites, w,
                                              (size_t)n_tips, cudaMemcpyHostToDevice, h->copy_stream),
                         "upload masks");
                PLK_CUDA(h, cudaMemcpyAsync(h->d_arrive.as<int>() + c, h->h_gen + slot, sizeof(int),
                                            cudaMemcpyHostToDevice, h->copy_stream),
                         "arrival flag");
            }
            PLK_CUDA(h, launch_check_codes(h->d_codes.as<uint8_t>(), n_tips, n_sites, (int)stride, all,
                                           h->d_flag.as<int>(), h->flag_gen, h->copy_stream),
                     "check kernel launch");
        } else {
            PLK_CUDA(h, cudaMemcpyAsync(h->d_mask_raw.p, masks8 ? (const void*)masks8 : (const void*)masks,
                                        n_cells * eb, cudaMemcpyHostToDevice, h->copy_stream),
                     "upload masks");
            PLK_CUDA(h, launch_encode_small(h->d_mask_raw.p, eb, n_tips, n_sites, code_stride(n_sites), all,
                                            h->d_codes.as<uint8_t>(), h->d_flag.as<int>(), h->flag_gen,
                                            h->copy_stream),
                     "encode kernel launch");
        }
        h->codes_streamed = stream_codes;
        // the empty-cell flag comes back with the next result fetch (no wait
        // here); the code table is the identity, so none is uploaded (the
        // P(t) kernel takes the code as the state set)
        PLK_CUDA(h, cudaMemcpyAsync(h->h_flag, h->d_flag.p, sizeof(int), cudaMemcpyDeviceToHost, h->copy_stream),
                 "read flag");
        PLK_CUDA(h, cudaEventRecord(h->codes_ready, h->copy_stream), "cudaEventRecord");
        h->codes_pending = true;
        h->flag_pending = true;
    } else {
        const size_t stride = (size_t)code_stride(n_sites);
        std::vector<uint8_t> codes((size_t)n_tips * stride, 0);
        std::map<uint32_t, int> index;
        for (size_t i = 0; i < n_cells; ++i) {
            const uint32_t m = masks[i] & all;
            if (m == 0) bad = true;
            auto it = index.find(m);
            int c;
            if (it == index.end()) {
                c = (int)table.size();
                if (c >= kMaxCodes) return fail(h, PLK_ERR_UNSUPPORTED, "more than 256 distinct tip state sets");
                index.emplace(m, c);
                table.push_back(m);
            } else c = it->second;
            codes[(i / n_sites) * stride + (i % n_sites)] = (uint8_t)c;
        }
        PLK_CUDA(h, upload(h, h->d_codes, codes), "upload tip codes");
        PLK_CUDA(h, upload(h, h->d_code_mask, table), "upload code table");
        PLK_CUDA(h, cudaStreamSynchronize(h->stream), "upload tip codes");
    }
    h->n_tips = n_tips;
    h->n_sites = n_sites;
    h->S = n_states;
    h->n_codes = (int)table.size();
    h->code_mask = table;
    h->bad_tip = bad;
    h->have_aln = true;
    h->variant = -1;
    h->have_lnl = false;
    return PLK_OK;
}

}  // namespace

extern "C" {

plk_status plk_set_alignment(plk_handle* h, int n_tips, int n_sites, int n_states, const uint32_t* masks) {
    return set_alignment_impl(h, n_tips, n_sites, n_states, masks, nullptr);
}

plk_status plk_set_alignment8(plk_handle* h, int n_tips, int n_sites, int n_states, const uint8_t* masks) {
    if (!h) return PLK_ERR_ARG;
    if (n_tips < 1 || n_sites < 1 || n_states < 1 || n_states > 8 || !masks)
        return fail(h, PLK_ERR_ARG, "byte masks need n_tips >= 1, n_sites >= 1, 1 <= n_states <= 8");
    if (n_states <= 4 && !h->patterns) return set_alignment_impl(h, n_tips, n_sites, n_states, nullptr, masks);
    // more states, or patterns compressed on the host: through the 32-bit path
    const std::vector<uint32_t> wide(masks, masks + (size_t)n_tips * n_sites);
    return set_alignment_impl(h, n_tips, n_sites, n_states, wide.data(), nullptr);
}

plk_status plk_set_tree(plk_handle* h, int n_nodes, const int* left, const int* right, const double* bl) {
    if (!h) return PLK_ERR_ARG;
    if (n_nodes < 2 || !left || !right || !bl) return fail(h, PLK_ERR_ARG, "tree needs n_nodes >= 2 and three arrays");
    PLK_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
    int n_leaves = 0;
    for (int v = 0; v < n_nodes; ++v)
        if (left[v] < 0 && right[v] < 0) ++n_leaves;
    std::vector<int> post, rank;
    int root = -1;
    std::string err;
    if (!check_tree(n_leaves, n_nodes, left, right, &root, &post, &rank, &err)) return fail(h, PLK_ERR_ARG, err);
    for (int v = 0; v < n_nodes; ++v)
        if (!std::isfinite(bl[v])) return fail(h, PLK_ERR_ARG, "non-finite branch length at node " + std::to_string(v));
    h->left.assign(left, left + n_nodes);
    h->right.assign(right, right + n_nodes);
    h->bl.assign(bl, bl + n_nodes);
    h->post = post;
    h->rank = rank;
    h->root = root;
    h->n_nodes = n_nodes;
    h->tree_tips = n_leaves;
    h->prog = build_program(n_leaves, n_nodes, left, right, root, rank);
    PLK_CUDA(h,
             upload_group(h, h->d_tree_block,
                          {part(h->d_ops, h->prog.ops), part(h->d_order, post), part(h->d_left, h->left),
                           part(h->d_right, h->right), part(h->d_rank, rank)}),
             "upload tree");
    // default rate model: the reference's empty rate_model
    h->root_quirk = true;
    h->cut_off.clear();
    h->cut_rate.clear();
    h->clade_of_node.clear();
    h->clade_rate.clear();
    h->teff_dirty = true;
    h->have_tree = true;
    h->variant = -1;
    h->have_lnl = false;
    return PLK_OK;
}

plk_status plk_set_rate_model(plk_handle* h, int root_quirk, int n_cut, const float* cut_off,
                              const float* cut_rate, const int* clade_of_node, int n_clades,
                              const float* clade_rate) {
    if (!h) return PLK_ERR_ARG;
    if (!h->have_tree) return fail(h, PLK_ERR_STATE, "set the tree before the rate model");
    if (n_cut < 0 || n_clades < 0 || (n_cut > 0 && (!cut_off || !cut_rate)) || (n_clades > 0 && !clade_rate))
        return fail(h, PLK_ERR_ARG, "bad rate model arrays");
    for (int i = 1; i < n_cut; ++i)
        if (cut_off[i] < cut_off[i - 1]) return fail(h, PLK_ERR_ARG, "cut-offs must ascend");
    h->root_quirk = root_quirk != 0;
    h->cut_off.assign(cut_off, cut_off + n_cut);
    h->cut_rate.assign(cut_rate, cut_rate + n_cut);
    h->clade_rate.assign(clade_rate, clade_rate + n_clades);
    if (clade_of_node) {
        h->clade_of_node.assign(clade_of_node, clade_of_node + h->n_nodes);
        for (int c : h->clade_of_node)
            if (c >= n_clades) return fail(h, PLK_ERR_ARG, "clade number without a rate");
    } else h->clade_of_node.clear();
    h->teff_dirty = true;
    h->have_lnl = false;
    return PLK_OK;
}

plk_status plk_set_model(plk_handle* h, int S, const double* Q, const double* root_w, int reversible,
                         int n_cats, const double* cat_rates, const double* cat_weights, int p_mode) {
    if (!h) return PLK_ERR_ARG;
    if (S < 1 || S > kMaxStates || !Q || !root_w) return fail(h, PLK_ERR_ARG, "model needs 1 <= n_states <= 24, Q and root weights");
    if (n_cats < 1 || n_cats > kMaxCats || !cat_rates || !cat_weights)
        return fail(h, PLK_ERR_ARG, "model needs 1 <= n_cats <= 16 with rates and weights");
    if (p_mode != PLK_P_TAYLOR20 && p_mode != PLK_P_EXACT) return fail(h, PLK_ERR_ARG, "unknown p_mode");
    for (int i = 0; i < S * S; ++i)
        if (!std::isfinite(Q[i])) return fail(h, PLK_ERR_ARG, "non-finite Q entry");
    for (int k = 0; k < n_cats; ++k)
        if (!(cat_rates[k] >= 0.0) || !std::isfinite(cat_rates[k]) || !std::isfinite(cat_weights[k]))
            return fail(h, PLK_ERR_ARG, "bad category rate or weight");
    PLK_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
    h->Q.assign(Q, Q + S * S);
    h->root_w.assign(root_w, root_w + S);
    h->cat_rate.assign(cat_rates, cat_rates + n_cats);
    h->cat_w.assign(cat_weights, cat_weights + n_cats);
    if (h->C != n_cats) h->variant = -1;
    h->C = n_cats;
    h->reversible = reversible;
    h->lam.assign(S, 0.0);
    h->L.assign((size_t)S * S, 0.0);
    h->R.assign((size_t)S * S, 0.0);
    if (p_mode == PLK_P_TAYLOR20) h->p_kind = 0;
    else if (reversible) {
        if (!reversible_eigen(S, Q, root_w, h->lam.data(), h->L.data(), h->R.data()))
            return fail(h, PLK_ERR_ARG, "eigen form needs positive root weights (frequencies)");
        h->p_kind = 1;
    } else h->p_kind = 2;
    PLK_CUDA(h,
             upload_group(h, h->d_model_block,
                          {part(h->d_Q, h->Q), part(h->d_rootw, h->root_w), part(h->d_catr, h->cat_rate),
                           part(h->d_catw, h->cat_w), part(h->d_lam, h->lam), part(h->d_L, h->L),
                           part(h->d_R, h->R)}),
             "upload model");
    h->have_model = true;
    h->have_lnl = false;
    return PLK_OK;
}

plk_status plk_loglik_async(plk_handle* h, int precision) {
    plk_status s = ready(h);
    if (s != PLK_OK) return s;
    if (precision != PLK_FP64 && precision != PLK_FP32S) return fail(h, PLK_ERR_ARG, "unknown precision");
    h->lnl_pending = false;
    if (h->bad_tip) return fail(h, PLK_ERR_TIP, "a tip cell allows no state of the model");
    plk_handle::EvSet* ev = nullptr;
    if (h->profiling) {
        if (h->ev_used == h->evs.size()) {
            plk_handle::EvSet e{};
            for (auto& x : e.e) PLK_CUDA(h, cudaEventCreate(&x), "cudaEventCreate");
            h->evs.push_back(e);
        }
        ev = &h->evs[h->ev_used++];
        PLK_CUDA(h, cudaEventRecord(ev->e[0], h->stream), "cudaEventRecord");
    }
    if ((s = build_pmats(h, precision == PLK_FP32S && tuned_paired(h), precision == PLK_FP32S && tuned_tc20(h))) !=
        PLK_OK)
        return s;
    if (ev) PLK_CUDA(h, cudaEventRecord(ev->e[1], h->stream), "cudaEventRecord");
    if ((s = run_prune(h, precision, nullptr, ev ? &ev->e[2] : nullptr)) != PLK_OK) return s;
    if (h->patterns)  // every pattern's lnL counts once per site showing it
        PLK_CUDA(h, launch_weighted_sum(h->d_site_lnl.as<double>(), h->d_pattern_w.as<double>(), h->n_sites,
                                        h->d_lnl.as<double>(), h->stream),
                 "weighted sum kernel launch");
    if (ev) PLK_CUDA(h, cudaEventRecord(ev->e[3], h->stream), "cudaEventRecord");
    h->lnl_pending = true;
    return PLK_OK;
}

plk_status plk_loglik_result(plk_handle* h, double* lnl_out) {
    if (!h) return PLK_ERR_ARG;
    if (!lnl_out) return fail(h, PLK_ERR_ARG, "lnl_out is NULL");
    *lnl_out = 0.0;
    if (!h->lnl_pending) return fail(h, PLK_ERR_STATE, "no evaluation enqueued (plk_loglik_async)");
    double v = 0.0;
    PLK_CUDA(h, cudaMemcpyAsync(&v, h->d_lnl.p, sizeof(double), cudaMemcpyDeviceToHost, h->stream), "copy lnL");
    PLK_CUDA(h, cudaStreamSynchronize(h->stream), "likelihood kernels");
    h->lnl_pending = false;
    if (h->flag_pending) {  // the alignment's empty-cell check, read back with this result
        h->flag_pending = false;
        h->bad_tip = *h->h_flag == h->flag_gen;
    }
    if (h->bad_tip) return fail(h, PLK_ERR_TIP, "a tip cell allows no state of the model");
    *lnl_out = v;
    h->have_lnl = true;
    if (!std::isfinite(v)) {
        clear_counters(h);  // e.g. a bounded device wait ran out in the pass
        return fail(h, PLK_ERR_NUMERIC, "log-likelihood is not finite");
    }
    return PLK_OK;
}

plk_status plk_loglik(plk_handle* h, int precision, double* lnl_out) {
    if (!h) return PLK_ERR_ARG;
    if (!lnl_out) return fail(h, PLK_ERR_ARG, "lnl_out is NULL");
    *lnl_out = 0.0;
    plk_status s = plk_loglik_async(h, precision);
    if (s != PLK_OK) return s;
    return plk_loglik_result(h, lnl_out);
}

plk_status plk_loglik_err(plk_handle* h, double* lnl_fast, double* lnl_fp64, double* abs_err, double* rel_err) {
    if (!h) return PLK_ERR_ARG;
    if (!lnl_fast || !lnl_fp64 || !abs_err || !rel_err) return fail(h, PLK_ERR_ARG, "an output pointer is NULL");
    *lnl_fast = *lnl_fp64 = *abs_err = *rel_err = 0.0;
    // the FP64 plain form first, so that the handle's per-site values are the
    // fast form's afterwards (as after plk_loglik(h, PLK_FP32S, ...))
    double d = 0.0, f = 0.0;
    plk_status s = plk_loglik(h, PLK_FP64, &d);
    if (s != PLK_OK) return s;
    if ((s = plk_loglik(h, PLK_FP32S, &f)) != PLK_OK) return s;
    *lnl_fast = f;
    *lnl_fp64 = d;
    *abs_err = std::fabs(f - d);
    *rel_err = d != 0.0 ? *abs_err / std::fabs(d) : *abs_err;
    return PLK_OK;
}

plk_status plk_set_stream(plk_handle* h, void* stream) {
    if (!h) return PLK_ERR_ARG;
    PLK_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
    PLK_CUDA(h, cudaStreamSynchronize(h->stream), "switch stream");
    h->stream = stream ? static_cast<cudaStream_t>(stream) : h->own_stream;
    return PLK_OK;
}

plk_status plk_set_profiling(plk_handle* h, int on) {
    if (!h) return PLK_ERR_ARG;
    h->profiling = on != 0;
    h->ev_used = 0;
    return PLK_OK;
}

plk_status plk_kernel_times(plk_handle* h, double* ms_out, int* n_evals, int reset) {
    if (!h || !ms_out) return PLK_ERR_ARG;
    PLK_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
    PLK_CUDA(h, cudaStreamSynchronize(h->stream), "kernel timing");
    double tot[3] = {0, 0, 0};
    for (size_t i = 0; i < h->ev_used; ++i)
        for (int p = 0; p < 3; ++p) {
            float ms = 0.f;
            PLK_CUDA(h, cudaEventElapsedTime(&ms, h->evs[i].e[p], h->evs[i].e[p + 1]), "cudaEventElapsedTime");
            tot[p] += ms;
        }
    for (int p = 0; p < 3; ++p) ms_out[p] = tot[p];
    if (n_evals) *n_evals = (int)h->ev_used;
    if (reset) h->ev_used = 0;
    return PLK_OK;
}

int plk_prune_variant(const plk_handle* h) { return h ? h->variant : -1; }

plk_status plk_test_withhold_stage(plk_handle* h) {
    if (!h) return PLK_ERR_ARG;
    h->withhold_stage = true;
    return PLK_OK;
}

plk_status plk_site_loglik(plk_handle* h, double* out) {
    if (!h) return PLK_ERR_ARG;
    if (!out) return fail(h, PLK_ERR_ARG, "out is NULL");
    if (!h->have_lnl) return fail(h, PLK_ERR_STATE, "no likelihood computed yet (plk_loglik)");
    PLK_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
    if (!h->patterns) {
        PLK_CUDA(h, cudaMemcpyAsync(out, h->d_site_lnl.p, sizeof(double) * h->n_sites, cudaMemcpyDeviceToHost, h->stream),
                 "copy site lnL");
        PLK_CUDA(h, cudaStreamSynchronize(h->stream), "copy site lnL");
        return PLK_OK;
    }
    std::vector<double> per_pattern(h->n_sites);
    PLK_CUDA(h, cudaMemcpyAsync(per_pattern.data(), h->d_site_lnl.p, sizeof(double) * h->n_sites,
                                cudaMemcpyDeviceToHost, h->stream), "copy site lnL");
    PLK_CUDA(h, cudaStreamSynchronize(h->stream), "copy site lnL");
    for (int s = 0; s < h->n_sites_full; ++s) out[s] = per_pattern[h->site_pattern[s]];
    return PLK_OK;
}

int plk_n_internal(const plk_handle* h) { return h ? (int)h->post.size() : 0; }

plk_status plk_node_states(plk_handle* h, int mode, int precision, double* out) {
    plk_status s = ready(h);
    if (s != PLK_OK) return s;
    if (!out) return fail(h, PLK_ERR_ARG, "out is NULL");
    if (mode != PLK_NODES_COND && mode != PLK_NODES_MARGINAL) return fail(h, PLK_ERR_ARG, "unknown node-state mode");
    if (precision != PLK_FP64 && precision != PLK_FP32S) return fail(h, PLK_ERR_ARG, "unknown precision");
    if (h->flag_pending) {  // the alignment's empty-cell check
        PLK_CUDA(h, cudaStreamSynchronize(h->stream), "tip check");
        h->flag_pending = false;
        h->bad_tip = *h->h_flag == h->flag_gen;
    }
    if (h->bad_tip) return fail(h, PLK_ERR_TIP, "a tip cell allows no state of the model");
    if ((s = build_pmats(h)) != PLK_OK) return s;
    void* cond = nullptr;
    if ((s = run_prune(h, precision, &cond)) != PLK_OK) return s;
    const int n_int = (int)h->post.size();
    const size_t out_n = (size_t)n_int * h->n_sites * h->S;
    PLK_CUDA(h, h->d_nodes_out.ensure(out_n * sizeof(double)), "allocate node output");
    if (mode == PLK_NODES_COND) {
        PLK_CUDA(h, launch_cond_normalise(cond, h->d_catw.as<double>(), n_int, h->C, h->n_sites, h->S, precision,
                                          h->d_nodes_out.as<double>(), h->stream),
                 "normalise kernel launch");
    } else {
        const size_t tsz = precision == PLK_FP64 ? sizeof(double) : sizeof(float);
        PLK_CUDA(h, h->d_outside.ensure((size_t)n_int * h->C * h->n_sites * h->S * tsz), "allocate outside vectors");
        PreorderArgs p{};
        const bool fp64 = precision == PLK_FP64;
        p.order = h->d_order.as<int>(); p.left = h->d_left.as<int>(); p.right = h->d_right.as<int>();
        p.rank = h->d_rank.as<int>(); p.n_int = n_int; p.n_tips = h->n_tips; p.n_sites = h->n_sites;
        p.n_codes = h->n_codes; p.S = h->S; p.C = h->C; p.codes = h->d_codes.as<uint8_t>();
        p.site_stride = code_stride(h->n_sites);
        p.P = fp64 ? (const void*)h->d_P64.p : (const void*)h->d_P32.p;
        p.tipT = fp64 ? (const void*)h->d_tip64.p : (const void*)h->d_tip32.p;
        p.root_w = h->d_rootw.as<double>(); p.cat_w = h->d_catw.as<double>();
        p.cond = cond; p.outside = h->d_outside.p; p.out = h->d_nodes_out.as<double>();
        PLK_CUDA(h, launch_preorder(p, precision, h->stream), "pre-order kernel launch");
    }
    if (!h->patterns) {
        PLK_CUDA(h, cudaMemcpyAsync(out, h->d_nodes_out.p, out_n * sizeof(double), cudaMemcpyDeviceToHost, h->stream),
                 "copy node states");
        PLK_CUDA(h, cudaStreamSynchronize(h->stream), "node-state kernels");
    } else {
        // [rank][pattern][S] on the device -> [rank][site][S] for the caller
        std::vector<double> per_pattern(out_n);
        PLK_CUDA(h, cudaMemcpyAsync(per_pattern.data(), h->d_nodes_out.p, out_n * sizeof(double),
                                    cudaMemcpyDeviceToHost, h->stream), "copy node states");
        PLK_CUDA(h, cudaStreamSynchronize(h->stream), "node-state kernels");
        const size_t S = (size_t)h->S;
        for (int r = 0; r < n_int; ++r)
            for (int s = 0; s < h->n_sites_full; ++s)
                std::copy_n(&per_pattern[((size_t)r * h->n_sites + h->site_pattern[s]) * S], S,
                            out + ((size_t)r * h->n_sites_full + s) * S);
    }
    h->have_lnl = true;
    return PLK_OK;
}

plk_status plk_node_states_err(plk_handle* h, int mode, double* out, double* max_abs_err) {
    if (!h) return PLK_ERR_ARG;
    if (!out || !max_abs_err) return fail(h, PLK_ERR_ARG, "an output pointer is NULL");
    *max_abs_err = 0.0;
    const size_t n = (size_t)h->post.size() * (size_t)(h->patterns ? h->n_sites_full : h->n_sites) * (size_t)h->S;
    std::vector<double> ref;
    try {
        ref.resize(n);
    } catch (const std::bad_alloc&) {
        return fail(h, PLK_ERR_ALLOC, "host allocation for the FP64 node states failed");
    }
    plk_status s = plk_node_states(h, mode, PLK_FP64, ref.data());
    if (s != PLK_OK) return s;
    if ((s = plk_node_states(h, mode, PLK_FP32S, out)) != PLK_OK) return s;
    double m = 0.0;
    for (size_t i = 0; i < n; ++i) {
        const double e = std::fabs(out[i] - ref[i]);
        if (!(e <= m)) m = e;  // a NaN difference propagates
    }
    *max_abs_err = m;
    return PLK_OK;
}

plk_status plk_simulate(int n_nodes, const int* left, const int* right, const double* bl, int n_states,
                        const double* Q, const double* freqs, int n_cats, const double* cat_rates, int n_sites,
                        uint64_t seed, int n_threads, uint32_t* masks_out) {
    if (n_nodes < 2 || !left || !right || !bl || n_states < 2 || n_states > kMaxStates || !Q || !freqs ||
        n_cats < 1 || n_cats > kMaxCats || !cat_rates || n_sites < 1 || !masks_out)
        return fail(nullptr, PLK_ERR_ARG, "bad arguments to plk_simulate");
    int n_leaves = 0;
    for (int v = 0; v < n_nodes; ++v)
        if (left[v] < 0 && right[v] < 0) ++n_leaves;
    std::vector<int> post, rank;
    int root = -1;
    std::string err;
    if (!check_tree(n_leaves, n_nodes, left, right, &root, &post, &rank, &err)) return fail(nullptr, PLK_ERR_ARG, err);
    if (!simulate_sites(n_leaves, n_nodes, left, right, root, bl, n_states, Q, freqs, n_cats, cat_rates, n_sites, seed,
                        n_threads, masks_out))
        return fail(nullptr, PLK_ERR_ARG, "simulation needs a reversible Q with positive frequencies");
    return PLK_OK;
}

int plk_fit_n_params(int n_states, int n_cats) {
    if (n_states < 2 || n_states > kMaxStates || n_cats < 1 || n_cats > kMaxCats) return 0;
    return gtr_n_params(n_states, n_cats);
}

plk_status plk_fit_gtr(plk_handle* h, int precision, const double* freqs, int n_cats, const double* x0,
                       double step, double ftol, double xtol, int max_evals, double* x_out, double* lnl_out,
                       int* n_evals_out) {
    if (!h) return PLK_ERR_ARG;
    if (!h->have_aln || !h->have_tree) return fail(h, PLK_ERR_STATE, "set the alignment and tree before fitting");
    const int S = h->S;
    if (S < 2 || !freqs || n_cats < 1 || n_cats > kMaxCats || !(step > 0.0) || max_evals < 1 || !x_out || !lnl_out)
        return fail(h, PLK_ERR_ARG, "bad arguments to plk_fit_gtr");
    for (int i = 0; i < S; ++i)
        if (!(freqs[i] > 0.0)) return fail(h, PLK_ERR_ARG, "frequencies must be positive");
    const int n = gtr_n_params(S, n_cats);
    std::vector<double> start(n, 0.0), steps(n, step);
    if (x0) std::copy(x0, x0 + n, start.begin());
    std::vector<double> Q((size_t)S * S), cr(n_cats), cw(n_cats);
    auto set_x = [&](const double* x, bool* ok) -> plk_status {
        double scale = 1.0;
        *ok = gtr_model_from_x(S, x, n_cats, freqs, Q.data(), cr.data(), cw.data(), &scale);
        if (!*ok) return PLK_OK;
        for (int c = 0; c < n_cats; ++c) cr[c] *= scale;
        return plk_set_model(h, S, Q.data(), freqs, 1, n_cats, cr.data(), cw.data(), PLK_P_EXACT);
    };
    auto run = [&](auto& opt) -> plk_status {
        while (!opt.done()) {
            bool ok = false;
            plk_status s = set_x(opt.point().data(), &ok);
            if (s != PLK_OK) return s;
            double f = HUGE_VAL;
            if (ok) {
                double l = 0.0;
                s = plk_loglik(h, precision, &l);
                if (s == PLK_OK) f = -l;
                else if (s != PLK_ERR_NUMERIC) return s;
            }
            opt.tell(f);
        }
        const std::vector<double>& bx = opt.best_x();
        std::copy(bx.begin(), bx.end(), x_out);
        bool ok = false;
        plk_status s = set_x(bx.data(), &ok);
        if (s != PLK_OK) return s;
        *lnl_out = -opt.best_f();
        if (n_evals_out) *n_evals_out = opt.evals();
        return PLK_OK;
    };
    if (h->fit_method == PLK_FIT_QUASI_NEWTON || h->fit_method == PLK_FIT_NEWTON_START) {
        QuasiNewton qn(n, start.data(), steps.data(), ftol, xtol, max_evals, h->fit_method == PLK_FIT_NEWTON_START);
        return run(qn);
    }
    NelderMead nm(n, start.data(), steps.data(), ftol, xtol, max_evals);
    return run(nm);
}

plk_status plk_set_fit_method(plk_handle* h, int method) {
    if (!h) return PLK_ERR_ARG;
    if (method != PLK_FIT_NELDER_MEAD && method != PLK_FIT_QUASI_NEWTON && method != PLK_FIT_NEWTON_START)
        return fail(h, PLK_ERR_ARG, "unknown fit method");
    h->fit_method = method;
    return PLK_OK;
}

plk_status plk_q_matrix(int n, int reversible, const unsigned* spec, const double* rates, const double* freqs,
                        double* Q_out) {
    if (n < 1 || n > kMaxStates || !spec || !rates || !Q_out) return fail(nullptr, PLK_ERR_ARG, "bad arguments to plk_q_matrix");
    q_matrix(n, reversible != 0, spec, rates, freqs, Q_out);
    return PLK_OK;
}

plk_status plk_pmat_host(int n, const double* Q, const double* root_w, int reversible, double t, int p_mode,
                         double* P_out) {
    if (n < 1 || n > kMaxStates || !Q || !P_out) return fail(nullptr, PLK_ERR_ARG, "bad arguments to plk_pmat_host");
    if (p_mode == PLK_P_TAYLOR20) {
        pmat_taylor20_host(n, Q, t, P_out);
        return PLK_OK;
    }
    if (p_mode != PLK_P_EXACT) return fail(nullptr, PLK_ERR_ARG, "unknown p_mode");
    if (reversible) {
        if (!root_w) return fail(nullptr, PLK_ERR_ARG, "reversible eigen form needs root weights");
        std::vector<double> lam(n), L((size_t)n * n), R((size_t)n * n);
        if (!reversible_eigen(n, Q, root_w, lam.data(), L.data(), R.data()))
            return fail(nullptr, PLK_ERR_ARG, "eigen form needs positive frequencies");
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                double acc = 0.0;
                for (int m = 0; m < n; ++m) acc += L[i * n + m] * std::exp(lam[m] * t) * R[m * n + j];
                P_out[i * n + j] = acc;
            }
        return PLK_OK;
    }
    pmat_series_host(n, Q, t, P_out);
    return PLK_OK;
}

plk_status plk_discrete_gamma(double alpha, int K, double* rates_out) {
    if (!(alpha > 0.0) || !std::isfinite(alpha) || K < 1 || K > kMaxCats || !rates_out)
        return fail(nullptr, PLK_ERR_ARG, "discrete Gamma needs alpha > 0 and 1 <= K <= 16");
    discrete_gamma(alpha, K, rates_out);
    return PLK_OK;
}

plk_status plk_effective_lengths(int n_nodes, const int* left, const int* right, const double* bl,
                                 int root_quirk, int n_cut, const float* cut_off, const float* cut_rate,
                                 const int* clade_of_node, int n_clades, const float* clade_rate,
                                 double* out) {
    if (n_nodes < 2 || !left || !right || !bl || !out || n_cut < 0 || n_clades < 0 ||
        (n_cut > 0 && (!cut_off || !cut_rate)) || (n_clades > 0 && !clade_rate))
        return fail(nullptr, PLK_ERR_ARG, "bad arguments to plk_effective_lengths");
    int n_leaves = 0;
    for (int v = 0; v < n_nodes; ++v)
        if (left[v] < 0 && right[v] < 0) ++n_leaves;
    std::vector<int> post, rank;
    int root = -1;
    std::string err;
    if (!check_tree(n_leaves, n_nodes, left, right, &root, &post, &rank, &err)) return fail(nullptr, PLK_ERR_ARG, err);
    std::vector<float> co(cut_off, cut_off + n_cut), cr(cut_rate, cut_rate + n_cut);
    std::vector<float> crt(clade_rate, clade_rate + n_clades);
    std::vector<int> con;
    if (clade_of_node) con.assign(clade_of_node, clade_of_node + n_nodes);
    effective_lengths(n_nodes, left, right, root, bl, root_quirk != 0, co, cr, con, crt, out);
    return PLK_OK;
}

}  // extern "C"
