// C ABI of the batch engine (include/plk.h, "batches").
//
// A batch holds many 4-state alignments, each with its own tree and model --
// the many trees treeator scores one simpleML at a time
// (src/treeator.cpp:705-990) and the per-partition models of partition_models
// (src/partition_models.h:30-165) -- and scores them all in one persistent
// launch.  The launch sequence (clear the work-queue head, upload the models
// from pinned host memory, P(t) for every node, the post-order pass, the
// per-item reduction, download the lnLs) is captured once into a CUDA graph
// and replayed for every evaluation.  An autotuner picks the sites per thread
// and the CTAs per SM of the persistent kernel on the batch itself.  NNI
// scoring (plk_nni.cu) reuses the same table.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "plk_batch.h"
#include "plk_internal.h"

using namespace plk;

namespace {

struct BBuf {
    void* p = nullptr;
    size_t bytes = 0;
    BBuf() = default;
    BBuf(const BBuf&) = delete;
    BBuf& operator=(const BBuf&) = delete;
    ~BBuf() { if (p) cudaFree(p); }
    cudaError_t ensure(size_t n) {
        if (n <= bytes && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        if (n == 0) n = 16;
        cudaError_t e = cudaMalloc(&p, n);
        if (e == cudaSuccess) bytes = n;
        return e;
    }
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
};

struct ItemHost {
    int n_tips = 0, n_sites = 0, n_nodes = 0, n_int = 0;
    Program prog;
    std::vector<double> t_eff;     // by internal id
    std::vector<int2> child;       // by internal id
    std::vector<uint8_t> codes;    // [n_tips][stride]
    std::vector<double> model;     // lam L R root_w cat_rate cat_w
    std::vector<NniMoveDev> moves; // internal ids
    std::vector<int> move_report;  // (caller's node id, which) per move
    std::vector<int> caller_id;    // caller's node id of every internal id
    bool has_model = false;
};

// Work units of one tile size plus their per-item index.
struct UnitSet {
    BBuf units, ptr, idx, sums, move_off;
    int n_units = 0;
    int spt = 0;
    std::vector<int2> host_units;
};

constexpr int kThreads = 128;

}  // namespace

struct plk_batch {
    int device = 0;
    int C = 1;
    int n_sms = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    std::vector<ItemHost> items;
    bool layout_dirty = true;
    // device layout
    BBuf d_items, d_codes, d_ops, d_teff, d_node_item, d_child, d_model, d_P32, d_tip32, d_lnl, d_counter;
    BBuf d_P32p, d_tip32p;  // paired layouts (C = 2, 4, 8)
    BBuf d_moves, d_move_item, d_nni_out, d_unit_move_sums, d_scr_D, d_scr_ED, d_scr_O, d_scr_EO;
    BBuf d_blen_ueo, d_blen_ues, d_blen_ieo, d_blen_ei, d_blen_out;  // branch-length derivative slots
    double* h_model = nullptr;  // pinned staging of the models
    double* h_lnl = nullptr;    // pinned lnL download
    size_t h_model_n = 0, h_lnl_n = 0;
    int n_nodes_total = 0, max_ops = 0, max_tips = 0, max_depth = 0, max_int = 0, total_moves = 0;
    UnitSet lnl_units, nni_units;
    // tuning of the lnL kernel
    BatchForm form;
    int grid = 0;
    size_t smem = 0;
    double tuned_ms = 0.0;
    bool tuned = false;
    // optimiser of plk_batch_fit_gtr
    int fit_method = PLK_FIT_NELDER_MEAD;
    // graph
    cudaGraphExec_t exec = nullptr;
    bool use_graph = true;
    // CUDA events around the device work of the last plk_batch_loglik (0, 1)
    // and plk_batch_nni_loglik (2, 3), and their elapsed times
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    double last_ms[2] = {0.0, 0.0};
    ~plk_batch() {
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
        if (exec) cudaGraphExecDestroy(exec);
        if (h_model) cudaFreeHost(h_model);
        if (h_lnl) cudaFreeHost(h_lnl);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

plk_status bfail(plk_batch* b, plk_status s, const std::string& m) {
    if (b) b->err = m;
    else report_error(s, m);
    return s;
}

#define PLK_BCUDA(b, expr, what)                                                                    \
    do {                                                                                            \
        cudaError_t _e = (expr);                                                                    \
        if (_e != cudaSuccess)                                                                      \
            return bfail(b, _e == cudaErrorMemoryAllocation ? PLK_ERR_ALLOC : PLK_ERR_CUDA,          \
                         std::string(what) + ": " + cudaGetErrorString(_e));                        \
    } while (0)

BatchDev device_view(plk_batch* b, const UnitSet& us) {
    BatchDev d{};
    d.n_items = (int)b->items.size();
    d.n_units = us.n_units;
    d.n_nodes_total = b->n_nodes_total;
    d.C = b->C;
    d.max_depth = b->max_depth;
    d.items = b->d_items.as<BatchItemDev>();
    d.codes = b->d_codes.as<uint8_t>();
    d.ops = b->d_ops.as<Op>();
    d.t_eff = b->d_teff.as<double>();
    d.node_item = b->d_node_item.as<int2>();
    d.child = b->d_child.as<int2>();
    d.model = b->d_model.as<double>();
    d.P32 = b->d_P32.as<float>();
    d.tip32 = b->d_tip32.as<float>();
    d.P32p = nullptr;  // the plain layout only, unless lnl_view asks for the paired one
    d.tip32p = nullptr;
    d.write_std = 1;
    d.units = us.units.as<int2>();
    d.unit_sums = us.sums.as<double>();
    d.item_unit_ptr = us.ptr.as<int>();
    d.item_units = us.idx.as<int>();
    d.lnl = b->d_lnl.as<double>();
    d.counter = b->d_counter.as<int>();
    d.moves = b->d_moves.as<NniMoveDev>();
    d.unit_move_off = us.move_off.as<long long>();
    d.unit_move_sums = b->d_unit_move_sums.as<double>();
    d.nni_out = b->d_nni_out.as<double>();
    d.move_item = b->d_move_item.as<int>();
    d.total_moves = b->total_moves;
    d.scratch_int = b->max_int;
    d.scr_D = b->d_scr_D.as<float4>();
    d.scr_ED = b->d_scr_ED.as<int>();
    d.scr_O = b->d_scr_O.as<float4>();
    d.scr_EO = b->d_scr_EO.as<int>();
    return d;
}

// The view for the lnL kernels: P(t) written in the layouts that `form`
// reads (both while tuning).
BatchDev lnl_view(plk_batch* b, const BatchForm* form) {
    BatchDev d = device_view(b, b->lnl_units);
    const bool has_paired = b->d_P32p.p != nullptr && (b->C == 2 || b->C == 4 || b->C == 8);
    if (has_paired && (!form || form->paired)) {
        d.P32p = b->d_P32p.as<float>();
        d.tip32p = b->d_tip32p.as<float>();
    }
    if (form && form->paired) d.write_std = 0;
    return d;
}

// Work units for tiles of 128 * spt sites: items with the longest op lists
// first, so the persistent grid ends on the cheapest units.
plk_status build_units(plk_batch* b, UnitSet& us, int spt, bool with_moves) {
    const int tile = kThreads * spt;
    std::vector<int> order(b->items.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return b->items[x].prog.ops.size() > b->items[y].prog.ops.size();
    });
    std::vector<int2> units;
    std::vector<std::vector<int>> per_item(b->items.size());
    for (int i : order) {
        const int tiles = (b->items[i].n_sites + tile - 1) / tile;
        for (int t = 0; t < tiles; ++t) {
            per_item[i].push_back((int)units.size());
            units.push_back(make_int2(i, t));
        }
    }
    std::vector<int> ptr(b->items.size() + 1, 0), idx;
    for (size_t i = 0; i < b->items.size(); ++i) {
        ptr[i + 1] = ptr[i] + (int)per_item[i].size();
        idx.insert(idx.end(), per_item[i].begin(), per_item[i].end());
    }
    us.n_units = (int)units.size();
    PLK_BCUDA(b, us.units.ensure(units.size() * sizeof(int2)), "allocate units");
    PLK_BCUDA(b, us.sums.ensure(units.size() * 2 * sizeof(double)), "allocate unit sums");
    PLK_BCUDA(b, us.ptr.ensure(ptr.size() * sizeof(int)), "allocate unit index");
    PLK_BCUDA(b, us.idx.ensure(std::max<size_t>(idx.size(), 1) * sizeof(int)), "allocate unit index");
    PLK_BCUDA(b, cudaMemcpy(us.units.p, units.data(), units.size() * sizeof(int2), cudaMemcpyHostToDevice), "upload units");
    PLK_BCUDA(b, cudaMemcpy(us.ptr.p, ptr.data(), ptr.size() * sizeof(int), cudaMemcpyHostToDevice), "upload units");
    if (!idx.empty())
        PLK_BCUDA(b, cudaMemcpy(us.idx.p, idx.data(), idx.size() * sizeof(int), cudaMemcpyHostToDevice), "upload units");
    if (with_moves) {
        std::vector<long long> off(units.size());
        long long tot = 0;
        for (size_t u = 0; u < units.size(); ++u) {
            off[u] = tot;
            tot += (long long)b->items[units[u].x].moves.size();
        }
        PLK_BCUDA(b, us.move_off.ensure(std::max<size_t>(off.size(), 1) * sizeof(long long)), "allocate move offsets");
        PLK_BCUDA(b, cudaMemcpy(us.move_off.p, off.data(), off.size() * sizeof(long long), cudaMemcpyHostToDevice),
                  "upload move offsets");
        PLK_BCUDA(b, b->d_unit_move_sums.ensure((size_t)std::max<long long>(tot, 1) * 2 * sizeof(double)),
                  "allocate move partial sums");
    }
    us.spt = spt;
    us.host_units = units;
    return PLK_OK;
}

plk_status build_layout(plk_batch* b) {
    const int C = b->C;
    std::vector<BatchItemDev> it(b->items.size());
    std::vector<Op> ops;
    std::vector<double> teff;
    std::vector<int2> node_item, child;
    std::vector<NniMoveDev> moves;
    std::vector<int> move_item;
    size_t codes_bytes = 0;
    int tips_total = 0;
    b->max_ops = b->max_tips = b->max_depth = b->max_int = 0;
    for (size_t i = 0; i < b->items.size(); ++i) {
        const ItemHost& h = b->items[i];
        BatchItemDev& d = it[i];
        std::memset(&d, 0, sizeof(d));
        d.codes_off = (long long)codes_bytes;
        d.ops_off = (int)ops.size();
        d.n_ops = (int)h.prog.ops.size();
        d.node_off = (int)teff.size();
        d.tip_off = tips_total;
        d.n_tips = h.n_tips;
        d.n_sites = h.n_sites;
        d.site_stride = code_stride(h.n_sites);
        d.model_off = (int)i * batch_model_stride(C);
        d.moves_off = (int)moves.size();
        d.n_moves = (int)h.moves.size();
        d.move_out_off = (int)moves.size();
        d.n_int = h.n_int;
        codes_bytes += h.codes.size();
        ops.insert(ops.end(), h.prog.ops.begin(), h.prog.ops.end());
        teff.insert(teff.end(), h.t_eff.begin(), h.t_eff.end());
        child.insert(child.end(), h.child.begin(), h.child.end());
        for (int v = 0; v < h.n_nodes; ++v) node_item.push_back(make_int2((int)i, v));
        moves.insert(moves.end(), h.moves.begin(), h.moves.end());
        for (size_t m = 0; m < h.moves.size(); ++m) move_item.push_back((int)i);
        tips_total += h.n_tips;
        b->max_ops = std::max(b->max_ops, d.n_ops);
        b->max_tips = std::max(b->max_tips, h.n_tips);
        b->max_depth = std::max(b->max_depth, h.prog.max_depth);
        b->max_int = std::max(b->max_int, h.n_int);
    }
    b->n_nodes_total = (int)teff.size();
    b->total_moves = (int)moves.size();
    PLK_BCUDA(b, b->d_items.ensure(it.size() * sizeof(BatchItemDev)), "allocate batch table");
    PLK_BCUDA(b, b->d_codes.ensure(codes_bytes), "allocate tip codes");
    PLK_BCUDA(b, b->d_ops.ensure(ops.size() * sizeof(Op)), "allocate programs");
    PLK_BCUDA(b, b->d_teff.ensure(teff.size() * sizeof(double)), "allocate lengths");
    PLK_BCUDA(b, b->d_node_item.ensure(node_item.size() * sizeof(int2)), "allocate node map");
    PLK_BCUDA(b, b->d_child.ensure(child.size() * sizeof(int2)), "allocate child table");
    PLK_BCUDA(b, b->d_model.ensure(it.size() * batch_model_stride(C) * sizeof(double)), "allocate models");
    PLK_BCUDA(b, b->d_P32.ensure((size_t)b->n_nodes_total * C * 16 * sizeof(float)), "allocate P");
    PLK_BCUDA(b, b->d_tip32.ensure((size_t)tips_total * C * 16 * 4 * sizeof(float)), "allocate tip tables");
    if (C == 2 || C == 4 || C == 8) {
        PLK_BCUDA(b, b->d_P32p.ensure((size_t)b->n_nodes_total * C * 16 * sizeof(float)), "allocate P");
        PLK_BCUDA(b, b->d_tip32p.ensure((size_t)tips_total * C * 16 * 4 * sizeof(float)), "allocate tip tables");
    }
    PLK_BCUDA(b, b->d_lnl.ensure(it.size() * sizeof(double)), "allocate lnL");
    PLK_BCUDA(b, b->d_counter.ensure(sizeof(int)), "allocate counter");
    PLK_BCUDA(b, b->d_moves.ensure(std::max<size_t>(moves.size(), 1) * sizeof(NniMoveDev)), "allocate moves");
    PLK_BCUDA(b, b->d_move_item.ensure(std::max<size_t>(move_item.size(), 1) * sizeof(int)), "allocate moves");
    PLK_BCUDA(b, b->d_nni_out.ensure(std::max<size_t>(moves.size(), 1) * sizeof(double)), "allocate NNI output");
    PLK_BCUDA(b, cudaMemcpy(b->d_items.p, it.data(), it.size() * sizeof(BatchItemDev), cudaMemcpyHostToDevice), "upload table");
    size_t off = 0;
    for (const ItemHost& h : b->items) {
        PLK_BCUDA(b, cudaMemcpy(b->d_codes.as<uint8_t>() + off, h.codes.data(), h.codes.size(), cudaMemcpyHostToDevice),
                  "upload tip codes");
        off += h.codes.size();
    }
    PLK_BCUDA(b, cudaMemcpy(b->d_ops.p, ops.data(), ops.size() * sizeof(Op), cudaMemcpyHostToDevice), "upload programs");
    PLK_BCUDA(b, cudaMemcpy(b->d_teff.p, teff.data(), teff.size() * sizeof(double), cudaMemcpyHostToDevice), "upload lengths");
    PLK_BCUDA(b, cudaMemcpy(b->d_node_item.p, node_item.data(), node_item.size() * sizeof(int2), cudaMemcpyHostToDevice),
              "upload node map");
    PLK_BCUDA(b, cudaMemcpy(b->d_child.p, child.data(), child.size() * sizeof(int2), cudaMemcpyHostToDevice),
              "upload child table");
    if (!moves.empty()) {
        PLK_BCUDA(b, cudaMemcpy(b->d_moves.p, moves.data(), moves.size() * sizeof(NniMoveDev), cudaMemcpyHostToDevice),
                  "upload moves");
        PLK_BCUDA(b, cudaMemcpy(b->d_move_item.p, move_item.data(), move_item.size() * sizeof(int), cudaMemcpyHostToDevice),
                  "upload moves");
    }
    const size_t mn = it.size() * batch_model_stride(C);
    if (mn > b->h_model_n) {
        if (b->h_model) cudaFreeHost(b->h_model);
        b->h_model = nullptr;
        PLK_BCUDA(b, cudaMallocHost(&b->h_model, mn * sizeof(double)), "allocate pinned models");
        b->h_model_n = mn;
    }
    const size_t ln = std::max(it.size(), moves.size());
    if (ln > b->h_lnl_n) {
        if (b->h_lnl) cudaFreeHost(b->h_lnl);
        b->h_lnl = nullptr;
        PLK_BCUDA(b, cudaMallocHost(&b->h_lnl, ln * sizeof(double)), "allocate pinned lnL");
        b->h_lnl_n = ln;
    }
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    b->lnl_units.spt = 0;
    b->nni_units.spt = 0;
    b->tuned = false;
    b->layout_dirty = false;
    return PLK_OK;
}

// The evaluation sequence (graph body).
plk_status enqueue_eval(plk_batch* b) {
    const BatchDev d = lnl_view(b, &b->form);
    const size_t mn = b->items.size() * batch_model_stride(b->C);
    PLK_BCUDA(b, cudaMemsetAsync(b->d_counter.p, 0, sizeof(int), b->stream), "clear work queue");
    PLK_BCUDA(b, cudaMemcpyAsync(b->d_model.p, b->h_model, mn * sizeof(double), cudaMemcpyHostToDevice, b->stream),
              "upload models");
    PLK_BCUDA(b, launch_batch_pmat(d, b->stream), "batch P(t) launch");
    PLK_BCUDA(b, launch_batch_prune(d, b->form, b->grid, b->smem, b->stream), "batch post-order launch");
    PLK_BCUDA(b, launch_batch_reduce(d, b->stream), "batch reduce launch");
    PLK_BCUDA(b, cudaMemcpyAsync(b->h_lnl, b->d_lnl.p, b->items.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                 b->stream),
              "download lnL");
    return PLK_OK;
}

// Autotuner over the kernel forms -- categories in pairs or one at a time,
// sites per thread 1 or 2, tip codes staged in shared memory (where they fit)
// or read from global -- times CTAs per SM 1 .. occupancy, two launches of
// the persistent kernel after a warm-up each.  PLK_BATCH_SPT and
// PLK_BATCH_PAIRED (0 / 1) pin those choices.
plk_status tune(plk_batch* b) {
    cudaEvent_t e0, e1;
    PLK_BCUDA(b, cudaEventCreate(&e0), "cudaEventCreate");
    PLK_BCUDA(b, cudaEventCreate(&e1), "cudaEventCreate");
    double best = 1e30;
    BatchForm best_form;
    int best_grid = 0;
    size_t best_smem = 0;
    const char* force_spt = getenv("PLK_BATCH_SPT");
    const char* force_paired = getenv("PLK_BATCH_PAIRED");
    std::vector<BatchForm> forms;
    for (int paired = 0; paired <= 1; ++paired)
        for (int spt = 1; spt <= 2; ++spt)
            for (int codes = 1; codes >= 0; --codes) {
                BatchForm f;
                f.spt = spt;
                f.codes_smem = codes != 0;
                f.paired = paired != 0;
                if (!batch_form_valid(b->C, f)) continue;
                if (force_spt && atoi(force_spt) != spt) continue;
                if (force_paired && atoi(force_paired) != paired) continue;
                const size_t smem = batch_smem_bytes(b->C, f, b->max_ops, b->max_tips, b->max_depth);
                if (smem == 0 || smem > 227 * 1024) continue;
                if (f.codes_smem && smem > 160 * 1024) continue;
                forms.push_back(f);
            }
    for (const BatchForm& f : forms) {
        const size_t smem = batch_smem_bytes(b->C, f, b->max_ops, b->max_tips, b->max_depth);
        const int occ = batch_occupancy(b->C, f, smem);
        if (occ < 1) continue;
        if (b->lnl_units.spt != f.spt) {
            plk_status s = build_units(b, b->lnl_units, f.spt, false);
            if (s != PLK_OK) return s;
        }
        const BatchDev d = lnl_view(b, nullptr);
        for (int per_sm = 1; per_sm <= occ; ++per_sm) {
            const int grid = std::min(b->lnl_units.n_units, per_sm * b->n_sms);
            if (grid < 1) continue;
            float ms = 0.f;
            for (int rep = 0; rep < 3; ++rep) {  // warm-up, then two timed launches
                PLK_BCUDA(b, cudaMemsetAsync(b->d_counter.p, 0, sizeof(int), b->stream), "clear work queue");
                if (rep == 1) PLK_BCUDA(b, cudaEventRecord(e0, b->stream), "cudaEventRecord");
                PLK_BCUDA(b, launch_batch_prune(d, f, grid, smem, b->stream), "batch post-order launch");
            }
            PLK_BCUDA(b, cudaEventRecord(e1, b->stream), "cudaEventRecord");
            PLK_BCUDA(b, cudaEventSynchronize(e1), "tune");
            PLK_BCUDA(b, cudaEventElapsedTime(&ms, e0, e1), "tune");
            if (ms < best) {
                best = ms;
                best_form = f;
                best_grid = grid;
                best_smem = smem;
            }
            if (grid == b->lnl_units.n_units) break;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best_grid == 0) return bfail(b, PLK_ERR_UNSUPPORTED, "no batch kernel configuration fits these trees");
    b->form = best_form;
    b->grid = best_grid;
    b->smem = best_smem;
    b->tuned_ms = best / 2.0;
    if (b->lnl_units.spt != best_form.spt) {
        plk_status s = build_units(b, b->lnl_units, best_form.spt, false);
        if (s != PLK_OK) return s;
    }
    b->tuned = true;
    return PLK_OK;
}

plk_status prepare_layout(plk_batch* b) {
    PLK_BCUDA(b, cudaSetDevice(b->device), "cudaSetDevice");
    if (b->items.empty()) return bfail(b, PLK_ERR_STATE, "batch is empty");
    for (size_t i = 0; i < b->items.size(); ++i)
        if (!b->items[i].has_model) return bfail(b, PLK_ERR_STATE, "item " + std::to_string(i) + " has no model");
    if (b->layout_dirty) {
        plk_status s = build_layout(b);
        if (s != PLK_OK) return s;
    }
    const int stride = batch_model_stride(b->C);
    for (size_t i = 0; i < b->items.size(); ++i)
        std::memcpy(b->h_model + i * stride, b->items[i].model.data(), stride * sizeof(double));
    return PLK_OK;
}

plk_status prepare(plk_batch* b) {
    plk_status s = prepare_layout(b);
    if (s != PLK_OK) return s;
    const int stride = batch_model_stride(b->C);
    if (!b->tuned) {
        // models must be on the device before timing the kernels
        PLK_BCUDA(b, cudaMemcpyAsync(b->d_model.p, b->h_model, b->items.size() * stride * sizeof(double),
                                     cudaMemcpyHostToDevice, b->stream),
                  "upload models");
        PLK_BCUDA(b, launch_batch_pmat(lnl_view(b, nullptr), b->stream), "batch P(t) launch");
        s = tune(b);
        if (s != PLK_OK) return s;
    }
    if (b->use_graph && !b->exec) {
        cudaGraph_t g = nullptr;
        PLK_BCUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        s = enqueue_eval(b);
        cudaError_t e = cudaStreamEndCapture(b->stream, &g);
        if (s != PLK_OK || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            b->use_graph = false;  // run the same sequence without a graph
        } else {
            e = cudaGraphInstantiate(&b->exec, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                b->exec = nullptr;
                cudaGetLastError();
                b->use_graph = false;
            }
        }
    }
    return PLK_OK;
}

// Relabel internal nodes n_tips + post-order rank, then enumerate the NNI
// rearrangements of the rooted tree: for an internal node v whose parent u
// is not the root, swap one of v's children with v's sibling (two moves);
// across the root edge between two internal root children v (left) and c,
// swap v's right child with either child of c (two moves).  A binary tree
// with n tips gets 2(n - 3) moves: every internal edge of the unrooted tree
// and both of its interchanges once.
void relabel_and_enumerate(int n_tips, int n_nodes, const int* left, const int* right, const double* bl,
                           const std::vector<int>& rank, int root, ItemHost* h, std::vector<int>* L2,
                           std::vector<int>* R2, std::vector<double>* B2) {
    std::vector<int> nid(n_nodes), oid(n_nodes);
    for (int v = 0; v < n_nodes; ++v) {
        nid[v] = v < n_tips ? v : n_tips + rank[v];
        oid[nid[v]] = v;
    }
    L2->assign(n_nodes, -1);
    R2->assign(n_nodes, -1);
    B2->assign(n_nodes, 0.0);
    for (int v = 0; v < n_nodes; ++v) {
        (*L2)[nid[v]] = left[v] >= 0 ? nid[left[v]] : -1;
        (*R2)[nid[v]] = right[v] >= 0 ? nid[right[v]] : -1;
        (*B2)[nid[v]] = bl[v];
    }
    const int r2 = nid[root];
    std::vector<int> parent(n_nodes, -1);
    for (int v = 0; v < n_nodes; ++v) {
        if ((*L2)[v] >= 0) parent[(*L2)[v]] = v;
        if ((*R2)[v] >= 0) parent[(*R2)[v]] = v;
    }
    h->caller_id = oid;
    auto binary = [&](int v) { return v >= n_tips && (*L2)[v] >= 0 && (*R2)[v] >= 0; };
    h->moves.clear();
    h->move_report.clear();
    auto add = [&](int kind, int which, int v, int u, int c, int x, int y, int z, int p, int q) {
        NniMoveDev m{};
        m.kind = kind; m.v = v; m.u = u; m.c = c; m.x = x; m.y = y; m.z = z; m.p = p; m.q = q;
        h->moves.push_back(m);
        h->move_report.push_back(oid[v]);
        h->move_report.push_back(which);
    };
    for (int v = n_tips; v < n_nodes; ++v) {
        if (v == r2 || !binary(v)) continue;
        const int u = parent[v];
        if (!binary(u)) continue;
        const int c = (*L2)[u] == v ? (*R2)[u] : (*L2)[u];
        const int a = (*L2)[v], bb = (*R2)[v];
        if (u != r2) {
            add(0, 0, v, u, -1, a, c, bb, -1, -1);   // v' = (a, c), u' = (v', b)
            add(0, 1, v, u, -1, c, bb, a, -1, -1);   // v' = (c, b), u' = (v', a)
        } else if ((*L2)[u] == v && binary(c)) {
            const int d = (*L2)[c], e = (*R2)[c];
            add(1, 2, v, u, c, a, d, -1, bb, e);     // v' = (a, d), c' = (b, e)
            add(1, 3, v, u, c, a, e, -1, d, bb);     // v' = (a, e), c' = (d, b)
        }
    }
}

}  // namespace

namespace {
// the pair of timing events (2 which, 2 which + 1), created on first use
plk_status batch_events(plk_batch* b, int which) {
    for (int i = 2 * which; i < 2 * which + 2; ++i)
        if (!b->ev[i]) PLK_BCUDA(b, cudaEventCreate(&b->ev[i]), "cudaEventCreate");
    return PLK_OK;
}
}  // namespace

extern "C" {

plk_status plk_batch_create(plk_batch** out, int device, int n_cats) {
    if (!out) return report_error(PLK_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (n_cats < 1 || n_cats > 8) return report_error(PLK_ERR_ARG, "batches support 1..8 rate categories");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return report_error(PLK_ERR_NODEV, "no CUDA device");
    if (device < 0 || device >= n) return report_error(PLK_ERR_ARG, "device index out of range");
    if ((e = cudaSetDevice(device)) != cudaSuccess) return report_error(PLK_ERR_CUDA, cudaGetErrorString(e));
    plk_batch* b = new (std::nothrow) plk_batch();
    if (!b) return report_error(PLK_ERR_ALLOC, "host allocation failed");
    b->device = device;
    b->C = n_cats;
    cudaDeviceGetAttribute(&b->n_sms, cudaDevAttrMultiProcessorCount, device);
    if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess) {
        delete b;
        return report_error(PLK_ERR_CUDA, cudaGetErrorString(e));
    }
    if (const char* g = getenv("PLK_BATCH_NOGRAPH")) b->use_graph = atoi(g) == 0;
    *out = b;
    return PLK_OK;
}

void plk_batch_destroy(plk_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    delete b;
}

const char* plk_batch_last_error(const plk_batch* b) { return b ? b->err.c_str() : plk_last_error(nullptr); }

int plk_batch_n_items(const plk_batch* b) { return b ? (int)b->items.size() : 0; }

plk_status plk_batch_add(plk_batch* b, int n_tips, int n_sites, const uint32_t* masks, int n_nodes, const int* left,
                         const int* right, const double* bl, int* item_out) {
    if (!b) return PLK_ERR_ARG;
    if (n_tips < 2 || n_sites < 1 || !masks || n_nodes < 3 || !left || !right || !bl)
        return bfail(b, PLK_ERR_ARG, "batch item needs >= 2 tips, >= 1 site and a tree");
    ItemHost h;
    std::vector<int> post, rank;
    int root = -1;
    std::string err;
    int n_leaves = 0;
    for (int v = 0; v < n_nodes; ++v)
        if (left[v] < 0 && right[v] < 0) ++n_leaves;
    if (n_leaves != n_tips) return bfail(b, PLK_ERR_ARG, "tree tips and alignment rows differ");
    if (!check_tree(n_tips, n_nodes, left, right, &root, &post, &rank, &err)) return bfail(b, PLK_ERR_ARG, err);
    for (int v = 0; v < n_nodes; ++v)
        if (!std::isfinite(bl[v])) return bfail(b, PLK_ERR_ARG, "non-finite branch length");
    std::vector<int> L2, R2;
    std::vector<double> B2;
    relabel_and_enumerate(n_tips, n_nodes, left, right, bl, rank, root, &h, &L2, &R2, &B2);
    std::vector<int> post2, rank2;
    int root2 = -1;
    if (!check_tree(n_tips, n_nodes, L2.data(), R2.data(), &root2, &post2, &rank2, &err))
        return bfail(b, PLK_ERR_ARG, err);
    h.n_tips = n_tips;
    h.n_sites = n_sites;
    h.n_nodes = n_nodes;
    h.n_int = (int)post2.size();
    h.prog = build_program(n_tips, n_nodes, L2.data(), R2.data(), root2, rank2);
    h.t_eff.assign(n_nodes, 0.0);
    effective_lengths(n_nodes, L2.data(), R2.data(), root2, B2.data(), false, {}, {}, {}, {}, h.t_eff.data());
    h.child.resize(n_nodes);
    for (int v = 0; v < n_nodes; ++v) h.child[v] = make_int2(L2[v], R2[v]);
    const int stride = code_stride(n_sites);
    h.codes.assign((size_t)n_tips * stride, 0);
    for (int t = 0; t < n_tips; ++t)
        for (int s = 0; s < n_sites; ++s) {
            const uint32_t m = masks[(size_t)t * n_sites + s] & 0xFu;
            if (m == 0) return bfail(b, PLK_ERR_TIP, "a tip cell allows no state");
            h.codes[(size_t)t * stride + s] = (uint8_t)m;
        }
    h.model.assign(batch_model_stride(b->C), 0.0);
    b->items.push_back(std::move(h));
    b->layout_dirty = true;
    if (item_out) *item_out = (int)b->items.size() - 1;
    return PLK_OK;
}

plk_status plk_batch_set_model(plk_batch* b, int item, const double* Q, const double* freqs, const double* cat_rates,
                               const double* cat_weights) {
    if (!b) return PLK_ERR_ARG;
    if (item < 0 || item >= (int)b->items.size() || !Q || !freqs || !cat_rates || !cat_weights)
        return bfail(b, PLK_ERR_ARG, "bad arguments to plk_batch_set_model");
    std::vector<double>& m = b->items[item].model;
    if (!reversible_eigen(4, Q, freqs, m.data(), m.data() + 4, m.data() + 20))
        return bfail(b, PLK_ERR_ARG, "reversible model needs positive frequencies");
    for (int s = 0; s < 4; ++s) m[36 + s] = freqs[s];
    for (int k = 0; k < b->C; ++k) {
        if (!(cat_rates[k] >= 0.0) || !std::isfinite(cat_weights[k]))
            return bfail(b, PLK_ERR_ARG, "bad category rate or weight");
        m[40 + k] = cat_rates[k];
        m[40 + b->C + k] = cat_weights[k];
    }
    b->items[item].has_model = true;
    return PLK_OK;
}

plk_status plk_batch_loglik(plk_batch* b, double* lnl_out) {
    if (!b || !lnl_out) return b ? bfail(b, PLK_ERR_ARG, "lnl_out is NULL") : PLK_ERR_ARG;
    plk_status s = prepare(b);
    if (s != PLK_OK) return s;
    if ((s = batch_events(b, 0)) != PLK_OK) return s;
    PLK_BCUDA(b, cudaEventRecord(b->ev[0], b->stream), "cudaEventRecord");
    if (b->exec) PLK_BCUDA(b, cudaGraphLaunch(b->exec, b->stream), "graph launch");
    else if ((s = enqueue_eval(b)) != PLK_OK) return s;
    PLK_BCUDA(b, cudaEventRecord(b->ev[1], b->stream), "cudaEventRecord");
    PLK_BCUDA(b, cudaStreamSynchronize(b->stream), "batch evaluation");
    float ms = 0.0f;
    PLK_BCUDA(b, cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]), "cudaEventElapsedTime");
    b->last_ms[0] = ms;
    std::memcpy(lnl_out, b->h_lnl, b->items.size() * sizeof(double));
    for (size_t i = 0; i < b->items.size(); ++i)
        if (!std::isfinite(lnl_out[i])) return bfail(b, PLK_ERR_NUMERIC, "a log-likelihood is not finite");
    return PLK_OK;
}

plk_status plk_batch_tuning(const plk_batch* b, int* spt, int* grid, double* ms, int* uses_graph) {
    if (!b) return PLK_ERR_ARG;
    if (spt) *spt = b->form.spt;
    if (grid) *grid = b->grid;
    if (ms) *ms = b->tuned_ms;
    if (uses_graph) *uses_graph = b->exec != nullptr;
    return PLK_OK;
}

plk_status plk_batch_form(const plk_batch* b, int* paired, int* codes_smem) {
    if (!b) return PLK_ERR_ARG;
    if (paired) *paired = b->form.paired ? 1 : 0;
    if (codes_smem) *codes_smem = b->form.codes_smem ? 1 : 0;
    return PLK_OK;
}

plk_status plk_batch_features(plk_batch* b, float* out) {
    if (!b || !out) return b ? bfail(b, PLK_ERR_ARG, "out is NULL") : PLK_ERR_ARG;
    PLK_BCUDA(b, cudaSetDevice(b->device), "cudaSetDevice");
    if (b->items.empty()) return bfail(b, PLK_ERR_STATE, "batch is empty");
    if (b->layout_dirty) {
        plk_status s = build_layout(b);
        if (s != PLK_OK) return s;
    }
    BBuf feat;
    const size_t n = b->items.size() * kNumFeatures;
    PLK_BCUDA(b, feat.ensure(n * sizeof(float)), "allocate features");
    PLK_BCUDA(b, launch_features(device_view(b, b->lnl_units), feat.as<float>(), b->stream), "features launch");
    PLK_BCUDA(b, cudaMemcpyAsync(out, feat.p, n * sizeof(float), cudaMemcpyDeviceToHost, b->stream), "download features");
    PLK_BCUDA(b, cudaStreamSynchronize(b->stream), "features");
    return PLK_OK;
}

}  // extern "C"

namespace {

// Sets the model of every item whose point(i) is not null from that GTR
// parameter vector (the plk_fit_gtr parameterisation, tree-length scale folded
// into the category rates), in parallel over items; in_domain[i] = 0 where the
// vector gives no valid model (that item's model is left unchanged).
template <class PointFn>
plk_status set_gtr_models(plk_batch* b, const double* freqs, PointFn point, std::vector<char>& in_domain) {
    const int n_items = (int)b->items.size();
    const int C = b->C;
    const int n_threads = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<plk_status> st(n_threads, PLK_OK);
    std::vector<std::thread> pool;
    for (int t = 0; t < n_threads; ++t)
        pool.emplace_back([&, t]() {
            std::vector<double> Q(16), cr(C), cw(C);
            for (int i = t; i < n_items; i += n_threads) {
                const double* x = point(i);
                if (!x) continue;
                double scale = 1.0;
                in_domain[i] = gtr_model_from_x(4, x, C, freqs + (size_t)i * 4, Q.data(), cr.data(), cw.data(), &scale);
                if (!in_domain[i]) continue;
                for (int k = 0; k < C; ++k) cr[k] *= scale;
                const plk_status s = plk_batch_set_model(b, i, Q.data(), freqs + (size_t)i * 4, cr.data(), cw.data());
                if (s != PLK_OK) st[t] = s;
            }
        });
    for (auto& th : pool) th.join();
    for (plk_status s : st)
        if (s != PLK_OK) return s;
    return PLK_OK;
}

struct FitOut {
    double* x;
    double* lnl;
    int* evals;
    int* rounds;
    const double* target;
    double target_tol;
    int* hits;
};

// Advances every item's optimiser (NelderMead or QuasiNewton) in lockstep:
// each round sets the model of the point every unfinished fit asks for and
// evaluates the whole batch once.
template <class Opt>
plk_status run_fits(plk_batch* b, const double* freqs, std::vector<Opt>& opts, const FitOut& out) {
    const int n_items = (int)b->items.size();
    const int C = b->C;
    const int np = gtr_n_params(4, C);
    std::vector<char> in_domain(n_items, 1);
    std::vector<double> lnl(n_items);
    // every item needs a model before the first evaluation
    for (int i = 0; i < n_items; ++i)
        if (!b->items[i].has_model) {
            std::vector<double> Q(16), cr(C), cw(C);
            double scale = 1.0;
            std::vector<double> zero(np, 0.0);
            gtr_model_from_x(4, zero.data(), C, freqs + (size_t)i * 4, Q.data(), cr.data(), cw.data(), &scale);
            plk_status s = plk_batch_set_model(b, i, Q.data(), freqs + (size_t)i * 4, cr.data(), cw.data());
            if (s != PLK_OK) return s;
        }
    int rounds = 0;
    std::vector<int> hit(n_items, -1);
    for (;;) {
        bool any = false;
        for (const auto& o : opts) any = any || !o.done();
        if (!any) break;
        plk_status s = set_gtr_models(
            b, freqs, [&](int i) { return opts[i].done() ? nullptr : opts[i].point().data(); }, in_domain);
        if (s != PLK_OK) return s;
        s = plk_batch_loglik(b, lnl.data());
        if (s != PLK_OK && s != PLK_ERR_NUMERIC) return s;
        ++rounds;
        for (int i = 0; i < n_items; ++i) {
            if (opts[i].done()) continue;
            const bool ok = in_domain[i] && std::isfinite(lnl[i]);
            opts[i].tell(ok ? -lnl[i] : HUGE_VAL);
            // first evaluation that comes within target_tol of the target
            if (out.target && hit[i] < 0 && ok && lnl[i] >= out.target[i] - out.target_tol) hit[i] = opts[i].evals();
        }
    }
    if (out.hits) std::copy(hit.begin(), hit.end(), out.hits);
    for (int i = 0; i < n_items; ++i) {
        const std::vector<double>& bx = opts[i].best_x();
        std::copy(bx.begin(), bx.end(), out.x + (size_t)i * np);
        out.lnl[i] = -opts[i].best_f();
        if (out.evals) out.evals[i] = opts[i].evals();
    }
    if (out.rounds) *out.rounds = rounds;
    return PLK_OK;
}

}  // namespace

extern "C" {

plk_status plk_batch_eval_gtr(plk_batch* b, const double* freqs, const double* x, double* lnl_out) {
    if (!b || !freqs || !x || !lnl_out) return b ? bfail(b, PLK_ERR_ARG, "bad arguments to plk_batch_eval_gtr") : PLK_ERR_ARG;
    const int n_items = (int)b->items.size();
    if (n_items == 0) return bfail(b, PLK_ERR_STATE, "batch is empty");
    const int np = gtr_n_params(4, b->C);
    std::vector<char> in_domain(n_items, 1);
    plk_status s = set_gtr_models(b, freqs, [&](int i) { return x + (size_t)i * np; }, in_domain);
    if (s != PLK_OK) return s;
    for (int i = 0; i < n_items; ++i)
        if (!in_domain[i] && !b->items[i].has_model)
            return bfail(b, PLK_ERR_ARG, "parameter vector of item " + std::to_string(i) + " gives no valid model");
    s = plk_batch_loglik(b, lnl_out);
    if (s != PLK_OK && s != PLK_ERR_NUMERIC) return s;
    for (int i = 0; i < n_items; ++i)
        if (!in_domain[i]) lnl_out[i] = -HUGE_VAL;
    return PLK_OK;
}

plk_status plk_batch_fit_gtr(plk_batch* b, const double* freqs, const double* x0, const double* step, double ftol,
                             double xtol, int max_evals, double* x_out, double* lnl_out, int* evals_out,
                             int* rounds_out, const double* target_lnl, double target_tol, int* hit_evals_out) {
    if (!b || !freqs || !x_out || !lnl_out || max_evals < 1)
        return b ? bfail(b, PLK_ERR_ARG, "bad arguments to plk_batch_fit_gtr") : PLK_ERR_ARG;
    const int n_items = (int)b->items.size();
    if (n_items == 0) return bfail(b, PLK_ERR_STATE, "batch is empty");
    const int np = gtr_n_params(4, b->C);
    std::vector<double> starts((size_t)n_items * np, 0.0), steps((size_t)n_items * np, 0.5);
    if (x0) std::copy(x0, x0 + (size_t)n_items * np, starts.begin());
    if (step) std::copy(step, step + (size_t)n_items * np, steps.begin());
    FitOut out{x_out, lnl_out, evals_out, rounds_out, target_lnl, target_tol, hit_evals_out};
    if (b->fit_method == PLK_FIT_QUASI_NEWTON || b->fit_method == PLK_FIT_NEWTON_START) {
        std::vector<QuasiNewton> opts;
        opts.reserve(n_items);
        for (int i = 0; i < n_items; ++i)
            opts.emplace_back(np, &starts[(size_t)i * np], &steps[(size_t)i * np], ftol, xtol, max_evals,
                              b->fit_method == PLK_FIT_NEWTON_START);
        return run_fits(b, freqs, opts, out);
    }
    std::vector<NelderMead> opts;
    opts.reserve(n_items);
    for (int i = 0; i < n_items; ++i)
        opts.emplace_back(np, &starts[(size_t)i * np], &steps[(size_t)i * np], ftol, xtol, max_evals);
    return run_fits(b, freqs, opts, out);
}

plk_status plk_batch_set_fit_method(plk_batch* b, int method) {
    if (!b) return PLK_ERR_ARG;
    if (method != PLK_FIT_NELDER_MEAD && method != PLK_FIT_QUASI_NEWTON && method != PLK_FIT_NEWTON_START)
        return bfail(b, PLK_ERR_ARG, "unknown fit method");
    b->fit_method = method;
    return PLK_OK;
}

plk_status plk_nni_moves_host(int n_nodes, const int* left, const int* right, int* moves_out, int* n_moves_out) {
    if (n_nodes < 3 || !left || !right || !n_moves_out) return report_error(PLK_ERR_ARG, "bad arguments to plk_nni_moves_host");
    int n_leaves = 0;
    for (int v = 0; v < n_nodes; ++v)
        if (left[v] < 0 && right[v] < 0) ++n_leaves;
    std::vector<int> post, rank;
    int root = -1;
    std::string err;
    if (!check_tree(n_leaves, n_nodes, left, right, &root, &post, &rank, &err)) return report_error(PLK_ERR_ARG, err);
    std::vector<double> bl(n_nodes, 0.0), B2;
    std::vector<int> L2, R2;
    ItemHost h;
    relabel_and_enumerate(n_leaves, n_nodes, left, right, bl.data(), rank, root, &h, &L2, &R2, &B2);
    *n_moves_out = (int)h.moves.size();
    if (moves_out) std::copy(h.move_report.begin(), h.move_report.end(), moves_out);
    return PLK_OK;
}

int plk_batch_nni_count(const plk_batch* b, int item) {
    if (!b || item < 0 || item >= (int)b->items.size()) return 0;
    return (int)b->items[item].moves.size();
}

plk_status plk_batch_nni_moves(const plk_batch* b, int item, int* moves) {
    if (!b || !moves || item < 0 || item >= (int)b->items.size()) return PLK_ERR_ARG;
    const std::vector<int>& r = b->items[item].move_report;
    std::copy(r.begin(), r.end(), moves);
    return PLK_OK;
}

plk_status plk_batch_nni_loglik(plk_batch* b, double* out) {
    if (!b || !out) return b ? bfail(b, PLK_ERR_ARG, "out is NULL") : PLK_ERR_ARG;
    plk_status s = prepare_layout(b);
    if (s != PLK_OK) return s;
    if (b->total_moves == 0) return PLK_OK;
    if (b->nni_units.spt != 1) {
        s = build_units(b, b->nni_units, 1, true);
        if (s != PLK_OK) return s;
    }
    // tip codes staged in shared memory or read from global, whichever lets
    // more CTAs share an SM; one persistent CTA per resident slot
    const size_t smem_staged = nni_smem_bytes(b->C, true, b->max_ops, b->max_tips, b->max_depth);
    const size_t smem_global = nni_smem_bytes(b->C, false, b->max_ops, b->max_tips, b->max_depth);
    if (smem_global > 227 * 1024) return bfail(b, PLK_ERR_UNSUPPORTED, "trees too large for NNI scoring");
    const int occ_staged = smem_staged <= 227 * 1024 ? nni_occupancy(b->C, true, smem_staged, false) : 0;
    const int occ_global = nni_occupancy(b->C, false, smem_global, false);
    const bool codes_smem = occ_staged >= occ_global && occ_staged > 0;
    const size_t smem = codes_smem ? smem_staged : smem_global;
    const int per_sm = std::max(1, codes_smem ? occ_staged : occ_global);
    const int grid = std::max(1, std::min(b->nni_units.n_units, per_sm * b->n_sms));
    const size_t slice = (size_t)b->max_int * kThreads;
    PLK_BCUDA(b, b->d_scr_D.ensure((size_t)grid * slice * b->C * sizeof(float4)), "allocate NNI scratch");
    PLK_BCUDA(b, b->d_scr_O.ensure((size_t)grid * slice * b->C * sizeof(float4)), "allocate NNI scratch");
    PLK_BCUDA(b, b->d_scr_ED.ensure((size_t)grid * slice * sizeof(int)), "allocate NNI scratch");
    PLK_BCUDA(b, b->d_scr_EO.ensure((size_t)grid * slice * sizeof(int)), "allocate NNI scratch");
    const BatchDev d = device_view(b, b->nni_units);
    const size_t mn = b->items.size() * batch_model_stride(b->C);
    plk_status se = batch_events(b, 1);
    if (se != PLK_OK) return se;
    PLK_BCUDA(b, cudaEventRecord(b->ev[2], b->stream), "cudaEventRecord");
    PLK_BCUDA(b, cudaMemsetAsync(b->d_counter.p, 0, sizeof(int), b->stream), "clear work queue");
    PLK_BCUDA(b, cudaMemcpyAsync(b->d_model.p, b->h_model, mn * sizeof(double), cudaMemcpyHostToDevice, b->stream),
              "upload models");
    PLK_BCUDA(b, launch_batch_pmat(d, b->stream), "batch P(t) launch");
    PLK_BCUDA(b, launch_batch_nni(d, codes_smem, grid, smem, b->stream), "NNI kernel launch");
    PLK_BCUDA(b, launch_batch_nni_reduce(d, b->stream), "NNI reduce launch");
    PLK_BCUDA(b, cudaMemcpyAsync(b->h_lnl, b->d_nni_out.p, (size_t)b->total_moves * sizeof(double),
                                 cudaMemcpyDeviceToHost, b->stream),
              "download NNI lnL");
    PLK_BCUDA(b, cudaEventRecord(b->ev[3], b->stream), "cudaEventRecord");
    PLK_BCUDA(b, cudaStreamSynchronize(b->stream), "NNI scoring");
    float nms = 0.0f;
    PLK_BCUDA(b, cudaEventElapsedTime(&nms, b->ev[2], b->ev[3]), "cudaEventElapsedTime");
    b->last_ms[1] = nms;
    std::memcpy(out, b->h_lnl, (size_t)b->total_moves * sizeof(double));
    return PLK_OK;
}

plk_status plk_batch_device_ms(const plk_batch* b, double* loglik_ms, double* nni_ms) {
    if (!b) return PLK_ERR_ARG;
    if (loglik_ms) *loglik_ms = b->last_ms[0];
    if (nni_ms) *nni_ms = b->last_ms[1];
    return PLK_OK;
}

}  // extern "C"

namespace {

// d lnL / dt and d2 lnL / dt2 of every edge slot of every item into deriv
// ([slot][2], item after item; item i's slots start at item_edge_off[i]).
plk_status blen_pass(plk_batch* b, std::vector<double>& deriv, std::vector<int>& item_edge_off) {
    const int n_items = (int)b->items.size();
    if (n_items == 0) return bfail(b, PLK_ERR_STATE, "batch is empty");
    for (const auto& it : b->items)
        if (!it.has_model) return bfail(b, PLK_ERR_STATE, "every item needs a model (plk_batch_set_model)");
    plk_status s = prepare_layout(b);
    if (s != PLK_OK) return s;
    if (b->nni_units.spt != 1) {
        s = build_units(b, b->nni_units, 1, true);
        if (s != PLK_OK) return s;
    }
    // as for NNI scoring: staged or global tip codes by resident CTAs per SM
    const size_t smem_staged = nni_smem_bytes(b->C, true, b->max_ops, b->max_tips, b->max_depth);
    const size_t smem_global = nni_smem_bytes(b->C, false, b->max_ops, b->max_tips, b->max_depth);
    if (smem_global > 227 * 1024) return bfail(b, PLK_ERR_UNSUPPORTED, "trees too large for branch-length derivatives");
    const int occ_staged = smem_staged <= 227 * 1024 ? nni_occupancy(b->C, true, smem_staged, true) : 0;
    const int occ_global = nni_occupancy(b->C, false, smem_global, true);
    const bool codes_smem = occ_staged >= occ_global && occ_staged > 0;
    const size_t smem = codes_smem ? smem_staged : smem_global;
    const int per_sm = std::max(1, codes_smem ? occ_staged : occ_global);
    const int grid = std::max(1, std::min(b->nni_units.n_units, per_sm * b->n_sms));
    const size_t slice = (size_t)b->max_int * kThreads;
    PLK_BCUDA(b, b->d_scr_D.ensure((size_t)grid * slice * b->C * sizeof(float4)), "allocate scratch");
    PLK_BCUDA(b, b->d_scr_O.ensure((size_t)grid * slice * b->C * sizeof(float4)), "allocate scratch");
    PLK_BCUDA(b, b->d_scr_ED.ensure((size_t)grid * slice * sizeof(int)), "allocate scratch");
    PLK_BCUDA(b, b->d_scr_EO.ensure((size_t)grid * slice * sizeof(int)), "allocate scratch");
    // edge slots: 2 per internal node of every item, per unit and per item
    item_edge_off.assign(n_items, 0);
    std::vector<int> edge_item;
    int total_slots = 0;
    for (int i = 0; i < n_items; ++i) {
        item_edge_off[i] = total_slots;
        total_slots += 2 * b->items[i].n_int;
        edge_item.insert(edge_item.end(), 2 * b->items[i].n_int, i);
    }
    const std::vector<int2>& units = b->nni_units.host_units;
    std::vector<long long> unit_edge_off(units.size());
    long long unit_slots = 0;
    for (size_t u = 0; u < units.size(); ++u) {
        unit_edge_off[u] = unit_slots;
        unit_slots += 2 * b->items[units[u].x].n_int;
    }
    PLK_BCUDA(b, b->d_blen_ueo.ensure(unit_edge_off.size() * sizeof(long long)), "allocate edge slots");
    PLK_BCUDA(b, b->d_blen_ues.ensure((size_t)unit_slots * 2 * sizeof(double)), "allocate edge slots");
    PLK_BCUDA(b, b->d_blen_ieo.ensure(item_edge_off.size() * sizeof(int)), "allocate edge slots");
    PLK_BCUDA(b, b->d_blen_ei.ensure(edge_item.size() * sizeof(int)), "allocate edge slots");
    PLK_BCUDA(b, b->d_blen_out.ensure((size_t)total_slots * 2 * sizeof(double)), "allocate edge slots");
    PLK_BCUDA(b, cudaMemcpyAsync(b->d_blen_ueo.p, unit_edge_off.data(), unit_edge_off.size() * sizeof(long long),
                                 cudaMemcpyHostToDevice, b->stream), "upload edge slots");
    PLK_BCUDA(b, cudaMemcpyAsync(b->d_blen_ieo.p, item_edge_off.data(), item_edge_off.size() * sizeof(int),
                                 cudaMemcpyHostToDevice, b->stream), "upload edge slots");
    PLK_BCUDA(b, cudaMemcpyAsync(b->d_blen_ei.p, edge_item.data(), edge_item.size() * sizeof(int),
                                 cudaMemcpyHostToDevice, b->stream), "upload edge slots");
    BlenDev bd{b->d_blen_ueo.as<long long>(), b->d_blen_ues.as<double>(), b->d_blen_ieo.as<int>(),
               b->d_blen_ei.as<int>(), total_slots, b->d_blen_out.as<double>()};
    deriv.assign((size_t)total_slots * 2, 0.0);
    const BatchDev d = device_view(b, b->nni_units);
    const size_t mn = (size_t)n_items * batch_model_stride(b->C);
    PLK_BCUDA(b, cudaMemsetAsync(b->d_counter.p, 0, sizeof(int), b->stream), "clear work queue");
    PLK_BCUDA(b, cudaMemcpyAsync(b->d_model.p, b->h_model, mn * sizeof(double), cudaMemcpyHostToDevice, b->stream),
              "upload models");
    PLK_BCUDA(b, launch_batch_pmat(d, b->stream), "batch P(t) launch");
    PLK_BCUDA(b, launch_batch_blen(d, bd, codes_smem, grid, smem, b->stream), "branch-length kernel launch");
    PLK_BCUDA(b, launch_batch_blen_reduce(d, bd, b->stream), "branch-length reduce launch");
    PLK_BCUDA(b, cudaMemcpyAsync(deriv.data(), b->d_blen_out.p, deriv.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                 b->stream), "download derivatives");
    PLK_BCUDA(b, cudaStreamSynchronize(b->stream), "branch-length derivatives");
    return PLK_OK;
}

// the lengths as the kernels see them, packed in layout order
plk_status upload_lengths(plk_batch* b) {
    std::vector<double> teff;
    teff.reserve(b->n_nodes_total);
    for (const auto& it : b->items) teff.insert(teff.end(), it.t_eff.begin(), it.t_eff.end());
    PLK_BCUDA(b, cudaMemcpyAsync(b->d_teff.p, teff.data(), teff.size() * sizeof(double), cudaMemcpyHostToDevice,
                                 b->stream), "upload lengths");
    PLK_BCUDA(b, cudaStreamSynchronize(b->stream), "upload lengths");
    return PLK_OK;
}

}  // namespace

extern "C" {

plk_status plk_batch_edge_derivatives(plk_batch* b, double* out) {
    if (!b || !out) return b ? bfail(b, PLK_ERR_ARG, "out is NULL") : PLK_ERR_ARG;
    std::vector<double> deriv;
    std::vector<int> ieo;
    plk_status s = blen_pass(b, deriv, ieo);
    if (s != PLK_OK) return s;
    size_t off = 0;
    for (size_t i = 0; i < b->items.size(); ++i) {
        const ItemHost& h = b->items[i];
        for (int v = 0; v < 2 * h.n_nodes; ++v) out[off + v] = 0.0;
        for (int slot = 0; slot < 2 * h.n_int; ++slot) {
            const int2 ch = h.child[h.n_tips + slot / 2];
            const int v = (slot % 2 == 0) ? ch.x : ch.y;
            if (v < 0) continue;
            out[off + 2 * h.caller_id[v]] = deriv[2 * (ieo[i] + slot)];
            out[off + 2 * h.caller_id[v] + 1] = deriv[2 * (ieo[i] + slot) + 1];
        }
        off += 2 * (size_t)h.n_nodes;
    }
    return PLK_OK;
}

plk_status plk_batch_optimize_branches(plk_batch* b, int max_iter, double tol, double* lnl_out, int* iters_out) {
    if (!b || max_iter < 1 || !(tol > 0.0)) return b ? bfail(b, PLK_ERR_ARG, "bad arguments to plk_batch_optimize_branches") : PLK_ERR_ARG;
    const int n_items = (int)b->items.size();
    if (n_items == 0) return bfail(b, PLK_ERR_STATE, "batch is empty");
    std::vector<double> cur(n_items), trial(n_items), deriv;
    std::vector<int> item_edge_off;
    plk_status s = plk_batch_loglik(b, cur.data());
    if (s != PLK_OK) return s;
    std::vector<char> done(n_items, 0);
    int it_n = 0;
    const double t_min = 1e-8, t_max = 20.0;
    for (; it_n < max_iter; ++it_n) {
        bool any = false;
        for (char d : done) any = any || !d;
        if (!any) break;
        if ((s = blen_pass(b, deriv, item_edge_off)) != PLK_OK) return s;
        // one Newton step per edge (all edges of an item at once), halved
        // until the item's lnL does not drop.  An item has converged when the
        // quadratic model predicts less than tol of gain from another step:
        // sum over its free edges of g^2 / (2 |c|) (an edge in a convex
        // direction counts as not converged; an edge held at a bound by its
        // slope does not count).
        std::vector<std::vector<double>> old(n_items), step(n_items);
        for (int i = 0; i < n_items; ++i) {
            ItemHost& h = b->items[i];
            old[i] = h.t_eff;
            step[i].assign(h.n_nodes, 0.0);
            if (done[i]) continue;
            double predicted = 0.0;
            for (int slot = 0; slot < 2 * h.n_int; ++slot) {
                const int2 ch = h.child[h.n_tips + slot / 2];
                const int v = (slot % 2 == 0) ? ch.x : ch.y;
                if (v < 0) continue;
                // the two root edges act through their sum (reversible model,
                // root weights = frequencies): only the first one moves
                if (slot / 2 == h.n_int - 1 && slot % 2 == 1) continue;
                const double g = deriv[2 * (item_edge_off[i] + slot)], c = deriv[2 * (item_edge_off[i] + slot) + 1];
                const double t = h.t_eff[v];
                const bool held = (t <= t_min * 1.000001 && g <= 0.0) || (t >= t_max * 0.999999 && g >= 0.0);
                if (!held) predicted += c < 0.0 ? g * g / (-2.0 * c) : HUGE_VAL;
                double tn;
                if (c < 0.0) tn = t - g / c;                 // Newton on a concave direction
                else tn = g > 0.0 ? 2.0 * t + 1e-3 : 0.5 * t;  // otherwise move along the slope
                tn = std::min(std::max(tn, std::max(t_min, 0.1 * t)), std::min(t_max, 10.0 * t + 0.05));
                step[i][v] = tn - t;
            }
            if (predicted < tol) {
                done[i] = 1;
                step[i].assign(h.n_nodes, 0.0);
            }
        }
        {
            bool any = false;
            for (char d : done) any = any || !d;
            if (!any) break;
        }
        std::vector<char> accepted(n_items, 0);
        for (int half = 0; half < 6; ++half) {
            for (int i = 0; i < n_items; ++i) {
                if (done[i] || accepted[i]) continue;
                const double f = std::ldexp(1.0, -half);
                for (int v = 0; v < b->items[i].n_nodes; ++v) b->items[i].t_eff[v] = old[i][v] + f * step[i][v];
            }
            if ((s = upload_lengths(b)) != PLK_OK) return s;
            s = plk_batch_loglik(b, trial.data());
            if (s != PLK_OK && s != PLK_ERR_NUMERIC) return s;
            bool pending = false;
            for (int i = 0; i < n_items; ++i) {
                if (done[i] || accepted[i]) continue;
                if (std::isfinite(trial[i]) && trial[i] >= cur[i] - 1e-12 * std::fabs(cur[i])) accepted[i] = 1;
                else pending = true;
            }
            if (!pending) break;
        }
        for (int i = 0; i < n_items; ++i) {
            if (done[i]) continue;
            if (!accepted[i]) {  // no step helps: keep the old lengths, the item has converged
                b->items[i].t_eff = old[i];
                done[i] = 1;
                continue;
            }
            cur[i] = trial[i];
        }
        if ((s = upload_lengths(b)) != PLK_OK) return s;
    }
    if (lnl_out) std::copy(cur.begin(), cur.end(), lnl_out);
    if (iters_out) *iters_out = it_n;
    return PLK_OK;
}

plk_status plk_batch_branch_lengths(const plk_batch* b, int item, double* bl_out) {
    if (!b || !bl_out || item < 0 || item >= (int)b->items.size()) return PLK_ERR_ARG;
    const ItemHost& h = b->items[item];
    for (int v = 0; v < h.n_nodes; ++v) bl_out[h.caller_id[v]] = h.t_eff[v];
    return PLK_OK;
}

}  // extern "C"
