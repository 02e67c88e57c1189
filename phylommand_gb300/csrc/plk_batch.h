// Device-side layout of a batch (plk_batch.cu, plk_nni.cu, plk_batch_api.cpp).
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#include "plk_internal.h"

namespace plk {

// One alignment + tree + model of a batch; offsets into the concatenated
// device arrays.  Internal nodes are numbered n_tips + post-order rank.
struct BatchItemDev {
    long long codes_off;  // bytes into codes ([n_tips][site_stride])
    int ops_off, n_ops;   // into ops
    int node_off;         // into t_eff, child and P32 ([node_off + v][C][16])
    int tip_off;          // into tip32 ([tip_off + t][C][16][4])
    int n_tips, n_sites, site_stride;
    int model_off;        // doubles into model: lam[4] L[16] R[16] root_w[4] cat_rate[C] cat_w[C]
    int moves_off, n_moves;  // into moves (NNI rearrangements of this tree)
    int move_out_off;     // into the NNI output
    int n_int;            // internal nodes (the root is n_tips + n_int - 1)
    int pad[2];
};
static_assert(sizeof(BatchItemDev) == 64, "BatchItemDev is 64 bytes");

// One NNI rearrangement of an item's tree (local node ids).
//   kind 0: parent u is not the root; the new v' joins children x and y of the
//           old tree, and the new u' joins v' with z (u's outside vector stays).
//   kind 1: v and c are the root's children; v' joins x and y, c' joins p and q.
struct NniMoveDev {
    int kind, v, u, c;
    int x, y, z, p;
    int q, pad0, pad1, pad2;
};

struct BatchDev {
    int n_items, n_units, n_nodes_total, C;
    int max_depth, pad;
    const BatchItemDev* items;
    const uint8_t* codes;
    const Op* ops;
    const double* t_eff;      // [n_nodes_total]
    const int2* node_item;    // [n_nodes_total] (item, local node id)
    const int2* child;        // [n_nodes_total] (left, right) local ids, -1 = none
    const double* model;      // per item, see BatchItemDev::model_off
    float* P32;               // [n_nodes_total][C][16]
    float* tip32;             // [n_tips_total][C][16][4]
    float* P32p;              // paired layout of P32 (plk_prune4p.cuh), or null
    float* tip32p;            // paired layout of tip32, or null
    int write_std, pad2;      // batch_pmat_kernel writes P32 / tip32 when non-zero
    const int2* units;        // [n_units] (item, tile index), largest trees first
    double* unit_sums;        // [n_units][2]
    const int* item_unit_ptr; // [n_items + 1]
    const int* item_units;    // units of each item in site order
    double* lnl;              // [n_items]
    int* counter;             // work-queue head, zeroed before each launch
    // NNI
    const NniMoveDev* moves;
    const long long* unit_move_off;  // [n_units] offset of each unit's per-move partials
    double* unit_move_sums;          // [sum over units of n_moves][2]: 16-byte SiteSum32 records (store_site_record)
    double* nni_out;                 // [sum over items of n_moves]
    const int* move_item;            // [total moves] item of each output move
    int total_moves, scratch_int;    // scratch_int: max internal nodes of any item
    float4* scr_D;                   // per CTA: [scratch_int][C][128]
    int* scr_ED;                     // per CTA: [scratch_int][128]
    float4* scr_O;
    int* scr_EO;
};

inline int batch_model_stride(int C) { return 40 + 2 * C; }

// One form of the batch post-order kernel: sites per thread, tip codes staged
// in shared memory or read from global, categories in pairs on the FP32x2
// pipe (C = 2, 4, 8; reads P32p / tip32p) or one at a time.
struct BatchForm {
    int spt = 1;
    bool codes_smem = false;
    bool paired = false;
};
bool batch_form_valid(int C, const BatchForm& f);
size_t batch_smem_bytes(int C, const BatchForm& f, int max_ops, int max_tips, int max_depth);
int batch_occupancy(int C, const BatchForm& f, size_t smem);
cudaError_t launch_batch_pmat(const BatchDev& b, cudaStream_t st);
cudaError_t launch_batch_prune(const BatchDev& b, const BatchForm& f, int grid, size_t smem, cudaStream_t st);
cudaError_t launch_batch_reduce(const BatchDev& b, cudaStream_t st);

// NNI scoring (plk_nni.cu): one tile per work unit, grid CTAs with their own
// scratch slices; then the per-(item, move) reduction.
size_t nni_smem_bytes(int C, bool codes_smem, int max_ops, int max_tips, int max_depth);
cudaError_t launch_batch_nni(const BatchDev& b, bool codes_smem, int grid, size_t smem, cudaStream_t st);
// resident CTAs per SM of the NNI (blen = false) or branch-length kernel
int nni_occupancy(int C, bool codes_smem, size_t smem, bool blen);
cudaError_t launch_batch_nni_reduce(const BatchDev& b, cudaStream_t st);

// Branch-length derivatives of every edge of every item (plk_nni.cu): per
// work unit the sums over its sites of d lnL / dt and d2 lnL / dt2 for each
// edge slot (slot i = child i % 2 of internal node n_tips + i / 2), then per
// item over its units in site order.  Same units, scratch and shared memory
// as the NNI kernel.
struct BlenDev {
    const long long* unit_edge_off;  // [n_units] first slot of each unit in unit_edge_sums
    double* unit_edge_sums;          // [slots][2]
    const int* item_edge_off;        // [n_items] first global slot of each item
    const int* edge_item;            // [total_slots]
    int total_slots;
    double* edge_out;                // [total_slots][2] (d1, d2)
};
cudaError_t launch_batch_blen(const BatchDev& b, const BlenDev& bd, bool codes_smem, int grid, size_t smem,
                              cudaStream_t st);
cudaError_t launch_batch_blen_reduce(const BatchDev& b, const BlenDev& bd, cudaStream_t st);

// Summary statistics of every item (plk_features.cu): out[n_items][43].
constexpr int kNumFeatures = 43;
cudaError_t launch_features(const BatchDev& b, float* out, cudaStream_t st);

}  // namespace plk
