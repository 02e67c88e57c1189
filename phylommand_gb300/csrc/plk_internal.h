// Internal declarations shared by the host code (plk_api.cpp, plk_host.cpp)
// and the device code (plk_kernels.cu) of libplk.
#pragma once

#include <cmath>
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/plk.h"

namespace plk {

constexpr int kMaxStates = 24;   // bitset<SIZE=24> in the reference (src/constants.h:25)
constexpr int kMaxCats = 16;
constexpr int kMaxCodes = 256;   // distinct tip state-sets per alignment (1 byte per cell)

// Source of one child vector in a post-order op.
constexpr int kSrcAcc = -1;    // the previous op's result, still in registers
constexpr int kSrcPop = -2;    // popped from the per-thread spill stack
constexpr int kSrcNone = -3;   // no second child (unary node)

// One internal node of the post-order program.  A thread walks the ops in
// order for its site(s); s0/s1 >= 0 name a tip (its id), else kSrc*.
// e0/e1 are the child node ids whose edge P(t) applies.
struct Op {
    int node;   // node id
    int rank;   // post-order rank (left subtree, right subtree, node)
    int e0, e1; // child ids (e1 = -1 for a unary node)
    int s0, s1; // sources of the two child vectors
    int push;   // 1: push the result onto the spill stack
    int pad;
};
static_assert(sizeof(Op) == 32, "Op is 32 bytes");

// Post-order program: ops plus the deepest spill stack it needs.
struct Program {
    std::vector<Op> ops;
    int max_depth = 0;
};

// Records msg as the handle-less error (plk_last_error(NULL)) and returns s.
plk_status report_error(plk_status s, const std::string& msg);

// ---- host model math (plk_host.cpp) --------------------------------------
unsigned rate_pos(unsigned n, bool tr, unsigned row, unsigned col);
void q_matrix(int n, bool tr, const unsigned* spec, const double* rates, const double* freqs,
              double* Q);
// Symmetric eigendecomposition by cyclic Jacobi rotations: A = V diag(w) V^T.
void jacobi_eigen(int n, const double* A, double* w, double* V);
// Eigen system of a reversible Q with weights pi: Q = L diag(lam) R with
// L = D^-1/2 V, R = V^T D^1/2 (D = diag(pi)).
bool reversible_eigen(int n, const double* Q, const double* pi, double* lam, double* L,
                      double* R);
void pmat_taylor20_host(int n, const double* Q, double t, double* P);
void pmat_series_host(int n, const double* Q, double t, double* P);
void discrete_gamma(double alpha, int K, double* rates);
// Effective branch lengths (rate_model over the tree, src/rate_model.cpp:103-127).
void effective_lengths(int n_nodes, const int* left, const int* right, int root,
                       const double* bl, bool root_quirk, const std::vector<float>& cut_off,
                       const std::vector<float>& cut_rate, const std::vector<int>& clade_of_node,
                       const std::vector<float>& clade_rate, double* t_eff);
// Checks the tree; fills root, internal post-order and rank; message on error.
bool check_tree(int n_tips, int n_nodes, const int* left, const int* right, int* root,
                std::vector<int>* internal_postorder, std::vector<int>* rank, std::string* err);
// Register-allocated post-order program (Sethi-Ullman child order).
Program build_program(int n_tips, int n_nodes, const int* left, const int* right, int root,
                      const std::vector<int>& rank);

// ---- simulation (plk_sim.cpp) -------------------------------------------------
bool simulate_sites(int n_tips, int n_nodes, const int* left, const int* right, int root, const double* bl,
                    int S, const double* Q, const double* freqs, int n_cats, const double* cat_rates,
                    int n_sites, uint64_t seed, int n_threads, uint32_t* masks);

// ---- fitting (plk_fit.cpp) ---------------------------------------------------
// Nelder-Mead minimiser as a state machine: evaluate point(), report the
// objective with tell(), repeat until done().
class NelderMead {
  public:
    NelderMead(int n, const double* x0, double step, double ftol_abs, double xtol, int max_evals);
    // initial simplex x0 + steps[i] e_i (one step per coordinate)
    NelderMead(int n, const double* x0, const double* steps, double ftol_abs, double xtol, int max_evals);
    bool done() const { return state_ == State::Done; }
    bool converged_ok() const { return converged_; }
    const std::vector<double>& point() const { return point_; }
    void tell(double f);
    const std::vector<double>& best_x() const;
    double best_f() const;
    int evals() const { return evals_; }

  private:
    enum class State { Init, Reflect, Expand, ContractOut, ContractIn, Shrink, Done };
    void order();
    bool converged() const;
    void begin_iteration();
    void start_shrink();
    int n_;
    double ftol_, xtol_;
    int max_evals_;
    int evals_ = 0;
    bool converged_ = false;
    State state_;
    int init_i_ = 0, shrink_i_ = 0;
    std::vector<std::vector<double>> simplex_;
    std::vector<double> fvals_, point_, centroid_, xr_;
    double fr_ = 0.0;
};
// Quasi-Newton minimiser with central-difference gradients (step 1e-2): the
// first inverse Hessian is the inverse of the central differences' diagonal
// curvature, or with full_hessian of a finite-difference Hessian at the start
// (off-diagonal terms from n (n - 1) / 2 mixed differences; made positive
// definite); later ones BFGS updates; backtracking Armijo line search.  Same
// ask/tell interface as NelderMead.  Stops when an iteration lowers f by at most ftol_abs and moves
// every coordinate by at most xtol, after three iterations in a row that
// lower f by at most ftol_abs, when the line search fails, or at max_evals.
class QuasiNewton {
  public:
    QuasiNewton(int n, const double* x0, const double* steps, double ftol_abs, double xtol, int max_evals,
                bool full_hessian);
    bool done() const { return state_ == State::Done; }
    const std::vector<double>& point() const { return point_; }
    void tell(double f);
    const std::vector<double>& best_x() const { return x_; }
    double best_f() const { return f_; }
    int evals() const { return evals_; }

  private:
    enum class State { Start, Grad, Hess, Line, Done };
    void start_gradient();
    void next_grad_point();
    void finish_gradient();
    void next_hess_point();
    void finish_hessian();
    void start_line();
    std::vector<double> hmix_;  // forward mixed differences f(x + h e_i + h e_j), i < j
    std::vector<std::pair<int, int>> pairs_;
    std::vector<double> curv_;  // central-difference curvature of the first gradient
    int hi_ = 0;
    int n_;
    double ftol_, xtol_, h_;
    int max_evals_, evals_ = 0;
    State state_ = State::Start;
    std::vector<double> x_, g_, point_, fplus_, dir_, x_prev_, g_prev_, max_step_;
    std::vector<double> H_;  // inverse Hessian, row-major
    double f_ = HUGE_VAL, f_prev_ = HUGE_VAL, t_ = 1.0, slope_ = 0.0;
    int gi_ = 0, backtracks_ = 0, iter_ = 0, flat_ = 0;
    bool have_prev_ = false;
    bool full_hessian_ = false;
};
// GTR(+Gamma) parameters of the fits (see plk_fit.cpp); false outside the domain.
bool gtr_model_from_x(int S, const double* x, int n_cats, const double* freqs, double* Q, double* cat_rates,
                      double* cat_weights, double* scale);
int gtr_n_params(int S, int n_cats);

// ---- device launches (plk_kernels.cu) -------------------------------------
struct DeviceModel {
    int S, C, n_nodes, n_tips, n_codes;
    const double* t_eff;      // [n_nodes]
    const double* cat_rate;   // [C]
    const double* Q;          // [S*S]
    const double* eig_lam;    // [S]
    const double* eig_L;      // [S*S]
    const double* eig_R;      // [S*S]
    const uint32_t* code_mask;// [n_codes]
    double* P64;              // [n_nodes][C][S][S]
    float* P32;               // [n_nodes][C][S][S]
    double* tip64;            // [n_tips][C][n_codes][S]
    float* tip32;             // [n_tips][C][n_codes][S]
    // when set (4 states, C = 2, 4, 8): also the paired layouts prune4p_kernel
    // reads (plk_prune4p.cuh), so that no relayout launch is needed
    float* P32p;
    float* tip32p;
    // when set (20 states, the tcgen05 forms tuned): also their B-operand
    // images and [state][code] tip tables (plk_prune20u.cu), ncs20 codes per
    // row (n_codes rounded up to 4)
    float* B20;
    float* T20;
    int ncs20;
    int b20_bf16;  // B20 holds the split-BF16 images (the kind::f16 form) instead of split TF32
};
// p_kind: 0 taylor20, 1 eigen (reversible), 2 series (non-reversible)
cudaError_t launch_pmat(const DeviceModel& m, int p_kind, cudaStream_t st);
// unique id of the current CUDA context (0 when it cannot be had): launch
// set-up caches key on it, since a device reset resets kernel attributes
unsigned long long current_ctx_id();
// copies bytes (both addresses 16-byte aligned) from mapped pinned host
// memory with loads over the host link instead of a DMA copy
cudaError_t launch_arena_copy(void* dst, const void* src_mapped, size_t bytes, cudaStream_t st);
// the empty-cell check of byte masks copied in place as codes (the streamed
// alignment): *bad = gen when a cell of sites < n_sites allows no state
cudaError_t launch_check_codes(const uint8_t* codes, int n_tips, int n_sites, int stride, uint32_t all, int* bad,
                               int gen, cudaStream_t st);

struct PruneArgs {
    const Op* ops;
    int n_ops;
    int max_depth;
    const uint8_t* codes;      // [n_tips][site_stride]
    int site_stride;
    int n_sites;
    int n_codes;
    int C;
    const void* P;             // T [n_nodes][C][S][S]
    const void* tipT;          // T [n_tips][C][n_codes][S]
    const double* root_w;      // [S]
    const double* cat_w;       // [C]
    double* site_lnl;          // [n_sites]
    double* block_sum;         // [2 * n_blocks] (sum, compensation)
    void* cond;                // T [n_int][C][n_sites][S] or null
    void* work;                // T scratch of the generic kernel [n_int][C][n_sites][S]
    // topology for the generic kernel (device arrays)
    const int* order;          // internal nodes in post-order [n_int]
    const int* left;           // [n_nodes]
    const int* right;          // [n_nodes]
    const int* rank;           // [n_nodes], -1 for tips
    int n_int;
    int n_tips;
    // FP32 kernel choice (picked by the autotuner).  4 states: 0 =
    // prune4_kernel, 1/2 = prune4s_kernel with 1/2 sites per thread, 3/4 =
    // prune4p_kernel (category pairs on FP32x2) with 1/2 sites per thread,
    // 5/6 = the same reading the tip codes from global memory, 7/8 =
    // prune4p_kernel with two threads per site (codes from global memory /
    // staged in shared memory), 9 = prune4p_bulk_kernel (TMA-fed stage ring),
    // 10/11 = prune4p_kernel with 1/2 sites per thread and each op's tip
    // codes staged with its tables, 12/13/14 = prune4w_kernel (warp-
    // independent, nothing staged) with 1/2/4 sites per thread, 15/16/17 =
    // the same with 1/2/4 sites per thread and the tables in shared memory,
    // 18 = two sites per thread pair, each thread half of the pairs.
    // 20 states: 0 = prune_generic_kernel, 1 / 2 = prune20_kernel on CUDA
    // cores / mma.sync tensor cores (TF32, three-product split) with 4 warps
    // per tile, 3 / 4 = the same with 8 warps, 5 = prune20u_kernel on
    // tcgen05 tensor cores (TMEM accumulators), 6 = its compact form
    // prune20v_kernel (three CTAs per SM), 7 = prune20v_kernel with split
    // BF16 products (kind::f16, FP32 accumulate).
    int variant;
    int n_nodes;
    void* scratch;             // kernel-specific scratch (prune20_scratch_bytes)
    // The last CTA of the kernel that stores the block sums adds them up into
    // *lnl_out (finish_grid_sum), counting arrivals in *grid_done, which is
    // zero between launches; with grid_done null only the block sums and
    // per-site values are written.
    unsigned* grid_done;
    double* lnl_out;
    // one arrival counter per 128-site tile, zero between launches: with it
    // the 20-state compact form combines the categories of a tile in the
    // tile's last CTA (no combine launch)
    unsigned* tile_done;
    // the paired P(t) and tip layouts are already in scratch (written by the
    // P(t) kernel): prune4p skips its relayout
    int paired_ready;
    // test of the failure path (plk_test_withhold_stage): the TMA-fed form
    // never stages its first op, the shared-table form never copies its
    // tables, so their bounded waits run out
    int withhold_first_stage;
    // streamed tip codes (plk_set_alignment8, 4 states): the codes of sites
    // [c chunk_sites, (c + 1) chunk_sites) have landed once arrive[c] holds
    // arrive_gen.  The warp-independent forms wait for their tile's chunk
    // (bounded); null for every other launch, which runs after all chunks.
    const int* arrive;
    int arrive_gen;
    int chunk_sites;
};
// Fused 20-state FP32 kernels (plk_prune20.cu): mode 1 = CUDA cores, 2 =
// tensor cores.  Launches the relayout, the pass and the per-site combine
// (which also finishes the total); *n_blocks = the number of block sums.
bool prune20_fits(const PruneArgs& a, int mode);
size_t prune20_scratch_bytes(const PruneArgs& a, int n_nodes);
cudaError_t launch_prune20(const PruneArgs& a, int n_nodes, int mode, void* scratch, int* n_blocks,
                           cudaStream_t st);
// Per-site log(sum_k w_k L_k 2^e_k) from the FP32 category root sums and
// exponents ([C][n_sites] each), the block sums and the total.
cudaError_t launch_combine20(const float* cat_L, const int* cat_E, const PruneArgs& a, int* n_blocks,
                             cudaStream_t st);
// 20 states on tcgen05 tensor cores with TMEM accumulators (plk_prune20u.cu):
// the B-operand relayout, the pass and the per-site combine.  form 0 =
// prune20u_kernel (spill stack in TMEM, three-slot stage ring), 1 =
// prune20v_kernel (the compact form: three CTAs per SM, spills in global
// memory), 2 = prune20v_kernel with split-BF16 products (kind::f16).
bool prune20u_fits(const PruneArgs& a, int form);
// Where the B-operand images and the transposed tip tables sit in the
// scratch, and their row length (n_codes rounded up to 4).
void prune20u_scratch_parts(void* scratch, const PruneArgs& a, int n_nodes, float** B, float** T);
int prune20u_codes_padded(int n_codes);
size_t prune20u_scratch_bytes(const PruneArgs& a, int n_nodes);
cudaError_t launch_prune20u(const PruneArgs& a, int n_nodes, void* scratch, int form, int* n_blocks,
                            cudaStream_t st);
// Staged 4-state FP32 kernel with categories in pairs on the packed FP32x2
// pipe (plk_prune4p.cu), C = 2, 4 or 8; needs prune4p_scratch_bytes of
// a.scratch for the paired P(t) and tip tables.
bool prune4p_fits(const PruneArgs& a, int spt, int tps = 1);
// Where the paired P(t) and tip layouts sit in prune4p's scratch.
void prune4p_scratch_parts(void* scratch, int n_nodes, int C, float** Pp, float** Tp);
size_t prune4p_scratch_bytes(const PruneArgs& a);
// codes: 0 = the tile's tip codes staged in shared memory (global memory when
// they do not fit), 1 = read from global memory at their use, 2 = each op's
// codes staged with its tables (tps 1).  tps: threads per site, 0 = the
// TMA-fed form.
cudaError_t launch_prune4p(const PruneArgs& a, int spt, int codes, int tps, int* n_blocks, cudaStream_t st);
// The paired P(t) and tip layouts written from the P(t) kernel's FP32
// copies (when the P(t) kernel did not write them itself).
cudaError_t launch_relayout4p(const PruneArgs& a, float* Pp, float* Tp, cudaStream_t st);
// Warp-independent 4-state FP32 kernel (plk_prune4w.cu): every warp walks the
// op list over its own 32 x spt sites (spt = 1, 2, 4 sites per thread),
// reading the paired layouts of prune4p's scratch through L1, spills in
// tensor memory; C = 2, 4 or 8.
// ts = 1: the tree's tables copied into shared memory first (when they fit).
// tps = 2: two threads per site, each with half of the category pairs.
bool prune4w_fits(const PruneArgs& a, int spt, int ts = 0, int tps = 1);
cudaError_t launch_prune4w(const PruneArgs& a, int spt, int ts, int tps, int* n_blocks, cudaStream_t st);
// Staged 4-state FP32 kernel (plk_prune4s.cu): spt sites per thread.
bool prune4s_fits(const PruneArgs& a, int spt);
cudaError_t launch_prune4s(const PruneArgs& a, int spt, int* n_blocks, cudaStream_t st);
// Chooses the kernel for (S, C, precision); returns the number of blocks used
// for the partial sums in *n_blocks.
cudaError_t launch_prune(const PruneArgs& a, int S, int precision, bool store, int* n_blocks,
                         cudaStream_t st);
// *out = compensated sum_i w[i] x[i] (one CTA)
cudaError_t launch_weighted_sum(const double* x, const double* w, int n, double* out, cudaStream_t st);
// codes[t * stride + s] = masks[t * n_sites + s] & all (alphabets of <= 4
// states; masks of elem_bytes 4 or 1), padding bytes 0; *bad |= 1 if a cell
// allows no state.
cudaError_t launch_encode_small(const void* masks, int elem_bytes, int n_tips, int n_sites, int stride, uint32_t all,
                                uint8_t* codes, int* bad, int gen, cudaStream_t st);
// Row stride of the tip-code matrix: n_sites rounded up to 16 bytes.
inline int code_stride(int n_sites) { return (n_sites + 15) & ~15; }

struct PreorderArgs {
    const int* order;   // internal nodes in post-order [n_int]
    const int* left;
    const int* right;
    const int* rank;    // [n_nodes], -1 for tips
    int n_int, n_tips, n_sites, n_codes, S, C;
    const uint8_t* codes;
    int site_stride;
    const void* P;
    const void* tipT;
    const double* root_w;
    const double* cat_w;
    const void* cond;   // T [n_int][C][n_sites][S]
    void* outside;      // T [n_int][C][n_sites][S]
    double* out;        // [n_int][n_sites][S] normalised
};
cudaError_t launch_preorder(const PreorderArgs& a, int precision, cudaStream_t st);
cudaError_t launch_cond_normalise(const void* cond, const double* cat_w, int n_int, int C,
                                  int n_sites, int S, int precision, double* out,
                                  cudaStream_t st);

}  // namespace plk
