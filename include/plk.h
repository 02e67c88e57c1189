/* plk.h — C ABI of the GB300 phylogenetic likelihood engine (libplk.so).
 *
 * The engine replaces the likelihood path of phylommand's treeator:
 *   simpleML::set_char            src/simpleML.h:41-57           -> plk_set_alignment
 *   tree::tree_file_parser result src/tree.cpp:69-237            -> plk_set_tree
 *   rate_model (time slices, clade rates)
 *                                 src/rate_model.cpp:103-127,
 *                                 src/rate_model.h:64-67         -> plk_set_rate_model
 *   sub_model Q / P(t)            src/sub_model.cpp:99-127,
 *                                 src/marth/marth.cpp:129-140    -> plk_q_matrix, plk_set_model
 *   simpleML::calculate_log_likelihood
 *                                 src/simpleML.h:58-90,
 *                                 src/simpleML.cpp:127-197       -> plk_loglik
 *   simpleML::get_log_likelihood_from_root
 *                                 src/simpleML.h:123-141         -> plk_loglik, plk_site_loglik
 *   simpleML::draw_normalized_likelihood_on_nodes
 *                                 src/simpleML.cpp:199-231       -> plk_node_states
 *   opt_function (the NLopt objective)
 *                                 src/treeator.cpp:1122-1129     -> plk_loglik per call
 *
 * Conventions
 *  - All arrays are caller-owned host memory, copied in on every plk_set_*;
 *    the handle owns every device buffer.  No device pointer escapes.
 *  - Every entry point returns a plk_status (0 = success, negative = error)
 *    and never throws; plk_last_error() gives the message of the last failure.
 *  - A handle is used from one host thread at a time (as the reference's
 *    simpleML object is); several handles may coexist, each on its own stream.
 *  - Tree: nodes 0..n_tips-1 are the tips, tip i being row i of the alignment;
 *    left[v] / right[v] are child ids or -1.  The root is the one node that is
 *    nobody's child.  branch_length[v] is the length of the edge above v.
 *    A node with one child follows the reference: its vector is the child's
 *    transported vector.
 *  - State sets: bit s of a mask means state s is allowed (the reference's
 *    bitset<24>); a gap or unknown is the all-states mask.
 */
#ifndef PLK_H
#define PLK_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PLK_API_VERSION 1

typedef struct plk_handle plk_handle;
typedef int plk_status;

/* status codes */
#define PLK_OK 0
#define PLK_ERR_ARG (-1)      /* bad argument (sizes, ids, values) */
#define PLK_ERR_ALLOC (-2)    /* device or host allocation failed */
#define PLK_ERR_CUDA (-3)     /* a CUDA call failed */
#define PLK_ERR_STATE (-4)    /* call order: e.g. plk_loglik before plk_set_tree */
#define PLK_ERR_TIMEOUT (-5)  /* a bounded device wait gave up */
#define PLK_ERR_NUMERIC (-6)  /* non-finite likelihood */
#define PLK_ERR_TIP (-7)      /* a tip cell allows no state (simpleML::check_nodes) */
#define PLK_ERR_NODEV (-8)    /* no CUDA device */
#define PLK_ERR_UNSUPPORTED (-9)

/* arithmetic of the partial vectors */
#define PLK_FP64 0   /* plain: FP64 partials, reference operation order */
#define PLK_FP32S 1  /* fast: FP32 partials, per-site power-of-two scaling,
                        FP64 P(t), scaler logs and compensated site sum */

/* construction of P(t) = exp(Q t) */
#define PLK_P_TAYLOR20 0 /* the reference's (I + Q t / 2^20)^(2^20),
                            src/marth/marth.cpp:129-140, same operation order */
#define PLK_P_EXACT 1    /* exp(Q t): eigendecomposition for a reversible Q
                            (FP64 Jacobi on the host, FP64 P on the device),
                            scaling and squaring for a non-reversible Q */

/* node-state outputs */
#define PLK_NODES_COND 0     /* per site, sum_k w_k L_k[s] / sum over s of the
                                post-order conditional vector (the intent of
                                simpleML::draw_normalized_likelihood_on_nodes) */
#define PLK_NODES_MARGINAL 1 /* per site, normalised marginal posterior from a
                                pre-order pass (absent in the reference) */

/* ---- handle ------------------------------------------------------------ */
/* Create a handle on CUDA device `device`. */
plk_status plk_create(plk_handle** out, int device);
/* Free the handle and every device buffer it owns.  NULL is accepted. */
void plk_destroy(plk_handle* h);
/* Message of the last failed call on h (or of the last failed plk_create
 * when h is NULL).  Valid until the next call on h. */
const char* plk_last_error(const plk_handle* h);
const char* plk_status_string(plk_status s);
int plk_api_version(void);

/* ---- inputs ------------------------------------------------------------ */
/* Alignment: masks[tip * n_sites + site], bit s = state s allowed;
 * 1 <= n_states <= 24 (the reference's bitset<SIZE=24>, src/constants.h:25).
 * Replaces simpleML::set_char for every (tip, site). */
plk_status plk_set_alignment(plk_handle* h, int n_tips, int n_sites, int n_states,
                             const uint32_t* masks);
/* The same with one byte per cell (bit s = state s allowed), for alphabets
 * of at most 8 states: a quarter of the host-to-device traffic.  For <= 4
 * states without site patterns the bytes go to the device as they are and are
 * encoded there; otherwise they are widened on the host first.  With 4 states
 * and at least 16,384 sites the bytes are the codes themselves: they are
 * copied in place in site chunks (PLK_STREAM_CHUNKS, default 2; 0 turns this
 * off) and the next FP32 evaluation starts while they land.  As with every
 * upload from pinned memory, the copy is asynchronous: keep the buffer
 * unchanged until the next evaluation has returned. */
plk_status plk_set_alignment8(plk_handle* h, int n_tips, int n_sites, int n_states,
                              const uint8_t* masks);

/* Site patterns (off by default, as the reference evaluates every site; its
 * unfinished MLtree.h declares n_patterns / char_per_pattern for this).  On:
 * the next plk_set_alignment keeps one column per distinct site pattern and
 * its count; the kernels evaluate patterns, plk_loglik sums pattern lnL x
 * count (compensated), plk_site_loglik and plk_node_states still return every
 * input site.  Changing the setting drops the current alignment. */
plk_status plk_set_patterns(plk_handle* h, int on);
/* Columns the kernels evaluate: the distinct patterns, or n_sites when off;
 * 0 before an alignment. */
int plk_n_patterns(const plk_handle* h);

/* Tree topology and raw branch lengths (see the conventions above). */
plk_status plk_set_tree(plk_handle* h, int n_nodes, const int* left, const int* right,
                        const double* branch_length);

/* Branch-length modifiers of rate_model (src/rate_model.cpp:103-127), applied
 * on the host to give the effective length of every edge as
 * simpleML::calculate_likelihood does (src/simpleML.cpp:127-184):
 *   t_eff(v) = time_mod(bl(v), (float)dist(parent)) * clade_rate(clade of parent)
 * root_quirk = 1 reproduces the reference exactly: the recursion starts at a
 * root distance of 0, so every edge whose parent lies at distance 0 (the two
 * root-child edges at least) gets length 0.  root_quirk = 0 gives every edge
 * its own length.  n_cut time slices: cut_off[i] (ascending), cut_rate[i].
 * clade_of_node[v] >= 0 marks v as MRCA of clade number clade_of_node[v]
 * (may be NULL); clade_rate[c] for c < n_clades.  Default after plk_set_tree:
 * root_quirk = 1, no slices, no clades. */
plk_status plk_set_rate_model(plk_handle* h, int root_quirk, int n_cut, const float* cut_off,
                              const float* cut_rate, const int* clade_of_node, int n_clades,
                              const float* clade_rate);

/* Substitution model.  Q is row-major n_states x n_states (rows sum to 0);
 * root_weights[s] weights the root vector (the frequencies for a reversible
 * model, all 1 for a non-reversible one, src/simpleML.h:128-135).  For
 * reversible = 1 and p_mode = PLK_P_EXACT, Q must satisfy
 * root_weights[i] Q[i][j] = root_weights[j] Q[j][i].  Rate categories: n_cats
 * rates r_k multiply every effective length; weights w_k mix the site
 * likelihoods.  n_cats = 1, r = w = 1 is the reference's model. */
plk_status plk_set_model(plk_handle* h, int n_states, const double* Q,
                         const double* root_weights, int reversible, int n_cats,
                         const double* cat_rates, const double* cat_weights, int p_mode);

/* ---- evaluation ---------------------------------------------------------- */
/* Total log-likelihood (sites summed with a compensated sum).  Builds P(t)
 * for every edge and category on the device, runs the post-order pass, and
 * reduces on the device; one device-to-host copy of 8 bytes. */
plk_status plk_loglik(plk_handle* h, int precision, double* lnl_out);
/* The fast form's log-likelihood with its error against the FP64 plain
 * form of the same inputs (which holds the reference's CPU value within
 * 1e-12): evaluates both, writes the FP32S value, the FP64 value, |delta lnL|
 * and |delta lnL| / |lnL FP64|.  Afterwards plk_site_loglik gives the fast
 * form's per-site values.  Replaces the error estimate of simpleML's
 * calculate_log_likelihood (src/simpleML.h:58-90), which has none: the
 * reference computes in FP64 only. */
plk_status plk_loglik_err(plk_handle* h, double* lnl_fast, double* lnl_fp64, double* abs_err, double* rel_err);
/* plk_loglik split in two: enqueue the whole evaluation on the handle's
 * stream without waiting, then fetch (waits for the stream).  Lets a caller
 * overlap host work with the device or queue evaluations back to back. */
plk_status plk_loglik_async(plk_handle* h, int precision);
plk_status plk_loglik_result(plk_handle* h, double* lnl_out);
/* Run the handle's work on an existing CUDA stream (a cudaStream_t passed as
 * void*); NULL returns to the handle's own stream. */
plk_status plk_set_stream(plk_handle* h, void* cuda_stream);
/* Kernel timing: with profiling on, every evaluation records CUDA events on
 * the handle's stream around its P(t) kernel, its post-order pass (whose last
 * CTA also adds up the total) and the site-pattern weighting (zero time
 * without site patterns).
 * plk_kernel_times waits for the stream and returns the summed milliseconds
 * of each phase (ms_out[3]) over the evaluations recorded since the last
 * reset, and their number. */
plk_status plk_set_profiling(plk_handle* h, int on);
plk_status plk_kernel_times(plk_handle* h, double* ms_out, int* n_evals, int reset);
/* The FP32 post-order kernel the autotuner chose for the current tree and
 * alignment.  4 states: 0 = prune4_kernel (partials in registers, P(t) from
 * global memory), 1 / 2 = prune4s_kernel with 1 / 2 sites per thread (P(t)
 * rows and tip tables staged in shared memory), 3 / 4 = prune4p_kernel (the
 * same with the categories in pairs on packed FP32x2), 5 / 6 = prune4p_kernel
 * reading the tip codes from global memory, 7 / 8 = prune4p_kernel with two
 * threads per site (each takes half of the category pairs; codes from global
 * memory / staged), 9 = prune4p_bulk_kernel (TMA-fed stage ring), 10 / 11 =
 * prune4p_kernel with 1 / 2 sites per thread and each op's tip codes staged
 * with its tables two ops ahead (the fast forms when the codes exceed L2),
 * 12 / 13 / 14 = prune4w_kernel (every warp walks the op list alone over its
 * own 32 x 1 / 2 / 4 sites, tables through L1, spill stack in TMEM), 15 / 16
 * / 17 = the same with the tree's tables in shared memory, 18 = two threads
 * per site pair with the tables in shared memory.  20 states: 1 / 2 =
 * prune20_kernel on CUDA cores / mma.sync tensor cores with 4 warps per tile,
 * 3 / 4 = the same with 8 warps, 5 = prune20u_kernel (tcgen05 tensor cores,
 * TMEM accumulators, spill stack in TMEM), 6 = prune20v_kernel (its compact
 * form: spills in global memory, split TF32), 7 = the compact form with
 * split-BF16 products (tcgen05 kind::f16, five CTAs per SM).  -1 = not tuned
 * yet or another kernel applies (FP64, other state counts, more than 8
 * categories). */
int plk_prune_variant(const plk_handle* h);
/* Test of the failure path: the next FP32 evaluation that runs one of the
 * mbarrier-driven post-order forms -- the TMA-fed 4-state form (candidate 9),
 * the shared-table warp-independent forms (15-18: their table copy), the
 * tcgen05 20-state forms (5-7: the first MMA commit) -- withholds the first
 * stage of every tile or CTA, so every bounded mbarrier wait of that launch
 * runs out; with a streamed alignment the warp-independent forms (12-18) wait
 * for an arrival no copy writes.  The tiles' sites come out NaN, the
 * evaluation fails with PLK_ERR_NUMERIC, and the handle stays usable.  No
 * effect on the other forms. */
plk_status plk_test_withhold_stage(plk_handle* h);
/* Per-site log-likelihoods of the last plk_loglik (n_sites doubles). */
plk_status plk_site_loglik(plk_handle* h, double* out);
/* Node-state output for every internal node: out[(rank * n_sites + site) *
 * n_states + s], internal nodes ranked in post-order (left subtree, right
 * subtree, node), the order draw_normalized_likelihood_on_nodes visits them. */
plk_status plk_node_states(plk_handle* h, int mode, int precision, double* out);
/* plk_node_states in the fast form (FP32S) into out, plus the largest
 * absolute difference from the FP64 plain form's node states over every
 * internal node, site and state (src/simpleML.cpp:199-231 prints FP64
 * values only). */
plk_status plk_node_states_err(plk_handle* h, int mode, double* out, double* max_abs_err);
/* Number of internal nodes of the current tree (rows of plk_node_states). */
int plk_n_internal(const plk_handle* h);

/* ---- maximum-likelihood fit ----------------------------------------------------
 * The likelihood calls of treeator's NLopt optimisation (opt_function,
 * src/treeator.cpp:1122-1129, maximised by LN_NELDERMEAD at
 * src/treeator.cpp:791-805), run inside the engine with its own Nelder-Mead
 * (Nelder & Mead 1965).  Fits a reversible GTR(+Gamma) model on the handle's
 * alignment and tree over
 *   x = (log exchangeabilities relative to the last one,
 *        log Gamma shape alpha  (only when n_cats > 1),
 *        log tree-length scale  (multiplies every branch length))
 * with fixed frequencies freqs[n_states] and Q normalised to mean rate 1.
 * x0 = NULL starts at x = 0 (all exchangeabilities 1, alpha 1, scale 1).  The
 * simplex starts at x0 + step * e_i; the fit stops when the spread of -lnL
 * over the simplex is <= ftol and every coordinate's extent is <= xtol, or
 * after max_evals evaluations.  x_out receives plk_fit_n_params values; the
 * handle keeps the fitted model. */
plk_status plk_fit_gtr(plk_handle* h, int precision, const double* freqs, int n_cats, const double* x0,
                       double step, double ftol, double xtol, int max_evals, double* x_out,
                       double* lnl_out, int* n_evals_out);
int plk_fit_n_params(int n_states, int n_cats);
/* Optimiser of plk_fit_gtr on this handle: PLK_FIT_NELDER_MEAD (default) or
 * PLK_FIT_QUASI_NEWTON (defined with the batch fit below). */
plk_status plk_set_fit_method(plk_handle* h, int method);

/* ---- batches: many alignments, trees and models in one launch -------------------
 * The reference scores one tree per simpleML object in treeator's loop over
 * the tree file (src/treeator.cpp:705-990), and maps sites to models through
 * partition_models (src/partition_models.h:30-165).  A batch holds many
 * 4-state alignments, each with its own tree and reversible model, and scores
 * all of them in one persistent launch (work units = site tiles of a tree,
 * largest trees first) replayed from a captured CUDA graph; an autotuner picks
 * the sites per thread and CTAs per SM on the batch itself.  FP32 partials
 * with per-site scaling, FP64 P(t) and sums; effective lengths are the raw
 * branch lengths (no root quirk); n_cats is fixed per batch (1..8). */
typedef struct plk_batch plk_batch;
plk_status plk_batch_create(plk_batch** out, int device, int n_cats);
void plk_batch_destroy(plk_batch* b);
const char* plk_batch_last_error(const plk_batch* b);
int plk_batch_n_items(const plk_batch* b);
/* Append an item: masks[n_tips * n_sites] (bits 0..3), tree as in plk_set_tree. */
plk_status plk_batch_add(plk_batch* b, int n_tips, int n_sites, const uint32_t* masks, int n_nodes,
                         const int* left, const int* right, const double* branch_length, int* item_out);
/* Model of one item: reversible Q (4 x 4) with frequencies freqs (the root
 * weights), category rates and weights (n_cats each; rates may carry a tree
 * scale).  Cheap: call it per optimiser step, then plk_batch_loglik. */
plk_status plk_batch_set_model(plk_batch* b, int item, const double* Q, const double* freqs,
                               const double* cat_rates, const double* cat_weights);
/* lnL of every item (n_items doubles), one graph replay. */
plk_status plk_batch_loglik(plk_batch* b, double* lnl_out);
/* Device time (CUDA events on the batch's stream) of the last
 * plk_batch_loglik (from the graph launch to its last copy) and of the last
 * plk_batch_nni_loglik (from its first upload to the download of the
 * scores), in ms; 0 before the first call.  A measurement helper with no
 * counterpart in the reference (treeator times nothing). */
plk_status plk_batch_device_ms(const plk_batch* b, double* loglik_ms, double* nni_ms);
/* The autotuner's choice: sites per thread, persistent grid size, ms of one
 * post-order launch, and whether evaluations replay a CUDA graph. */
plk_status plk_batch_tuning(const plk_batch* b, int* sites_per_thread, int* grid, double* ms,
                            int* uses_graph);
/* The autotuned form of the post-order kernel: paired = 1 when categories
 * go in pairs on the packed FP32x2 pipe (2, 4 or 8 categories; same per-site
 * bits as one at a time), codes_smem = 1 when each tile's tip codes are
 * staged in shared memory rather than read from global memory. */
plk_status plk_batch_form(const plk_batch* b, int* paired, int* codes_smem);

/* NNI neighbours of every item: the trees one nearest-neighbour interchange
 * away, with branch lengths kept on their edges -- what `treebender --nni`
 * writes out for treeator to re-score tree by tree (src/tree.cpp:2482-2548,
 * src/treebender.cpp:897-915), scored here without building the trees:
 * post-order messages, pre-order outside vectors, then each interchange from
 * the vectors around its edge.  A binary tree with n tips has 2(n - 3) moves.
 * plk_batch_nni_moves describes move m of an item as moves[2m] = node v (the
 * caller's id) and moves[2m+1] = which:
 *   0  swap right(v) with v's sibling          (parent of v not the root)
 *   1  swap left(v)  with v's sibling          (parent of v not the root)
 *   2  swap right(v) with left(c)              (v, c the root's children)
 *   3  swap right(v) with right(c)
 * plk_batch_nni_loglik writes, item after item, the lnL of every move. */
/* Summary statistics of every item (the warm-start network's inputs), 43
 * floats per item: base frequencies (4), mean pairwise proportions of the
 * substitution types A<->G, A<->C, A<->T, G<->C, G<->T, C<->T (6), histogram of
 * per-site collision entropy -ln(sum_s c_s (c_s - 1) / (m (m - 1))) (c_s the
 * counts of m unambiguous taxa) in 32 bins over [0, ln 4] (32), mean
 * p-distance (1).  Every statistic is a pairwise one, taken over at most 32
 * taxa (rows floor(q n / 32), q < 32), so none drifts with the number of
 * taxa. */
plk_status plk_batch_features(plk_batch* b, float* out);
/* Maximum-likelihood fits of every item at once: one Nelder-Mead per item
 * (the parameterisation of plk_fit_gtr: log exchangeabilities relative to the
 * last, log alpha, log tree-length scale; n_params = plk_fit_n_params(4,
 * n_cats)), advanced in lockstep so that each round evaluates every
 * unfinished fit's next point in one batch launch.  freqs[n_items][4] fixed;
 * x0[n_items][n_params] or NULL (all zero); step[n_items][n_params] initial
 * simplex steps (vertex i = x0 + step_i e_i) or NULL (all 0.5).  Outputs
 * per item: x_out, lnl_out, evals_out (may be
 * NULL); rounds_out = batch evaluations used.  Stopping rule of every fit:
 * the simplex's lnL spread <= ftol and its extent <= xtol in every
 * coordinate, or max_evals.  Optional: with target_lnl[n_items],
 * hit_evals_out[i] = the number of evaluations after which item i first
 * reached lnL >= target_lnl[i] - target_tol (-1 if never). */
plk_status plk_batch_fit_gtr(plk_batch* b, const double* freqs, const double* x0, const double* step,
                             double ftol, double xtol, int max_evals, double* x_out, double* lnl_out,
                             int* evals_out, int* rounds_out, const double* target_lnl,
                             double target_tol, int* hit_evals_out);
/* Optimiser of plk_batch_fit_gtr (and, with plk_set_fit_method, of
 * plk_fit_gtr).  PLK_FIT_NELDER_MEAD (default) is the counterpart of the
 * reference's NLopt LN_NELDERMEAD; PLK_FIT_QUASI_NEWTON is BFGS on
 * central-difference gradients (step 1e-2, 2 n evaluations per gradient; the
 * first inverse Hessian from their diagonal curvature); PLK_FIT_NEWTON_START
 * is the same with a full finite-difference Hessian at the start (n (n - 1)
 * / 2 more evaluations, so the first step is a Newton step).  Same stopping
 * tolerances (or three iterations in a row improving lnL by at most ftol). */
#define PLK_FIT_NELDER_MEAD 0
#define PLK_FIT_QUASI_NEWTON 1
#define PLK_FIT_NEWTON_START 2
plk_status plk_batch_set_fit_method(plk_batch* b, int method);
/* lnL of every item at the GTR parameter vector x[n_items][n_params] (the
 * parameterisation of plk_batch_fit_gtr) in one batch evaluation; the items
 * keep these models.  -HUGE_VAL where a vector gives no valid model. */
plk_status plk_batch_eval_gtr(plk_batch* b, const double* freqs, const double* x, double* lnl_out);

/* ---- warm-start network --------------------------------------------------------
 * No counterpart in the reference (its optimiser starts from fixed values,
 * src/treeator.cpp:612-615).  A fully connected network n_in -> n_hidden
 * (x n_hidden_layers, ReLU) -> n_out that maps plk_batch_features rows to a
 * starting point of plk_batch_fit_gtr.  BF16 weights and activations in the
 * tensor-core GEMMs, FP32 accumulation, FP32 master weights; trained with
 * Adam on the mean squared error.  Parameters are one flat FP32 vector: per
 * layer W[out][in] then b[out].  Weights start He-normal from `seed`. */
typedef struct plk_mlp plk_mlp;
plk_status plk_mlp_create(plk_mlp** out, int device, int n_in, int n_hidden, int n_hidden_layers,
                          int n_out, uint64_t seed);
void plk_mlp_destroy(plk_mlp* m);
const char* plk_mlp_last_error(const plk_mlp* m);
int plk_mlp_n_params(const plk_mlp* m);
plk_status plk_mlp_get_params(const plk_mlp* m, float* out);
plk_status plk_mlp_set_params(plk_mlp* m, const float* in);
/* y[batch][n_out] = network(x[batch][n_in]); host buffers. */
plk_status plk_mlp_forward(plk_mlp* m, int batch, const float* x, float* y);
/* Gradient of the loss (mean over batch x n_out of squared error against
 * t[batch][n_out]) into grad[n_params] (may be NULL); loss may be NULL. */
plk_status plk_mlp_gradients(plk_mlp* m, int batch, const float* x, const float* t, float* grad,
                             float* loss);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) at learning rate lr; loss before
 * the step into *loss (may be NULL). */
plk_status plk_mlp_train_step(plk_mlp* m, int batch, const float* x, const float* t, float lr,
                              float* loss);

/* ---- branch lengths (no counterpart in the reference: its branch lengths
 * are fixed inputs, src/tree.cpp:136, 176) ------------------------------------
 * First and second derivatives of every item's lnL with respect to the length
 * of the edge above every node, from one post-order and one pre-order pass
 * (P(t) = L diag(exp(lambda t)) R: the derivatives weight the same eigen
 * terms by lambda r and (lambda r)^2).  out: item after item, [n_nodes][2] in
 * the caller's node ids (d1, d2); the root's pair is 0. */
plk_status plk_batch_edge_derivatives(plk_batch* b, double* out);
/* Maximum-likelihood branch lengths of every item under its current model:
 * each iteration takes one Newton step on every edge of an item at once (a
 * step along the slope where the curvature is not negative; lengths within
 * [1e-8, 20], at most x10 per step; of the two root edges only the first
 * moves, their sum being what counts), halving the item's steps until its lnL
 * does not drop.  An item stops when the Newton model predicts less than tol
 * of lnL gain from another step (sum over its edges of d1^2 / (2 |d2|); edges
 * held at a length bound by their slope do not count), or when no halved
 * step keeps its lnL.
 * lnl_out[n_items] (may be NULL), iters_out = iterations run. */
plk_status plk_batch_optimize_branches(plk_batch* b, int max_iter, double tol, double* lnl_out, int* iters_out);
/* An item's current branch lengths in the caller's node ids. */
plk_status plk_batch_branch_lengths(const plk_batch* b, int item, double* bl_out);

int plk_batch_nni_count(const plk_batch* b, int item);
/* The same moves of one tree on the host (no device): *n_moves_out moves,
 * 2 ints each in moves_out (may be NULL to query the count). */
plk_status plk_nni_moves_host(int n_nodes, const int* left, const int* right, int* moves_out,
                              int* n_moves_out);
plk_status plk_batch_nni_moves(const plk_batch* b, int item, int* moves);
plk_status plk_batch_nni_loglik(plk_batch* b, double* lnl_out);

/* ---- simulation -------------------------------------------------------------
 * Seeded simulation of n_sites sites down a tree (the engine's counterpart of
 * simpleML::simulate_chars, src/simpleML.cpp:233-292, which draws from the
 * clock-seeded rand()): root state from freqs, then each edge from the row of
 * exp(Q * branch_length * r_k) of the parent's state, one of the n_cats rate
 * categories drawn uniformly per site.  Q must be reversible with freqs.
 * masks_out[tip * n_sites + site] = 1 << state.  Counter-based random numbers
 * keyed by (seed, site, node): the result does not depend on n_threads. */
plk_status plk_simulate(int n_nodes, const int* left, const int* right, const double* branch_length,
                        int n_states, const double* Q, const double* freqs, int n_cats,
                        const double* cat_rates, int n_sites, uint64_t seed, int n_threads,
                        uint32_t* masks_out);

/* ---- input formats (host only) ----------------------------------------------
 * Character matrix text -> state-set masks, restating the reference's
 * matrix_parser (src/matrix_parser.cpp:27-225): FASTA ('>' name lines; a
 * character outside the alphabet is an empty cell), relaxed PHYLIP ("n_taxa
 * n_char" header, a name up to the first blank then the cells of the line)
 * and the MATRIX of a NEXUS DATA block (ntax checked; in both, characters
 * outside the alphabet are skipped).  alphabet[256]: the state set of every
 * character, -1 outside the alphabet; NULL = the DNA alphabet with IUPAC
 * ambiguity codes in the order A, G, C, T ('-' and '.' empty).  Empty cells
 * (and the tails of short rows) come out as all states, as treeator sets them
 * (src/treeator.cpp:463-466).  Two calls: with masks_out / names_out NULL
 * only the sizes; then masks_out[n_taxa][n_sites] and the names,
 * NUL-terminated one after another, in names_out (names_cap bytes). */
#define PLK_FORMAT_FASTA 0
#define PLK_FORMAT_PHYLIP 1
#define PLK_FORMAT_NEXUS 2
plk_status plk_parse_alignment(const char* text, size_t len, int format, const int32_t* alphabet,
                               int* n_taxa_out, int* n_sites_out, uint32_t* masks_out, char* names_out,
                               size_t names_cap);
/* The first tree of Newick text -> the engine's node arrays, restating
 * tree::tree_file_parser (src/tree.cpp:69-237): comments in [], quoted
 * labels, branch lengths read as atof reads them, a node with a third child
 * resolved by a zero-length node over the first two.  Tips come first: tip i
 * is the taxon names[i] (n_taxa NUL-separated names, as plk_parse_alignment
 * returns them) or, with names NULL, the i-th tip in the text; internal nodes
 * follow in post-order.  Two calls: with left/right/bl NULL only
 * *n_nodes_out. */
plk_status plk_parse_newick(const char* text, size_t len, int n_taxa, const char* names, int* n_nodes_out,
                            int* left, int* right, double* bl);

/* ---- host helpers (FP64, no device work) ---------------------------------- */
/* Q as sub_model::calc_Q_matrix (src/sub_model.cpp:99-114): off-diagonal
 * Q[i][j] = rates[rate_spec[pos(i,j)]] * (reversible ? freq_j : 1), diagonal =
 * -row sum; pos as sub_model::get_rate_pos (src/sub_model.cpp:3-29): upper
 * triangle row-major for reversible models.  freqs holds n_states - 1 values
 * (the last is 1 - their sum, src/sub_model.cpp:44-53) or NULL for 1/n. */
plk_status plk_q_matrix(int n_states, int reversible, const unsigned* rate_spec,
                        const double* rates, const double* freqs, double* Q_out);
/* P(t) on the host with the engine's own FP64 code (either p_mode). */
plk_status plk_pmat_host(int n_states, const double* Q, const double* root_weights,
                         int reversible, double t, int p_mode, double* P_out);
/* Mean rates of K equal-probability categories of a mean-1 Gamma(alpha)
 * (Yang 1994). */
plk_status plk_discrete_gamma(double alpha, int K, double* rates_out);
/* Effective length of the edge above every node under a rate model, as
 * plk_set_rate_model defines it (the handle uses this same function).
 * clade_of_node may be NULL. */
plk_status plk_effective_lengths(int n_nodes, const int* left, const int* right,
                                 const double* branch_length, int root_quirk, int n_cut,
                                 const float* cut_off, const float* cut_rate,
                                 const int* clade_of_node, int n_clades, const float* clade_rate,
                                 double* t_eff_out);

/* ---- measurement helper -------------------------------------------------------
 * No counterpart in the reference (which has no GPU path).  Measures the FP32
 * multiply-add rate of `device`: every thread of a grid of 4 CTAs per SM runs
 * independent fma.rn.f32 chains (packed = 0) or fma.rn.f32x2 chains
 * (packed = 1), or fma.rn.f64 chains (packed = 2: the FP64 rate), for
 * `iters` iterations of 64 lane-FMAs, timed with CUDA events after a warm-up
 * launch.  Writes TFLOP/s (2 flops per lane-FMA) and the launch time in ms
 * (ms_out may be NULL).  1 <= iters <= 2^24.  The post-order passes' FP32
 * roofline, and the FP64 plain form's, are quoted against these numbers. */
plk_status plk_measure_fp32_peak(int device, int packed, int iters, double* tflops_out, double* ms_out);

/* ---- allocation-free entry point ----------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory when they need the result -- work recorded into a CUDA stream
 * capture (cudaMalloc cannot be captured), programs whose device memory is
 * owned by another allocator, or callers that cannot afford cudaMalloc /
 * cudaFree synchronising the device.
 *
 * Compensated (TwoSum) sum of n_sites per-site log-likelihoods in device
 * memory (d_site_lnl), written to one double in device memory (d_lnl_out), on
 * cuda_stream (a cudaStream_t as void*, NULL = default stream), asynchronously.
 * Allocates nothing: its block partial sums live in a 64 KiB file-scope device
 * array that every GPU loading the library keeps until exit.
 *  - 1 <= n_sites <= 1,048,576; anything else returns PLK_ERR_ARG with a
 *    message in plk_last_error(NULL).
 *  - The first call on a device (that device current) resolves the array's
 *    device address; make that first call before any stream capture.  After
 *    a device reset the next call resolves it again (the context changed):
 *    make that call before any capture too.
 *  - All calls share the array: calls that overlap on the GPU race. */
plk_status plk_sum_sites_noalloc(const double* d_site_lnl, int n_sites, double* d_lnl_out,
                                 void* cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* PLK_H */
