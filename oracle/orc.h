/* Test infrastructure: the CPU oracle.
 *
 * A plain C99, FP64 restatement of the reference likelihood path
 * (src/simpleML.cpp, src/simpleML.h, src/sub_model.cpp, src/marth/marth.cpp,
 * src/rate_model.cpp), extended with the parts the reference lacks (rate
 * categories, an independent exact matrix exponential, a pre-order marginal
 * pass).  Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of
 * bench.py load it, and only to check or to time a CPU baseline; the product
 * (libplk) never calls it.
 *
 * Tree convention: nodes 0..n_tips-1 are tips (row i of the tip matrix);
 * left[v], right[v] are child ids or -1; a node with no children is a tip.
 * The root is the one node that is nobody's child.
 */
#ifndef ORC_H
#define ORC_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_P_TAYLOR20 = 0, ORC_P_EXACT = 1, ORC_P_GIVEN = 2 };

/* Index of the rate parameter for Q[row][col] (src/sub_model.cpp:3-29). */
unsigned orc_rate_pos(unsigned n_states, int tr, unsigned row, unsigned col);
/* Q as sub_model::calc_Q_matrix builds it (src/sub_model.cpp:99-114).
 * freqs holds n_states-1 stored values (or NULL for 1/n); the last frequency is
 * 1 - sum of the others, as sub_model::get_freq (src/sub_model.cpp:44-53). */
void orc_q_matrix(unsigned n_states, int tr, const unsigned* rate_spec, const double* rates,
                  const double* freqs, double* Q);
/* P = (I + Q t / 2^20)^(2^20), marth::square_matrix::exponential(P, t, 20)
 * (src/marth/marth.cpp:129-140, 106-111, 50-61), same operation order. */
void orc_pmat_taylor20(unsigned S, const double* Q, double t, double* P);
/* exp(Q t) by scaling and squaring with a degree-24 Taylor sum: an algorithm
 * independent of the product's eigendecomposition, used to check it. */
void orc_pmat_exact(unsigned S, const double* Q, double t, double* P);
/* Effective branch length of the edge above every node, as
 * simpleML::calculate_likelihood passes it to branch_likelihood
 * (src/simpleML.cpp:127-184): get_time_mod_branch_length(bl, (float)dist(parent))
 * (src/rate_model.cpp:103-127) times get_rate_clade(clade of parent).
 * root_dist0 is the distance the recursion starts at (0.0 in the reference).
 * cut_off/cut_rate describe the time slices (may be n_cut = 0);
 * clade_of_node[v] >= 0 marks v as the MRCA of clade number clade_of_node[v];
 * clade_rate[c] is that clade's rate (float, as the reference stores it). */
void orc_effective_lengths(int n_nodes, const int* left, const int* right, const double* bl,
                           double root_dist0, int n_cut, const float* cut_off,
                           const float* cut_rate, const int* clade_of_node, int n_clades,
                           const float* clade_rate, double* t_eff);
/* Discrete Gamma rate categories, mean of each of K equal-probability
 * categories (Yang 1994), Gamma(alpha, rate alpha).  Quantiles by bisection on
 * a series / continued-fraction regularized incomplete gamma. */
void orc_discrete_gamma(double alpha, int K, double* rates);

/* Full likelihood evaluation in FP64.
 *   tips       [n_tips * n_sites] state masks, bit s = state s allowed
 *   t_eff      [n_nodes] effective length of the edge above each node
 *   Q          [S*S], root_w [S] (frequencies for a reversible model, 1 else)
 *   cat_rate/cat_weight [C]
 *   p_mode     ORC_P_TAYLOR20 / ORC_P_EXACT / ORC_P_GIVEN (then Pgiven holds
 *              [n_nodes * C * S * S], P of the edge above node v, category k)
 *   per_site_pmat  1: rebuild P for every (site, edge) as the reference does
 *              (same values, reference cost; used to time the reference)
 * Outputs (any may be NULL):
 *   site_lnl   [n_sites]
 *   cond       [n_internal * n_sites * C * S] raw conditional vectors, internal
 *              nodes in post-order rank
 *   cond_norm  [n_internal * n_sites * S]   sum_k w_k cond / sum over states
 *   marginal   [n_internal * n_sites * S]   normalised pre-order marginals
 * Returns the total lnL (sites summed in ascending order), or 0.0 when a tip
 * cell has no allowed state (simpleML::check_nodes, src/simpleML.cpp:52-71). */
double orc_loglik(int n_tips, int n_nodes, const int* left, const int* right, int n_sites,
                  int S, const uint32_t* tips, const double* t_eff, const double* Q,
                  const double* root_w, int C, const double* cat_rate,
                  const double* cat_weight, int p_mode, const double* Pgiven,
                  int per_site_pmat, int n_threads, double* site_lnl, double* cond,
                  double* cond_norm, double* marginal);

/* Post-order rank list of internal nodes (left subtree, right subtree, node). */
int orc_internal_postorder(int n_nodes, const int* left, const int* right, int* out);

#ifdef __cplusplus
}
#endif
#endif
