// Host-side FP64 model math and tree preparation for libplk.
//
//  * rate_pos / q_matrix    — sub_model::get_rate_pos and calc_Q_matrix
//                             (src/sub_model.cpp:3-29, 99-114; get_freq :44-53)
//  * pmat_taylor20_host     — marth::square_matrix::exponential(P, t, 20)
//                             (src/marth/marth.cpp:129-140, multiply :50-61)
//  * jacobi_eigen / reversible_eigen / pmat_series_host — exact exp(Qt),
//                             which the reference lacks (cyclic Jacobi,
//                             Golub & Van Loan 4th ed. section 8.5; scaling and
//                             squaring with a Taylor sum)
//  * discrete_gamma         — Yang (1994) mean-per-category Gamma rates
//  * effective_lengths      — rate_model::get_time_mod_branch_length and
//                             get_rate_clade as simpleML::calculate_likelihood
//                             applies them (src/rate_model.cpp:103-127,
//                             src/rate_model.h:64-67, src/simpleML.cpp:127-184)
//  * check_tree / build_program — flattening of the reference's pointer tree
//                             walk into a register-allocated op list
#include <algorithm>
#include <cmath>
#include <cstring>

#include "plk_internal.h"

namespace plk {

unsigned rate_pos(unsigned n, bool tr, unsigned row, unsigned col) {
    const unsigned npos = tr ? (n * n - n) / 2 : n * n - n;
    if (row == col) return npos;
    if (tr) {
        const unsigned lo = std::min(row, col), hi = std::max(row, col);
        // rows 0..lo-1 of the strict upper triangle hold (n-1) + ... + (n-lo) slots
        unsigned pos = 0;
        for (unsigned i = 1; i <= lo; ++i) pos += n - i;
        return pos + (hi - lo - 1);
    }
    return row * (n - 1) + col - (col > row ? 1u : 0u);
}

void q_matrix(int n, bool tr, const unsigned* spec, const double* rates, const double* freqs,
              double* Q) {
    // last frequency = 1 - sum of the stored ones, subtracted in index order
    double last = 1.0;
    if (freqs)
        for (int i = 0; i < n - 1; ++i) last -= freqs[i];
    for (int i = 0; i < n; ++i) {
        double neg = 0.0;
        for (int j = 0; j < n; ++j) {
            if (i == j) continue;
            double v = rates[spec[rate_pos((unsigned)n, tr, (unsigned)i, (unsigned)j)]];
            if (tr) {
                const double f = freqs ? (j == n - 1 ? last : freqs[j]) : 1.0 / n;
                v *= f;
            }
            neg -= v;
            Q[i * n + j] = v;
        }
        Q[i * n + i] = neg;
    }
}

void pmat_taylor20_host(int n, const double* Q, double t, double* P) {
    std::vector<double> A((size_t)n * n), B((size_t)n * n);
    const double two20 = 1048576.0;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            volatile double qt = Q[i * n + j] * t;  // rounded product, then exact /2^20
            A[i * n + j] = (i == j ? 1.0 : 0.0) + qt / two20;
        }
    for (int it = 0; it < 20; ++it) {
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                double acc = 0.0;
                for (int k = 0; k < n; ++k) {
                    volatile double prod = A[i * n + k] * A[k * n + j];
                    acc = acc + prod;
                }
                B[i * n + j] = acc;
            }
        A.swap(B);
    }
    std::memcpy(P, A.data(), sizeof(double) * n * n);
}

void jacobi_eigen(int n, const double* Ain, double* w, double* V) {
    std::vector<double> A(Ain, Ain + (size_t)n * n);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) V[i * n + j] = (i == j) ? 1.0 : 0.0;
    double scale = 0.0;
    for (int i = 0; i < n * n; ++i) scale = std::max(scale, std::fabs(A[i]));
    if (scale == 0.0) scale = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) off += A[p * n + q] * A[p * n + q];
        if (std::sqrt(off) <= 1e-17 * scale) break;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = A[p * n + q];
                if (std::fabs(apq) <= 1e-300) continue;
                // rotation that zeroes A[p][q]: tan(phi) = t, smaller root
                const double theta = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) /
                                 (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {  // columns p, q
                    const double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {  // rows p, q
                    const double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double vkp = V[k * n + p], vkq = V[k * n + q];
                    V[k * n + p] = c * vkp - s * vkq;
                    V[k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < n; ++i) w[i] = A[i * n + i];
}

bool reversible_eigen(int n, const double* Q, const double* pi, double* lam, double* L,
                      double* R) {
    std::vector<double> B((size_t)n * n), V((size_t)n * n), sq(n);
    for (int i = 0; i < n; ++i) {
        if (!(pi[i] > 0.0)) return false;
        sq[i] = std::sqrt(pi[i]);
    }
    // B = D^1/2 Q D^-1/2, symmetrised against rounding
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            const double bij = sq[i] * Q[i * n + j] / sq[j];
            const double bji = sq[j] * Q[j * n + i] / sq[i];
            B[i * n + j] = 0.5 * (bij + bji);
        }
    jacobi_eigen(n, B.data(), lam, V.data());
    for (int i = 0; i < n; ++i)
        for (int m = 0; m < n; ++m) {
            L[i * n + m] = V[i * n + m] / sq[i];
            R[m * n + i] = V[i * n + m] * sq[i];
        }
    return true;
}

void pmat_series_host(int n, const double* Q, double t, double* P) {
    double norm = 0.0;
    for (int i = 0; i < n; ++i) {
        double r = 0.0;
        for (int j = 0; j < n; ++j) r += std::fabs(Q[i * n + j] * t);
        norm = std::max(norm, r);
    }
    int s = 0;
    while (norm > 0.125 && s < 1000) { norm *= 0.5; ++s; }
    const double f = std::ldexp(t, -s);
    const size_t nn = (size_t)n * n;
    std::vector<double> A(nn), term(nn), nt(nn);
    for (size_t i = 0; i < nn; ++i) A[i] = Q[i] * f;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) P[i * n + j] = term[i * n + j] = (i == j) ? 1.0 : 0.0;
    for (int m = 1; m <= 18; ++m) {
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                double acc = 0.0;
                for (int k = 0; k < n; ++k) acc += term[i * n + k] * A[k * n + j];
                nt[i * n + j] = acc / m;
            }
        term.swap(nt);
        for (size_t i = 0; i < nn; ++i) P[i] += term[i];
    }
    for (int it = 0; it < s; ++it) {
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                double acc = 0.0;
                for (int k = 0; k < n; ++k) acc += P[i * n + k] * P[k * n + j];
                nt[i * n + j] = acc;
            }
        std::memcpy(P, nt.data(), sizeof(double) * nn);
    }
}

// Regularized lower incomplete gamma P(a, x): power series below a + 1,
// continued fraction for the upper tail above.
static double inc_gamma_p(double a, double x) {
    if (x <= 0.0) return 0.0;
    const double log_pref = a * std::log(x) - x - std::lgamma(a);
    if (x < a + 1.0) {
        double sum = 1.0 / a, term = sum;
        for (int k = 1; k < 100000; ++k) {
            term *= x / (a + k);
            sum += term;
            if (term < sum * 1e-17) break;
        }
        return std::exp(log_pref) * sum;
    }
    // upper tail Q(a,x) = e^-x x^a / Gamma(a) * 1/(x+1-a- 1(1-a)/(x+3-a- ...))
    const double tiny = 1e-300;
    double b = x + 1.0 - a, c = 1.0 / tiny, d = 1.0 / b, f = d;
    for (int k = 1; k < 100000; ++k) {
        const double an = -k * (k - a);
        b += 2.0;
        d = an * d + b;
        if (std::fabs(d) < tiny) d = tiny;
        c = b + an / c;
        if (std::fabs(c) < tiny) c = tiny;
        d = 1.0 / d;
        const double delta = c * d;
        f *= delta;
        if (std::fabs(delta - 1.0) < 1e-16) break;
    }
    return 1.0 - std::exp(log_pref) * f;
}

// x with P(a, x) = p: bracketing by doubling, then Newton steps kept inside
// the bracket (bisection when a step leaves it).
static double inc_gamma_p_inverse(double a, double p) {
    double lo = 0.0, hi = std::max(1.0, a);
    while (inc_gamma_p(a, hi) < p) { lo = hi; hi *= 2.0; }
    double x = 0.5 * (lo + hi);
    for (int it = 0; it < 200; ++it) {
        const double fx = inc_gamma_p(a, x) - p;
        if (fx < 0) lo = x; else hi = x;
        const double dens = std::exp((a - 1.0) * std::log(x) - x - std::lgamma(a));
        double nx = (dens > 0) ? x - fx / dens : 0.5 * (lo + hi);
        if (!(nx > lo && nx < hi)) nx = 0.5 * (lo + hi);
        if (std::fabs(nx - x) <= 1e-16 * std::max(1.0, x) || hi - lo <= 1e-16 * hi) { x = nx; break; }
        x = nx;
    }
    return x;
}

void discrete_gamma(double alpha, int K, double* rates) {
    if (K <= 1) { rates[0] = 1.0; return; }
    // Gamma(shape alpha, rate alpha) has mean 1; the partial first moment up
    // to the quantile b is P(alpha + 1, alpha b), so the mean rate of category
    // k is K * (P(alpha+1, alpha b_{k+1}) - P(alpha+1, alpha b_k)).
    double prev = 0.0;
    for (int k = 0; k < K; ++k) {
        double cum = 1.0;
        if (k < K - 1) {
            const double y = inc_gamma_p_inverse(alpha, double(k + 1) / K);  // alpha * b
            cum = inc_gamma_p(alpha + 1.0, y);
        }
        rates[k] = (cum - prev) * K;
        prev = cum;
    }
}

// get_time_mod_branch_length (src/rate_model.cpp:103-127) with its float
// distance and cut-offs.  `strict_last` = true keeps the reference's final
// test (distance > last cut-off, so a branch starting exactly there -- the
// root-child edges when there are no slices -- gets 0).
static double time_mod_length(double bl, float d, const std::vector<float>& cut,
                              const std::vector<float>& rate, bool strict_last) {
    const double end = d + bl;
    double len = 0.0, prev = -0.0;
    for (size_t i = 0; i < cut.size(); ++i) {
        if (d < cut[i] && end > prev) {
            if (d >= prev && end <= cut[i]) len += (end - d) * rate[i];
            else if (d < prev && end <= cut[i]) len += (end - prev) * rate[i];
            else if (d >= prev && end > cut[i]) len += (cut[i] - d) * rate[i];
            else if (d < prev && end > cut[i]) len += (cut[i] - prev) * rate[i];
        }
        prev = cut[i];
    }
    if (d < prev && end > prev) len += end - prev;
    else if (strict_last ? (d > prev) : (d >= prev)) len = bl;
    return len;
}

void effective_lengths(int n_nodes, const int* left, const int* right, int root,
                       const double* bl, bool root_quirk, const std::vector<float>& cut_off,
                       const std::vector<float>& cut_rate, const std::vector<int>& clade_of_node,
                       const std::vector<float>& clade_rate, double* t_eff) {
    for (int v = 0; v < n_nodes; ++v) t_eff[v] = 0.0;
    struct Frame { int node; int clade; double dist; };
    std::vector<Frame> st;
    st.push_back({root, 0, 0.0});
    while (!st.empty()) {
        const Frame f = st.back();
        st.pop_back();
        const int u = f.node;
        if (left[u] < 0 && right[u] < 0) continue;
        int clade = f.clade;
        if (!clade_of_node.empty() && clade_of_node[u] >= 0) clade = clade_of_node[u];
        const double rate = clade < (int)clade_rate.size() ? (double)clade_rate[clade] : 1.0;
        const int kids[2] = {left[u], right[u]};
        for (int c = 0; c < 2; ++c) {
            const int v = kids[c];
            if (v < 0) continue;
            t_eff[v] = time_mod_length(bl[v], (float)f.dist, cut_off, cut_rate, root_quirk) * rate;
            st.push_back({v, clade, f.dist + bl[v]});
        }
    }
}

bool check_tree(int n_tips, int n_nodes, const int* left, const int* right, int* root,
                std::vector<int>* post, std::vector<int>* rank, std::string* err) {
    if (n_tips < 1 || n_nodes <= n_tips) {
        *err = "tree needs at least one tip and one internal node";
        return false;
    }
    std::vector<int> parent(n_nodes, -1);
    for (int v = 0; v < n_nodes; ++v) {
        const bool tip = left[v] < 0 && right[v] < 0;
        if ((v < n_tips) != tip) {
            *err = "node " + std::to_string(v) +
                   (v < n_tips ? " is a tip id but has children" : " is internal but has no child");
            return false;
        }
        const int kids[2] = {left[v], right[v]};
        for (int c = 0; c < 2; ++c) {
            const int k = kids[c];
            if (k < 0) continue;
            if (k >= n_nodes || k == v) { *err = "child id out of range at node " + std::to_string(v); return false; }
            if (parent[k] >= 0) { *err = "node " + std::to_string(k) + " has two parents"; return false; }
            parent[k] = v;
        }
    }
    int r = -1;
    for (int v = 0; v < n_nodes; ++v)
        if (parent[v] < 0) {
            if (r >= 0) { *err = "tree has more than one root"; return false; }
            r = v;
        }
    if (r < 0) { *err = "tree has no root (cycle)"; return false; }
    // iterative post-order (left subtree, right subtree, node)
    post->clear();
    rank->assign(n_nodes, -1);
    std::vector<std::pair<int, int>> st;
    st.push_back({r, 0});
    int visited = 0;
    while (!st.empty()) {
        auto& f = st.back();
        const int u = f.first;
        if (f.second == 0) {
            ++visited;
            f.second = 1;
            if (left[u] >= 0) { st.push_back({left[u], 0}); continue; }
        }
        if (f.second == 1) {
            f.second = 2;
            if (right[u] >= 0) { st.push_back({right[u], 0}); continue; }
        }
        if (left[u] >= 0 || right[u] >= 0) {
            (*rank)[u] = (int)post->size();
            post->push_back(u);
        }
        st.pop_back();
    }
    if (visited != n_nodes) { *err = "tree is not connected"; return false; }
    *root = r;
    return true;
}

Program build_program(int n_tips, int n_nodes, const int* left, const int* right, int root,
                      const std::vector<int>& rank) {
    (void)n_nodes;
    Program prog;
    // Sethi-Ullman number: registers (spill slots + accumulator) a subtree needs
    std::vector<int> need(n_nodes, 0);
    {
        std::vector<int> order;
        for (int v = 0; v < n_nodes; ++v)
            if (rank[v] >= 0) order.push_back(v);
        std::sort(order.begin(), order.end(), [&](int a, int b) { return rank[a] < rank[b]; });
        for (int u : order) {
            const int l = left[u], r = right[u];
            const int nl = l >= 0 ? need[l] : 0, nr = r >= 0 ? need[r] : 0;
            need[u] = (nl == nr) ? nl + 1 : std::max(nl, nr);
        }
    }
    auto is_tip = [&](int v) { return v < n_tips; };
    struct Frame { int u; int stage; int first; int second; };
    std::vector<Frame> st;
    st.push_back({root, 0, -1, -1});
    while (!st.empty()) {
        Frame& f = st.back();
        const int u = f.u, l = left[u], r = right[u];
        if (f.stage == 0) {
            // evaluation order: the internal child needing more registers first
            int first = -1, second = -1;
            if (l >= 0 && r >= 0) {
                if (!is_tip(l) && !is_tip(r)) {
                    if (need[l] >= need[r]) { first = l; second = r; } else { first = r; second = l; }
                } else if (!is_tip(l)) { first = l; second = r; }
                else if (!is_tip(r)) { first = r; second = l; }
                else { first = -1; second = -1; }
            } else {
                const int c = l >= 0 ? l : r;
                if (!is_tip(c)) first = c;
            }
            f.first = first;
            f.second = second;
            f.stage = 1;
            if (first >= 0) { st.push_back({first, 0, -1, -1}); continue; }
        }
        if (f.stage == 1) {
            f.stage = 2;
            if (f.first >= 0 && f.second >= 0 && !is_tip(f.second)) {
                prog.ops.back().push = 1;
                st.push_back({f.second, 0, -1, -1});
                continue;
            }
        }
        Op op{};
        op.node = u;
        op.rank = rank[u];
        op.push = 0;
        if (l >= 0 && r >= 0) {
            if (is_tip(l) && is_tip(r)) { op.e0 = l; op.s0 = l; op.e1 = r; op.s1 = r; }
            else if (f.second >= 0 && !is_tip(f.second)) {
                op.e0 = f.first; op.s0 = kSrcPop; op.e1 = f.second; op.s1 = kSrcAcc;
            } else {
                op.e0 = f.first; op.s0 = kSrcAcc; op.e1 = f.second; op.s1 = f.second;
            }
        } else {
            const int c = l >= 0 ? l : r;
            op.e0 = c;
            op.s0 = is_tip(c) ? c : kSrcAcc;
            op.e1 = -1;
            op.s1 = kSrcNone;
        }
        prog.ops.push_back(op);
        st.pop_back();
    }
    int sp = 0;
    for (const Op& op : prog.ops) {
        if (op.s0 == kSrcPop) --sp;
        if (op.push) ++sp;
        prog.max_depth = std::max(prog.max_depth, sp);
    }
    return prog;
}

}  // namespace plk
