/* Test infrastructure: the CPU oracle (see orc.h).  FP64, compiled with
 * -ffp-contract=off so that every multiply and add is rounded on its own, as
 * the reference's x86-64 build does.  Each function names the reference code it
 * restates; the parts the reference lacks say what they follow instead. */
#include "orc.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ---- Q matrix (src/sub_model.cpp:3-29, 44-53, 99-114) ---------------- */

unsigned orc_rate_pos(unsigned n, int tr, unsigned row, unsigned col) {
    unsigned npos = tr ? (n * n - n) / 2 : n * n - n;
    if (row == col) return npos;
    unsigned pos = 0;
    if (tr) {
        /* upper triangle, row-major: (r,c) with r<c and (c,r) share a slot */
        unsigned i = row < col ? row : col;
        unsigned j = row < col ? col - row : row - col;
        while (i) { pos += n - i; --i; }
        pos += j - 1;
    } else {
        pos = row * (n - 1) + col;
        if (col > row) --pos;
    }
    return pos;
}

static double orc_freq(unsigned n, const double* freqs, unsigned j) {
    if (freqs == NULL) return 1.0 / n;
    if (j == n - 1) {
        double f = 1.0;
        for (unsigned i = 0; i < n - 1; ++i) f -= freqs[i];
        return f;
    }
    return freqs[j];
}

void orc_q_matrix(unsigned n, int tr, const unsigned* spec, const double* rates,
                  const double* freqs, double* Q) {
    for (unsigned i = 0; i < n; ++i) {
        double neg_sum = 0.0;
        for (unsigned j = 0; j < n; ++j) {
            if (i == j) continue;
            double v = rates[spec[orc_rate_pos(n, tr, i, j)]];
            if (tr) v *= orc_freq(n, freqs, j);
            neg_sum -= v;
            Q[i * n + j] = v;
        }
        Q[i * n + i] = neg_sum;
    }
}

/* ---- P(t) ---------------------------------------------------------------- */

/* prod = A * A with prod[i][j] = 0, += A[i][k]*A[k][j], k ascending
 * (src/marth/marth.cpp:50-61, power(2) at :106-111). */
static void square_into(unsigned S, const double* A, double* out) {
    for (unsigned i = 0; i < S; ++i)
        for (unsigned j = 0; j < S; ++j) {
            double acc = 0;
            for (unsigned k = 0; k < S; ++k) acc += A[i * S + k] * A[k * S + j];
            out[i * S + j] = acc;
        }
}

void orc_pmat_taylor20(unsigned S, const double* Q, double t, double* P) {
    /* src/marth/marth.cpp:129-140: identity, add (q*t)/2^20, square 20 times */
    double* tmp = (double*)malloc(sizeof(double) * S * S);
    const double scale = pow(2, 20);
    for (unsigned x = 0; x < S; ++x)
        for (unsigned y = 0; y < S; ++y) {
            double q = (Q[x * S + y] * t) / scale;
            P[x * S + y] = (x == y ? 1.0 : 0.0) + q;
        }
    for (int it = 0; it < 20; ++it) {
        square_into(S, P, tmp);
        memcpy(P, tmp, sizeof(double) * S * S);
    }
    free(tmp);
}

void orc_pmat_exact(unsigned S, const double* Q, double t, double* P) {
    /* scaling and squaring: A = Q t / 2^s with ||A||_inf <= 1/8, Taylor to
     * degree 24 (truncation < 1e-40), then s squarings. */
    double norm = 0.0;
    for (unsigned i = 0; i < S; ++i) {
        double r = 0.0;
        for (unsigned j = 0; j < S; ++j) r += fabs(Q[i * S + j] * t);
        if (r > norm) norm = r;
    }
    int s = 0;
    while (norm > 0.125) { norm *= 0.5; ++s; }
    double f = ldexp(t, -s);
    size_t n2 = (size_t)S * S;
    double* A = (double*)malloc(sizeof(double) * n2);
    double* term = (double*)malloc(sizeof(double) * n2);
    double* nt = (double*)malloc(sizeof(double) * n2);
    for (size_t i = 0; i < n2; ++i) A[i] = Q[i] * f;
    for (unsigned i = 0; i < S; ++i)
        for (unsigned j = 0; j < S; ++j) {
            term[i * S + j] = (i == j) ? 1.0 : 0.0;
            P[i * S + j] = term[i * S + j];
        }
    for (int m = 1; m <= 24; ++m) {
        for (unsigned i = 0; i < S; ++i)
            for (unsigned j = 0; j < S; ++j) {
                double acc = 0;
                for (unsigned k = 0; k < S; ++k) acc += term[i * S + k] * A[k * S + j];
                nt[i * S + j] = acc / m;
            }
        memcpy(term, nt, sizeof(double) * n2);
        for (size_t i = 0; i < n2; ++i) P[i] += term[i];
    }
    for (int i = 0; i < s; ++i) {
        square_into(S, P, nt);
        memcpy(P, nt, sizeof(double) * n2);
    }
    free(A); free(term); free(nt);
}

/* ---- effective branch lengths (src/rate_model.cpp:103-127,
 *      src/rate_model.h:64-67, src/simpleML.cpp:127-184) ------------------ */

static double time_mod_length(double branch_length, float distance_to_root, int n_cut,
                              const float* cut_off, const float* cut_rate) {
    const double branch_end = distance_to_root + branch_length;
    double new_len = 0.0;
    double previous = -0.0;
    for (int i = 0; i < n_cut; ++i) {
        if (distance_to_root < cut_off[i] && branch_end > previous) {
            if (distance_to_root >= previous && branch_end <= cut_off[i])
                new_len += (branch_end - distance_to_root) * cut_rate[i];
            else if (distance_to_root < previous && branch_end <= cut_off[i])
                new_len += (branch_end - previous) * cut_rate[i];
            else if (distance_to_root >= previous && branch_end > cut_off[i])
                new_len += (cut_off[i] - distance_to_root) * cut_rate[i];
            else if (distance_to_root < previous && branch_end > cut_off[i])
                new_len += (cut_off[i] - previous) * cut_rate[i];
        }
        previous = cut_off[i];
    }
    if (distance_to_root < previous && branch_end > previous) new_len += branch_end - previous;
    else if (distance_to_root > previous) new_len = branch_length;
    return new_len;
}

static int find_root(int n_nodes, const int* left, const int* right) {
    char* is_child = (char*)calloc((size_t)n_nodes, 1);
    for (int v = 0; v < n_nodes; ++v) {
        if (left[v] >= 0) is_child[left[v]] = 1;
        if (right[v] >= 0) is_child[right[v]] = 1;
    }
    int root = -1;
    for (int v = 0; v < n_nodes; ++v)
        if (!is_child[v]) { root = v; break; }
    free(is_child);
    return root;
}

typedef struct { int node; int clade; double dist; int stage; } frame_t;

void orc_effective_lengths(int n_nodes, const int* left, const int* right, const double* bl,
                           double root_dist0, int n_cut, const float* cut_off,
                           const float* cut_rate, const int* clade_of_node, int n_clades,
                           const float* clade_rate, double* t_eff) {
    for (int v = 0; v < n_nodes; ++v) t_eff[v] = 0.0;
    int root = find_root(n_nodes, left, right);
    if (root < 0) return;
    frame_t* st = (frame_t*)malloc(sizeof(frame_t) * (size_t)(n_nodes + 1));
    int sp = 0;
    st[sp].node = root; st[sp].clade = 0; st[sp].dist = root_dist0; ++sp;
    while (sp > 0) {
        frame_t f = st[--sp];
        int u = f.node;
        if (left[u] < 0 && right[u] < 0) continue;
        int clade = f.clade;
        if (clade_of_node && clade_of_node[u] >= 0) clade = clade_of_node[u];
        /* rate_model::get_rate_clade: rates[clade] if defined, else 1 */
        double rate = (clade < n_clades) ? (double)clade_rate[clade] : 1.0;
        int kids[2] = {left[u], right[u]};
        for (int c = 0; c < 2; ++c) {
            int v = kids[c];
            if (v < 0) continue;
            t_eff[v] = time_mod_length(bl[v], (float)f.dist, n_cut, cut_off, cut_rate) * rate;
            st[sp].node = v; st[sp].clade = clade; st[sp].dist = f.dist + bl[v]; ++sp;
        }
    }
    free(st);
}

/* ---- discrete Gamma (Yang 1994, mean per category) ------------------------ */

/* regularized lower incomplete gamma P(a, x): power series for x < a + 1,
 * Legendre continued fraction (modified Lentz) for the complement otherwise. */
static double reg_lower_gamma(double a, double x) {
    if (x <= 0.0) return 0.0;
    double lpre = a * log(x) - x - lgamma(a);
    if (x < a + 1.0) {
        double term = 1.0 / a, sum = term, ap = a;
        for (int n = 0; n < 10000; ++n) {
            ap += 1.0;
            term *= x / ap;
            sum += term;
            if (fabs(term) < fabs(sum) * 1e-17) break;
        }
        return sum * exp(lpre);
    }
    const double tiny = 1e-300;
    double b = x + 1.0 - a, c = 1.0 / tiny, d = 1.0 / b, h = d;
    for (int i = 1; i < 10000; ++i) {
        double an = -i * (i - a);
        b += 2.0;
        d = an * d + b; if (fabs(d) < tiny) d = tiny;
        c = b + an / c; if (fabs(c) < tiny) c = tiny;
        d = 1.0 / d;
        double del = d * c;
        h *= del;
        if (fabs(del - 1.0) < 1e-17) break;
    }
    return 1.0 - exp(lpre) * h;
}

void orc_discrete_gamma(double alpha, int K, double* rates) {
    if (K <= 1) { rates[0] = 1.0; return; }
    /* y_k solves P(alpha, y_k) = k/K (y = alpha * quantile of the mean-1 law) */
    double prev_mass = 0.0;
    for (int k = 0; k < K; ++k) {
        double mass;
        if (k == K - 1) mass = 1.0;
        else {
            double p = (double)(k + 1) / K, lo = 0.0, hi = alpha + 1.0;
            while (reg_lower_gamma(alpha, hi) < p) hi *= 2.0;
            for (int it = 0; it < 200; ++it) {
                double mid = 0.5 * (lo + hi);
                if (reg_lower_gamma(alpha, mid) < p) lo = mid; else hi = mid;
            }
            mass = reg_lower_gamma(alpha + 1.0, 0.5 * (lo + hi));
        }
        rates[k] = (mass - prev_mass) * K;
        prev_mass = mass;
    }
}

/* ---- traversal helpers --------------------------------------------------- */

int orc_internal_postorder(int n_nodes, const int* left, const int* right, int* out) {
    int root = find_root(n_nodes, left, right);
    if (root < 0) return 0;
    int* st = (int*)malloc(sizeof(int) * (size_t)(2 * n_nodes + 2));
    char* seen = (char*)calloc((size_t)n_nodes, 1);
    int sp = 0, n = 0;
    st[sp++] = root;
    while (sp > 0) {
        int u = st[sp - 1];
        if (left[u] < 0 && right[u] < 0) { --sp; continue; }
        if (!seen[u]) {
            seen[u] = 1;
            if (right[u] >= 0) st[sp++] = right[u];
            if (left[u] >= 0) st[sp++] = left[u];
        } else {
            --sp;
            out[n++] = u;
        }
    }
    free(st); free(seen);
    return n;
}

/* ---- likelihood ------------------------------------------------------------ */

typedef struct {
    int n_tips, n_nodes, n_sites, S, C, n_int, per_site_pmat, p_mode;
    const int *left, *right, *order;
    int* rank;
    const uint32_t* tips;
    const double *t_eff, *Q, *root_w, *cat_rate, *cat_weight;
    double* P; /* [n_nodes][C][S][S] */
    double *site_lnl, *cond_out, *cond_norm, *marginal;
    int bad_tip;
    int site_lo, site_hi;
} job_t;

static void edge_pmat(const job_t* J, int v, int k, double* out) {
    double t = J->t_eff[v] * J->cat_rate[k];
    if (J->p_mode == ORC_P_TAYLOR20) orc_pmat_taylor20((unsigned)J->S, J->Q, t, out);
    else orc_pmat_exact((unsigned)J->S, J->Q, t, out);
}

/* D[i] = sum_j x[j] P[i][j] (src/simpleML.cpp:186-197, j ascending) */
static void child_vec(const job_t* J, int v, int k, int site, const double* cond_site,
                      const double* Pv, double* D, double* xbuf) {
    const int S = J->S;
    const double* x;
    if (v < J->n_tips) {
        uint32_t m = J->tips[(size_t)v * J->n_sites + site];
        for (int j = 0; j < S; ++j) xbuf[j] = ((m >> j) & 1u) ? 1.0 : 0.0;
        x = xbuf;
    } else {
        x = cond_site + ((size_t)J->rank[v] * J->C + k) * S;
    }
    for (int i = 0; i < S; ++i) {
        double pi = 0.0;
        for (int j = 0; j < S; ++j) pi += x[j] * Pv[i * S + j];
        D[i] = pi;
    }
}

static void* run_sites(void* arg) {
    job_t* J = (job_t*)arg;
    const int S = J->S, C = J->C, n_int = J->n_int;
    double* cs = (double*)malloc(sizeof(double) * (size_t)n_int * C * S);
    double* Dl = (double*)malloc(sizeof(double) * (size_t)J->n_nodes * C * S);
    double* out = (double*)malloc(sizeof(double) * (size_t)n_int * C * S);
    double* tmpP = (double*)malloc(sizeof(double) * (size_t)S * S);
    double* xbuf = (double*)malloc(sizeof(double) * (size_t)S);
    double* Dtmp = (double*)malloc(sizeof(double) * (size_t)S);
    for (int site = J->site_lo; site < J->site_hi; ++site) {
        long site_exp = 0;
        /* check_nodes: a tip cell with no allowed state fails the whole call */
        for (int t = 0; t < J->n_tips; ++t)
            if ((J->tips[(size_t)t * J->n_sites + site] & ((S >= 32) ? 0xffffffffu : ((1u << S) - 1u))) == 0)
                J->bad_tip = 1;
        for (int r = 0; r < n_int; ++r) {
            int u = J->order[r];
            for (int k = 0; k < C; ++k) {
                double* cu = cs + ((size_t)r * C + k) * S;
                int l = J->left[u], rr = J->right[u];
                const double* Pl = NULL;
                const double* Pr = NULL;
                if (l >= 0) {
                    if (J->per_site_pmat) { edge_pmat(J, l, k, tmpP); Pl = tmpP; }
                    else Pl = J->P + ((size_t)l * C + k) * S * S;
                    child_vec(J, l, k, site, cs, Pl, Dl + ((size_t)l * C + k) * S, xbuf);
                    for (int i = 0; i < S; ++i) cu[i] = Dl[((size_t)l * C + k) * S + i];
                }
                if (rr >= 0) {
                    if (J->per_site_pmat) { edge_pmat(J, rr, k, tmpP); Pr = tmpP; }
                    else Pr = J->P + ((size_t)rr * C + k) * S * S;
                    double* Dr = Dl + ((size_t)rr * C + k) * S;
                    child_vec(J, rr, k, site, cs, Pr, Dr, xbuf);
                    for (int i = 0; i < S; ++i) {
                        if (l >= 0) cu[i] *= Dr[i];
                        else cu[i] = Dr[i];
                    }
                }
            }
            /* power-of-two rescaling below 2^-256 (exact; absent in the
             * reference, whose trees never get there) */
            double mx = 0.0;
            for (int q = 0; q < C * S; ++q) if (cs[(size_t)r * C * S + q] > mx) mx = cs[(size_t)r * C * S + q];
            if (mx > 0.0 && mx < 0x1p-256) {
                int e;
                frexp(mx, &e);
                for (int q = 0; q < C * S; ++q) cs[(size_t)r * C * S + q] = ldexp(cs[(size_t)r * C * S + q], -e);
                site_exp += e;
            }
        }
        /* root: sum_k w_k sum_s L[s] * (tr ? pi_s : 1)  (src/simpleML.h:123-141) */
        int rroot = n_int - 1;
        double lsum = 0.0;
        for (int k = 0; k < C; ++k) {
            const double* R = cs + ((size_t)rroot * C + k) * S;
            double lk = 0.0;
            for (int s = 0; s < S; ++s) lk += R[s] * J->root_w[s];
            lsum += J->cat_weight[k] * lk;
        }
        if (J->site_lnl) J->site_lnl[site] = site_exp ? log(lsum) + (double)site_exp * 0.69314718055994530942 : log(lsum);
        if (J->cond_out)
            for (int r = 0; r < n_int; ++r)
                memcpy(J->cond_out + (((size_t)r * J->n_sites + site) * C) * S,
                       cs + (size_t)r * C * S, sizeof(double) * (size_t)C * S);
        if (J->cond_norm)
            for (int r = 0; r < n_int; ++r) {
                double* o = J->cond_norm + ((size_t)r * J->n_sites + site) * S;
                double tot = 0.0;
                for (int s = 0; s < S; ++s) {
                    double a = 0.0;
                    for (int k = 0; k < C; ++k) a += J->cat_weight[k] * cs[((size_t)r * C + k) * S + s];
                    o[s] = a;
                }
                for (int s = 0; s < S; ++s) tot += o[s];
                for (int s = 0; s < S; ++s) o[s] /= tot;
            }
        if (J->marginal) {
            /* pre-order: Out(root) = root weights; for child v of u with
             * sibling w: Out(v)[b] = sum_a Out(u)[a] D_w[a] P_v[a][b]. */
            for (int k = 0; k < C; ++k)
                for (int s = 0; s < S; ++s) out[((size_t)rroot * C + k) * S + s] = J->root_w[s];
            for (int r = n_int - 1; r >= 0; --r) {
                int u = J->order[r];
                int kids[2] = {J->left[u], J->right[u]};
                for (int c = 0; c < 2; ++c) {
                    int v = kids[c], w = kids[1 - c];
                    if (v < 0 || v < J->n_tips) continue;
                    for (int k = 0; k < C; ++k) {
                        const double* Pv = J->P + ((size_t)v * C + k) * S * S;
                        if (J->per_site_pmat) { edge_pmat(J, v, k, tmpP); Pv = tmpP; }
                        const double* Ou = out + ((size_t)r * C + k) * S;
                        const double* Dw = (w >= 0) ? Dl + ((size_t)w * C + k) * S : NULL;
                        for (int a = 0; a < S; ++a) Dtmp[a] = Ou[a] * (Dw ? Dw[a] : 1.0);
                        double* Ov = out + ((size_t)J->rank[v] * C + k) * S;
                        for (int b = 0; b < S; ++b) {
                            double acc = 0.0;
                            for (int a = 0; a < S; ++a) acc += Dtmp[a] * Pv[a * S + b];
                            Ov[b] = acc;
                        }
                    }
                    double* Ov0 = out + (size_t)J->rank[v] * C * S;
                    double mo = 0.0;
                    for (int q = 0; q < C * S; ++q) if (Ov0[q] > mo) mo = Ov0[q];
                    if (mo > 0.0 && mo < 0x1p-256) {
                        int e;
                        frexp(mo, &e);
                        for (int q = 0; q < C * S; ++q) Ov0[q] = ldexp(Ov0[q], -e);
                    }
                }
            }
            for (int r = 0; r < n_int; ++r) {
                double* o = J->marginal + ((size_t)r * J->n_sites + site) * S;
                double tot = 0.0;
                for (int s = 0; s < S; ++s) {
                    double a = 0.0;
                    for (int k = 0; k < C; ++k)
                        a += J->cat_weight[k] * out[((size_t)r * C + k) * S + s] * cs[((size_t)r * C + k) * S + s];
                    o[s] = a;
                    tot += a;
                }
                for (int s = 0; s < S; ++s) o[s] /= tot;
            }
        }
    }
    free(cs); free(Dl); free(out); free(tmpP); free(xbuf); free(Dtmp);
    return NULL;
}

double orc_loglik(int n_tips, int n_nodes, const int* left, const int* right, int n_sites,
                  int S, const uint32_t* tips, const double* t_eff, const double* Q,
                  const double* root_w, int C, const double* cat_rate,
                  const double* cat_weight, int p_mode, const double* Pgiven,
                  int per_site_pmat, int n_threads, double* site_lnl, double* cond,
                  double* cond_norm, double* marginal) {
    int* order = (int*)malloc(sizeof(int) * (size_t)n_nodes);
    int n_int = orc_internal_postorder(n_nodes, left, right, order);
    int* rank = (int*)malloc(sizeof(int) * (size_t)n_nodes);
    for (int v = 0; v < n_nodes; ++v) rank[v] = -1;
    for (int r = 0; r < n_int; ++r) rank[order[r]] = r;
    size_t pm = (size_t)n_nodes * C * S * S;
    double* P = (double*)calloc(pm, sizeof(double));
    job_t base;
    memset(&base, 0, sizeof(base));
    base.n_tips = n_tips; base.n_nodes = n_nodes; base.n_sites = n_sites; base.S = S; base.C = C;
    base.n_int = n_int; base.per_site_pmat = per_site_pmat; base.p_mode = p_mode;
    base.left = left; base.right = right; base.order = order; base.rank = rank; base.tips = tips;
    base.t_eff = t_eff; base.Q = Q; base.root_w = root_w; base.cat_rate = cat_rate;
    base.cat_weight = cat_weight; base.P = P; base.site_lnl = NULL;
    base.cond_out = cond; base.cond_norm = cond_norm; base.marginal = marginal;
    if (p_mode == ORC_P_GIVEN) {
        memcpy(P, Pgiven, sizeof(double) * pm);
        base.per_site_pmat = 0;
    } else if (!per_site_pmat) {
        for (int v = 0; v < n_nodes; ++v)
            for (int k = 0; k < C; ++k) edge_pmat(&base, v, k, P + ((size_t)v * C + k) * S * S);
    }
    double* sl = (double*)malloc(sizeof(double) * (size_t)(n_sites > 0 ? n_sites : 1));
    base.site_lnl = sl;
    if (n_threads < 1) n_threads = 1;
    if (n_threads > n_sites) n_threads = n_sites > 0 ? n_sites : 1;
    job_t* jobs = (job_t*)malloc(sizeof(job_t) * (size_t)n_threads);
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)n_threads);
    for (int i = 0; i < n_threads; ++i) {
        jobs[i] = base;
        jobs[i].site_lo = (int)((long long)n_sites * i / n_threads);
        jobs[i].site_hi = (int)((long long)n_sites * (i + 1) / n_threads);
        if (n_threads > 1) pthread_create(&th[i], NULL, run_sites, &jobs[i]);
    }
    if (n_threads == 1) run_sites(&jobs[0]);
    else for (int i = 0; i < n_threads; ++i) pthread_join(th[i], NULL);
    int bad = 0;
    for (int i = 0; i < n_threads; ++i) bad |= jobs[i].bad_tip;
    double total = 0.0;
    for (int s = 0; s < n_sites; ++s) total += sl[s];
    if (site_lnl) memcpy(site_lnl, sl, sizeof(double) * (size_t)n_sites);
    free(jobs); free(th); free(sl); free(P); free(order); free(rank);
    return bad ? 0.0 : total;
}
