// Derivative-free maximum-likelihood fitting for libplk.
//
// The reference maximises lnL with NLopt's LN_NELDERMEAD and no stopping
// criteria (src/treeator.cpp:791-805, objective opt_function at :1122-1129).
// libplk does not link NLopt; NelderMead below is written from Nelder &
// Mead (1965), "A simplex method for function minimization", with the usual
// coefficients (reflection 1, expansion 2, contraction 1/2, shrink 1/2) and
// explicit stopping rules.  It is a state machine that asks for one point at
// a time, so one loop drives a single fit and a batch of fits can be advanced
// together with all their requested points evaluated in one GPU launch.
#include <algorithm>
#include <cmath>
#include <numeric>

#include "plk_internal.h"

namespace plk {

NelderMead::NelderMead(int n, const double* x0, double step, double ftol_abs, double xtol, int max_evals)
    : n_(n), ftol_(ftol_abs), xtol_(xtol), max_evals_(max_evals) {
    simplex_.assign((size_t)(n + 1), std::vector<double>(x0, x0 + n));
    for (int i = 0; i < n; ++i) simplex_[i + 1][i] += step;
    fvals_.assign((size_t)(n + 1), HUGE_VAL);
    point_ = simplex_[0];
    state_ = State::Init;
    init_i_ = 0;
}

NelderMead::NelderMead(int n, const double* x0, const double* steps, double ftol_abs, double xtol, int max_evals)
    : NelderMead(n, x0, 0.0, ftol_abs, xtol, max_evals) {
    for (int i = 0; i < n; ++i) simplex_[i + 1][i] = x0[i] + steps[i];
    point_ = simplex_[0];
}

void NelderMead::order() {
    std::vector<int> idx(n_ + 1);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return fvals_[a] < fvals_[b]; });
    std::vector<std::vector<double>> s(n_ + 1);
    std::vector<double> f(n_ + 1);
    for (int i = 0; i <= n_; ++i) {
        s[i] = simplex_[idx[i]];
        f[i] = fvals_[idx[i]];
    }
    simplex_.swap(s);
    fvals_.swap(f);
}

bool NelderMead::converged() const {
    if (!(fvals_[n_] - fvals_[0] <= ftol_)) return false;
    double diam = 0.0;
    for (int i = 1; i <= n_; ++i)
        for (int j = 0; j < n_; ++j) diam = std::max(diam, std::fabs(simplex_[i][j] - simplex_[0][j]));
    return diam <= xtol_;
}

// Start an iteration: order, test convergence, propose the reflection.
void NelderMead::begin_iteration() {
    order();
    if (converged()) { state_ = State::Done; converged_ = true; return; }
    if (evals_ >= max_evals_) { state_ = State::Done; return; }
    centroid_.assign(n_, 0.0);
    for (int i = 0; i < n_; ++i)
        for (int j = 0; j < n_; ++j) centroid_[j] += simplex_[i][j] / n_;
    point_.resize(n_);
    for (int j = 0; j < n_; ++j) point_[j] = centroid_[j] + (centroid_[j] - simplex_[n_][j]);
    state_ = State::Reflect;
}

void NelderMead::start_shrink() {
    for (int i = 1; i <= n_; ++i)
        for (int j = 0; j < n_; ++j) simplex_[i][j] = simplex_[0][j] + 0.5 * (simplex_[i][j] - simplex_[0][j]);
    shrink_i_ = 1;
    point_ = simplex_[1];
    state_ = State::Shrink;
}

void NelderMead::tell(double f) {
    if (state_ == State::Done) return;
    if (!std::isfinite(f)) f = HUGE_VAL;  // outside the model's domain: reject the point
    ++evals_;
    switch (state_) {
        case State::Init:
            fvals_[init_i_] = f;
            if (++init_i_ <= n_) { point_ = simplex_[init_i_]; return; }
            begin_iteration();
            return;
        case State::Reflect:
            xr_ = point_;
            fr_ = f;
            if (fr_ < fvals_[0]) {
                for (int j = 0; j < n_; ++j) point_[j] = centroid_[j] + 2.0 * (xr_[j] - centroid_[j]);
                state_ = State::Expand;
            } else if (fr_ < fvals_[n_ - 1]) {
                simplex_[n_] = xr_;
                fvals_[n_] = fr_;
                begin_iteration();
            } else if (fr_ < fvals_[n_]) {
                for (int j = 0; j < n_; ++j) point_[j] = centroid_[j] + 0.5 * (xr_[j] - centroid_[j]);
                state_ = State::ContractOut;
            } else {
                for (int j = 0; j < n_; ++j) point_[j] = centroid_[j] + 0.5 * (simplex_[n_][j] - centroid_[j]);
                state_ = State::ContractIn;
            }
            return;
        case State::Expand:
            if (f < fr_) { simplex_[n_] = point_; fvals_[n_] = f; }
            else { simplex_[n_] = xr_; fvals_[n_] = fr_; }
            begin_iteration();
            return;
        case State::ContractOut:
            if (f <= fr_) { simplex_[n_] = point_; fvals_[n_] = f; begin_iteration(); }
            else start_shrink();
            return;
        case State::ContractIn:
            if (f < fvals_[n_]) { simplex_[n_] = point_; fvals_[n_] = f; begin_iteration(); }
            else start_shrink();
            return;
        case State::Shrink:
            fvals_[shrink_i_] = f;
            if (++shrink_i_ <= n_) { point_ = simplex_[shrink_i_]; return; }
            begin_iteration();
            return;
        case State::Done:
            return;
    }
}

const std::vector<double>& NelderMead::best_x() const {
    int b = 0;
    for (int i = 1; i <= n_; ++i)
        if (fvals_[i] < fvals_[b]) b = i;
    return simplex_[b];
}

double NelderMead::best_f() const { return *std::min_element(fvals_.begin(), fvals_.end()); }

// ---------------------------------------------------------------------------
// Quasi-Newton (BFGS, Nocedal & Wright 2006, ch. 6) on central-difference
// gradients.  At the start point the full Hessian is taken by finite
// differences (the diagonal comes free with the central differences, the
// n (n - 1) / 2 off-diagonal terms from forward mixed differences), shifted
// by a multiple of the identity until Cholesky succeeds, and inverted: the
// first step is a Newton step.  Later iterations use the BFGS update of the
// inverse Hessian.  Steps are capped at 1 in the max norm; the line search
// shortens the step (quadratic interpolation, within [0.1, 0.5] of the last
// trial) until the Armijo condition holds.
// ---------------------------------------------------------------------------
QuasiNewton::QuasiNewton(int n, const double* x0, const double* steps, double ftol_abs, double xtol, int max_evals,
                         bool full_hessian)
    : n_(n), ftol_(ftol_abs), xtol_(xtol), h_(1e-2), max_evals_(max_evals), full_hessian_(full_hessian) {
    x_.assign(x0, x0 + n);
    max_step_.assign(steps, steps + n);
    point_ = x_;
    g_.assign(n, 0.0);
    fplus_.assign(n, 0.0);
    dir_.assign(n, 0.0);
    curv_.assign(n, 0.0);
    H_.assign((size_t)n * n, 0.0);
}

void QuasiNewton::start_gradient() {
    gi_ = 0;
    next_grad_point();
    state_ = State::Grad;
}

// evaluation k of a gradient: coordinate k / 2, +h for even k, -h for odd k
void QuasiNewton::next_grad_point() {
    point_ = x_;
    point_[gi_ / 2] += (gi_ % 2 == 0) ? h_ : -h_;
}

void QuasiNewton::next_hess_point() {
    point_ = x_;
    point_[pairs_[hi_].first] += h_;
    point_[pairs_[hi_].second] += h_;
}

// H = finite-difference Hessian at the start, made positive definite by a
// growing multiple of the identity (Cholesky as the test), inverted into H_
void QuasiNewton::finish_hessian() {
    const int n = n_;
    std::vector<double> A((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) {
        const double c = curv_[i];
        // no usable curvature: a step of about max_step_ along the gradient
        A[(size_t)i * n + i] = (std::isfinite(c) && c > 1e-12) ? c : std::max(std::fabs(g_[i]), 1e-12) / max_step_[i];
    }
    for (size_t p = 0; p < pairs_.size(); ++p) {
        const int i = pairs_[p].first, j = pairs_[p].second;
        const double v = (hmix_[p] - fplus_[i] - fplus_[j] + f_) / (h_ * h_);
        if (std::isfinite(v) && curv_[i] > 1e-12 && curv_[j] > 1e-12) A[(size_t)i * n + j] = A[(size_t)j * n + i] = v;
    }
    double dmax = 0.0;
    for (int i = 0; i < n; ++i) dmax = std::max(dmax, A[(size_t)i * n + i]);
    std::vector<double> Lc((size_t)n * n);
    double mu = 0.0;
    bool ok = false;
    for (int attempt = 0; attempt < 30 && !ok; ++attempt) {
        ok = true;
        for (int i = 0; i < n && ok; ++i)
            for (int j = 0; j <= i; ++j) {
                double s = A[(size_t)i * n + j] + (i == j ? mu : 0.0);
                for (int k = 0; k < j; ++k) s -= Lc[(size_t)i * n + k] * Lc[(size_t)j * n + k];
                if (i == j) {
                    if (!(s > 0.0)) { ok = false; break; }
                    Lc[(size_t)i * n + i] = std::sqrt(s);
                } else {
                    Lc[(size_t)i * n + j] = s / Lc[(size_t)j * n + j];
                }
            }
        if (!ok) mu = (mu == 0.0) ? 1e-6 * dmax : 10.0 * mu;
    }
    if (!ok) {
        for (int i = 0; i < n; ++i) H_[(size_t)i * n + i] = 1.0 / A[(size_t)i * n + i];
    } else {
        // columns of the inverse: solve L L^T x = e_c
        std::vector<double> y(n), x(n);
        for (int c = 0; c < n; ++c) {
            for (int i = 0; i < n; ++i) {
                double s = (i == c) ? 1.0 : 0.0;
                for (int k = 0; k < i; ++k) s -= Lc[(size_t)i * n + k] * y[k];
                y[i] = s / Lc[(size_t)i * n + i];
            }
            for (int i = n - 1; i >= 0; --i) {
                double s = y[i];
                for (int k = i + 1; k < n; ++k) s -= Lc[(size_t)k * n + i] * x[k];
                x[i] = s / Lc[(size_t)i * n + i];
            }
            for (int i = 0; i < n; ++i) H_[(size_t)i * n + c] = x[i];
        }
    }
    start_line();
}

void QuasiNewton::finish_gradient() {
    if (!have_prev_ && !full_hessian_) {
        // first inverse Hessian: diagonal Newton where the curvature is positive
        for (int k = 0; k < n_; ++k)
            H_[(size_t)k * n_ + k] =
                curv_[k] > 1e-12 ? 1.0 / curv_[k] : max_step_[k] / std::max(std::fabs(g_[k]), 1e-12);
        start_line();
        return;
    }
    if (!have_prev_ && hmix_.empty() && n_ > 1) {
        // first iterate: the mixed differences of the full Hessian
        for (int i = 0; i < n_; ++i)
            for (int j = i + 1; j < n_; ++j) pairs_.emplace_back(i, j);
        hmix_.assign(pairs_.size(), HUGE_VAL);
        hi_ = 0;
        next_hess_point();
        state_ = State::Hess;
        return;
    }
    if (!have_prev_ && n_ == 1) {
        H_[0] = curv_[0] > 1e-12 ? 1.0 / curv_[0] : max_step_[0] / std::max(std::fabs(g_[0]), 1e-12);
    }
    if (have_prev_) {
        std::vector<double> s(n_), y(n_), Hy(n_, 0.0);
        double sy = 0.0, ss = 0.0, yy = 0.0;
        for (int i = 0; i < n_; ++i) {
            s[i] = x_[i] - x_prev_[i];
            y[i] = g_[i] - g_prev_[i];
            sy += s[i] * y[i];
            ss += s[i] * s[i];
            yy += y[i] * y[i];
        }
        if (sy > 1e-12 * std::sqrt(ss * yy)) {
            const double rho = 1.0 / sy;
            double yHy = 0.0;
            for (int i = 0; i < n_; ++i) {
                for (int j = 0; j < n_; ++j) Hy[i] += H_[(size_t)i * n_ + j] * y[j];
                yHy += y[i] * Hy[i];
            }
            for (int i = 0; i < n_; ++i)
                for (int j = 0; j < n_; ++j)
                    H_[(size_t)i * n_ + j] += -rho * (s[i] * Hy[j] + Hy[i] * s[j]) + (rho * rho * yHy + rho) * s[i] * s[j];
        }
    }
    start_line();
}

void QuasiNewton::start_line() {
    for (int attempt = 0; attempt < 2; ++attempt) {
        double m = 0.0;
        slope_ = 0.0;
        for (int i = 0; i < n_; ++i) {
            double d = 0.0;
            for (int j = 0; j < n_; ++j) d -= H_[(size_t)i * n_ + j] * g_[j];
            dir_[i] = d;
            m = std::max(m, std::fabs(d));
        }
        if (m > 1.0)
            for (double& d : dir_) d /= m;
        for (int i = 0; i < n_; ++i) slope_ += g_[i] * dir_[i];
        if (slope_ < 0.0) break;
        // not a descent direction: fall back to the steepest descent scaled by
        // the initial steps
        std::fill(H_.begin(), H_.end(), 0.0);
        const double gn = std::sqrt(std::inner_product(g_.begin(), g_.end(), g_.begin(), 0.0));
        for (int i = 0; i < n_; ++i) H_[(size_t)i * n_ + i] = max_step_[i] / std::max(gn, 1e-300);
    }
    if (!(slope_ < 0.0)) {
        state_ = State::Done;
        return;
    }
    t_ = 1.0;
    backtracks_ = 0;
    for (int i = 0; i < n_; ++i) point_[i] = x_[i] + t_ * dir_[i];
    state_ = State::Line;
}

void QuasiNewton::tell(double f) {
    if (state_ == State::Done) return;
    if (!std::isfinite(f)) f = HUGE_VAL;
    ++evals_;
    switch (state_) {
        case State::Start:
            f_ = f;
            if (!std::isfinite(f_)) { state_ = State::Done; return; }
            start_gradient();
            break;
        case State::Grad: {
            const int k = gi_ / 2;
            if (gi_ % 2 == 0) {
                fplus_[k] = f;
            } else {
                const double fp = fplus_[k], fm = f;
                double curv = 0.0;
                if (std::isfinite(fp) && std::isfinite(fm)) {
                    g_[k] = (fp - fm) / (2.0 * h_);
                    curv = (fp - 2.0 * f_ + fm) / (h_ * h_);
                } else if (std::isfinite(fp)) {
                    g_[k] = (fp - f_) / h_;
                } else if (std::isfinite(fm)) {
                    g_[k] = (f_ - fm) / h_;
                } else {
                    g_[k] = 0.0;
                }
                if (!have_prev_) curv_[k] = curv;
            }
            if (++gi_ < 2 * n_) next_grad_point();
            else finish_gradient();
            break;
        }
        case State::Hess:
            hmix_[hi_] = f;
            if (++hi_ < (int)pairs_.size()) next_hess_point();
            else finish_hessian();
            break;
        case State::Line:
            if (f <= f_ + 1e-4 * t_ * slope_) {
                double moved = 0.0;
                for (int i = 0; i < n_; ++i) moved = std::max(moved, std::fabs(point_[i] - x_[i]));
                x_prev_ = x_;
                g_prev_ = g_;
                f_prev_ = f_;
                x_ = point_;
                f_ = f;
                have_prev_ = true;
                ++iter_;
                // converged: a small decrease with a small step, or three
                // small decreases in a row (a flat direction)
                flat_ = (f_prev_ - f_ <= ftol_) ? flat_ + 1 : 0;
                if ((f_prev_ - f_ <= ftol_ && moved <= xtol_) || flat_ >= 3) {
                    state_ = State::Done;
                    return;
                }
                start_gradient();
            } else {
                if (++backtracks_ > 30) {
                    state_ = State::Done;  // no decrease along a descent direction: at the noise floor
                    return;
                }
                // minimiser of the quadratic through f_, slope_ and this trial
                double tn = 0.5 * t_;
                if (std::isfinite(f)) {
                    const double denom = 2.0 * (f - f_ - slope_ * t_);
                    if (denom > 0.0) tn = -slope_ * t_ * t_ / denom;
                }
                t_ = std::min(std::max(tn, 0.1 * t_), 0.5 * t_);
                for (int i = 0; i < n_; ++i) point_[i] = x_[i] + t_ * dir_[i];
            }
            break;
        case State::Done:
            return;
    }
    if (evals_ >= max_evals_) state_ = State::Done;
}

// GTR(+Gamma) parameter vector of the fits:
//   x[0 .. npos-2]   log exchangeabilities relative to the last one (fixed 1)
//   x[npos-1]        log Gamma shape alpha (absent when n_cats == 1)
//   x[last]          log tree-length scale (multiplies every branch length)
// Q is normalised to mean rate 1 under the fixed frequencies.
bool gtr_model_from_x(int S, const double* x, int n_cats, const double* freqs, double* Q, double* cat_rates,
                      double* cat_weights, double* scale) {
    const int npos = S * (S - 1) / 2;
    std::vector<double> exch(npos, 1.0);
    for (int i = 0; i < npos - 1; ++i) exch[i] = std::exp(x[i]);
    std::vector<unsigned> spec(npos);
    std::iota(spec.begin(), spec.end(), 0u);
    q_matrix(S, true, spec.data(), exch.data(), freqs, Q);
    // the engine's q_matrix derives the last frequency; use the given one
    double mu = 0.0;
    for (int i = 0; i < S; ++i) mu -= freqs[i] * Q[i * S + i];
    if (!(mu > 0.0) || !std::isfinite(mu)) return false;
    for (int i = 0; i < S * S; ++i) Q[i] /= mu;
    int k = npos - 1;
    if (n_cats > 1) {
        const double alpha = std::exp(x[k++]);
        if (!(alpha > 1e-4 && alpha < 1e4)) return false;
        discrete_gamma(alpha, n_cats, cat_rates);
    } else cat_rates[0] = 1.0;
    for (int c = 0; c < n_cats; ++c) cat_weights[c] = 1.0 / n_cats;
    *scale = std::exp(x[k]);
    return *scale > 0.0 && std::isfinite(*scale);
}

int gtr_n_params(int S, int n_cats) { return S * (S - 1) / 2 - 1 + (n_cats > 1 ? 1 : 0) + 1; }

}  // namespace plk
