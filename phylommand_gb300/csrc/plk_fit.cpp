// Derivative-free maximum-likelihood fitting for libplk.
//
// The reference maximises lnL with NLopt's LN_NELDERMEAD and no stopping
// criteria (src/treeator.cpp:791-805, objective opt_function at :1122-1129).
// NLopt is not part of this build; NelderMead below is written from Nelder &
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
