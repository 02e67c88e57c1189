// Seeded sequence simulation on the host (the engine's counterpart of
// simpleML::simulate_chars, src/simpleML.cpp:233-292, which draws from rand()
// seeded by the clock).  Sites are independent, so they are split over
// threads; every random number comes from a counter-based generator keyed by
// (seed, site, node), so the output does not depend on the thread count.
//
// Generator: SplitMix64 (Steele, Lea & Flood 2014, "Fast splittable
// pseudorandom number generators") applied to a hashed counter.
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "plk_internal.h"

namespace plk {

namespace {

inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// uniform in [0, 1) from the counter (seed, a, b)
inline double uniform01(uint64_t seed, uint64_t a, uint64_t b) {
    const uint64_t h = splitmix64(seed ^ splitmix64(a * 0xD1B54A32D192ED03ull + splitmix64(b)));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

inline int draw(const double* cum, int S, double u) {
    for (int s = 0; s < S - 1; ++s)
        if (u < cum[s]) return s;
    return S - 1;
}

}  // namespace

bool simulate_sites(int n_tips, int n_nodes, const int* left, const int* right, int root, const double* bl,
                    int S, const double* Q, const double* freqs, int n_cats, const double* cat_rates,
                    int n_sites, uint64_t seed, int n_threads, uint32_t* masks) {
    // cumulative P(t * r_k) rows for every (edge, category), exact exp(Q t)
    std::vector<double> lam(S), L((size_t)S * S), R((size_t)S * S);
    if (!reversible_eigen(S, Q, freqs, lam.data(), L.data(), R.data())) return false;
    std::vector<double> cum((size_t)n_nodes * n_cats * S * S);
    for (int v = 0; v < n_nodes; ++v)
        for (int k = 0; k < n_cats; ++k) {
            double* c = &cum[(((size_t)v * n_cats) + k) * S * S];
            const double t = bl[v] * cat_rates[k];
            for (int i = 0; i < S; ++i) {
                double acc = 0.0;
                for (int j = 0; j < S; ++j) {
                    double p = 0.0;
                    for (int m = 0; m < S; ++m) p += L[i * S + m] * std::exp(lam[m] * t) * R[m * S + j];
                    acc += p > 0.0 ? p : 0.0;
                    c[i * S + j] = acc;
                }
                for (int j = 0; j < S; ++j) c[i * S + j] /= acc;
            }
        }
    std::vector<double> cum_pi(S);
    double a = 0.0;
    for (int s = 0; s < S; ++s) cum_pi[s] = (a += freqs[s]);
    for (int s = 0; s < S; ++s) cum_pi[s] /= a;
    // pre-order list of (parent, child) edges
    std::vector<std::pair<int, int>> edges;
    std::vector<int> st = {root};
    while (!st.empty()) {
        const int u = st.back();
        st.pop_back();
        for (int c : {left[u], right[u]})
            if (c >= 0) {
                edges.push_back({u, c});
                st.push_back(c);
            }
    }
    auto work = [&](int lo, int hi) {
        std::vector<int> state(n_nodes);
        for (int site = lo; site < hi; ++site) {
            const int k = std::min(n_cats - 1, (int)(uniform01(seed, (uint64_t)site, 0xC47u) * n_cats));
            state[root] = draw(cum_pi.data(), S, uniform01(seed, (uint64_t)site, 0x5EEDu));
            for (const auto& e : edges) {
                const double* c = &cum[(((size_t)e.second * n_cats) + k) * S * S + (size_t)state[e.first] * S];
                state[e.second] = draw(c, S, uniform01(seed, (uint64_t)site, (uint64_t)e.second + 1));
            }
            for (int t = 0; t < n_tips; ++t) masks[(size_t)t * n_sites + site] = 1u << state[t];
        }
    };
    if (n_threads < 1) n_threads = 1;
    if (n_threads > n_sites) n_threads = n_sites > 0 ? n_sites : 1;
    std::vector<std::thread> pool;
    for (int i = 0; i < n_threads; ++i)
        pool.emplace_back(work, (int)((long long)n_sites * i / n_threads), (int)((long long)n_sites * (i + 1) / n_threads));
    for (auto& th : pool) th.join();
    return true;
}

}  // namespace plk
