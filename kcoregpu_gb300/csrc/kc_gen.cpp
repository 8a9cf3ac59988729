// Seeded synthetic graph generators for the benchmark shapes (R-MAT,
// Chung-Lu power law, Erdos-Renyi).  Counter-based randomness makes every
// output independent of the thread count and identical on x86 and Arm hosts.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#include <omp.h>

#include "kc_internal.h"

namespace kc {

static inline uint32_t ceil_log2(uint32_t n) {
    uint32_t s = 0;
    while (s < 32 && (1ull << s) < (uint64_t)n) ++s;
    return s;
}

// Vose alias table over non-negative weights.
struct Alias {
    std::vector<double> prob;
    std::vector<uint32_t> alias;
    void build(const std::vector<double>& w) {
        const size_t n = w.size();
        prob.assign(n, 0.0);
        alias.assign(n, 0);
        double sum = 0;
        for (double x : w) sum += x;
        std::vector<double> p(n);
        std::vector<uint32_t> small, large;
        small.reserve(n); large.reserve(n);
        for (size_t i = 0; i < n; ++i) {
            p[i] = w[i] * (double)n / sum;
            (p[i] < 1.0 ? small : large).push_back((uint32_t)i);
        }
        while (!small.empty() && !large.empty()) {
            uint32_t s = small.back(); small.pop_back();
            uint32_t l = large.back(); large.pop_back();
            prob[s] = p[s];
            alias[s] = l;
            p[l] = (p[l] + p[s]) - 1.0;
            (p[l] < 1.0 ? small : large).push_back(l);
        }
        for (uint32_t l : large) { prob[l] = 1.0; alias[l] = l; }
        for (uint32_t s : small) { prob[s] = 1.0; alias[s] = s; }
    }
    inline uint32_t sample(uint64_t r) const {
        const uint32_t n = (uint32_t)prob.size();
        uint32_t i = (uint32_t)(((unsigned __int128)r * n) >> 64);
        double u = (double)(mix64(r) >> 11) * (1.0 / 9007199254740992.0);
        return u < prob[i] ? i : alias[i];
    }
};

// Draws undirected pairs from `draw(counter, &u, &v)` until `m` distinct
// non-loop pairs exist; keeps the first-drawn copy of every pair and the
// first m pairs in draw order, so the result is deterministic.
template <class Draw>
static void distinct_pairs(uint64_t m, uint64_t space, Draw draw, uint32_t* src, uint32_t* dst) {
    if (m > space) m = space;
    std::vector<uint64_t> keep;   // packed (min<<32 | max)
    std::vector<uint64_t> order;  // draw index of each kept pair
    uint64_t ctr = 0;
    while (keep.size() < m) {
        uint64_t need = m - keep.size();
        uint64_t batch = need + need / 8 + 1024;
        std::vector<std::pair<uint64_t, uint64_t>> fresh(batch);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < (int64_t)batch; ++i) {
            uint32_t u, v;
            draw(ctr + (uint64_t)i, u, v);
            uint64_t a = u < v ? u : v, b = u < v ? v : u;
            fresh[i] = {u == v ? ~0ull : (a << 32 | b), ctr + (uint64_t)i};
        }
        ctr += batch;
        // merge with already-kept pairs, dedup keeping the earliest draw
        std::vector<std::pair<uint64_t, uint64_t>> all;
        all.reserve(keep.size() + fresh.size());
        for (size_t i = 0; i < keep.size(); ++i) all.push_back({keep[i], order[i]});
        for (auto& f : fresh) if (f.first != ~0ull) all.push_back(f);
        std::sort(all.begin(), all.end());
        size_t w = 0;
        for (size_t i = 0; i < all.size(); ++i)
            if (i == 0 || all[i].first != all[i - 1].first) all[w++] = all[i];
        all.resize(w);
        std::sort(all.begin(), all.end(), [](const auto& x, const auto& y) { return x.second < y.second; });
        if (all.size() > m) all.resize(m);
        keep.resize(all.size());
        order.resize(all.size());
        for (size_t i = 0; i < all.size(); ++i) { keep[i] = all[i].first; order[i] = all[i].second; }
    }
    for (uint64_t i = 0; i < m; ++i) { src[i] = (uint32_t)(keep[i] >> 32); dst[i] = (uint32_t)keep[i]; }
}

}  // namespace kc

using namespace kc;

extern "C" {

int kc_gen_rmat(uint32_t n, uint64_t ne, double a, double b, double c, uint64_t seed,
                uint32_t* src, uint32_t* dst) {
    if (n == 0 || (ne && (!src || !dst)) || a < 0 || b < 0 || c < 0 || a + b + c > 1.0 + 1e-12) {
        set_error_msg("kc_gen_rmat: bad argument");
        return KC_ERR_INVALID;
    }
    const uint32_t scale = ceil_log2(n);
    const double ab = a + b, abc = a + b + c;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)ne; ++i) {
        for (uint64_t attempt = 0;; ++attempt) {
            uint64_t u = 0, v = 0;
            for (uint32_t l = 0; l < scale; ++l) {
                double r = rnd_unit(seed, ((uint64_t)i << 8) ^ attempt, l);
                uint64_t bu, bv;
                if (r < a) { bu = 0; bv = 0; }
                else if (r < ab) { bu = 0; bv = 1; }
                else if (r < abc) { bu = 1; bv = 0; }
                else { bu = 1; bv = 1; }
                u = (u << 1) | bu;
                v = (v << 1) | bv;
            }
            if (u < n && v < n) { src[i] = (uint32_t)u; dst[i] = (uint32_t)v; break; }
        }
    }
    std::vector<uint32_t> perm;
    seeded_permutation(n, seed ^ 0xA5A5A5A5ull, perm);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)ne; ++i) { src[i] = perm[src[i]]; dst[i] = perm[dst[i]]; }
    return KC_OK;
}

int kc_gen_chung_lu(uint32_t n, uint64_t m, double gamma, double max_w, uint64_t seed,
                    uint32_t* src, uint32_t* dst) {
    if (n < 2 || gamma <= 1.0 || max_w <= 0 || (m && (!src || !dst))) {
        set_error_msg("kc_gen_chung_lu: bad argument");
        return KC_ERR_INVALID;
    }
    const double beta = 1.0 / (gamma - 1.0);
    const double target = 2.0 * (double)m;
    // w_i = max_w * (i0 / (i + i0))^beta; find i0 so that sum w_i = 2m (bisection
    // on log i0; the sum grows with i0).
    // Fixed-order summation (1024 fixed chunks, then in order) so the result
    // does not depend on the thread count.
    auto wsum = [&](double i0) {
        const int64_t nch = 1024;
        std::vector<double> part(nch, 0.0);
#pragma omp parallel for schedule(static)
        for (int64_t c = 0; c < nch; ++c) {
            double s = 0;
            for (int64_t i = (int64_t)n * c / nch; i < (int64_t)n * (c + 1) / nch; ++i)
                s += std::pow(i0 / ((double)i + i0), beta);
            part[c] = s;
        }
        double s = 0;
        for (double x : part) s += x;
        return s * max_w;
    };
    double lo = 1e-6, hi = (double)n * 1e3;
    for (int it = 0; it < 80; ++it) {
        double mid = std::sqrt(lo * hi);
        if (wsum(mid) < target) lo = mid; else hi = mid;
    }
    const double i0 = std::sqrt(lo * hi);
    std::vector<double> w(n);
    for (uint32_t i = 0; i < n; ++i) w[i] = max_w * std::pow(i0 / ((double)i + i0), beta);
    Alias al;
    al.build(w);
    const uint64_t space = (uint64_t)n * (n - 1) / 2;
    distinct_pairs(m, space, [&](uint64_t k, uint32_t& u, uint32_t& v) {
        u = al.sample(rnd(seed, 1, 2 * k));
        v = al.sample(rnd(seed, 1, 2 * k + 1));
    }, src, dst);
    std::vector<uint32_t> perm;
    seeded_permutation(n, seed ^ 0xC3C3C3C3ull, perm);
    const uint64_t mm = std::min(m, space);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)mm; ++i) { src[i] = perm[src[i]]; dst[i] = perm[dst[i]]; }
    return KC_OK;
}

int kc_gen_er(uint32_t n, uint64_t m, uint64_t seed, uint32_t* src, uint32_t* dst) {
    if (n < 2 || (m && (!src || !dst))) {
        set_error_msg("kc_gen_er: bad argument");
        return KC_ERR_INVALID;
    }
    const uint64_t space = (uint64_t)n * (n - 1) / 2;
    distinct_pairs(m, space, [&](uint64_t k, uint32_t& u, uint32_t& v) {
        u = (uint32_t)(((unsigned __int128)rnd(seed, 2, 2 * k) * n) >> 64);
        v = (uint32_t)(((unsigned __int128)rnd(seed, 2, 2 * k + 1) * n) >> 64);
    }, src, dst);
    return KC_OK;
}

}  // extern "C"
