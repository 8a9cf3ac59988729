/*
 * kc_gen_oracle.c - TEST INFRASTRUCTURE ONLY.  A second, independent
 * implementation of the seeded benchmark workloads (R-MAT, Chung-Lu, Erdos-
 * Renyi, the 4,096-graph batch) and of the reference CSR build
 * (src/graph.cpp:84-122: self-loops dropped, symmetrised, deduplicated,
 * neighbours ascending, V = max id + 1).  bench.py's reference arm builds its
 * input graphs with it, so that arm never maps the product library, and the
 * CPU tests require its CSR bytes to equal the product generator's.
 *
 * The workload definitions (one per generator, stated once here):
 *   rnd(seed, stream, ctr) = f(f(seed ^ K1) ^ f(stream * K2 + ctr)), f = the
 *     splitmix64 finaliser; unit(...) = (rnd >> 11) * 2^-53.
 *   R-MAT(n, ne, a, b, c, seed): scale = ceil(log2 n); draw i, attempt t picks
 *     one quadrant per bit l with unit(seed, (i << 8) ^ t, l) against a, a+b,
 *     a+b+c; endpoints >= n are redrawn (t + 1); then every id is relabelled
 *     by a seeded Fisher-Yates permutation (seed ^ 0xA5A5A5A5).
 *   Chung-Lu(n, m, gamma, max_w, seed): w_i = max_w (i0 / (i + i0))^(1/(gamma-1))
 *     with i0 found by 80 geometric bisection steps so that sum w_i = 2m (the
 *     sum over 1,024 fixed chunks, in order); endpoints by Vose alias sampling
 *     of rnd(seed, 1, 2k) and rnd(seed, 1, 2k+1); the first m distinct
 *     non-loop pairs in draw order, each as (min, max); relabelled with
 *     seed ^ 0xC3C3C3C3.
 *   ER(n, m, seed): endpoints floor(rnd(seed, 2, 2k|2k+1) * n / 2^64); the
 *     first m distinct non-loop pairs in draw order as (min, max).
 *   batch(G, seed_base, nmin, nmax, dmin, dmax, a, b, c): graph g, seed s =
 *     seed_base + g: n = floor(exp(ln nmin + unit(s,7,0) (ln nmax - ln nmin))),
 *     d = dmin + unit(s,7,1) (dmax - dmin), m = round(n d / 2); even g ER(n, m, s),
 *     odd g R-MAT(n, m, a, b, c, s); each graph CSR-built on its own.
 *
 * Compiled without floating-point contraction (as the product generator is),
 * so both evaluate every expression with the same roundings on any host.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

static inline uint64_t g_mix(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
static inline uint64_t g_rnd(uint64_t seed, uint64_t stream, uint64_t ctr) {
    return g_mix(g_mix(seed ^ 0xD1B54A32D192ED03ull) ^ g_mix(stream * 0x9E3779B97F4A7C15ull + ctr));
}
static inline double g_unit(uint64_t seed, uint64_t stream, uint64_t ctr) {
    return (double)(g_rnd(seed, stream, ctr) >> 11) * (1.0 / 9007199254740992.0);
}
/* floor(r * n / 2^64) */
static inline uint32_t g_scale(uint64_t r, uint32_t n) {
    return (uint32_t)(((unsigned __int128)r * n) >> 64);
}

static uint32_t* g_permutation(uint32_t n, uint64_t seed) {
    uint32_t* p = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
    if (!p) return NULL;
    for (uint32_t i = 0; i < n; ++i) p[i] = i;
    for (uint32_t i = n; i > 1; --i) {
        const uint32_t j = g_scale(g_rnd(seed, 0x5EED, i), i);
        const uint32_t t = p[i - 1];
        p[i - 1] = p[j];
        p[j] = t;
    }
    return p;
}

int kco_gen_rmat(uint32_t n, uint64_t ne, double a, double b, double c, uint64_t seed, uint32_t* src,
                 uint32_t* dst) {
    if (n == 0) return -8;
    uint32_t scale = 0;
    while (scale < 32 && (1ull << scale) < (uint64_t)n) ++scale;
    const double ab = a + b, abc = a + b + c;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)ne; ++i) {
        for (uint64_t t = 0;; ++t) {
            uint64_t u = 0, v = 0;
            for (uint32_t l = 0; l < scale; ++l) {
                const double r = g_unit(seed, ((uint64_t)i << 8) ^ t, l);
                const uint64_t bu = r < ab ? 0 : 1;
                const uint64_t bv = (r < a || (r >= ab && r < abc)) ? 0 : 1;
                u = (u << 1) | bu;
                v = (v << 1) | bv;
            }
            if (u < n && v < n) { src[i] = (uint32_t)u; dst[i] = (uint32_t)v; break; }
        }
    }
    uint32_t* p = g_permutation(n, seed ^ 0xA5A5A5A5ull);
    if (!p) return -3;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)ne; ++i) { src[i] = p[src[i]]; dst[i] = p[dst[i]]; }
    free(p);
    return 0;
}

/* Open-addressing set of packed (min << 32 | max) pairs; 0 marks an empty
 * slot (pair (0,0) is a self-loop and never stored). */
typedef struct { uint64_t* slot; uint64_t mask; } g_set;

static int g_set_init(g_set* s, uint64_t m) {
    uint64_t cap = 1024;
    while (cap < 2 * m + 16) cap <<= 1;
    s->slot = (uint64_t*)calloc(cap, sizeof(uint64_t));
    s->mask = cap - 1;
    return s->slot ? 0 : -3;
}
static int g_set_insert(g_set* s, uint64_t key) {   /* 1 when new */
    uint64_t h = g_mix(key) & s->mask;
    for (;;) {
        if (s->slot[h] == 0) { s->slot[h] = key; return 1; }
        if (s->slot[h] == key) return 0;
        h = (h + 1) & s->mask;
    }
}

/* The first m distinct non-loop pairs in draw order; draw(k) gives the
 * endpoints of draw k.  Draws are computed in parallel blocks and kept in
 * order by one thread. */
typedef void (*g_draw_fn)(const void* ctx, uint64_t k, uint32_t* u, uint32_t* v);

static int g_distinct(uint64_t m, g_draw_fn draw, const void* ctx, uint32_t* src, uint32_t* dst) {
    g_set s;
    if (g_set_init(&s, m)) return -3;
    const int64_t blk = 1 << 20;
    uint64_t* keys = (uint64_t*)malloc(sizeof(uint64_t) * blk);
    if (!keys) { free(s.slot); return -3; }
    uint64_t kept = 0, ctr = 0;
    while (kept < m) {
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < blk; ++i) {
            uint32_t u, v;
            draw(ctx, ctr + (uint64_t)i, &u, &v);
            const uint64_t lo = u < v ? u : v, hi = u < v ? v : u;
            keys[i] = u == v ? 0 : (lo << 32 | hi);
        }
        for (int64_t i = 0; i < blk && kept < m; ++i) {
            if (keys[i] == 0 || !g_set_insert(&s, keys[i])) continue;
            src[kept] = (uint32_t)(keys[i] >> 32);
            dst[kept] = (uint32_t)keys[i];
            ++kept;
        }
        ctr += (uint64_t)blk;
    }
    free(keys);
    free(s.slot);
    return 0;
}

typedef struct { uint32_t n; uint64_t seed; } g_er_ctx;
static void g_er_draw(const void* c, uint64_t k, uint32_t* u, uint32_t* v) {
    const g_er_ctx* x = (const g_er_ctx*)c;
    *u = g_scale(g_rnd(x->seed, 2, 2 * k), x->n);
    *v = g_scale(g_rnd(x->seed, 2, 2 * k + 1), x->n);
}

int kco_gen_er(uint32_t n, uint64_t m, uint64_t seed, uint32_t* src, uint32_t* dst) {
    if (n < 2) return -8;
    const uint64_t space = (uint64_t)n * (n - 1) / 2;
    if (m > space) m = space;
    g_er_ctx c = {n, seed};
    return g_distinct(m, g_er_draw, &c, src, dst);
}

typedef struct { uint32_t n; uint64_t seed; const double* prob; const uint32_t* alias; } g_cl_ctx;
static inline uint32_t g_alias_sample(const g_cl_ctx* x, uint64_t r) {
    const uint32_t i = g_scale(r, x->n);
    const double u = (double)(g_mix(r) >> 11) * (1.0 / 9007199254740992.0);
    return u < x->prob[i] ? i : x->alias[i];
}
static void g_cl_draw(const void* c, uint64_t k, uint32_t* u, uint32_t* v) {
    const g_cl_ctx* x = (const g_cl_ctx*)c;
    *u = g_alias_sample(x, g_rnd(x->seed, 1, 2 * k));
    *v = g_alias_sample(x, g_rnd(x->seed, 1, 2 * k + 1));
}

static double g_cl_sum(uint32_t n, double i0, double beta, double max_w) {
    enum { NCH = 1024 };
    double part[NCH];
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < NCH; ++c) {
        double s = 0;
        for (int64_t i = (int64_t)n * c / NCH; i < (int64_t)n * (c + 1) / NCH; ++i) s += pow(i0 / ((double)i + i0), beta);
        part[c] = s;
    }
    double s = 0;
    for (int c = 0; c < NCH; ++c) s += part[c];
    return s * max_w;
}

int kco_gen_chung_lu(uint32_t n, uint64_t m, double gamma, double max_w, uint64_t seed, uint32_t* src,
                     uint32_t* dst) {
    if (n < 2 || gamma <= 1.0 || max_w <= 0) return -8;
    const double beta = 1.0 / (gamma - 1.0);
    const double target = 2.0 * (double)m;
    double lo = 1e-6, hi = (double)n * 1e3;
    for (int it = 0; it < 80; ++it) {
        const double mid = sqrt(lo * hi);
        if (g_cl_sum(n, mid, beta, max_w) < target) lo = mid; else hi = mid;
    }
    const double i0 = sqrt(lo * hi);
    double* w = (double*)malloc(sizeof(double) * n);
    double* prob = (double*)malloc(sizeof(double) * n);
    uint32_t* alias = (uint32_t*)malloc(sizeof(uint32_t) * n);
    uint32_t* small = (uint32_t*)malloc(sizeof(uint32_t) * n);
    uint32_t* large = (uint32_t*)malloc(sizeof(uint32_t) * n);
    if (!w || !prob || !alias || !small || !large) {
        free(w); free(prob); free(alias); free(small); free(large);
        return -3;
    }
    double sum = 0;
    for (uint32_t i = 0; i < n; ++i) { w[i] = max_w * pow(i0 / ((double)i + i0), beta); sum += w[i]; }
    /* Vose's alias method; w becomes the scaled probabilities */
    uint32_t ns = 0, nl = 0;
    for (uint32_t i = 0; i < n; ++i) {
        prob[i] = 0;
        alias[i] = 0;
        w[i] = w[i] * (double)n / sum;
        if (w[i] < 1.0) small[ns++] = i; else large[nl++] = i;
    }
    while (ns && nl) {
        const uint32_t s = small[--ns], l = large[--nl];
        prob[s] = w[s];
        alias[s] = l;
        w[l] = (w[l] + w[s]) - 1.0;
        if (w[l] < 1.0) small[ns++] = l; else large[nl++] = l;
    }
    for (uint32_t k = 0; k < nl; ++k) { prob[large[k]] = 1.0; alias[large[k]] = large[k]; }
    for (uint32_t k = 0; k < ns; ++k) { prob[small[k]] = 1.0; alias[small[k]] = small[k]; }
    free(small); free(large); free(w);
    const uint64_t space = (uint64_t)n * (n - 1) / 2;
    if (m > space) m = space;
    g_cl_ctx c = {n, seed, prob, alias};
    int rc = g_distinct(m, g_cl_draw, &c, src, dst);
    free(prob); free(alias);
    if (rc) return rc;
    uint32_t* p = g_permutation(n, seed ^ 0xC3C3C3C3ull);
    if (!p) return -3;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)m; ++i) { src[i] = p[src[i]]; dst[i] = p[dst[i]]; }
    free(p);
    return 0;
}

static int g_cmp_u32(const void* x, const void* y) {
    const uint32_t a = *(const uint32_t*)x, b = *(const uint32_t*)y;
    return a < b ? -1 : a > b;
}

/* Reference CSR of ne directed pairs (graph.cpp:84-122).  *off_out (V+1) and
 * *nbr_out (E) are malloc'ed; free them with kco_free. */
int kco_build_csr(const uint32_t* src, const uint32_t* dst, uint64_t ne, uint32_t* V_out, uint64_t* E_out,
                  uint32_t** off_out, uint32_t** nbr_out) {
    uint32_t vmax = 0;
    for (uint64_t i = 0; i < ne; ++i)
        if (src[i] != dst[i]) {
            const uint32_t x = src[i] > dst[i] ? src[i] : dst[i];
            if (x > vmax) vmax = x;
        }
    if (vmax == 0xFFFFFFFFu) return -8;
    const uint32_t V = vmax + 1;
    uint64_t* start = (uint64_t*)calloc((size_t)V + 1, sizeof(uint64_t));
    if (!start) return -3;
    for (uint64_t i = 0; i < ne; ++i)
        if (src[i] != dst[i]) { start[src[i] + 1]++; start[dst[i] + 1]++; }
    for (uint32_t v = 0; v < V; ++v) start[v + 1] += start[v];
    const uint64_t raw_n = start[V];
    uint32_t* raw = (uint32_t*)malloc(sizeof(uint32_t) * (raw_n ? raw_n : 1));
    uint64_t* cur = (uint64_t*)malloc(sizeof(uint64_t) * ((size_t)V + 1));
    uint32_t* deg = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)V + 1));
    if (!raw || !cur || !deg) { free(start); free(raw); free(cur); free(deg); return -3; }
    memcpy(cur, start, sizeof(uint64_t) * V);
    for (uint64_t i = 0; i < ne; ++i)
        if (src[i] != dst[i]) { raw[cur[src[i]]++] = dst[i]; raw[cur[dst[i]]++] = src[i]; }
    free(cur);
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t v = 0; v < (int64_t)V; ++v) {
        uint32_t* b = raw + start[v];
        const uint64_t len = start[v + 1] - start[v];
        qsort(b, len, sizeof(uint32_t), g_cmp_u32);
        uint64_t k = 0;
        for (uint64_t j = 0; j < len; ++j)
            if (j == 0 || b[j] != b[j - 1]) b[k++] = b[j];
        deg[v] = (uint32_t)k;
    }
    uint64_t E = 0;
    for (uint32_t v = 0; v < V; ++v) E += deg[v];
    if (E > 0xFFFFFFFFull) { free(start); free(raw); free(deg); return -8; }
    uint32_t* off = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)V + 1));
    uint32_t* nbr = (uint32_t*)malloc(sizeof(uint32_t) * (E ? E : 1));
    if (!off || !nbr) { free(start); free(raw); free(deg); free(off); free(nbr); return -3; }
    off[0] = 0;
    for (uint32_t v = 0; v < V; ++v) off[v + 1] = off[v] + deg[v];
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t v = 0; v < (int64_t)V; ++v)
        memcpy(nbr + off[v], raw + start[v], sizeof(uint32_t) * deg[v]);
    free(start); free(raw); free(deg);
    *V_out = V;
    *E_out = E;
    *off_out = off;
    *nbr_out = nbr;
    return 0;
}

void kco_free(void* p) { free(p); }

/* The batch: per-graph sizes as in the header comment; returns the segmented
 * CSR (vbase/abase ngraphs+1 entries; graph g's V_g+1 local offsets at
 * vbase[g]+g; its local neighbour ids at abase[g]).  All four arrays are
 * malloc'ed (kco_free). */
int kco_gen_batch(uint32_t ngraphs, uint64_t seed_base, uint32_t nmin, uint32_t nmax, double dmin, double dmax,
                  double a, double b, double c, uint64_t** vbase, uint64_t** abase, uint32_t** offsets,
                  uint32_t** neighbors) {
    if (ngraphs == 0 || nmin < 2 || nmax < nmin || dmin <= 0 || dmax < dmin) return -8;
    uint32_t* gV = (uint32_t*)calloc(ngraphs, sizeof(uint32_t));
    uint64_t* gE = (uint64_t*)calloc(ngraphs, sizeof(uint64_t));
    uint32_t** gO = (uint32_t**)calloc(ngraphs, sizeof(uint32_t*));
    uint32_t** gN = (uint32_t**)calloc(ngraphs, sizeof(uint32_t*));
    if (!gV || !gE || !gO || !gN) { free(gV); free(gE); free(gO); free(gN); return -3; }
    int bad = 0;
    const int nested = omp_get_max_active_levels();
    omp_set_max_active_levels(1);
#pragma omp parallel for schedule(dynamic, 1) reduction(| : bad)
    for (int64_t g = 0; g < (int64_t)ngraphs; ++g) {
        const uint64_t s = seed_base + (uint64_t)g;
        const double u1 = g_unit(s, 7, 0), u2 = g_unit(s, 7, 1);
        const uint32_t n = (uint32_t)floor(exp(log((double)nmin) + u1 * (log((double)nmax) - log((double)nmin))));
        const double d = dmin + u2 * (dmax - dmin);
        const uint64_t m = (uint64_t)llround((double)n * d / 2.0);
        uint32_t* S = (uint32_t*)malloc(sizeof(uint32_t) * (m ? m : 1));
        uint32_t* T = (uint32_t*)malloc(sizeof(uint32_t) * (m ? m : 1));
        int rc = (!S || !T) ? -3 : (g % 2 == 0) ? kco_gen_er(n, m, s, S, T) : kco_gen_rmat(n, m, a, b, c, s, S, T);
        if (rc == 0) rc = kco_build_csr(S, T, m, &gV[g], &gE[g], &gO[g], &gN[g]);
        free(S); free(T);
        if (rc) bad = 1;
    }
    omp_set_max_active_levels(nested);
    uint64_t* vb = bad ? NULL : (uint64_t*)malloc(8 * ((size_t)ngraphs + 1));
    uint64_t* ab = bad ? NULL : (uint64_t*)malloc(8 * ((size_t)ngraphs + 1));
    uint32_t *O = NULL, *N = NULL;
    if (vb && ab) {
        vb[0] = ab[0] = 0;
        for (uint32_t g = 0; g < ngraphs; ++g) { vb[g + 1] = vb[g] + gV[g]; ab[g + 1] = ab[g] + gE[g]; }
        O = (uint32_t*)malloc(4 * ((size_t)vb[ngraphs] + ngraphs));
        N = (uint32_t*)malloc(4 * (size_t)(ab[ngraphs] ? ab[ngraphs] : 1));
    }
    const int ok = vb && ab && O && N;
    for (uint32_t g = 0; g < ngraphs; ++g) {
        if (ok) {
            memcpy(O + vb[g] + g, gO[g], 4 * ((size_t)gV[g] + 1));
            if (gE[g]) memcpy(N + ab[g], gN[g], 4 * (size_t)gE[g]);
        }
        free(gO[g]);
        free(gN[g]);
    }
    free(gV); free(gE); free(gO); free(gN);
    if (!ok) { free(vb); free(ab); free(O); free(N); return -3; }
    *vbase = vb;
    *abase = ab;
    *offsets = O;
    *neighbors = N;
    return 0;
}
