/*
 * Seeded workload generators of the oracle (TEST INFRASTRUCTURE ONLY).
 *
 * The CPU-only legs (the benchmark's reference arm, fixture scripts) build
 * their inputs here, so that they never load the product library.  The
 * streams are defined by the workload, not by any implementation: a tested
 * equality (tests/test_oracle_gen.py) shows that these functions return the
 * same bytes as the product's generators for the same arguments.
 *
 * Random source: xoshiro256** (Blackman and Vigna, 2018) seeded through
 * splitmix64 from (seed, stream); bounded integers by Lemire's multiply-shift
 * method with rejection of the biased low products (Lemire, 2019), on the
 * high 32 bits of each draw; unit doubles from the high 53 bits.
 *
 * Random digraph with a Hamiltonian chain (stream 1):
 *   1. Fisher-Yates shuffle of 0..n-1 (i from n-1 down to 1, j uniform in
 *      [0, i]) gives the chain order perm;
 *   2. chain arcs perm[i] -> perm[i+1] in order, each with a weight uniform in
 *      [wmin, wmax];
 *   3. extra arcs: draw u, then v, uniform in [0, n); reject self-loops and
 *      pairs already present; the weight is drawn after acceptance;
 *   4. CSR rows in generation order (stable counting sort by source).
 * Pairs (one stream per pair: 2^32 + index): source uniform; a hop count d
 * log-uniform in [lo, hi] (floor(exp(log lo + (log(hi+1) - log lo) u)),
 * clipped); when d <= bfs_cap, a FIFO BFS from the source over arcs in row
 * order for d levels, and the target uniform over the deepest non-empty
 * level reached (unless that is the source alone); otherwise, or in that
 * case, a uniform target other than the source.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    uint64_t a, b, c, d;
} xs256;

static uint64_t sm64(uint64_t *state) {
    uint64_t z = (*state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static void xs_seed(xs256 *r, uint64_t seed, uint64_t stream) {
    uint64_t st = seed ^ (stream * 0xD1B54A32D192ED03ull);
    r->a = sm64(&st);
    r->b = sm64(&st);
    r->c = sm64(&st);
    r->d = sm64(&st);
}

static inline uint64_t rol64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static inline uint64_t xs_next(xs256 *r) {
    const uint64_t out = rol64(r->b * 5, 7) * 9;
    const uint64_t t = r->b << 17;
    r->c ^= r->a;
    r->d ^= r->b;
    r->b ^= r->c;
    r->a ^= r->d;
    r->c ^= t;
    r->d = rol64(r->d, 45);
    return out;
}

static inline uint64_t xs_bounded(xs256 *r, uint64_t range) {
    if (range <= 1) return 0;
    const uint32_t bound = (uint32_t)range;
    uint64_t prod = (xs_next(r) >> 32) * range;
    if ((uint32_t)prod < bound) {
        const uint32_t reject_below = (uint32_t)(0u - bound) % bound;
        while ((uint32_t)prod < reject_below) prod = (xs_next(r) >> 32) * range;
    }
    return prod >> 32;
}

static inline double xs_unit(xs256 *r) { return (double)(xs_next(r) >> 11) / 9007199254740992.0; }

/* Open-addressed set of (u, v) arcs, Fibonacci hashing, linear probing. */
typedef struct {
    uint64_t *slot; /* 0 = empty, else (u << 32 | v) + 1 */
    uint64_t mask;
    int shift;
} arcset;

static int arcset_new(arcset *s, uint64_t expected) {
    int bits = 10;
    while ((1ull << bits) < 2 * expected) bits++;
    s->slot = (uint64_t *)calloc(1ull << bits, sizeof(uint64_t));
    s->mask = (1ull << bits) - 1;
    s->shift = 64 - bits;
    return s->slot ? 0 : -1;
}

/* inserts (u, v); returns 1 if it was new */
static int arcset_put(arcset *s, uint32_t u, uint32_t v) {
    const uint64_t key = (((uint64_t)u << 32) | v) + 1;
    uint64_t i = (key * 0x9E3779B97F4A7C15ull) >> s->shift;
    for (;; i = (i + 1) & s->mask) {
        if (s->slot[i] == key) return 0;
        if (s->slot[i] == 0) {
            s->slot[i] = key;
            return 1;
        }
    }
}

int oracle_gen_random_chain(int32_t n, int64_t e_total, uint32_t wmin, uint32_t wmax, uint64_t seed,
                            int32_t *off, int32_t *col, uint32_t *w, int32_t *perm_out) {
    if (n < 2 || e_total < n - 1 || wmax < wmin) return -1;
    if ((double)e_total > 0.5 * (double)n * (double)(n - 1)) return -1;
    xs256 r;
    xs_seed(&r, seed, 1);
    int32_t *perm = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    int32_t *src = (int32_t *)malloc(sizeof(int32_t) * (size_t)e_total);
    int32_t *dst = (int32_t *)malloc(sizeof(int32_t) * (size_t)e_total);
    uint32_t *wt = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)e_total);
    int32_t *next = (int32_t *)malloc(sizeof(int32_t) * ((size_t)n + 1));
    arcset set;
    set.slot = NULL;
    if (!perm || !src || !dst || !wt || !next || arcset_new(&set, (uint64_t)e_total)) {
        free(perm);
        free(src);
        free(dst);
        free(wt);
        free(next);
        free(set.slot);
        return -2;
    }
    const uint64_t span = (uint64_t)wmax - wmin + 1;
    for (int32_t i = 0; i < n; i++) perm[i] = i;
    for (int32_t i = n - 1; i >= 1; i--) {
        const int32_t j = (int32_t)xs_bounded(&r, (uint64_t)i + 1);
        const int32_t x = perm[i];
        perm[i] = perm[j];
        perm[j] = x;
    }
    int64_t k = 0;
    for (; k < n - 1; k++) {
        src[k] = perm[k];
        dst[k] = perm[k + 1];
        wt[k] = wmin + (uint32_t)xs_bounded(&r, span);
        arcset_put(&set, (uint32_t)src[k], (uint32_t)dst[k]);
    }
    while (k < e_total) {
        const uint32_t u = (uint32_t)xs_bounded(&r, (uint64_t)n);
        const uint32_t v = (uint32_t)xs_bounded(&r, (uint64_t)n);
        if (u == v || !arcset_put(&set, u, v)) continue;
        src[k] = (int32_t)u;
        dst[k] = (int32_t)v;
        wt[k] = wmin + (uint32_t)xs_bounded(&r, span);
        k++;
    }
    /* rows in generation order */
    for (int32_t i = 0; i <= n; i++) next[i] = 0;
    for (int64_t i = 0; i < k; i++) next[src[i] + 1]++;
    for (int32_t i = 0; i < n; i++) next[i + 1] += next[i];
    memcpy(off, next, sizeof(int32_t) * ((size_t)n + 1));
    for (int64_t i = 0; i < k; i++) {
        const int32_t at = next[src[i]]++;
        col[at] = dst[i];
        w[at] = wt[i];
    }
    if (perm_out) memcpy(perm_out, perm, sizeof(int32_t) * (size_t)n);
    free(perm);
    free(src);
    free(dst);
    free(wt);
    free(next);
    free(set.slot);
    return 0;
}

typedef struct {
    int32_t n;
    const int32_t *off, *col;
    int32_t npairs, lo, hi, bfs_cap;
    uint64_t seed;
    int32_t *S, *T, *want;
    int32_t claimed;
    pthread_mutex_t lock;
} pairjob;

static void *pair_thread(void *arg) {
    pairjob *J = (pairjob *)arg;
    const int32_t n = J->n;
    int32_t *level = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    int32_t *fifo = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    if (!level || !fifo) {
        free(level);
        free(fifo);
        return NULL;
    }
    memset(level, 0xFF, sizeof(int32_t) * (size_t)n); /* -1: not seen */
    for (;;) {
        pthread_mutex_lock(&J->lock);
        const int32_t p = J->claimed < J->npairs ? J->claimed++ : -1;
        pthread_mutex_unlock(&J->lock);
        if (p < 0) break;
        xs256 r;
        xs_seed(&r, J->seed, 0x100000000ull + (uint64_t)p);
        const int32_t s = (int32_t)xs_bounded(&r, (uint64_t)n);
        const double a = log((double)J->lo), b = log((double)J->hi + 1.0);
        int32_t d = (int32_t)floor(exp(a + (b - a) * xs_unit(&r)));
        d = d < J->lo ? J->lo : d > J->hi ? J->hi : d;
        J->want[p] = d;
        J->S[p] = s;
        int32_t t = -1;
        if (d <= J->bfs_cap) {
            int32_t head = 0, tail = 0;
            int32_t deep_b = 0, deep_e = 1; /* deepest non-empty level: [deep_b, deep_e) */
            level[s] = 0;
            fifo[tail++] = s;
            for (int32_t depth = 0; depth < d && head < tail; depth++) {
                const int32_t end = tail;
                for (; head < end; head++) {
                    const int32_t u = fifo[head];
                    for (int32_t k = J->off[u]; k < J->off[u + 1]; k++) {
                        const int32_t v = J->col[k];
                        if (v < 0 || level[v] >= 0) continue;
                        level[v] = depth + 1;
                        fifo[tail++] = v;
                    }
                }
                if (tail > end) {
                    deep_b = end;
                    deep_e = tail;
                }
            }
            if (deep_e > deep_b && !(deep_b == 0 && deep_e == 1))
                t = fifo[deep_b + (int32_t)xs_bounded(&r, (uint64_t)(deep_e - deep_b))];
            for (int32_t i = 0; i < tail; i++) level[fifo[i]] = -1;
        }
        while (t < 0 || (t == s && n > 1)) t = (int32_t)xs_bounded(&r, (uint64_t)n);
        J->T[p] = t;
    }
    free(level);
    free(fifo);
    return NULL;
}

int oracle_gen_pairs(int32_t n, const int32_t *off, const int32_t *col, int32_t npairs, int32_t hop_lo,
                     int32_t hop_hi, int32_t bfs_cap_level, uint64_t seed, int32_t threads, int32_t *S,
                     int32_t *T, int32_t *want_hops) {
    if (n < 2 || npairs < 0 || hop_lo < 1 || hop_hi < hop_lo) return -1;
    pairjob J;
    J.n = n;
    J.off = off;
    J.col = col;
    J.npairs = npairs;
    J.lo = hop_lo;
    J.hi = hop_hi;
    J.bfs_cap = bfs_cap_level;
    J.seed = seed;
    J.S = S;
    J.T = T;
    J.want = want_hops;
    J.claimed = 0;
    pthread_mutex_init(&J.lock, NULL);
    if (threads < 1) threads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)threads);
    if (!th) return -2;
    for (int i = 0; i < threads; i++) pthread_create(&th[i], NULL, pair_thread, &J);
    for (int i = 0; i < threads; i++) pthread_join(th[i], NULL);
    free(th);
    pthread_mutex_destroy(&J.lock);
    return 0;
}
