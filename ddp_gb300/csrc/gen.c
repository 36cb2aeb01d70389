/*
 * Seeded workload generators for the GA* / dynamic A* path.
 *
 * These replace the reference's generator programs with deterministic,
 * seed-addressed C (same results on x86_64 and aarch64; no rand(), no
 * platform-dependent integer widths):
 *   - random digraph with a Hamiltonian chain (GA_star/GenerateCSR.cpp
 *     builds the CSR from an edge list; GA_star/randomGraph.py and
 *     genGraph.py draw the edges; the chain guarantees reachability),
 *   - 4-connected grid maze with random walls and a carved corridor
 *     (maze/create_maze.cpp:69-113, same arc order up/down/right/left),
 *   - insert/delete update batches (DA_star/genDynamicGraph.cpp:122-173
 *     writes Updates.txt; here deletes are drawn too, chain arcs protected),
 *   - source/target pairs with a target BFS hop distance.
 * All CSR outputs here use N+1 offsets (off[N] = E).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "ddp_gb300.h"

/* ---------------- PRNG: splitmix64 seeding, xoshiro256** stream -------- */
typedef struct {
    uint64_t s[4];
} rng_t;

static uint64_t splitmix64(uint64_t *x) {
    uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static void rng_seed(rng_t *r, uint64_t seed, uint64_t stream) {
    uint64_t x = seed ^ (stream * 0xD1B54A32D192ED03ull);
    for (int i = 0; i < 4; i++) r->s[i] = splitmix64(&x);
}

static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static inline uint64_t rng_next(rng_t *r) {
    uint64_t *s = r->s;
    uint64_t result = rotl(s[1] * 5, 7) * 9;
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return result;
}

/* uniform integer in [0, n) without modulo bias (Lemire) */
static inline uint64_t rng_below(rng_t *r, uint64_t n) {
    if (n <= 1) return 0;
    uint64_t x = rng_next(r) >> 32; /* 32-bit draws suffice for n < 2^32 */
    uint64_t m = x * n;
    uint32_t l = (uint32_t)m;
    if (l < (uint32_t)n) {
        uint32_t t = (uint32_t)(-(uint32_t)n) % (uint32_t)n;
        while (l < t) {
            x = rng_next(r) >> 32;
            m = x * n;
            l = (uint32_t)m;
        }
    }
    return m >> 32;
}

static inline double rng_unit(rng_t *r) { return (double)(rng_next(r) >> 11) * (1.0 / 9007199254740992.0); }

/* ---------------- (u,v) hash set with multiplicity ---------------------- */
typedef struct {
    uint64_t *keys; /* 0 = empty, 1 = tombstone, else (u<<32 | v) + 2 */
    uint64_t mask;
} pairset_t;

static int pairset_init(pairset_t *p, uint64_t expected) {
    uint64_t cap = 1024;
    while (cap < expected * 2) cap <<= 1;
    p->keys = (uint64_t *)calloc(cap, sizeof(uint64_t));
    p->mask = cap - 1;
    return p->keys ? 0 : -1;
}

static inline uint64_t pair_key(uint32_t u, uint32_t v) { return (((uint64_t)u << 32) | v) + 2; }

static inline uint64_t pair_hash(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    return k;
}

static int pairset_has(const pairset_t *p, uint32_t u, uint32_t v) {
    uint64_t k = pair_key(u, v), i = pair_hash(k) & p->mask;
    for (;;) {
        uint64_t c = p->keys[i];
        if (c == 0) return 0;
        if (c == k) return 1;
        i = (i + 1) & p->mask;
    }
}

static void pairset_add(pairset_t *p, uint32_t u, uint32_t v) {
    uint64_t k = pair_key(u, v), i = pair_hash(k) & p->mask;
    for (;;) {
        uint64_t c = p->keys[i];
        if (c == 0 || c == 1) {
            p->keys[i] = k;
            return;
        }
        i = (i + 1) & p->mask;
    }
}

static void pairset_del(pairset_t *p, uint32_t u, uint32_t v) {
    uint64_t k = pair_key(u, v), i = pair_hash(k) & p->mask;
    for (;;) {
        uint64_t c = p->keys[i];
        if (c == 0) return;
        if (c == k) {
            p->keys[i] = 1;
            return;
        }
        i = (i + 1) & p->mask;
    }
}

/* ---------------- random digraph with a Hamiltonian chain --------------- */
int ddp_gen_random_chain(int32_t n, int64_t e_total, uint32_t wmin, uint32_t wmax, uint64_t seed,
                         int32_t *off, int32_t *col, uint32_t *w, int32_t *perm_out) {
    if (n < 2 || e_total < n - 1 || wmax < wmin) return -1;
    if ((double)e_total > 0.5 * (double)n * (double)(n - 1)) return -1; /* too dense to sample */
    rng_t r;
    rng_seed(&r, seed, 1);
    int32_t *perm = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    int32_t *au = (int32_t *)malloc(sizeof(int32_t) * (size_t)e_total);
    int32_t *av = (int32_t *)malloc(sizeof(int32_t) * (size_t)e_total);
    uint32_t *aw = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)e_total);
    pairset_t ps;
    if (!perm || !au || !av || !aw || pairset_init(&ps, (uint64_t)e_total)) {
        free(perm);
        free(au);
        free(av);
        free(aw);
        return -2;
    }
    for (int32_t i = 0; i < n; i++) perm[i] = i;
    for (int32_t i = n - 1; i > 0; i--) {
        int32_t j = (int32_t)rng_below(&r, (uint64_t)i + 1);
        int32_t t = perm[i];
        perm[i] = perm[j];
        perm[j] = t;
    }
    uint64_t wspan = (uint64_t)wmax - wmin + 1;
    int64_t m = 0;
    for (int32_t i = 0; i + 1 < n; i++) {
        au[m] = perm[i];
        av[m] = perm[i + 1];
        aw[m] = wmin + (uint32_t)rng_below(&r, wspan);
        pairset_add(&ps, (uint32_t)perm[i], (uint32_t)perm[i + 1]);
        m++;
    }
    while (m < e_total) {
        uint32_t u = (uint32_t)rng_below(&r, (uint64_t)n);
        uint32_t v = (uint32_t)rng_below(&r, (uint64_t)n);
        if (u == v || pairset_has(&ps, u, v)) continue;
        pairset_add(&ps, u, v);
        au[m] = (int32_t)u;
        av[m] = (int32_t)v;
        aw[m] = wmin + (uint32_t)rng_below(&r, wspan);
        m++;
    }
    /* counting sort by source, stable in generation order */
    memset(off, 0, sizeof(int32_t) * ((size_t)n + 1));
    for (int64_t i = 0; i < m; i++) off[au[i] + 1]++;
    for (int32_t i = 0; i < n; i++) off[i + 1] += off[i];
    int32_t *fill = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    memcpy(fill, off, sizeof(int32_t) * (size_t)n);
    for (int64_t i = 0; i < m; i++) {
        int32_t k = fill[au[i]]++;
        col[k] = av[i];
        w[k] = aw[i];
    }
    if (perm_out) memcpy(perm_out, perm, sizeof(int32_t) * (size_t)n);
    free(fill);
    free(perm);
    free(au);
    free(av);
    free(aw);
    free(ps.keys);
    return 0;
}

/* ---------------- grid maze ---------------------------------------------- */
int ddp_gen_maze(int32_t rows, int32_t cols, uint32_t wall_permille, uint64_t seed,
                 int32_t *cell_node, int32_t *n_nodes, int64_t *n_arcs, int32_t *off, int32_t *col,
                 uint32_t *w, int32_t *xy) {
    if (rows < 1 || cols < 1 || wall_permille > 1000) return -1;
    rng_t r;
    rng_seed(&r, seed, 2);
    int64_t cells = (int64_t)rows * cols;
    uint8_t *wall = (uint8_t *)malloc((size_t)cells);
    if (!wall) return -2;
    for (int64_t i = 0; i < cells; i++) wall[i] = rng_below(&r, 1000) < wall_permille;
    /* carve a random monotone corridor (0,0) -> (rows-1, cols-1) */
    int32_t i = 0, j = 0;
    wall[0] = 0;
    while (i != rows - 1 || j != cols - 1) {
        if (i == rows - 1) j++;
        else if (j == cols - 1) i++;
        else if (rng_below(&r, 2)) j++;
        else i++;
        wall[(int64_t)i * cols + j] = 0;
    }
    int32_t n = 0;
    for (int64_t c = 0; c < cells; c++) cell_node[c] = wall[c] ? -1 : n++;
    int64_t m = 0;
    for (i = 0; i < rows; i++) {
        for (j = 0; j < cols; j++) {
            int64_t c = (int64_t)i * cols + j;
            if (wall[c]) continue;
            int32_t u = cell_node[c];
            off[u] = (int32_t)m;
            xy[2 * u] = j;
            xy[2 * u + 1] = i;
            /* arc order of maze/create_maze.cpp:93-111: up, down, right, left */
            if (i > 0 && !wall[c - cols]) { col[m] = cell_node[c - cols]; w[m++] = 1; }
            if (i < rows - 1 && !wall[c + cols]) { col[m] = cell_node[c + cols]; w[m++] = 1; }
            if (j < cols - 1 && !wall[c + 1]) { col[m] = cell_node[c + 1]; w[m++] = 1; }
            if (j > 0 && !wall[c - 1]) { col[m] = cell_node[c - 1]; w[m++] = 1; }
        }
    }
    off[n] = (int32_t)m;
    *n_nodes = n;
    *n_arcs = m;
    free(wall);
    return 0;
}

/* ---------------- update batches ---------------------------------------- */
typedef struct {
    int32_t u, v;
    uint32_t w;
} arc_t;

int ddp_gen_updates(int32_t n, int64_t e, const int32_t *off, const int32_t *col, const uint32_t *w,
                    const int32_t *protect_next, int32_t nbatches, int32_t per_batch,
                    int32_t inserts_per_batch, uint32_t wmin, uint32_t wmax, uint64_t seed,
                    int32_t *flag, int32_t *uu, int32_t *vv, uint32_t *ww) {
    if (n < 2 || inserts_per_batch > per_batch || wmax < wmin) return -1;
    rng_t r;
    rng_seed(&r, seed, 3);
    int64_t total_ins = (int64_t)nbatches * inserts_per_batch;
    pairset_t ps;
    if (pairset_init(&ps, (uint64_t)(e + total_ins))) return -2;
    arc_t *pool = (arc_t *)malloc(sizeof(arc_t) * (size_t)(e + total_ins + 1));
    arc_t *pending = (arc_t *)malloc(sizeof(arc_t) * (size_t)(inserts_per_batch + 1));
    if (!pool || !pending) {
        free(ps.keys);
        free(pool);
        free(pending);
        return -2;
    }
    int64_t np = 0;
    for (int32_t u = 0; u < n; u++) {
        for (int32_t k = off[u]; k < off[u + 1]; k++) {
            int32_t v = col[k];
            if (v < 0) continue;
            pairset_add(&ps, (uint32_t)u, (uint32_t)v);
            if (protect_next && protect_next[u] == v) continue;
            pool[np].u = u;
            pool[np].v = v;
            pool[np].w = w[k];
            np++;
        }
    }
    uint64_t wspan = (uint64_t)wmax - wmin + 1;
    int64_t o = 0;
    int32_t ndel = per_batch - inserts_per_batch;
    for (int32_t b = 0; b < nbatches; b++) {
        /* inserts: arcs absent from the pre-batch graph */
        for (int32_t k = 0; k < inserts_per_batch; k++) {
            uint32_t u, v;
            do {
                u = (uint32_t)rng_below(&r, (uint64_t)n);
                v = (uint32_t)rng_below(&r, (uint64_t)n);
            } while (u == v || pairset_has(&ps, u, v));
            pairset_add(&ps, u, v);
            pending[k].u = (int32_t)u;
            pending[k].v = (int32_t)v;
            pending[k].w = wmin + (uint32_t)rng_below(&r, wspan);
            flag[o] = 1;
            uu[o] = (int32_t)u;
            vv[o] = (int32_t)v;
            ww[o] = pending[k].w;
            o++;
        }
        /* deletes: uniform over live, unprotected arcs of the pre-batch graph */
        for (int32_t k = 0; k < ndel; k++) {
            if (np == 0) {
                flag[o] = 0;
                uu[o] = vv[o] = -1;
                ww[o] = 0;
                o++;
                continue;
            }
            int64_t idx = (int64_t)rng_below(&r, (uint64_t)np);
            arc_t a = pool[idx];
            pool[idx] = pool[np - 1];
            np--;
            pairset_del(&ps, (uint32_t)a.u, (uint32_t)a.v);
            flag[o] = 0;
            uu[o] = a.u;
            vv[o] = a.v;
            ww[o] = a.w;
            o++;
        }
        for (int32_t k = 0; k < inserts_per_batch; k++) pool[np++] = pending[k];
    }
    free(ps.keys);
    free(pool);
    free(pending);
    return 0;
}

/* ---------------- source/target pairs ----------------------------------- */
typedef struct {
    int32_t n;
    const int32_t *off, *col;
    int32_t npairs, hop_lo, hop_hi, bfs_cap;
    uint64_t seed;
    int32_t *S, *T, *want;
    int32_t next;
    pthread_mutex_t mu;
} pairs_ctx;

static void *pairs_worker(void *arg) {
    pairs_ctx *c = (pairs_ctx *)arg;
    int32_t n = c->n;
    int32_t *dist = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    int32_t *q = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    for (int32_t i = 0; i < n; i++) dist[i] = -1;
    for (;;) {
        pthread_mutex_lock(&c->mu);
        int32_t p = c->next < c->npairs ? c->next++ : -1;
        pthread_mutex_unlock(&c->mu);
        if (p < 0) break;
        rng_t r;
        rng_seed(&r, c->seed, 0x100000000ull + (uint64_t)p);
        int32_t s = (int32_t)rng_below(&r, (uint64_t)n);
        double lo = log((double)c->hop_lo), hi = log((double)c->hop_hi + 1.0);
        int32_t d = (int32_t)floor(exp(lo + (hi - lo) * rng_unit(&r)));
        if (d < c->hop_lo) d = c->hop_lo;
        if (d > c->hop_hi) d = c->hop_hi;
        c->want[p] = d;
        c->S[p] = s;
        int32_t t = -1;
        if (d <= c->bfs_cap) {
            /* truncated forward BFS from s to level d */
            int32_t qh = 0, qt = 0, level_begin = 0, level_end = 0;
            dist[s] = 0;
            q[qt++] = s;
            int32_t last_lvl_b = 0, last_lvl_e = 1;
            for (int32_t lvl = 0; lvl < d && qh < qt; lvl++) {
                level_begin = qh;
                level_end = qt;
                for (int32_t i = level_begin; i < level_end; i++) {
                    int32_t u = q[i];
                    for (int32_t k = c->off[u]; k < c->off[u + 1]; k++) {
                        int32_t v = c->col[k];
                        if (v >= 0 && dist[v] < 0) {
                            dist[v] = lvl + 1;
                            q[qt++] = v;
                        }
                    }
                }
                qh = level_end;
                if (qt > qh) {
                    last_lvl_b = qh;
                    last_lvl_e = qt;
                }
            }
            if (last_lvl_e > last_lvl_b && !(last_lvl_b == 0 && last_lvl_e == 1))
                t = q[last_lvl_b + (int32_t)rng_below(&r, (uint64_t)(last_lvl_e - last_lvl_b))];
            for (int32_t i = 0; i < qt; i++) dist[q[i]] = -1;
        }
        if (t < 0) {
            do {
                t = (int32_t)rng_below(&r, (uint64_t)n);
            } while (t == s && n > 1);
        }
        c->T[p] = t;
    }
    free(dist);
    free(q);
    return NULL;
}

int ddp_gen_pairs(int32_t n, const int32_t *off, const int32_t *col, int32_t npairs, int32_t hop_lo,
                  int32_t hop_hi, int32_t bfs_cap_level, uint64_t seed, int32_t threads, int32_t *S,
                  int32_t *T, int32_t *want_hops) {
    if (n < 2 || npairs < 0 || hop_lo < 1 || hop_hi < hop_lo) return -1;
    pairs_ctx c;
    c.n = n;
    c.off = off;
    c.col = col;
    c.npairs = npairs;
    c.hop_lo = hop_lo;
    c.hop_hi = hop_hi;
    c.bfs_cap = bfs_cap_level;
    c.seed = seed;
    c.S = S;
    c.T = T;
    c.want = want_hops;
    c.next = 0;
    pthread_mutex_init(&c.mu, NULL);
    if (threads < 1) threads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)threads);
    for (int i = 0; i < threads; i++) pthread_create(&th[i], NULL, pairs_worker, &c);
    for (int i = 0; i < threads; i++) pthread_join(th[i], NULL);
    free(th);
    pthread_mutex_destroy(&c.mu);
    return 0;
}

/* ---------------- 2D geometric k-NN graph -------------------------------- */
/* Points uniform on an integer grid [0, side)^2, numbered in Morton order,
 * each joined in both directions to its k nearest neighbours (ties by
 * index), duplicates removed; w = max(1, round(wscale * length / spacing))
 * with spacing = side / sqrt(n), i.e. wscale per mean point spacing. */
typedef struct {
    int32_t n, k, side, gcells;
    const int32_t *xy;
    const int32_t *cell_start, *cell_pts;
    int32_t *knn;
    int32_t next;
    pthread_mutex_t mu;
} knn_ctx;

static void *knn_worker(void *arg) {
    knn_ctx *c = (knn_ctx *)arg;
    const int32_t k = c->k, G = c->gcells;
    int64_t *bd = (int64_t *)malloc(sizeof(int64_t) * (size_t)k);
    int32_t *bi = (int32_t *)malloc(sizeof(int32_t) * (size_t)k);
    const double csz = (double)c->side / G;
    for (;;) {
        pthread_mutex_lock(&c->mu);
        int32_t start = c->next;
        c->next += 4096;
        pthread_mutex_unlock(&c->mu);
        if (start >= c->n) break;
        int32_t stop = start + 4096 < c->n ? start + 4096 : c->n;
        for (int32_t p = start; p < stop; p++) {
            const int64_t px = c->xy[2 * p], py = c->xy[2 * p + 1];
            int32_t cx = (int32_t)(px / csz), cy = (int32_t)(py / csz);
            if (cx >= G) cx = G - 1;
            if (cy >= G) cy = G - 1;
            int cnt = 0;
            for (int r = 1;; r++) {
                cnt = 0;
                for (int32_t yy = cy - r; yy <= cy + r; yy++) {
                    if (yy < 0 || yy >= G) continue;
                    for (int32_t xx = cx - r; xx <= cx + r; xx++) {
                        if (xx < 0 || xx >= G) continue;
                        const int32_t cell = yy * G + xx;
                        for (int32_t j = c->cell_start[cell]; j < c->cell_start[cell + 1]; j++) {
                            const int32_t q = c->cell_pts[j];
                            if (q == p) continue;
                            const int64_t dx = c->xy[2 * q] - px, dy = c->xy[2 * q + 1] - py;
                            const int64_t d = dx * dx + dy * dy;
                            /* insertion into the sorted top-k (distance, index) */
                            if (cnt < k || d < bd[cnt - 1] || (d == bd[cnt - 1] && q < bi[cnt - 1])) {
                                int pos = cnt < k ? cnt++ : k - 1;
                                while (pos > 0 && (bd[pos - 1] > d || (bd[pos - 1] == d && bi[pos - 1] > q))) {
                                    bd[pos] = bd[pos - 1];
                                    bi[pos] = bi[pos - 1];
                                    pos--;
                                }
                                bd[pos] = d;
                                bi[pos] = q;
                            }
                        }
                    }
                }
                /* the ring of radius r covers every point within r*csz */
                const double reach = r * csz;
                if (cnt == k && (double)bd[k - 1] < reach * reach) break;
                if (r > G) break;
            }
            for (int i = 0; i < k; i++) c->knn[(size_t)p * k + i] = i < cnt ? bi[i] : -1;
        }
    }
    free(bd);
    free(bi);
    return NULL;
}

int ddp_gen_geometric(int32_t n, int32_t k, int32_t side, uint32_t wscale, uint64_t seed, int32_t threads,
                      int32_t *xy, int32_t *off, int32_t *col, uint32_t *w, int64_t *n_arcs) {
    if (n < 2 || k < 1 || k >= n || side < 2) return -1;
    rng_t r;
    rng_seed(&r, seed, 5);
    for (int32_t i = 0; i < n; i++) {
        xy[2 * i] = (int32_t)rng_below(&r, (uint64_t)side);
        xy[2 * i + 1] = (int32_t)rng_below(&r, (uint64_t)side);
    }
    /* number the points along a Morton (Z-order) curve: nodes close in the
     * plane get close ids, so a search's state and arc reads stay local in
     * memory (the plane is what the search explores) */
    {
        uint64_t *key = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
        if (!key) return -2;
        for (int32_t i = 0; i < n; i++) {
            uint64_t m = 0, x = (uint32_t)xy[2 * i], y = (uint32_t)xy[2 * i + 1];
            for (int b = 0; b < 31; b++) m |= ((x >> b) & 1ull) << (2 * b) | ((y >> b) & 1ull) << (2 * b + 1);
            key[i] = (m << 1) >> 1;
        }
        /* LSD radix sort of (key, point) on 62-bit keys, 8 passes of 8 bits */
        uint64_t *k2 = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
        int32_t *p1 = (int32_t *)malloc(sizeof(int32_t) * (size_t)n), *p2 = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
        if (!k2 || !p1 || !p2) {
            free(key);
            free(k2);
            free(p1);
            free(p2);
            return -2;
        }
        for (int32_t i = 0; i < n; i++) p1[i] = i;
        for (int pass = 0; pass < 8; pass++) {
            int64_t cnt[257] = {0};
            const int sh = 8 * pass;
            for (int32_t i = 0; i < n; i++) cnt[((key[i] >> sh) & 255) + 1]++;
            for (int b = 0; b < 256; b++) cnt[b + 1] += cnt[b];
            for (int32_t i = 0; i < n; i++) {
                const int64_t d = cnt[(key[i] >> sh) & 255]++;
                k2[d] = key[i];
                p2[d] = p1[i];
            }
            uint64_t *tk = key;
            key = k2;
            k2 = tk;
            int32_t *tp = p1;
            p1 = p2;
            p2 = tp;
        }
        int32_t *nxy = (int32_t *)malloc(sizeof(int32_t) * 2 * (size_t)n);
        if (!nxy) return -2;
        for (int32_t i = 0; i < n; i++) {
            nxy[2 * i] = xy[2 * p1[i]];
            nxy[2 * i + 1] = xy[2 * p1[i] + 1];
        }
        memcpy(xy, nxy, sizeof(int32_t) * 2 * (size_t)n);
        free(nxy);
        free(key);
        free(k2);
        free(p1);
        free(p2);
    }
    /* grid buckets, about 2 points per cell */
    int32_t G = (int32_t)sqrt((double)n / 2.0);
    if (G < 1) G = 1;
    const double csz = (double)side / G;
    int32_t *cs = (int32_t *)calloc((size_t)G * G + 1, sizeof(int32_t));
    int32_t *cp = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    int32_t *cellof = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    int32_t *knn = (int32_t *)malloc(sizeof(int32_t) * (size_t)n * k);
    if (!cs || !cp || !cellof || !knn) {
        free(cs);
        free(cp);
        free(cellof);
        free(knn);
        return -2;
    }
    for (int32_t i = 0; i < n; i++) {
        int32_t cx = (int32_t)(xy[2 * i] / csz), cy = (int32_t)(xy[2 * i + 1] / csz);
        if (cx >= G) cx = G - 1;
        if (cy >= G) cy = G - 1;
        cellof[i] = cy * G + cx;
        cs[cellof[i] + 1]++;
    }
    for (int64_t c2 = 0; c2 < (int64_t)G * G; c2++) cs[c2 + 1] += cs[c2];
    {
        int32_t *fill = (int32_t *)malloc(sizeof(int32_t) * (size_t)G * G);
        memcpy(fill, cs, sizeof(int32_t) * (size_t)G * G);
        for (int32_t i = 0; i < n; i++) cp[fill[cellof[i]]++] = i;
        free(fill);
    }
    knn_ctx c;
    c.n = n;
    c.k = k;
    c.side = side;
    c.gcells = G;
    c.xy = xy;
    c.cell_start = cs;
    c.cell_pts = cp;
    c.knn = knn;
    c.next = 0;
    pthread_mutex_init(&c.mu, NULL);
    if (threads < 1) threads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)threads);
    for (int i = 0; i < threads; i++) pthread_create(&th[i], NULL, knn_worker, &c);
    for (int i = 0; i < threads; i++) pthread_join(th[i], NULL);
    free(th);
    pthread_mutex_destroy(&c.mu);
    /* symmetric rows: kNN(u) plus every v with u in kNN(v), sorted, unique */
    int32_t *deg = (int32_t *)calloc((size_t)n + 1, sizeof(int32_t));
    for (int64_t i = 0; i < (int64_t)n * k; i++)
        if (knn[i] >= 0) deg[knn[i] + 1]++;
    for (int32_t i = 0; i < n; i++) deg[i + 1] += deg[i];
    int32_t *rev = (int32_t *)malloc(sizeof(int32_t) * (size_t)(deg[n] > 0 ? deg[n] : 1));
    {
        int32_t *fill = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
        memcpy(fill, deg, sizeof(int32_t) * (size_t)n);
        for (int32_t u = 0; u < n; u++)
            for (int j = 0; j < k; j++) {
                int32_t v = knn[(size_t)u * k + j];
                if (v >= 0) rev[fill[v]++] = u;
            }
        free(fill);
    }
    const double spacing = (double)side / sqrt((double)n);
    int64_t m = 0;
    int32_t tmp[256];
    for (int32_t u = 0; u < n; u++) {
        off[u] = (int32_t)m;
        int t = 0;
        for (int j = 0; j < k; j++)
            if (knn[(size_t)u * k + j] >= 0 && t < 256) tmp[t++] = knn[(size_t)u * k + j];
        for (int32_t j = deg[u]; j < deg[u + 1] && t < 256; j++) tmp[t++] = rev[j];
        /* sort + unique (rows are short) */
        for (int a = 1; a < t; a++) {
            int32_t x = tmp[a];
            int b = a - 1;
            while (b >= 0 && tmp[b] > x) {
                tmp[b + 1] = tmp[b];
                b--;
            }
            tmp[b + 1] = x;
        }
        for (int a = 0; a < t; a++) {
            if (a > 0 && tmp[a] == tmp[a - 1]) continue;
            const int32_t v = tmp[a];
            const double dx = (double)xy[2 * v] - xy[2 * u], dy = (double)xy[2 * v + 1] - xy[2 * u + 1];
            const double len = sqrt(dx * dx + dy * dy);
            double ww = floor(wscale * len / spacing + 0.5);
            if (ww < 1) ww = 1;
            col[m] = v;
            w[m] = (uint32_t)ww;
            m++;
        }
    }
    off[n] = (int32_t)m;
    *n_arcs = m;
    free(cs);
    free(cp);
    free(cellof);
    free(knn);
    free(deg);
    free(rev);
    return 0;
}

/* ---------------- maze with every cell a node, and obstacle moves -------- */
/* CSR over all rows x cols cells (node = cell id); a wall cell has no arcs
 * and no open neighbour points to it.  Arc order per cell as
 * maze/create_maze.cpp:93-111: up, down, right, left. */
int ddp_gen_grid_from_walls(int32_t rows, int32_t cols, const uint8_t *wall, int32_t *off, int32_t *col,
                            uint32_t *w, int64_t *n_arcs) {
    if (rows < 1 || cols < 1 || !wall) return -1;
    int64_t m = 0;
    for (int32_t i = 0; i < rows; i++)
        for (int32_t j = 0; j < cols; j++) {
            const int64_t c = (int64_t)i * cols + j;
            off[c] = (int32_t)m;
            if (wall[c]) continue;
            if (i > 0 && !wall[c - cols]) { col[m] = (int32_t)(c - cols); w[m++] = 1; }
            if (i < rows - 1 && !wall[c + cols]) { col[m] = (int32_t)(c + cols); w[m++] = 1; }
            if (j < cols - 1 && !wall[c + 1]) { col[m] = (int32_t)(c + 1); w[m++] = 1; }
            if (j > 0 && !wall[c - 1]) { col[m] = (int32_t)(c - 1); w[m++] = 1; }
        }
    off[(int64_t)rows * cols] = (int32_t)m;
    *n_arcs = m;
    return 0;
}

/* Obstacle moves (the dynamic maze workload of maze/create_maze.cpp:137-251,
 * restated so that every batch is consistent with the update semantics):
 * per batch, `moves` wall cells open and `moves` open cells close (the two
 * sets disjoint, cells in `protect` never close).  An opened cell gets unit
 * arcs both ways to each neighbour open after the batch; a closed cell loses
 * its arcs both ways to each neighbour open before the batch.  Each pair is
 * listed once.  Inserts come first, then deletes; a delete never targets an
 * arc inserted in the same batch.  wall (rows x cols) is updated in place.
 * counts[b] receives each batch's line count; the lines go to
 * flag/u/v/w (capacity cap); returns -3 when cap is too small. */
int ddp_gen_maze_moves(int32_t rows, int32_t cols, uint8_t *wall, const uint8_t *protect, int32_t nbatches,
                       int32_t moves, uint64_t seed, int32_t *counts, int32_t *flag, int32_t *uu, int32_t *vv,
                       uint32_t *ww, int64_t cap, int64_t *total) {
    if (rows < 1 || cols < 1 || !wall || nbatches < 0 || moves < 0) return -1;
    const int64_t cells = (int64_t)rows * cols;
    rng_t r;
    rng_seed(&r, seed, 7);
    uint8_t *mark = (uint8_t *)calloc((size_t)cells, 1); /* 1 opening, 2 closing */
    int64_t *picked = (int64_t *)malloc(sizeof(int64_t) * (size_t)(2 * (moves > 0 ? moves : 1)));
    if (!mark || !picked) {
        free(mark);
        free(picked);
        return -2;
    }
    int64_t k = 0;
    int rc = 0;
    const int di[4] = {-1, 1, 0, 0}, dj[4] = {0, 0, 1, -1};
#define EMIT(F, A, B)                  \
    do {                               \
        if (k >= cap) { rc = -3; goto out; } \
        flag[k] = (F);                 \
        uu[k] = (int32_t)(A);          \
        vv[k] = (int32_t)(B);          \
        ww[k] = (F) ? 1u : 0u;         \
        k++;                           \
    } while (0)
    for (int32_t b = 0; b < nbatches; b++) {
        const int64_t k0 = k;
        int32_t nopen = 0, nclose = 0;
        /* pick cells to open (walls) and to close (open, unprotected) */
        for (int32_t tries = 0; nopen < moves && tries < 64 * moves + 1024; tries++) {
            const int64_t c = (int64_t)rng_below(&r, (uint64_t)cells);
            if (wall[c] && !mark[c]) { mark[c] = 1; picked[nopen++] = c; }
        }
        for (int32_t tries = 0; nclose < moves && tries < 64 * moves + 1024; tries++) {
            const int64_t c = (int64_t)rng_below(&r, (uint64_t)cells);
            if (!wall[c] && !mark[c] && !(protect && protect[c])) { mark[c] = 2; picked[nopen + nclose++] = c; }
        }
        /* inserts: opened cell <-> neighbours open after the batch */
        for (int32_t p = 0; p < nopen; p++) {
            const int64_t c = picked[p];
            const int32_t i = (int32_t)(c / cols), j = (int32_t)(c % cols);
            for (int q = 0; q < 4; q++) {
                const int32_t a = i + di[q], bj = j + dj[q];
                if (a < 0 || a >= rows || bj < 0 || bj >= cols) continue;
                const int64_t d = (int64_t)a * cols + bj;
                const int after_open = (!wall[d] && mark[d] != 2) || mark[d] == 1;
                if (!after_open) continue;
                if (mark[d] == 1 && d < c) continue; /* the pair is listed by d */
                EMIT(1, c, d);
                EMIT(1, d, c);
            }
        }
        /* deletes: closed cell <-> neighbours open before the batch */
        for (int32_t p = 0; p < nclose; p++) {
            const int64_t c = picked[nopen + p];
            const int32_t i = (int32_t)(c / cols), j = (int32_t)(c % cols);
            for (int q = 0; q < 4; q++) {
                const int32_t a = i + di[q], bj = j + dj[q];
                if (a < 0 || a >= rows || bj < 0 || bj >= cols) continue;
                const int64_t d = (int64_t)a * cols + bj;
                if (wall[d]) continue; /* no arc before the batch */
                if (mark[d] == 2 && d < c) continue;
                EMIT(0, c, d);
                EMIT(0, d, c);
            }
        }
        for (int32_t p = 0; p < nopen; p++) { wall[picked[p]] = 0; mark[picked[p]] = 0; }
        for (int32_t p = 0; p < nclose; p++) { wall[picked[nopen + p]] = 1; mark[picked[nopen + p]] = 0; }
        counts[b] = (int32_t)(k - k0);
    }
out:
#undef EMIT
    free(mark);
    free(picked);
    *total = k;
    return rc;
}
