/*
 * CPU oracle for the GA* / dynamic A* hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the parity tests,
 * the smoke check and the CPU-baseline leg of the benchmark call it.  The
 * product (libddp_gb300.so) never links, loads or calls it, and nothing in
 * the product falls back to it.
 *
 * It restates, operation for operation, the reference's serial CPU A*
 * (lkoshale/DDP):
 *   - heap insert / pop-min / decrease-key   GA_star/A_star_cpu.cpp:10-97
 *     (the same code lives in LIB/include/a_star.h:94-188)
 *   - main search loop                       GA_star/A_star_cpu.cpp:152-188
 *     (LIB/include/a_star.h:192-275), including its quirks:
 *       * Cx holds f = g + h, INF = INT_MAX, the relax test is evaluated in
 *         unsigned arithmetic (weights are unsigned);
 *       * the CSR has N offsets and no sentinel; the last row ends at E-1
 *         (A_star_cpu.cpp:170, a_star.h:235), so callers append an isolated
 *         sentinel node to make the quirk harmless;
 *       * the search stops when the target is popped, the reported cost is
 *         Cx[target] = g(t) + h(t);
 *   - the level-synchronous reverse BFS of GA_star/bfs_hx.cu:11-36,111-172
 *     (hop counts, -1 = unreachable, last row ends at E);
 *   - the reverse-CSR builder of DA_star/genOpCSR.cpp:31-53;
 *   - the update-batch semantics of DA_star/DA_dyn_cpu.cu: inserts build a
 *     diff CSR in batch order (insertDiff/createDiffGraph :1928-2005),
 *     deletes mark the first live (u,v) arc of the pre-batch graph dead
 *     (removeDelEdges :2008-2043), and the batch is folded into a new CSR of
 *     live base arcs followed by the inserted arcs of each row
 *     (mergeDiff :2080-2128).
 *
 * Decrease-key: the reference finds the heap slot of a node by a linear scan
 * (A_star_cpu.cpp:77-97).  A node is in the heap at most once (the open flag
 * guards every insert), so the slot it finds is unique; mode
 * ORACLE_HEAP_POSMAP keeps that slot in a position map instead and performs
 * exactly the same swaps, so both modes pop the same nodes in the same order
 * and return the same cost and path.  ORACLE_HEAP_SCAN keeps the reference's
 * O(|open|) scan and is the one timed as the reference's CPU cost.
 */
#include <limits.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define ORACLE_HEAP_SCAN 0
#define ORACLE_HEAP_POSMAP 1

typedef struct {
    int *pq;   /* heap of node ids */
    int size;
    int *pos;  /* node -> heap slot (POSMAP mode only), -1 when absent */
} heap_t;

static inline void heap_swap(heap_t *hp, int a, int b) {
    int t = hp->pq[a];
    hp->pq[a] = hp->pq[b];
    hp->pq[b] = t;
    if (hp->pos) {
        hp->pos[hp->pq[a]] = a;
        hp->pos[hp->pq[b]] = b;
    }
}

/* A_star_cpu.cpp:10-31 (insertPQ): append, then sift up on Cx. */
static void heap_insert(heap_t *hp, int node, const int *cx) {
    hp->pq[hp->size] = node;
    if (hp->pos) hp->pos[node] = hp->size;
    hp->size++;
    int i = hp->size - 1;
    while (i > 0) {
        if (cx[hp->pq[(i - 1) / 2]] > cx[hp->pq[i]]) {
            heap_swap(hp, i, (i - 1) / 2);
            i = (i - 1) / 2;
        } else {
            break;
        }
    }
}

/* A_star_cpu.cpp:33-74 (getMin): move the last slot to the root, sift down
 * preferring the left child on ties. */
static int heap_pop(heap_t *hp, const int *cx) {
    if (hp->size == 0) return -1;
    int min = hp->pq[0];
    hp->pq[0] = hp->pq[hp->size - 1];
    if (hp->pos) {
        hp->pos[hp->pq[0]] = 0;
        hp->pos[min] = -1;
    }
    hp->size--;
    int i = 0;
    int *pq = hp->pq;
    while (2 * i + 1 < hp->size) {
        if (2 * i + 2 >= hp->size) {
            if (cx[pq[2 * i + 1]] < cx[pq[i]]) {
                heap_swap(hp, 2 * i + 1, i);
                i = 2 * i + 1;
            } else {
                break;
            }
        } else {
            if (cx[pq[i]] > cx[pq[2 * i + 1]] && cx[pq[2 * i + 1]] <= cx[pq[2 * i + 2]]) {
                heap_swap(hp, 2 * i + 1, i);
                i = 2 * i + 1;
            } else if (cx[pq[i]] > cx[pq[2 * i + 2]] && cx[pq[2 * i + 2]] <= cx[pq[2 * i + 1]]) {
                heap_swap(hp, 2 * i + 2, i);
                i = 2 * i + 2;
            } else {
                break;
            }
        }
    }
    return min;
}

/* A_star_cpu.cpp:77-97 (updatePQ): locate the node, then sift up. */
static void heap_update(heap_t *hp, int node, const int *cx) {
    int index = -1;
    if (hp->pos) {
        index = hp->pos[node];
    } else {
        for (int i = 0; i < hp->size; i++)
            if (hp->pq[i] == node) index = i;
    }
    if (index > 0) {
        int i = index;
        while (i > 0) {
            if (cx[hp->pq[(i - 1) / 2]] > cx[hp->pq[i]]) {
                heap_swap(hp, i, (i - 1) / 2);
                i = (i - 1) / 2;
            } else {
                break;
            }
        }
    }
}

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/*
 * Serial A* of GA_star/A_star_cpu.cpp:152-203.
 *   off: N offsets (reference layout, no sentinel); col/w: E arcs; h: N ints.
 * Returns 1 when the target was popped, 0 when the open list ran dry.
 * out_cost = Cx[t] (INT_MAX when not found).  path (s..t) is written when
 * path != NULL, truncated to path_cap, *path_len = full length.
 * stats[0..2] (optional): pops, arcs scanned, successful relaxations.
 * out_search_s (optional): wall time of the search loop alone.
 */
int oracle_astar(int N, int E, const int *off, const int *col, const uint32_t *w,
                 const int *h, int s, int t, int mode, int *out_cost, int *path,
                 int path_cap, int *path_len, int64_t *stats, double *out_search_s) {
    if (N <= 0 || s < 0 || s >= N || t < 0 || t >= N) return -1;
    int *cx = (int *)malloc(sizeof(int) * (size_t)N);
    int *parent = (int *)malloc(sizeof(int) * (size_t)N);
    int *open = (int *)malloc(sizeof(int) * (size_t)N);
    heap_t hp;
    hp.pq = (int *)malloc(sizeof(int) * (size_t)N);
    hp.size = 0;
    hp.pos = NULL;
    if (mode == ORACLE_HEAP_POSMAP) {
        hp.pos = (int *)malloc(sizeof(int) * (size_t)N);
        memset(hp.pos, -1, sizeof(int) * (size_t)N);
    }
    memset(parent, -1, sizeof(int) * (size_t)N);
    memset(open, -1, sizeof(int) * (size_t)N);
    for (int i = 0; i < N; i++) cx[i] = INT_MAX;

    int64_t pops = 0, scans = 0, relax = 0;
    double t0 = now_s();
    cx[s] = h[s];
    heap_insert(&hp, s, cx);
    open[s] = 1;
    int found = 0;
    while (hp.size > 0 && !found) {
        int u = heap_pop(&hp, cx);
        pops++;
        open[u] = -1;
        if (u == t) {
            found = 1;
            break;
        }
        int begin = off[u];
        int end = E - 1; /* A_star_cpu.cpp:170: the last row ends at E-1 */
        if (u != N - 1) end = off[u + 1];
        for (int j = begin; j < end; j++) {
            int child = col[j];
            scans++;
            /* int - int, then unsigned arithmetic, as in the reference. */
            unsigned int cand = (unsigned int)(cx[u] - h[u]) + w[j] + (unsigned int)h[child];
            if ((unsigned int)cx[child] > cand) {
                cx[child] = (int)cand;
                relax++;
                if (open[child] == 1) {
                    heap_update(&hp, child, cx);
                } else {
                    heap_insert(&hp, child, cx);
                    open[child] = 1;
                }
                parent[child] = u;
            }
        }
    }
    double t1 = now_s();
    if (out_search_s) *out_search_s = t1 - t0;
    if (stats) {
        stats[0] = pops;
        stats[1] = scans;
        stats[2] = relax;
    }
    if (out_cost) *out_cost = found ? cx[t] : INT_MAX;
    int len = 0;
    if (found) {
        /* walk parents from t, then reverse (A_star_cpu.cpp:190-200) */
        int c = t;
        len = 1;
        while (parent[c] != -1 && len <= N) {
            c = parent[c];
            len++;
        }
        if (path) {
            int k = len - 1;
            c = t;
            if (k < path_cap) path[k] = c;
            while (parent[c] != -1 && k > 0) {
                c = parent[c];
                k--;
                if (k < path_cap) path[k] = c;
            }
        }
    }
    if (path_len) *path_len = len;
    free(cx);
    free(parent);
    free(open);
    free(hp.pq);
    free(hp.pos);
    return found;
}

/*
 * Level-synchronous BFS of GA_star/bfs_hx.cu:11-36,111-138, run on the
 * reverse graph from the target: dist[v] = hops from v to the target, -1 if
 * the target is unreachable from v.  Rows use the N-offset layout; the last
 * row ends at E (bfs_hx.cu:20-22).
 */
void oracle_bfs_hops(int N, int E, const int *roff, const int *rcol, int root, int *dist) {
    for (int i = 0; i < N; i++) dist[i] = -1;
    if (root < 0 || root >= N) return;
    int *cur = (int *)malloc(sizeof(int) * (size_t)N);
    int *nxt = (int *)malloc(sizeof(int) * (size_t)N);
    int ncur = 1, nnxt;
    cur[0] = root;
    dist[root] = 0;
    while (ncur > 0) {
        nnxt = 0;
        for (int i = 0; i < ncur; i++) {
            int u = cur[i];
            int b = roff[u], e = (u != N - 1) ? roff[u + 1] : E;
            for (int j = b; j < e; j++) {
                int c = rcol[j];
                if (c < 0) continue;
                if (dist[c] < 0) {
                    dist[c] = dist[u] + 1;
                    nxt[nnxt++] = c;
                }
            }
        }
        int *tmp = cur;
        cur = nxt;
        nxt = tmp;
        ncur = nnxt;
    }
    free(cur);
    free(nxt);
}

/*
 * Reverse CSR of DA_star/genOpCSR.cpp:31-53: row v of the result lists the
 * sources u of arcs u->v in increasing u (and within u, arc order).  Input
 * and output use the N-offset layout with the last row ending at E.
 */
void oracle_reverse_csr(int N, int E, const int *off, const int *col, const uint32_t *w,
                        int *roff, int *rcol, uint32_t *rw) {
    int *cnt = (int *)calloc((size_t)N + 1, sizeof(int));
    for (int u = 0; u < N; u++) {
        int b = off[u], e = (u != N - 1) ? off[u + 1] : E;
        for (int j = b; j < e; j++)
            if (col[j] >= 0) cnt[col[j] + 1]++;
    }
    for (int v = 0; v < N; v++) cnt[v + 1] += cnt[v];
    for (int v = 0; v < N; v++) roff[v] = cnt[v];
    for (int u = 0; u < N; u++) {
        int b = off[u], e = (u != N - 1) ? off[u + 1] : E;
        for (int j = b; j < e; j++) {
            int v = col[j];
            if (v < 0) continue;
            int k = cnt[v]++;
            rcol[k] = u;
            if (rw) rw[k] = w[j];
        }
    }
    free(cnt);
}

/*
 * One update batch with the semantics of DA_star/DA_dyn_cpu.cu:
 *   flag 1: insert u->v (weight w), appended to row u after the live base
 *           arcs, inserted arcs of a row keep batch order (createDiffGraph);
 *   flag 0: delete the first live u->v arc of the pre-batch graph
 *           (removeDelEdges; arcs inserted in the same batch are not seen);
 *   flag 2: set the weight of the first live u->v arc of the pre-batch graph
 *           (an extension for weight-change workloads; the reference has no
 *           such update, a delete plus an insert gives the same arc set).
 * The result is folded like mergeDiff: per row, live base arcs, then the
 * row's inserted arcs.  Input/output use the N-offset layout, last row ends
 * at E.  Output arrays must hold E + (#inserts) arcs.  Returns the new E,
 * and *n_deleted the number of deletes that found an arc.
 */
int oracle_apply_batch(int N, int E, const int *off, const int *col, const uint32_t *w,
                       int n, const int *flag, const int *u, const int *v, const uint32_t *uw,
                       int *noff, int *ncol, uint32_t *nw, int *n_deleted) {
    int *c = (int *)malloc(sizeof(int) * (size_t)(E > 0 ? E : 1));
    uint32_t *ww = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(E > 0 ? E : 1));
    memcpy(c, col, sizeof(int) * (size_t)E);
    memcpy(ww, w, sizeof(uint32_t) * (size_t)E);
    int ndel = 0;
    for (int i = 0; i < n; i++) {
        if (flag[i] != 0 && flag[i] != 2) continue;
        int a = u[i];
        if (a < 0 || a >= N) continue;
        int b = off[a], e = (a != N - 1) ? off[a + 1] : E;
        for (int j = b; j < e; j++) {
            if (c[j] == v[i]) {
                if (flag[i] == 0) {
                    c[j] = -1;
                    ndel++;
                } else {
                    ww[j] = uw[i];
                }
                break;
            }
        }
    }
    /* per-row insert lists in batch order */
    int *icnt = (int *)calloc((size_t)N + 1, sizeof(int));
    int nins = 0;
    for (int i = 0; i < n; i++)
        if (flag[i] == 1 && u[i] >= 0 && u[i] < N) {
            icnt[u[i] + 1]++;
            nins++;
        }
    for (int x = 0; x < N; x++) icnt[x + 1] += icnt[x];
    int *iv = (int *)malloc(sizeof(int) * (size_t)(nins > 0 ? nins : 1));
    uint32_t *iw = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(nins > 0 ? nins : 1));
    int *ifill = (int *)malloc(sizeof(int) * (size_t)N);
    for (int x = 0; x < N; x++) ifill[x] = icnt[x];
    for (int i = 0; i < n; i++)
        if (flag[i] == 1 && u[i] >= 0 && u[i] < N) {
            int k = ifill[u[i]]++;
            iv[k] = v[i];
            iw[k] = uw[i];
        }
    int k = 0;
    for (int x = 0; x < N; x++) {
        noff[x] = k;
        int b = off[x], e = (x != N - 1) ? off[x + 1] : E;
        for (int j = b; j < e; j++)
            if (c[j] != -1) {
                ncol[k] = c[j];
                nw[k] = ww[j];
                k++;
            }
        for (int j = icnt[x]; j < icnt[x + 1]; j++) {
            ncol[k] = iv[j];
            nw[k] = iw[j];
            k++;
        }
    }
    if (n_deleted) *n_deleted = ndel;
    free(c);
    free(ww);
    free(icnt);
    free(iv);
    free(iw);
    free(ifill);
    return k;
}

/* ------------------------------------------------------------------------ */
/* Many independent queries on a thread pool (CPU baseline timing).         */

typedef struct {
    int N, E;
    const int *off, *col, *roff, *rcol;
    const uint32_t *w;
    int hkind; /* 0: h = 0, 1: h = reverse-BFS hops x wmin (bfs_hx + scaling) */
    int wmin;
    int nq;
    const int *S, *T;
    int mode;
    double deadline;
    int *out_cost;
    double *out_search_s;
    double *out_h_s;
    volatile int next;
    volatile int done;
    pthread_mutex_t mu;
} many_ctx;

static void *many_worker(void *arg) {
    many_ctx *c = (many_ctx *)arg;
    int *h = (int *)malloc(sizeof(int) * (size_t)c->N);
    for (;;) {
        pthread_mutex_lock(&c->mu);
        int q = c->next;
        if (q < c->nq && now_s() < c->deadline) c->next = q + 1;
        else q = -1;
        pthread_mutex_unlock(&c->mu);
        if (q < 0) break;
        double h0 = now_s();
        if (c->hkind == 1) {
            oracle_bfs_hops(c->N, c->E, c->roff, c->rcol, c->T[q], h);
            for (int i = 0; i < c->N; i++) h[i] = h[i] < 0 ? 0 : h[i] * c->wmin;
        } else {
            memset(h, 0, sizeof(int) * (size_t)c->N);
        }
        double h1 = now_s();
        int cost;
        double ss = 0;
        oracle_astar(c->N, c->E, c->off, c->col, c->w, h, c->S[q], c->T[q], c->mode, &cost,
                     NULL, 0, NULL, NULL, &ss);
        c->out_cost[q] = cost;
        if (c->out_search_s) c->out_search_s[q] = ss;
        if (c->out_h_s) c->out_h_s[q] = h1 - h0;
        pthread_mutex_lock(&c->mu);
        c->done++;
        pthread_mutex_unlock(&c->mu);
    }
    free(h);
    return NULL;
}

/*
 * Runs queries 0..nq-1 on `threads` threads until all are done or
 * `budget_s` seconds have passed (no new query starts after that).  Unrun
 * queries keep out_cost = -1.  Returns the number of completed queries.
 */
int oracle_astar_many(int N, int E, const int *off, const int *col, const uint32_t *w,
                      const int *roff, const int *rcol, int hkind, int wmin, int nq,
                      const int *S, const int *T, int mode, int threads, double budget_s,
                      int *out_cost, double *out_search_s, double *out_h_s) {
    many_ctx c;
    memset(&c, 0, sizeof(c));
    c.N = N;
    c.E = E;
    c.off = off;
    c.col = col;
    c.w = w;
    c.roff = roff;
    c.rcol = rcol;
    c.hkind = hkind;
    c.wmin = wmin;
    c.nq = nq;
    c.S = S;
    c.T = T;
    c.mode = mode;
    c.deadline = now_s() + budget_s;
    c.out_cost = out_cost;
    c.out_search_s = out_search_s;
    c.out_h_s = out_h_s;
    pthread_mutex_init(&c.mu, NULL);
    for (int i = 0; i < nq; i++) out_cost[i] = -1;
    if (threads < 1) threads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)threads);
    for (int i = 0; i < threads; i++) pthread_create(&th[i], NULL, many_worker, &c);
    for (int i = 0; i < threads; i++) pthread_join(th[i], NULL);
    free(th);
    pthread_mutex_destroy(&c.mu);
    return c.done;
}
