/*
 * Text I/O in the reference's file formats.
 *   graph.txt   "N E", E cols, N offsets, E weights
 *               (LIB/include/graph.h:93-118, GA_star/A_star_cpu.cpp:105-140)
 *   Hx.txt      N ints (GA_star/bfs_hx.cu:158-172)
 *   Updates.txt repeated: "count", then count lines "flag u v w"
 *               (DA_star/DA_dyn_cpu.cu:1295-1326)
 * Files are read whole and parsed with a hand-written integer scanner; the
 * reference's iostream / fscanf parse takes seconds at 10^7 arcs.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ddp_gb300.h"

typedef struct {
    const char *p, *end;
} scan_t;

static int read_file(const char *path, char **buf, size_t *len) {
    FILE *f = fopen(path, "rb");
    if (!f) return -1;
    if (fseek(f, 0, SEEK_END) != 0) {
        fclose(f);
        return -1;
    }
    long sz = ftell(f);
    if (sz < 0) {
        fclose(f);
        return -1;
    }
    rewind(f);
    char *b = (char *)malloc((size_t)sz + 1);
    if (!b) {
        fclose(f);
        return -2;
    }
    size_t got = fread(b, 1, (size_t)sz, f);
    fclose(f);
    b[got] = 0;
    *buf = b;
    *len = got;
    return 0;
}

/* next integer (optional sign); returns 0 at end of input, -1 on junk */
static int scan_i64(scan_t *s, int64_t *out) {
    const char *p = s->p;
    while (p < s->end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) p++;
    if (p >= s->end) {
        s->p = p;
        return 0;
    }
    int neg = 0;
    if (*p == '-' || *p == '+') {
        neg = (*p == '-');
        p++;
    }
    if (p >= s->end || *p < '0' || *p > '9') {
        s->p = p;
        return -1;
    }
    int64_t v = 0;
    while (p < s->end && *p >= '0' && *p <= '9') {
        v = v * 10 + (*p - '0');
        p++;
    }
    s->p = p;
    *out = neg ? -v : v;
    return 1;
}

/* ---- parallel parse: the file is cut at whitespace into one chunk per
 * thread; pass 1 counts each chunk's tokens, pass 2 parses every token
 * straight into its place (token k of the body is col, offset or weight by
 * its index alone). */
typedef struct {
    const char *p, *end;
    int64_t first, count; /* body token index of the chunk's first token, tokens */
    int64_t N, E;
    int32_t *o, *c;
    uint32_t *w;
    int bad;
} chunk_t;

static int is_space(char ch) { return ch == ' ' || ch == '\n' || ch == '\r' || ch == '\t'; }

static void *count_chunk(void *arg) {
    chunk_t *k = (chunk_t *)arg;
    int64_t n = 0;
    int in = 0;
    for (const char *p = k->p; p < k->end; p++) {
        const int sp = is_space(*p);
        if (!sp && !in) n++;
        in = !sp;
    }
    k->count = n;
    return NULL;
}

static void *parse_chunk(void *arg) {
    chunk_t *k = (chunk_t *)arg;
    scan_t s = {k->p, k->end};
    int64_t x;
    for (int64_t t = k->first; t < k->first + k->count; t++) {
        if (scan_i64(&s, &x) != 1) {
            k->bad = 1;
            return NULL;
        }
        if (t < k->E) k->c[t] = (int32_t)x;
        else if (t < k->E + k->N) k->o[t - k->E] = (int32_t)x;
        else if (t < 2 * k->E + k->N) k->w[t - k->E - k->N] = (uint32_t)x;
    }
    return NULL;
}

int ddp_io_read_graph_text(const char *path, int32_t *n, int64_t *e, int32_t **off, int32_t **col,
                           uint32_t **w) {
    char *buf;
    size_t len;
    if (!path || !n || !e || !off || !col || !w) return DDP_ERR_INVALID;
    int rc = read_file(path, &buf, &len);
    if (rc) return rc == -2 ? DDP_ERR_OOM : DDP_ERR_IO;
    scan_t s = {buf, buf + len};
    int64_t N, E;
    if (scan_i64(&s, &N) != 1 || scan_i64(&s, &E) != 1 || N < 1 || E < 0 || N > INT32_MAX ||
        E > INT32_MAX) {
        free(buf);
        return DDP_ERR_IO;
    }
    int32_t *o = (int32_t *)malloc(sizeof(int32_t) * (size_t)(N + 1));
    int32_t *c = (int32_t *)malloc(sizeof(int32_t) * (size_t)(E > 0 ? E : 1));
    uint32_t *ww = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(E > 0 ? E : 1));
    if (!o || !c || !ww) {
        free(buf);
        free(o);
        free(c);
        free(ww);
        return DDP_ERR_OOM;
    }
    /* chunks: about 8 MB each, at most 32 threads */
    const char *body = s.p;
    const size_t blen = (size_t)(buf + len - body);
    int T = (int)(blen / (8u << 20)) + 1;
    if (T > 32) T = 32;
    chunk_t ch[32];
    const char *p = body;
    for (int i = 0; i < T; i++) {
        const char *q = (i == T - 1) ? buf + len : body + blen / (size_t)T * (size_t)(i + 1);
        if (q < p) q = p;
        while (q < buf + len && !is_space(*q)) q++; /* never split a number */
        ch[i].p = p;
        ch[i].end = q;
        ch[i].N = N;
        ch[i].E = E;
        ch[i].o = o;
        ch[i].c = c;
        ch[i].w = ww;
        ch[i].bad = 0;
        p = q;
    }
    pthread_t th[32];
    for (int i = 1; i < T; i++)
        if (pthread_create(&th[i], NULL, count_chunk, &ch[i])) count_chunk(&ch[i]), th[i] = 0;
    count_chunk(&ch[0]);
    for (int i = 1; i < T; i++)
        if (th[i]) pthread_join(th[i], NULL);
    int64_t total = 0;
    for (int i = 0; i < T; i++) {
        ch[i].first = total;
        total += ch[i].count;
    }
    int bad = total < 2 * E + N;
    if (!bad) {
        for (int i = 1; i < T; i++)
            if (pthread_create(&th[i], NULL, parse_chunk, &ch[i])) parse_chunk(&ch[i]), th[i] = 0;
        parse_chunk(&ch[0]);
        for (int i = 1; i < T; i++)
            if (th[i]) pthread_join(th[i], NULL);
        for (int i = 0; i < T; i++) bad |= ch[i].bad;
    }
    free(buf);
    if (bad) {
        free(o);
        free(c);
        free(ww);
        return DDP_ERR_IO;
    }
    o[N] = (int32_t)E;
    *n = (int32_t)N;
    *e = E;
    *off = o;
    *col = c;
    *w = ww;
    return DDP_OK;
}

/* buffered decimal writer (fprintf per number takes seconds at 10^7) */
typedef struct {
    FILE *f;
    char b[1 << 16];
    size_t n;
    int err;
} out_t;

static void out_flush(out_t *o) {
    if (o->n && fwrite(o->b, 1, o->n, o->f) != o->n) o->err = 1;
    o->n = 0;
}

static void out_i64(out_t *o, int64_t v, char sep) {
    if (o->n + 24 > sizeof(o->b)) out_flush(o);
    char t[24];
    int k = 0;
    uint64_t u = v < 0 ? (uint64_t)(-(v + 1)) + 1u : (uint64_t)v;
    do {
        t[k++] = (char)('0' + (int)(u % 10u));
        u /= 10u;
    } while (u);
    if (v < 0) o->b[o->n++] = '-';
    while (k) o->b[o->n++] = t[--k];
    o->b[o->n++] = sep;
}

int ddp_io_write_graph_text(const char *path, int32_t n, int64_t e, const int32_t *off,
                            const int32_t *col, const uint32_t *w) {
    if (!path || n < 1 || e < 0 || !off || (e > 0 && (!col || !w))) return DDP_ERR_INVALID;
    out_t *o = (out_t *)malloc(sizeof(out_t));
    if (!o) return DDP_ERR_OOM;
    o->f = fopen(path, "w");
    o->n = 0;
    o->err = 0;
    if (!o->f) {
        free(o);
        return DDP_ERR_IO;
    }
    out_i64(o, n, ' ');
    out_i64(o, e, '\n');
    for (int64_t i = 0; i < e; i++) out_i64(o, col[i], ' ');
    o->b[o->n++] = '\n';
    for (int32_t i = 0; i < n; i++) out_i64(o, off[i], ' ');
    o->b[o->n++] = '\n';
    for (int64_t i = 0; i < e; i++) out_i64(o, (int64_t)w[i], ' ');
    o->b[o->n++] = '\n';
    out_flush(o);
    const int bad = o->err | (fclose(o->f) != 0);
    free(o);
    return bad ? DDP_ERR_IO : DDP_OK;
}

/* ---- binary graph file: "DDPG" 1 (int32 each), n, e (int64), off[n+1],
 * col[e] (int32), w[e] (uint32), little-endian ---------------------------- */
int ddp_io_write_graph_bin(const char *path, int32_t n, int64_t e, const int32_t *off, const int32_t *col,
                           const uint32_t *w) {
    if (!path || n < 1 || e < 0 || !off || (e > 0 && (!col || !w))) return DDP_ERR_INVALID;
    FILE *f = fopen(path, "wb");
    if (!f) return DDP_ERR_IO;
    const int32_t hdr[2] = {0x47504444, 1}; /* "DDPG", version */
    const int64_t ne[2] = {n, e};
    int ok = fwrite(hdr, sizeof(hdr), 1, f) == 1 && fwrite(ne, sizeof(ne), 1, f) == 1 &&
             fwrite(off, sizeof(int32_t), (size_t)n + 1, f) == (size_t)n + 1 &&
             (e == 0 || (fwrite(col, sizeof(int32_t), (size_t)e, f) == (size_t)e &&
                         fwrite(w, sizeof(uint32_t), (size_t)e, f) == (size_t)e));
    ok = (fclose(f) == 0) && ok;
    return ok ? DDP_OK : DDP_ERR_IO;
}

int ddp_io_read_graph_bin(const char *path, int32_t *n, int64_t *e, int32_t **off, int32_t **col, uint32_t **w) {
    if (!path || !n || !e || !off || !col || !w) return DDP_ERR_INVALID;
    FILE *f = fopen(path, "rb");
    if (!f) return DDP_ERR_IO;
    int32_t hdr[2];
    int64_t ne[2];
    if (fread(hdr, sizeof(hdr), 1, f) != 1 || hdr[0] != 0x47504444 || hdr[1] != 1 ||
        fread(ne, sizeof(ne), 1, f) != 1 || ne[0] < 1 || ne[0] > INT32_MAX || ne[1] < 0 || ne[1] > INT32_MAX) {
        fclose(f);
        return DDP_ERR_IO;
    }
    const int64_t N = ne[0], E = ne[1];
    int32_t *o = (int32_t *)malloc(sizeof(int32_t) * (size_t)(N + 1));
    int32_t *c = (int32_t *)malloc(sizeof(int32_t) * (size_t)(E > 0 ? E : 1));
    uint32_t *ww = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(E > 0 ? E : 1));
    int ok = o && c && ww && fread(o, sizeof(int32_t), (size_t)N + 1, f) == (size_t)N + 1 &&
             (E == 0 || (fread(c, sizeof(int32_t), (size_t)E, f) == (size_t)E &&
                         fread(ww, sizeof(uint32_t), (size_t)E, f) == (size_t)E));
    fclose(f);
    if (ok) { /* offsets must be a CSR of E arcs */
        ok = o[0] == 0 && o[N] == E;
        for (int64_t i = 0; ok && i < N; i++) ok = o[i] <= o[i + 1];
    }
    if (!ok) {
        free(o);
        free(c);
        free(ww);
        return DDP_ERR_IO;
    }
    *n = (int32_t)N;
    *e = E;
    *off = o;
    *col = c;
    *w = ww;
    return DDP_OK;
}

int ddp_io_read_ints_text(const char *path, int64_t max, int32_t *out, int64_t *count) {
    char *buf;
    size_t len;
    if (!path || !out || max < 0) return DDP_ERR_INVALID;
    int rc = read_file(path, &buf, &len);
    if (rc) return rc == -2 ? DDP_ERR_OOM : DDP_ERR_IO;
    scan_t s = {buf, buf + len};
    int64_t k = 0, x;
    int r;
    while (k < max && (r = scan_i64(&s, &x)) == 1) out[k++] = (int32_t)x;
    free(buf);
    if (count) *count = k;
    return DDP_OK;
}

int ddp_io_write_ints_text(const char *path, int64_t n, const int32_t *vals) {
    if (!path || n < 0 || (n > 0 && !vals)) return DDP_ERR_INVALID;
    FILE *f = fopen(path, "w");
    if (!f) return DDP_ERR_IO;
    for (int64_t i = 0; i < n; i++) fprintf(f, "%d ", vals[i]);
    return fclose(f) == 0 ? DDP_OK : DDP_ERR_IO;
}

int ddp_io_read_updates_text(const char *path, int32_t *nbatches, int32_t **counts, int32_t **flag,
                             int32_t **u, int32_t **v, uint32_t **w) {
    char *buf;
    size_t len;
    if (!path || !nbatches || !counts || !flag || !u || !v || !w) return DDP_ERR_INVALID;
    int rc = read_file(path, &buf, &len);
    if (rc) return rc == -2 ? DDP_ERR_OOM : DDP_ERR_IO;
    /* first pass: count batches and lines */
    scan_t s = {buf, buf + len};
    int64_t x, nb = 0, total = 0;
    int r;
    while ((r = scan_i64(&s, &x)) == 1) {
        if (x < 0) {
            free(buf);
            return DDP_ERR_IO;
        }
        for (int64_t i = 0; i < 4 * x; i++) {
            int64_t y;
            if (scan_i64(&s, &y) != 1) {
                free(buf);
                return DDP_ERR_IO;
            }
        }
        nb++;
        total += x;
    }
    if (r < 0) {
        free(buf);
        return DDP_ERR_IO;
    }
    int32_t *cn = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nb > 0 ? nb : 1));
    int32_t *fl = (int32_t *)malloc(sizeof(int32_t) * (size_t)(total > 0 ? total : 1));
    int32_t *uu = (int32_t *)malloc(sizeof(int32_t) * (size_t)(total > 0 ? total : 1));
    int32_t *vv = (int32_t *)malloc(sizeof(int32_t) * (size_t)(total > 0 ? total : 1));
    uint32_t *ww = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(total > 0 ? total : 1));
    if (!cn || !fl || !uu || !vv || !ww) {
        free(buf);
        free(cn);
        free(fl);
        free(uu);
        free(vv);
        free(ww);
        return DDP_ERR_OOM;
    }
    s.p = buf;
    int64_t b = 0, k = 0;
    while (scan_i64(&s, &x) == 1) {
        cn[b++] = (int32_t)x;
        for (int64_t i = 0; i < x; i++) {
            int64_t a0, a1, a2, a3;
            scan_i64(&s, &a0);
            scan_i64(&s, &a1);
            scan_i64(&s, &a2);
            scan_i64(&s, &a3);
            fl[k] = (int32_t)a0;
            uu[k] = (int32_t)a1;
            vv[k] = (int32_t)a2;
            ww[k] = (uint32_t)a3;
            k++;
        }
    }
    free(buf);
    *nbatches = (int32_t)nb;
    *counts = cn;
    *flag = fl;
    *u = uu;
    *v = vv;
    *w = ww;
    return DDP_OK;
}

int ddp_io_write_updates_text(const char *path, int32_t nbatches, const int32_t *counts,
                              const int32_t *flag, const int32_t *u, const int32_t *v,
                              const uint32_t *w) {
    if (!path || nbatches < 0 || (nbatches > 0 && !counts)) return DDP_ERR_INVALID;
    FILE *f = fopen(path, "w");
    if (!f) return DDP_ERR_IO;
    int64_t k = 0;
    for (int32_t b = 0; b < nbatches; b++) {
        fprintf(f, "%d\n", counts[b]);
        for (int32_t i = 0; i < counts[b]; i++, k++)
            fprintf(f, "%d %d %d %u\n", flag[k], u[k], v[k], w[k]);
    }
    return fclose(f) == 0 ? DDP_OK : DDP_ERR_IO;
}

void ddp_free(void *p) { free(p); }
