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

int ddp_io_read_graph_text(const char *path, int32_t *n, int64_t *e, int32_t **off, int32_t **col,
                           uint32_t **w) {
    char *buf;
    size_t len;
    if (!path || !n || !e || !off || !col || !w) return DDP_ERR_INVALID;
    int rc = read_file(path, &buf, &len);
    if (rc) return rc == -2 ? DDP_ERR_OOM : DDP_ERR_IO;
    scan_t s = {buf, buf + len};
    int64_t N, E, x;
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
    int bad = 0;
    for (int64_t i = 0; i < E && !bad; i++) {
        if (scan_i64(&s, &x) != 1) bad = 1;
        else c[i] = (int32_t)x;
    }
    for (int64_t i = 0; i < N && !bad; i++) {
        if (scan_i64(&s, &x) != 1) bad = 1;
        else o[i] = (int32_t)x;
    }
    for (int64_t i = 0; i < E && !bad; i++) {
        if (scan_i64(&s, &x) != 1) bad = 1;
        else ww[i] = (uint32_t)x;
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

int ddp_io_write_graph_text(const char *path, int32_t n, int64_t e, const int32_t *off,
                            const int32_t *col, const uint32_t *w) {
    if (!path || n < 1 || e < 0 || !off || (e > 0 && (!col || !w))) return DDP_ERR_INVALID;
    FILE *f = fopen(path, "w");
    if (!f) return DDP_ERR_IO;
    fprintf(f, "%d %lld\n", n, (long long)e);
    for (int64_t i = 0; i < e; i++) fprintf(f, "%d ", col[i]);
    fprintf(f, "\n");
    for (int32_t i = 0; i < n; i++) fprintf(f, "%d ", off[i]);
    fprintf(f, "\n");
    for (int64_t i = 0; i < e; i++) fprintf(f, "%u ", w[i]);
    fprintf(f, "\n");
    return fclose(f) == 0 ? DDP_OK : DDP_ERR_IO;
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
