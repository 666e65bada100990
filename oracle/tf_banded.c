/*
 * RCM + banded LU with partial pivoting.  TEST INFRASTRUCTURE ONLY: the
 * oracle's stand-in for the Pardiso solve in the reference
 * (TissueFolding/TissueFolding/SourceCode/NewtonRaphsonSolver.cpp:382-404,
 * :418-683).  The factorization is the textbook unblocked band algorithm
 * (column pivot search inside the lower band, row swap over the active
 * columns, rank-1 update), so the upper band grows to kl+ku.
 */
#include "tf_banded.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct { int n; int* ptr; int* idx; } tfb_graph;

static int tfb_build_graph(int n, const int* ia, const int* ja, tfb_graph* g) {
    int* deg = (int*)calloc((size_t)n, sizeof(int));
    if (!deg) return 2;
    for (int i = 0; i < n; ++i)
        for (int p = ia[i]; p < ia[i + 1]; ++p) {
            int j = ja[p];
            if (j != i) { deg[i]++; deg[j]++; }
        }
    g->n = n;
    g->ptr = (int*)malloc(sizeof(int) * (size_t)(n + 1));
    g->ptr[0] = 0;
    for (int i = 0; i < n; ++i) g->ptr[i + 1] = g->ptr[i] + deg[i];
    g->idx = (int*)malloc(sizeof(int) * (size_t)(g->ptr[n] > 0 ? g->ptr[n] : 1));
    memset(deg, 0, sizeof(int) * (size_t)n);
    for (int i = 0; i < n; ++i)
        for (int p = ia[i]; p < ia[i + 1]; ++p) {
            int j = ja[p];
            if (j != i) {
                g->idx[g->ptr[i] + deg[i]++] = j;
                g->idx[g->ptr[j] + deg[j]++] = i;
            }
        }
    /* deduplicate each adjacency list (insertion sort + unique) */
    int* newptr = (int*)malloc(sizeof(int) * (size_t)(n + 1));
    int w = 0;
    newptr[0] = 0;
    for (int i = 0; i < n; ++i) {
        int b = g->ptr[i], e = g->ptr[i + 1];
        for (int p = b + 1; p < e; ++p) {
            int v = g->idx[p], q = p - 1;
            while (q >= b && g->idx[q] > v) { g->idx[q + 1] = g->idx[q]; --q; }
            g->idx[q + 1] = v;
        }
        int start = w;
        for (int p = b; p < e; ++p)
            if (p == b || g->idx[p] != g->idx[p - 1]) g->idx[w++] = g->idx[p];
        (void)start;
        newptr[i + 1] = w;
    }
    free(g->ptr);
    g->ptr = newptr;
    free(deg);
    return 0;
}

/* BFS from `root` over unvisited vertices; returns the last vertex reached
 * and the number of levels. */
static int tfb_bfs_far(const tfb_graph* g, int root, const char* done, int* queue, int* level, int* nlev) {
    int head = 0, tail = 0, last = root;
    for (int i = 0; i < g->n; ++i) level[i] = -1;
    level[root] = 0;
    queue[tail++] = root;
    while (head < tail) {
        int v = queue[head++];
        last = v;
        for (int p = g->ptr[v]; p < g->ptr[v + 1]; ++p) {
            int u = g->idx[p];
            if (!done[u] && level[u] < 0) { level[u] = level[v] + 1; queue[tail++] = u; }
        }
    }
    *nlev = level[last];
    /* among the deepest level prefer the smallest degree */
    int best = last;
    for (int i = 0; i < tail; ++i) {
        int v = queue[i];
        if (level[v] == *nlev) {
            int dv = g->ptr[v + 1] - g->ptr[v], db = g->ptr[best + 1] - g->ptr[best];
            if (dv < db) best = v;
        }
    }
    return best;
}

static void tfb_rcm(const tfb_graph* g, int* perm /* new -> old */) {
    int n = g->n, pos = 0;
    char* done = (char*)calloc((size_t)n, 1);
    int* queue = (int*)malloc(sizeof(int) * (size_t)n);
    int* level = (int*)malloc(sizeof(int) * (size_t)n);
    int* nb = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int seed = 0; seed < n; ++seed) {
        if (done[seed]) continue;
        /* pseudo-peripheral start vertex */
        int root = seed, nlev = 0, prev = -1;
        for (int it = 0; it < 8; ++it) {
            int far = tfb_bfs_far(g, root, done, queue, level, &nlev);
            if (nlev <= prev) break;
            prev = nlev;
            root = far;
        }
        int head = pos, tail = pos;
        perm[tail++] = root;
        done[root] = 1;
        while (head < tail) {
            int v = perm[head++];
            int k = 0;
            for (int p = g->ptr[v]; p < g->ptr[v + 1]; ++p) {
                int u = g->idx[p];
                if (!done[u]) { done[u] = 1; nb[k++] = u; }
            }
            for (int a = 1; a < k; ++a) {      /* sort by degree */
                int u = nb[a], du = g->ptr[u + 1] - g->ptr[u], b = a - 1;
                while (b >= 0 && (g->ptr[nb[b] + 1] - g->ptr[nb[b]]) > du) { nb[b + 1] = nb[b]; --b; }
                nb[b + 1] = u;
            }
            for (int a = 0; a < k; ++a) perm[tail++] = nb[a];
        }
        pos = tail;
    }
    for (int i = 0; i < n / 2; ++i) { int t = perm[i]; perm[i] = perm[n - 1 - i]; perm[n - 1 - i] = t; }
    free(done); free(queue); free(level); free(nb);
}

int tfb_solve_csr(int n, const int* ia, const int* ja, const double* a,
                  const double* b, double* x, int transpose, int refine) {
    if (n <= 0) return 0;
    tfb_graph g;
    if (tfb_build_graph(n, ia, ja, &g)) return 2;
    int* perm = (int*)malloc(sizeof(int) * (size_t)n);   /* new -> old */
    int* iperm = (int*)malloc(sizeof(int) * (size_t)n);  /* old -> new */
    tfb_rcm(&g, perm);
    for (int i = 0; i < n; ++i) iperm[perm[i]] = i;
    free(g.ptr); free(g.idx);

    /* bandwidths of the permuted operator M (M = A or A^T) */
    int kl = 0, ku = 0;
    for (int i = 0; i < n; ++i)
        for (int p = ia[i]; p < ia[i + 1]; ++p) {
            int r = iperm[i], c = iperm[ja[p]];
            if (transpose) { int t = r; r = c; c = t; }
            if (r - c > kl) kl = r - c;
            if (c - r > ku) ku = c - r;
        }
    const int kv = kl + ku;
    const long ldab = 2L * kl + ku + 1;
    double* ab = (double*)calloc((size_t)(ldab * n), sizeof(double));
    int* ipiv = (int*)malloc(sizeof(int) * (size_t)n);
    if (!ab || !ipiv) { free(perm); free(iperm); free(ab); free(ipiv); return 2; }
#define AB(r, c) ab[(long)(c) * ldab + (kv + (r) - (c))]
    for (int i = 0; i < n; ++i)
        for (int p = ia[i]; p < ia[i + 1]; ++p) {
            int r = iperm[i], c = iperm[ja[p]];
            if (transpose) { int t = r; r = c; c = t; }
            AB(r, c) += a[p];
        }
    int info = 0, ju = 0;
    for (int j = 0; j < n; ++j) {
        int km = kl < n - 1 - j ? kl : n - 1 - j;
        int jp = 0;
        double amax = fabs(AB(j, j));
        for (int p = 1; p <= km; ++p) {
            double v = fabs(AB(j + p, j));
            if (v > amax) { amax = v; jp = p; }
        }
        ipiv[j] = j + jp;
        if (AB(j + jp, j) == 0.0) { if (!info) info = j + 1; continue; }
        int jumax = j + ku + jp < n - 1 ? j + ku + jp : n - 1;
        if (jumax > ju) ju = jumax;
        if (jp != 0)
            for (int c = j; c <= ju; ++c) { double t = AB(j, c); AB(j, c) = AB(j + jp, c); AB(j + jp, c) = t; }
        const double piv = AB(j, j);
        for (int p = 1; p <= km; ++p) AB(j + p, j) /= piv;
        for (int c = j + 1; c <= ju; ++c) {
            const double t = AB(j, c);
            if (t != 0.0)
                for (int p = 1; p <= km; ++p) AB(j + p, c) -= AB(j + p, j) * t;
        }
    }
    if (info) { free(perm); free(iperm); free(ab); free(ipiv); return 1; }

    double* y = (double*)malloc(sizeof(double) * (size_t)n);
    double* r = (double*)malloc(sizeof(double) * (size_t)n);
    for (int i = 0; i < n; ++i) x[i] = 0.0;
    for (int pass = 0; pass <= refine; ++pass) {
        /* residual r = b - M x (in original numbering) */
        for (int i = 0; i < n; ++i) r[i] = b[i];
        if (pass > 0) {
            for (int i = 0; i < n; ++i)
                for (int p = ia[i]; p < ia[i + 1]; ++p) {
                    if (transpose) r[ja[p]] -= a[p] * x[i];
                    else r[i] -= a[p] * x[ja[p]];
                }
        }
        for (int i = 0; i < n; ++i) y[i] = r[perm[i]];
        for (int j = 0; j < n; ++j) {
            int km = kl < n - 1 - j ? kl : n - 1 - j;
            if (ipiv[j] != j) { double t = y[j]; y[j] = y[ipiv[j]]; y[ipiv[j]] = t; }
            for (int p = 1; p <= km; ++p) y[j + p] -= AB(j + p, j) * y[j];
        }
        for (int j = n - 1; j >= 0; --j) {
            y[j] /= AB(j, j);
            int r0 = j - kv > 0 ? j - kv : 0;
            for (int rr = r0; rr < j; ++rr) y[rr] -= AB(rr, j) * y[j];
        }
        for (int i = 0; i < n; ++i) x[perm[i]] += y[i];
    }
#undef AB
    free(y); free(r); free(perm); free(iperm); free(ab); free(ipiv);
    return 0;
}
