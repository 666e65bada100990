/*
 * tf_oracle.c -- CPU restatement of the reference's implicit prism step.
 * TEST INFRASTRUCTURE ONLY (see tf_oracle.h for the map to the reference).
 * Operation order follows the reference line by line so that results agree
 * with oracle/_ref to the last bits where the compiler keeps the same
 * rounding; each block cites the reference lines it restates (paths relative
 * to TissueFolding/TissueFolding/SourceCode/).
 */
#include "tf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "tf_banded.h"

struct tfo_model {
    int nn, ne;
    double* pos;        /* 3N current node positions (Node::Position) */
    int* conn;          /* 6E node ids */
    unsigned char* fixed;
    double* ext_visc;   /* 3N Node::externalViscosity */
    int* placement;     /* E ShapeBase::tissuePlacement */
    unsigned char* spans;
    double *lam, *mu, *eta;
    double* detdXde;    /* 6E */
    double* invdXde;    /* 54E */
    double *Fg, *invFg; /* 9E */
    double* area;       /* N Node::viscositySurface */
    int *nptr, *nadj;   /* node adjacency (sorted) */
    int* ia;            /* structural CSR of K, rows = DOF */
    int* ja;
    long nnz;
    double* a;          /* values of the last assembly */
    double* g;          /* gSum of the last assembly */
    double *Ke, *Kv, *fe, *fv; /* per-element scratch (lazily allocated) */
};

/* Gauss points (eta, nu, zeta) and weights, Prism.cpp:123-146 */
static double GP[6][3];
static const double GW = 1.0 / 6.0;
static double DNREF[6][3][6]; /* setShapeFunctionDerivatives, Prism.cpp:655-680 */
static int g_init = 0;

static void tfo_init_constants(void) {
    if (g_init) return;
    double s = 1.0 / pow(3, 0.5);
    double pts[6][3] = {{1.0 / 6.0, 1.0 / 6.0, s}, {2.0 / 3.0, 1.0 / 6.0, s}, {1.0 / 6.0, 2.0 / 3.0, s},
                        {1.0 / 6.0, 1.0 / 6.0, -s}, {2.0 / 3.0, 1.0 / 6.0, -s}, {1.0 / 6.0, 2.0 / 3.0, -s}};
    for (int p = 0; p < 6; ++p) {
        for (int k = 0; k < 3; ++k) GP[p][k] = pts[p][k];
        double eta = pts[p][0], nu = pts[p][1], zeta = pts[p][2];
        double alpha = (1 - zeta) / 2, beta = (1 + zeta) / 2, lambda = 1 - eta - nu;
        double d[3][6] = {{-alpha, alpha, 0, -beta, beta, 0},
                          {-alpha, 0, alpha, -beta, 0, beta},
                          {-lambda / 2, -eta / 2, -nu / 2, lambda / 2, eta / 2, nu / 2}};
        memcpy(DNREF[p], d, sizeof(d));
    }
    g_init = 1;
}

/* ShapeBase::determinant3by3Matrix(gsl_matrix*), ShapeBase.cpp:2050-2056 */
static double det3(const double M[9]) {
    double det = 0.0;
    det = M[0] * (M[4] * M[8] - M[5] * M[7]);
    det -= M[1] * (M[3] * M[8] - M[5] * M[6]);
    det += M[2] * (M[3] * M[7] - M[4] * M[6]);
    return det;
}

/* ShapeBase::InvertMatrix(gsl) ShapeBase.cpp:3767-3782: row-pivoted LU and
 * column-by-column inverse, same loop order as the GSL stand-in. */
static void inv3(const double Ain[9], double inv[9]) {
    double A[9];
    int p[3] = {0, 1, 2};
    memcpy(A, Ain, sizeof(A));
    for (int j = 0; j < 2; ++j) {
        double amax = fabs(A[3 * j + j]);
        int ip = j;
        for (int i = j + 1; i < 3; ++i) {
            double v = fabs(A[3 * i + j]);
            if (v > amax) { amax = v; ip = i; }
        }
        if (ip != j) {
            for (int k = 0; k < 3; ++k) { double t = A[3 * j + k]; A[3 * j + k] = A[3 * ip + k]; A[3 * ip + k] = t; }
            int t = p[j]; p[j] = p[ip]; p[ip] = t;
        }
        double ajj = A[3 * j + j];
        if (ajj != 0.0)
            for (int i = j + 1; i < 3; ++i) {
                double aij = A[3 * i + j] / ajj;
                A[3 * i + j] = aij;
                for (int k = j + 1; k < 3; ++k) A[3 * i + k] -= aij * A[3 * j + k];
            }
    }
    for (int c = 0; c < 3; ++c) {
        double x[3];
        for (int i = 0; i < 3; ++i) x[i] = (p[i] == c) ? 1.0 : 0.0;
        for (int i = 0; i < 3; ++i) {
            double s = x[i];
            for (int k = 0; k < i; ++k) s -= A[3 * i + k] * x[k];
            x[i] = s;
        }
        for (int ii = 2; ii >= 0; --ii) {
            double s = x[ii];
            for (int k = ii + 1; k < 3; ++k) s -= A[3 * ii + k] * x[k];
            x[ii] = s / A[3 * ii + ii];
        }
        for (int i = 0; i < 3; ++i) inv[3 * i + c] = x[i];
    }
}

/* C = A B (3x3), dgemm accumulation order */
static void mm3(const double A[9], const double B[9], double C[9]) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double acc = 0.0;
            for (int k = 0; k < 3; ++k) acc += A[3 * i + k] * B[3 * k + j];
            C[3 * i + j] = acc;
        }
}

void tfo_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int tfo_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static void build_structure(tfo_model* m) {
    int nn = m->nn, ne = m->ne;
    int* cnt = (int*)calloc((size_t)nn, sizeof(int));
    for (int e = 0; e < ne; ++e)
        for (int a = 0; a < 6; ++a) cnt[m->conn[6 * e + a]] += 6;
    int* ptr = (int*)malloc(sizeof(int) * (size_t)(nn + 1));
    ptr[0] = 0;
    for (int i = 0; i < nn; ++i) ptr[i + 1] = ptr[i] + cnt[i];
    int* tmp = (int*)malloc(sizeof(int) * (size_t)(ptr[nn] > 0 ? ptr[nn] : 1));
    memset(cnt, 0, sizeof(int) * (size_t)nn);
    for (int e = 0; e < ne; ++e)
        for (int a = 0; a < 6; ++a) {
            int A = m->conn[6 * e + a];
            for (int b = 0; b < 6; ++b) tmp[ptr[A] + cnt[A]++] = m->conn[6 * e + b];
        }
    m->nptr = (int*)malloc(sizeof(int) * (size_t)(nn + 1));
    m->nadj = (int*)malloc(sizeof(int) * (size_t)(ptr[nn] > 0 ? ptr[nn] : 1));
    int w = 0;
    m->nptr[0] = 0;
    for (int i = 0; i < nn; ++i) {
        int b = ptr[i], e = ptr[i + 1];
        for (int p = b + 1; p < e; ++p) { /* insertion sort */
            int v = tmp[p], q = p - 1;
            while (q >= b && tmp[q] > v) { tmp[q + 1] = tmp[q]; --q; }
            tmp[q + 1] = v;
        }
        for (int p = b; p < e; ++p)
            if (p == b || tmp[p] != tmp[p - 1]) m->nadj[w++] = tmp[p];
        m->nptr[i + 1] = w;
    }
    free(tmp); free(ptr); free(cnt);
    long nnz = 9L * w;
    m->nnz = nnz;
    m->ia = (int*)malloc(sizeof(int) * (size_t)(3 * nn + 1));
    m->ja = (int*)malloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
    m->ia[0] = 0;
    long q = 0;
    for (int i = 0; i < nn; ++i)
        for (int d = 0; d < 3; ++d) {
            for (int p = m->nptr[i]; p < m->nptr[i + 1]; ++p)
                for (int dd = 0; dd < 3; ++dd) m->ja[q++] = 3 * m->nadj[p] + dd;
            m->ia[3 * i + d + 1] = (int)q;
        }
    m->a = (double*)calloc((size_t)(nnz > 0 ? nnz : 1), sizeof(double));
    m->g = (double*)calloc((size_t)(3 * nn), sizeof(double));
}

/* position of entry (row 3A+i, col 3B+j) in the structural CSR */
static long entry_index(const tfo_model* m, int A, int B, int i, int j) {
    int lo = m->nptr[A], hi = m->nptr[A + 1] - 1;
    while (lo < hi) {
        int mid = (lo + hi) / 2;
        if (m->nadj[mid] < B) lo = mid + 1; else hi = mid;
    }
    int k = lo - m->nptr[A];
    return (long)m->ia[3 * A + i] + 3L * k + j;
}

/* Prism::calculateElementShapeFunctionDerivatives, Prism.cpp:705-728: per
 * Gauss point dX/dxi of the reference shape X (6 x 3), its determinant and
 * inverse. */
static void reference_geometry(tfo_model* m, int e, const double* X) {
    for (int p = 0; p < 6; ++p) {
        double Jt[9], J[9];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                double acc = 0.0;
                for (int a = 0; a < 6; ++a) acc += DNREF[p][r][a] * X[3 * a + c];
                Jt[3 * r + c] = acc;
            }
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) J[3 * r + c] = Jt[3 * c + r];
        m->detdXde[6 * e + p] = det3(J);
        inv3(J, &m->invdXde[54L * e + 9 * p]);
    }
}

void tfo_set_reference_shapes(tfo_model* m, const double* ref_pos) {
    /* ReferenceShape->Positions read from a mesh file
     * (ShapeBase::updateReferencePositionMatrixFromSave, ShapeBase.cpp:935-944) */
    for (int e = 0; e < m->ne; ++e) reference_geometry(m, e, &ref_pos[18L * e]);
}

tfo_model* tfo_create(int n_nodes, int n_elems, const double* pos0, const int* conn,
                      const unsigned char* fixed, const double* ext_visc, const int* node_placement,
                      const double* E, const double* nu, const double* eta) {
    tfo_init_constants();
    tfo_model* m = (tfo_model*)calloc(1, sizeof(tfo_model));
    m->nn = n_nodes;
    m->ne = n_elems;
    m->pos = (double*)malloc(sizeof(double) * 3 * (size_t)n_nodes);
    memcpy(m->pos, pos0, sizeof(double) * 3 * (size_t)n_nodes);
    m->conn = (int*)malloc(sizeof(int) * 6 * (size_t)n_elems);
    memcpy(m->conn, conn, sizeof(int) * 6 * (size_t)n_elems);
    m->fixed = (unsigned char*)malloc(3 * (size_t)n_nodes);
    memcpy(m->fixed, fixed, 3 * (size_t)n_nodes);
    m->ext_visc = (double*)malloc(sizeof(double) * 3 * (size_t)n_nodes);
    memcpy(m->ext_visc, ext_visc, sizeof(double) * 3 * (size_t)n_nodes);
    m->placement = (int*)malloc(sizeof(int) * (size_t)n_elems);
    m->spans = (unsigned char*)calloc((size_t)n_elems, 1);
    m->lam = (double*)malloc(sizeof(double) * (size_t)n_elems);
    m->mu = (double*)malloc(sizeof(double) * (size_t)n_elems);
    m->eta = (double*)malloc(sizeof(double) * (size_t)n_elems);
    m->detdXde = (double*)malloc(sizeof(double) * 6 * (size_t)n_elems);
    m->invdXde = (double*)malloc(sizeof(double) * 54 * (size_t)n_elems);
    m->Fg = (double*)malloc(sizeof(double) * 9 * (size_t)n_elems);
    m->invFg = (double*)malloc(sizeof(double) * 9 * (size_t)n_elems);
    m->area = (double*)calloc((size_t)n_nodes, sizeof(double));
    for (int e = 0; e < n_elems; ++e) {
        /* ShapeBase::setTissuePlacement, ShapeBase.cpp:705-770 */
        int hasA = 0, hasB = 0, hasL = 0;
        for (int a = 0; a < 6; ++a) {
            int p = node_placement[conn[6 * e + a]];
            if (p == 1) hasA = 1; else if (p == 0) hasB = 1; else if (p == 3) hasL = 1;
        }
        int pl;
        if (hasL) pl = 3;
        else if (hasA) { if (hasB) { pl = 2; m->spans[e] = 1; } else pl = 1; }
        else if (hasB) pl = 0;
        else pl = 2;
        m->placement[e] = pl;
        /* Prism::setElasticProperties, Prism.cpp:491-516 */
        double v = nu[e];
        if (v > 0.5) v = 0.5; else if (v < 0.0) v = 0.0;
        m->lam[e] = E[e] * v / (1 + v) / (1 - 2.0 * v);
        m->mu[e] = E[e] / 2.0 / (1 + v);
        m->eta[e] = eta[e];
        double X[18];
        for (int a = 0; a < 6; ++a)
            for (int c = 0; c < 3; ++c) X[3 * a + c] = pos0[3 * conn[6 * e + a] + c];
        reference_geometry(m, e, X);
        for (int k = 0; k < 9; ++k) {
            m->Fg[9L * e + k] = (k % 4 == 0) ? 1.0 : 0.0;
            m->invFg[9L * e + k] = (k % 4 == 0) ? 1.0 : 0.0;
        }
    }
    build_structure(m);
    return m;
}

void tfo_destroy(tfo_model* m) {
    if (!m) return;
    free(m->pos); free(m->conn); free(m->fixed); free(m->ext_visc); free(m->placement);
    free(m->spans); free(m->lam); free(m->mu); free(m->eta); free(m->detdXde); free(m->invdXde);
    free(m->Fg); free(m->invFg); free(m->area); free(m->nptr); free(m->nadj); free(m->ia);
    free(m->ja); free(m->a); free(m->g); free(m->Ke); free(m->Kv); free(m->fe); free(m->fv);
    free(m);
}

void tfo_set_Fg(tfo_model* m, const double* Fg) {
    /* ShapeBase::setFg */
    for (int e = 0; e < m->ne; ++e) {
        memcpy(&m->Fg[9L * e], &Fg[9L * e], 9 * sizeof(double));
        inv3(&m->Fg[9L * e], &m->invFg[9L * e]);
    }
}

void tfo_get_Fg(const tfo_model* m, double* Fg, double* invFg) {
    if (Fg) memcpy(Fg, m->Fg, sizeof(double) * 9 * (size_t)m->ne);
    if (invFg) memcpy(invFg, m->invFg, sizeof(double) * 9 * (size_t)m->ne);
}

void tfo_set_positions(tfo_model* m, const double* pos) { memcpy(m->pos, pos, sizeof(double) * 3 * (size_t)m->nn); }
void tfo_get_positions(const tfo_model* m, double* pos) { memcpy(pos, m->pos, sizeof(double) * 3 * (size_t)m->nn); }

void tfo_get_lame(const tfo_model* m, double* lam, double* mu) {
    memcpy(lam, m->lam, sizeof(double) * (size_t)m->ne);
    memcpy(mu, m->mu, sizeof(double) * (size_t)m->ne);
}

void tfo_get_placement(const tfo_model* m, int* placement) { memcpy(placement, m->placement, sizeof(int) * (size_t)m->ne); }

void tfo_get_ref_geometry(const tfo_model* m, double* detdXde, double* invdXde) {
    if (detdXde) memcpy(detdXde, m->detdXde, sizeof(double) * 6 * (size_t)m->ne);
    if (invdXde) memcpy(invdXde, m->invdXde, sizeof(double) * 54 * (size_t)m->ne);
}

/* Growth for one step with per-element rates (1/s): ShapeBase::
 * calculateFgFromRates :396-421 with identity rotation and unit tissue weight,
 * updateGrowthIncrement :567-586, growShapeByFg :1215-1251. */
void tfo_grow(tfo_model* m, double dt, const double* rates) {
    for (int e = 0; e < m->ne; ++e) {
        double inc[9] = {0};
        inc[0] = exp(rates[3 * e] * 1.0 * dt);
        inc[4] = exp(rates[3 * e + 1] * 1.0 * dt);
        inc[8] = exp(rates[3 * e + 2] * 1.0 * dt);
        double Fn[9];
        mm3(inc, &m->Fg[9L * e], Fn);
        memcpy(&m->Fg[9L * e], Fn, sizeof(Fn));
        inv3(Fn, &m->invFg[9L * e]);
    }
}

/* Prism::calculateBasalArea / calculateApicalArea, Prism.cpp:2424-2503 */
static double face_area(const double* pos, const int* ids) {
    const double Threshold = 1E-5;
    double s1[3], s2[3], Side1 = 0.0, Side2 = 0.0, costet = 0.0, Area = 0.0;
    for (int i = 0; i < 3; ++i) {
        s1[i] = pos[3 * ids[1] + i] - pos[3 * ids[0] + i];
        s2[i] = pos[3 * ids[2] + i] - pos[3 * ids[0] + i];
        costet += s1[i] * s2[i];
        Side1 += s1[i] * s1[i];
        Side2 += s2[i] * s2[i];
    }
    if (Side1 > Threshold && Side2 > Threshold) {
        Side1 = pow(Side1, 0.5);
        Side2 = pow(Side2, 0.5);
        costet /= (Side1 * Side2);
        double sinTetSq = 1 - costet * costet, sintet = 0;
        if (sinTetSq > Threshold) sintet = pow(sinTetSq, 0.5);
        Area = Side1 * Side2 * sintet / 2.0;
    }
    return Area;
}

/* Simulation::updateNodeViscositySurfaces, Simulation.cpp:7563-7581 and
 * ShapeBase::assignViscositySurfaceAreaToNodes, ShapeBase.cpp:4056-4078 */
void tfo_update_viscosity_surfaces(tfo_model* m, double* area_out) {
    for (int i = 0; i < m->nn; ++i) m->area[i] = 0;
    for (int e = 0; e < m->ne; ++e) {
        const int* c = &m->conn[6 * e];
        int pl = m->placement[e];
        int apical = (pl == 1) || (pl == 2 && m->spans[e]);
        int basal = (pl == 0) || (pl == 2 && m->spans[e]);
        if (apical) {
            int ids[3] = {c[3], c[4], c[5]};
            double A = face_area(m->pos, ids);
            for (int i = 0; i < 3; ++i) m->area[ids[i]] += A / 3;
        }
        if (basal) {
            int ids[3] = {c[0], c[1], c[2]};
            double A = face_area(m->pos, ids);
            for (int i = 0; i < 3; ++i) m->area[ids[i]] += A / 3;
        }
    }
    if (area_out) memcpy(area_out, m->area, sizeof(double) * (size_t)m->nn);
}

void tfo_set_viscosity_surfaces(tfo_model* m, const double* area) { memcpy(m->area, area, sizeof(double) * (size_t)m->nn); }

/* One element: ShapeBase::calculateForces3D (:2184-2235) with
 * Prism::calculateCurrNodalForces (Prism.cpp:749-874) per Gauss point, then
 * calculateImplicitKElastic (:2619-2639) and calculateImplicitKViscous
 * (:2641-2705).  `want_k` = 0 skips both tangents. */
static void element_eval(const tfo_model* m, int e, const double* uk, const double* vel, double dt,
                         int mode, int want_k, double* Ke, double* Kv, double* fe, double* fv) {
    const int* conn = &m->conn[6 * e];
    const double lambda = m->lam[e], mu = m->mu[e], eta = m->eta[e];
    const double* InvFg = &m->invFg[9L * e];
    double CurrShape[6][3], ve[18];
    for (int a = 0; a < 6; ++a)
        for (int d = 0; d < 3; ++d) {
            CurrShape[a][d] = uk[3 * conn[a] + d];
            ve[3 * a + d] = vel[3 * conn[a] + d];
        }
    double Tge[18] = {0}, Tgv[18] = {0};
    double Fe_gp[6][9], DN_gp[6][6][3], B_gp[6][6][18], S_gp[6][9], Sv_gp[6][9], detF_gp[6], lnJ_gp[6];
    double D81[6][3][3][3][3];
    for (int gp = 0; gp < 6; ++gp) {
        const double(*dN)[6] = DNREF[gp];
        const double* InvdXde = &m->invdXde[54L * e + 9 * gp];
        const double detdXde = m->detdXde[6 * e + gp];
        double Jt[9], Jac[9], F[9], Fe[9], C[9], InvC[9], S[9], InvJ[9];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                double acc = 0.0;
                for (int a = 0; a < 6; ++a) acc += dN[r][a] * CurrShape[a][c];
                Jt[3 * r + c] = acc;
            }
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) Jac[3 * r + c] = Jt[3 * c + r];
        mm3(Jac, InvdXde, F);
        mm3(F, InvFg, Fe);
        memcpy(Fe_gp[gp], Fe, sizeof(Fe));
        for (int i = 0; i < 3; ++i) /* C = Fe^T Fe, ShapeBase.cpp:2238-2243 */
            for (int j = 0; j < 3; ++j) {
                double acc = 0.0;
                for (int k = 0; k < 3; ++k) acc += Fe[3 * k + i] * Fe[3 * k + j];
                C[3 * i + j] = acc;
            }
        double detFe = det3(Fe);
        double lnJ = log(detFe);
        lnJ_gp[gp] = lnJ;
        inv3(C, InvC);
        for (int i = 0; i < 3; ++i) /* ShapeBase.cpp:2284-2297 */
            for (int j = 0; j < 3; ++j) {
                double Iij = ((i == j) ? 1.0 : 0.0) - InvC[3 * i + j];
                Iij = Iij * mu;
                double s = InvC[3 * i + j] * (lambda * lnJ);
                S[3 * i + j] = s + Iij;
            }
        if (want_k && mode == TFO_LITERAL) { /* ShapeBase.cpp:2299-2321 */
            double multiplier = 2 * (mu - lambda * lnJ);
            for (int I = 0; I < 3; ++I)
                for (int J = 0; J < 3; ++J)
                    for (int K = 0; K < 3; ++K)
                        for (int L = 0; L < 3; ++L) {
                            double Iijkl = 0.5 * (InvC[3 * I + K] * InvC[3 * J + L] + InvC[3 * I + L] * InvC[3 * J + K]);
                            D81[gp][I][J][K][L] = lambda * InvC[3 * I + J] * InvC[3 * K + L] + multiplier * Iijkl;
                        }
        }
        /* elastic stress, ShapeBase.cpp:2323-2341 */
        double tmp[9], St[9];
        mm3(Fe, S, tmp);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double acc = 0.0;
                for (int k = 0; k < 3; ++k) acc += tmp[3 * i + k] * Fe[3 * j + k];
                St[3 * i + j] = acc;
            }
        double rdet = 1.0 / detFe;
        for (int k = 0; k < 9; ++k) St[k] *= rdet;
        memcpy(S_gp[gp], St, sizeof(St));
        double compact[6] = {St[0], St[4], St[8], St[1], St[7], St[2]};
        inv3(Jac, InvJ);
        double detF = det3(F);
        detF_gp[gp] = detF;
        /* invJShFuncDerS and B, ShapeBase.cpp:2378-2411 */
        double DN[6][3];
        for (int a = 0; a < 6; ++a)
            for (int mm = 0; mm < 3; ++mm) {
                double acc = 0.0;
                for (int n = 0; n < 3; ++n) acc += InvJ[3 * n + mm] * dN[n][a];
                DN[a][mm] = acc;
            }
        memcpy(DN_gp[gp], DN, sizeof(DN));
        double B[6][18];
        memset(B, 0, sizeof(B));
        for (int a = 0; a < 6; ++a) {
            B[0][3 * a] = DN[a][0];
            B[1][3 * a + 1] = DN[a][1];
            B[2][3 * a + 2] = DN[a][2];
            B[3][3 * a] = DN[a][1]; B[3][3 * a + 1] = DN[a][0];
            B[4][3 * a + 1] = DN[a][2]; B[4][3 * a + 2] = DN[a][1];
            B[5][3 * a] = DN[a][2]; B[5][3 * a + 2] = DN[a][0];
        }
        memcpy(B_gp[gp], B, sizeof(B));
        double BT[18][6];
        for (int r = 0; r < 18; ++r)
            for (int k = 0; k < 6; ++k) {
                double v = B[k][r] * detF;
                BT[r][k] = v * detdXde;
            }
        double currge[18], currgv[18] = {0};
        for (int r = 0; r < 18; ++r) {
            double acc = 0.0;
            for (int k = 0; k < 6; ++k) acc += BT[r][k] * compact[k];
            currge[r] = acc;
        }
        memset(Sv_gp[gp], 0, sizeof(Sv_gp[gp]));
        if (eta != 0) { /* Prism.cpp:850-858, ShapeBase.cpp:2413-2617 */
            double l[6];
            for (int r = 0; r < 6; ++r) {
                double acc = 0.0;
                for (int c = 0; c < 18; ++c) acc += B[r][c] * ve[c];
                l[r] = acc;
            }
            double d[9] = {l[0], 0.5 * l[3], 0.5 * l[5], 0.5 * l[3], l[1], 0.5 * l[4], 0.5 * l[5], 0.5 * l[4], l[2]};
            double Sv[9];
            for (int k = 0; k < 9; ++k) Sv[k] = d[k] * eta;
            memcpy(Sv_gp[gp], Sv, sizeof(Sv));
            double cv[6] = {Sv[0], Sv[4], Sv[8], Sv[1], Sv[7], Sv[2]};
            for (int r = 0; r < 18; ++r) {
                double acc = 0.0;
                for (int k = 0; k < 6; ++k) acc += BT[r][k] * cv[k];
                currgv[r] = acc;
            }
        }
        for (int r = 0; r < 18; ++r) {
            Tge[r] += currge[r] * GW;
            Tgv[r] += currgv[r] * GW;
        }
    }
    /* element forces with the fixed-DOF mask, ShapeBase.cpp:2203-2227 */
    for (int a = 0; a < 6; ++a)
        for (int d = 0; d < 3; ++d) {
            int fx = m->fixed[3 * conn[a] + d];
            if (fe) fe[3 * a + d] = fx ? 0.0 : 0.0 - Tge[3 * a + d];
            if (fv) fv[3 * a + d] = fx ? 0.0 : 0.0 - Tgv[3 * a + d];
        }
    if (!want_k) return;

    /* elastic tangent, ShapeBase.cpp:2619-2639, :2786-2890 */
    if (Ke) {
        for (int k = 0; k < 324; ++k) Ke[k] = 0.0;
        for (int gp = 0; gp < 6; ++gp) {
            double cK[324];
            memset(cK, 0, sizeof(cK));
            const double* Fe = Fe_gp[gp];
            const double detF = detF_gp[gp], detdXde = m->detdXde[6 * e + gp];
            const double detFe = det3(Fe);
            for (int a = 0; a < 6; ++a)
                for (int b = 0; b < 6; ++b) {
                    const double* DNa = DN_gp[gp][a];
                    const double* DNb = DN_gp[gp][b];
                    double Keab[9];
                    if (mode == TFO_LITERAL) {
                        for (int i = 0; i < 3; ++i)
                            for (int k = 0; k < 3; ++k) {
                                double value = 0;
                                for (int j = 0; j < 3; ++j)
                                    for (int l = 0; l < 3; ++l)
                                        for (int I = 0; I < 3; ++I)
                                            for (int J = 0; J < 3; ++J)
                                                for (int K = 0; K < 3; ++K)
                                                    for (int L = 0; L < 3; ++L)
                                                        value += (Fe[3 * i + I] * Fe[3 * j + J] * Fe[3 * k + K] * Fe[3 * l + L] *
                                                                  D81[gp][I][J][K][L] * DNb[l] * DNa[j]);
                                value *= detF * detdXde;
                                value /= detFe;
                                value += 0.0;
                                Keab[3 * i + k] = value;
                            }
                    } else {
                        const double lnJ = lnJ_gp[gp];
                        double s = DNa[0] * DNb[0] + DNa[1] * DNb[1] + DNa[2] * DNb[2];
                        for (int i = 0; i < 3; ++i)
                            for (int k = 0; k < 3; ++k) {
                                double value = lambda * DNa[i] * DNb[k] +
                                               (mu - lambda * lnJ) * (((i == k) ? s : 0.0) + DNa[k] * DNb[i]);
                                value *= detF * detdXde;
                                value /= detFe;
                                Keab[3 * i + k] = value;
                            }
                    }
                    for (int i = 0; i < 3; ++i)
                        for (int j = 0; j < 3; ++j) cK[(3 * a + i) * 18 + 3 * b + j] += Keab[3 * i + j];
                }
            const double* Stress = S_gp[gp];
            for (int a = 0; a < 6; ++a)
                for (int b = 0; b < 6; ++b) {
                    const double* DNa = DN_gp[gp][a];
                    const double* DNb = DN_gp[gp][b];
                    double tmp1[3];
                    for (int j = 0; j < 3; ++j) {
                        double acc = 0.0;
                        for (int i = 0; i < 3; ++i) acc += DNa[i] * Stress[3 * i + j];
                        tmp1[j] = acc;
                    }
                    double Keab2 = 0.0;
                    for (int j = 0; j < 3; ++j) Keab2 += tmp1[j] * DNb[j];
                    double value = Keab2 * detF * detdXde;
                    for (int i = 0; i < 3; ++i) cK[(3 * a + i) * 18 + 3 * b + i] += value;
                }
            for (int k = 0; k < 324; ++k) Ke[k] += cK[k] * GW;
        }
    }
    /* viscous tangent, ShapeBase.cpp:2641-2705, :2892-3053, :3093-3103 */
    if (Kv) {
        for (int k = 0; k < 324; ++k) Kv[k] = 0.0;
        if (eta != 0) {
            for (int gp = 0; gp < 6; ++gp) {
                double cK[324];
                memset(cK, 0, sizeof(cK));
                const double detF = detF_gp[gp], detdXde = m->detdXde[6 * e + gp];
                double vg[9] = {0};
                for (int c = 0; c < 6; ++c)
                    for (int i = 0; i < 3; ++i)
                        for (int j = 0; j < 3; ++j) vg[3 * i + j] += ve[3 * c + i] * DN_gp[gp][c][j];
                double par[9];
                for (int k = 0; k < 9; ++k) par[k] = ((k % 4 == 0) ? 1.0 : 0.0) * (1.0 / dt);
                for (int k = 0; k < 9; ++k) par[k] -= vg[k];
                const double(*B)[18] = B_gp[gp];
                for (int a = 0; a < 6; ++a)
                    for (int b = 0; b < 6; ++b) {
                        double BaT[3][6], Bb[6][3], BaTBb[9], K1[9];
                        for (int i = 0; i < 6; ++i)
                            for (int j = 0; j < 3; ++j) {
                                BaT[j][i] = B[i][3 * a + j];
                                Bb[i][j] = B[i][3 * b + j];
                            }
                        for (int i = 3; i < 6; ++i)
                            for (int j = 0; j < 3; ++j) Bb[i][j] = 0.5 * Bb[i][j];
                        for (int p = 0; p < 3; ++p)
                            for (int q = 0; q < 3; ++q) {
                                double acc = 0.0;
                                for (int r = 0; r < 6; ++r) acc += BaT[p][r] * Bb[r][q];
                                BaTBb[3 * p + q] = acc;
                            }
                        mm3(BaTBb, par, K1);
                        for (int k = 0; k < 9; ++k) K1[k] *= detF;
                        for (int k = 0; k < 9; ++k) K1[k] *= detdXde;
                        for (int k = 0; k < 9; ++k) K1[k] *= eta;
                        for (int i = 0; i < 3; ++i)
                            for (int j = 0; j < 3; ++j) cK[(3 * b + j) * 18 + 3 * a + i] += K1[3 * i + j];
                    }
                const double* Sv = Sv_gp[gp];
                for (int a = 0; a < 6; ++a)
                    for (int b = 0; b < 6; ++b) {
                        const double* DNa = DN_gp[gp][a];
                        const double* DNb = DN_gp[gp][b];
                        double par2[9], K2[9];
                        for (int i = 0; i < 3; ++i)
                            for (int j = 0; j < 3; ++j) {
                                double o1 = DNa[i] * DNb[j];
                                double o2 = DNb[i] * DNa[j];
                                par2[3 * i + j] = o1 - o2;
                            }
                        mm3(Sv, par2, K2);
                        for (int k = 0; k < 9; ++k) K2[k] *= detF;
                        for (int k = 0; k < 9; ++k) K2[k] *= detdXde;
                        for (int i = 0; i < 3; ++i)
                            for (int j = 0; j < 3; ++j) cK[(3 * b + j) * 18 + 3 * a + i] += K2[3 * i + j];
                    }
                for (int k = 0; k < 324; ++k) Kv[k] += cK[k] * GW;
            }
        }
    }
}

static void velocity(const tfo_model* m, const double* uk, const double* un, double dt, double* vel) {
    /* NewtonRaphsonSolver::calculateDisplacementMatrix :148-152 */
    for (int i = 0; i < 3 * m->nn; ++i) {
        double v = uk[i];
        v -= un[i];
        vel[i] = v * (1.0 / dt);
    }
}

void tfo_element_eval(tfo_model* m, const double* uk, const double* un, double dt, int mode,
                      int e0, int count, double* Ke, double* Kv, double* fe, double* fv) {
    double* vel = (double*)malloc(sizeof(double) * 3 * (size_t)m->nn);
    velocity(m, uk, un, dt, vel);
    int want_k = (Ke != NULL) || (Kv != NULL);
#pragma omp parallel for schedule(dynamic, 16)
    for (int k = 0; k < count; ++k) {
        int e = e0 + k;
        element_eval(m, e, uk, vel, dt, mode, want_k, Ke ? &Ke[324L * k] : NULL, Kv ? &Kv[324L * k] : NULL,
                     fe ? &fe[18L * k] : NULL, fv ? &fv[18L * k] : NULL);
    }
    free(vel);
}

static void ensure_scratch(tfo_model* m) {
    if (m->Ke) return;
    m->Ke = (double*)malloc(sizeof(double) * 324 * (size_t)m->ne);
    m->Kv = (double*)malloc(sizeof(double) * 324 * (size_t)m->ne);
    m->fe = (double*)malloc(sizeof(double) * 18 * (size_t)m->ne);
    m->fv = (double*)malloc(sizeof(double) * 18 * (size_t)m->ne);
}

/* The body of one Newton iteration up to (not including) the solve:
 * Simulation.cpp:6473-6546 with NewtonRaphsonSolver.cpp:102-378. */
long tfo_assemble(tfo_model* m, const double* uk, const double* un, double dt, int mode) {
    ensure_scratch(m);
    const int N3 = 3 * m->nn;
    double* vel = (double*)malloc(sizeof(double) * (size_t)N3);
    velocity(m, uk, un, dt, vel);
#pragma omp parallel for schedule(dynamic, 16)
    for (int e = 0; e < m->ne; ++e)
        element_eval(m, e, uk, vel, dt, mode, 1, &m->Ke[324L * e], &m->Kv[324L * e], &m->fe[18L * e], &m->fv[18L * e]);
    double* ge = (double*)calloc((size_t)N3, sizeof(double));
    double* gvi = (double*)calloc((size_t)N3, sizeof(double));
    /* writeForcesTogeAndgvInternal :273-279 -> ShapeBase.cpp:2148-2165 */
    for (int e = 0; e < m->ne; ++e)
        for (int a = 0; a < 6; ++a)
            for (int d = 0; d < 3; ++d) {
                int I = 3 * m->conn[6 * e + a] + d;
                ge[I] = ge[I] + m->fe[18L * e + 3 * a + d];
                gvi[I] = gvi[I] + m->fv[18L * e + 3 * a + d];
            }
    /* writeImplicitElementalKToJacobian :281-295: all Kv, then all Ke */
    memset(m->a, 0, sizeof(double) * (size_t)m->nnz);
    for (int pass = 0; pass < 2; ++pass)
        for (int e = 0; e < m->ne; ++e) {
            if (pass == 0 && m->eta[e] == 0) continue;
            const double* Kel = pass == 0 ? &m->Kv[324L * e] : &m->Ke[324L * e];
            const int* c = &m->conn[6 * e];
            for (int a = 0; a < 6; ++a)
                for (int b = 0; b < 6; ++b) {
                    long base = entry_index(m, c[a], c[b], 0, 0);
                    for (int i = 0; i < 3; ++i) {
                        long row = base + (m->ia[3 * c[a] + i] - m->ia[3 * c[a]]);
                        for (int j = 0; j < 3; ++j) m->a[row + j] += Kel[(3 * a + i) * 18 + 3 * b + j];
                    }
                }
        }
    /* calculateExternalViscousForcesForNR :297-324 (surface based) */
    for (int i = 0; i < m->nn; ++i)
        for (int d = 0; d < 3; ++d) {
            double sv = m->area[i] * m->ext_visc[3 * i + d];
            double val = sv * vel[3 * i + d];
            m->g[3 * i + d] = val * -1.0;
        }
    /* addImplicitKViscousExternalToJacobian :326-348 */
    for (int i = 0; i < m->nn; ++i) {
        double apdt = m->area[i] / dt;
        for (int d = 0; d < 3; ++d) {
            long p = entry_index(m, i, i, d, d);
            m->a[p] = apdt * m->ext_visc[3 * i + d] + m->a[p];
        }
    }
    /* calculateSumOfInternalForces :363-367, addExernalForces :369-378 */
    for (int k = 0; k < N3; ++k) {
        double s = ge[k] + gvi[k] + m->g[k];
        m->g[k] = s + 0.0;
    }
    /* calcutateFixedK :237-255: gSum only; rows/cols are applied on export */
    for (int k = 0; k < N3; ++k)
        if (m->fixed[k]) m->g[k] = 0.0;
    free(ge); free(gvi); free(vel);
    return m->nnz;
}

/* A bounded sample of one K+f assembly for timing: the element loop over the
 * first `count` prisms (OpenMP) and their serial scatter into K and g in the
 * reference's order.  Returns the number of prisms processed. */
long tfo_assemble_sample(tfo_model* m, const double* uk, const double* un, double dt, int mode, int count) {
    if (count > m->ne) count = m->ne;
    const int N3 = 3 * m->nn;
    double* vel = (double*)malloc(sizeof(double) * (size_t)N3);
    velocity(m, uk, un, dt, vel);
    double* Ke = (double*)malloc(sizeof(double) * 324 * (size_t)count);
    double* Kv = (double*)malloc(sizeof(double) * 324 * (size_t)count);
    double* fe = (double*)malloc(sizeof(double) * 18 * (size_t)count);
    double* fv = (double*)malloc(sizeof(double) * 18 * (size_t)count);
#pragma omp parallel for schedule(dynamic, 16)
    for (int e = 0; e < count; ++e)
        element_eval(m, e, uk, vel, dt, mode, 1, &Ke[324L * e], &Kv[324L * e], &fe[18L * e], &fv[18L * e]);
    memset(m->a, 0, sizeof(double) * (size_t)m->nnz);
    for (int k = 0; k < N3; ++k) m->g[k] = 0.0;
    for (int e = 0; e < count; ++e)
        for (int a = 0; a < 6; ++a)
            for (int d = 0; d < 3; ++d) {
                int I = 3 * m->conn[6 * e + a] + d;
                m->g[I] = m->g[I] + fe[18L * e + 3 * a + d] + fv[18L * e + 3 * a + d];
            }
    for (int pass = 0; pass < 2; ++pass)
        for (int e = 0; e < count; ++e) {
            if (pass == 0 && m->eta[e] == 0) continue;
            const double* Kel = pass == 0 ? &Kv[324L * e] : &Ke[324L * e];
            const int* c = &m->conn[6 * e];
            for (int a = 0; a < 6; ++a)
                for (int b = 0; b < 6; ++b) {
                    long base = entry_index(m, c[a], c[b], 0, 0);
                    for (int i = 0; i < 3; ++i) {
                        long row = base + (m->ia[3 * c[a] + i] - m->ia[3 * c[a]]);
                        for (int j = 0; j < 3; ++j) m->a[row + j] += Kel[(3 * a + i) * 18 + 3 * b + j];
                    }
                }
        }
    free(vel); free(Ke); free(Kv); free(fe); free(fv);
    return count;
}

long tfo_structure_nnz(const tfo_model* m) { return m->nnz; }

void tfo_get_structure(const tfo_model* m, int* ia, int* ja) {
    memcpy(ia, m->ia, sizeof(int) * (size_t)(3 * m->nn + 1));
    memcpy(ja, m->ja, sizeof(int) * (size_t)m->nnz);
}

/* Values with calcutateFixedK applied (row and column zero, diagonal 1). */
void tfo_get_values(const tfo_model* m, double* a, double* g) {
    if (a)
        for (int r = 0; r < 3 * m->nn; ++r)
            for (int p = m->ia[r]; p < m->ia[r + 1]; ++p) {
                int c = m->ja[p];
                a[p] = (m->fixed[r] || m->fixed[c]) ? (r == c ? 1.0 : 0.0) : m->a[p];
            }
    if (g) memcpy(g, m->g, sizeof(double) * 3 * (size_t)m->nn);
}

/* constructiaForPardiso :686-707 */
long tfo_export_filtered(const tfo_model* m, double drop, int* ia, int* ja, double* a) {
    long q = 0;
    if (ia) ia[0] = 0;
    for (int r = 0; r < 3 * m->nn; ++r) {
        for (int p = m->ia[r]; p < m->ia[r + 1]; ++p) {
            int c = m->ja[p];
            double v = (m->fixed[r] || m->fixed[c]) ? (r == c ? 1.0 : 0.0) : m->a[p];
            if (v > drop || v < -drop) {
                if (ja) { ja[q] = c; a[q] = v; }
                ++q;
            }
        }
        if (ia) ia[r + 1] = (int)q;
    }
    return q;
}

void tfo_residual(tfo_model* m, const double* uk, const double* un, double dt, double* g) {
    const int N3 = 3 * m->nn;
    double* vel = (double*)malloc(sizeof(double) * (size_t)N3);
    velocity(m, uk, un, dt, vel);
    double* fe = (double*)malloc(sizeof(double) * 18 * (size_t)m->ne);
    double* fv = (double*)malloc(sizeof(double) * 18 * (size_t)m->ne);
#pragma omp parallel for schedule(dynamic, 64)
    for (int e = 0; e < m->ne; ++e) element_eval(m, e, uk, vel, dt, TFO_CLOSED, 0, NULL, NULL, &fe[18L * e], &fv[18L * e]);
    double* ge = (double*)calloc((size_t)N3, sizeof(double));
    double* gvi = (double*)calloc((size_t)N3, sizeof(double));
    for (int e = 0; e < m->ne; ++e)
        for (int a = 0; a < 6; ++a)
            for (int d = 0; d < 3; ++d) {
                int I = 3 * m->conn[6 * e + a] + d;
                ge[I] += fe[18L * e + 3 * a + d];
                gvi[I] += fv[18L * e + 3 * a + d];
            }
    for (int i = 0; i < m->nn; ++i)
        for (int d = 0; d < 3; ++d) {
            int k = 3 * i + d;
            double gv = (m->area[i] * m->ext_visc[k] * vel[k]) * -1.0;
            g[k] = m->fixed[k] ? 0.0 : (ge[k] + gvi[k] + gv);
        }
    free(ge); free(gvi); free(fe); free(fv); free(vel);
}

int tfo_solve(tfo_model* m, double* du) {
    const int N3 = 3 * m->nn;
    long nnz = tfo_export_filtered(m, 1E-13, NULL, NULL, NULL);
    int* ia = (int*)malloc(sizeof(int) * (size_t)(N3 + 1));
    int* ja = (int*)malloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
    double* a = (double*)malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
    tfo_export_filtered(m, 1E-13, ia, ja, a);
    /* Pardiso phase 33 with iparm[11] = 1 (transpose) and iparm[7] = 1 */
    int rc = tfb_solve_csr(N3, ia, ja, a, m->g, du, 1, 1);
    free(ia); free(ja); free(a);
    return rc;
}

/* Simulation::updateStepNR, Simulation.cpp:6449-6590 (preceded by the growth
 * and viscosity-surface updates of runOneStep :5906-5915). */
int tfo_step(tfo_model* m, double dt, const double* rates, int mode, int* iters,
             double* dunorm_hist, int max_hist) {
    if (rates) tfo_grow(m, dt, rates);
    tfo_update_viscosity_surfaces(m, NULL);
    const int N3 = 3 * m->nn;
    double* un = (double*)malloc(sizeof(double) * (size_t)N3);
    double* uk = (double*)malloc(sizeof(double) * (size_t)N3);
    double* du = (double*)malloc(sizeof(double) * (size_t)N3);
    memcpy(un, m->pos, sizeof(double) * (size_t)N3);
    memcpy(uk, un, sizeof(double) * (size_t)N3);
    int k = 0, converged = 0, capped = 0, rc = 0;
    const int maxIteration = 20;
    while (!converged) {
        tfo_assemble(m, uk, un, dt, mode);
        if (tfo_solve(m, du) != 0) { rc = -1; break; }
        double s = 0.0;
        for (int i = 0; i < N3; ++i) s += du[i] * du[i];
        double d = sqrt(s);
        if (k < max_hist) dunorm_hist[k] = d;
        converged = !(d > 1E-8);
        for (int i = 0; i < N3; ++i) uk[i] = uk[i] + du[i];
        k++;
        if (!converged && k > maxIteration) { capped = 1; converged = 1; }
    }
    memcpy(m->pos, uk, sizeof(double) * (size_t)N3);
    *iters = k;
    free(un); free(uk); free(du);
    return rc ? rc : capped;
}
