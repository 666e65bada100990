// Smoothed-aggregation algebraic multigrid: the preconditioner of the
// Krylov solve of A du = g (A = K^T) on large meshes, in place of the
// block-Jacobi one.  No counterpart in the reference, which factorises the
// system with Pardiso (NewtonRaphsonSolver.cpp:418-683); the solution it
// converges to is the same (the Krylov tolerance is unchanged).
//
// Set-up, once per handle, on the host from the block pattern and the
// reference node positions:
//   * greedy aggregation of the node graph: a node whose neighbours are all
//     free becomes an aggregate with them; left-over nodes join the
//     neighbouring aggregate they touch most.  Aggregates never cross
//     instances (the graph of a batch is disconnected);
//   * near-null space: the six rigid-body modes at level 0 (translations and
//     rotations about the aggregate centroid), zero on fixed DOFs; at coarser
//     levels the R factors of the level below;
//   * tentative prolongator per aggregate from a modified Gram-Schmidt QR of
//     its near-null-space rows (6 coarse DOFs per aggregate; a dependent
//     column is dropped and its coarse DOF gets a unit diagonal);
//   * block patterns of the smoothed prolongator P = (I - omega D^-1 A) P_t
//     (node i couples to the aggregates of its neighbours), of T = A P and of
//     the coarse matrix P^T T, with per output block the ordered list of the
//     products that make it (no atomics, reproducible).
//   Plain aggregation (tf_options.precond 3) keeps P = P_t.
// Numeric phase, once per time step (all on the device), level by level:
//   lambda_max of D^-1 A by power iteration (smoother weight and prolongator
//   smoothing weight omega = 4 / (3.15 lambda)); P; T = A P; A_{l+1} = P^T T;
//   6x6 block inverses; Gauss-Jordan inverse of the coarsest level per
//   instance (<= 16 nodes).
// Application (one V-cycle per preconditioner call, all kernels, capturable
// in a CUDA graph): damped block-Jacobi pre- and post-smoothing (one sweep
// each way at level 0, kCoarseSweeps on the coarser levels), residual,
// restriction, coarse correction.  Kernels of an instance whose Krylov
// solve has stopped return at once.
// Precision: the preconditioner is any fixed linear operator as far as the
// Krylov method is concerned, so the whole V-cycle -- its matrices (an FP32
// copy of the level-0 values and block inverses, the coarse operators and
// prolongators) and its vectors -- is FP32: half the bytes of its
// bandwidth-bound sweeps, and no FP32/FP64 conversions on the FP64 pipe.  The
// level-0 smoother reads S = D^-1 A in FP16 (entries of order one), a quarter
// of the FP64 bytes.
// The Krylov recurrences, their SpMVs with A and the convergence test are
// untouched FP64.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include <cuda_fp16.h>

#include "tf_internal.cuh"

namespace tf {

namespace {

constexpr int kT = 256;
constexpr int kCoarseNodes = 16;  // nodes per instance at the coarsest level (96 DOFs)
constexpr int kCoarseDofs = 6 * kCoarseNodes;
constexpr int kPowerIters = 16;
constexpr int kTailNodes = 256;   // levels with at most this many nodes per instance run fused
constexpr int kTailThreads = 1024;
// damped block-Jacobi sweeps before and after the coarse correction on the
// levels >= 1 (level 0 sweeps once each way): more sweeps on the small,
// launch-bound coarse levels cut the Krylov iterations (320,000-prism sheet:
// 88 / 64 / 58 per step with 1 / 2 / 3 sweeps, 80 / 68.7 / 68.4 ms; 1M-prism
// wing: 201 / 150 / 128, 177 / 153 / 144 ms) while extra level-0 sweeps,
// which cost a full-size SpMV each, barely do
constexpr int kCoarseSweeps = 3;

// ---- host set-up -----------------------------------------------------------------

struct HostLevel {
    int n = 0, bs = 3;
    std::vector<int> rowptr, colidx;   // block pattern of this level
    std::vector<int> seg0;             // [nseg+1] node offsets per instance
    std::vector<double> B;             // [n * bs * 6] near-null space rows
};

// Greedy aggregation; returns the aggregate of each node and their count.
int aggregate(const std::vector<int>& rowptr, const std::vector<int>& colidx, int n, std::vector<int>& agg) {
    agg.assign(n, -1);
    int na = 0;
    for (int i = 0; i < n; ++i) {
        if (agg[i] >= 0) continue;
        bool free = true;
        for (int p = rowptr[i]; p < rowptr[i + 1] && free; ++p) free = agg[colidx[p]] < 0;
        if (!free) continue;
        for (int p = rowptr[i]; p < rowptr[i + 1]; ++p) agg[colidx[p]] = na;
        agg[i] = na++;
    }
    std::vector<int> cnt;
    for (int i = 0; i < n; ++i) {
        if (agg[i] >= 0) continue;
        // join the neighbouring aggregate with most connections (smallest id on ties)
        int best = -1, bestc = 0;
        for (int p = rowptr[i]; p < rowptr[i + 1]; ++p) {
            const int a = agg[colidx[p]];
            if (a < 0) continue;
            int c = 0;
            for (int q = rowptr[i]; q < rowptr[i + 1]; ++q) c += agg[colidx[q]] == a;
            if (c > bestc || (c == bestc && a < best)) {
                best = a;
                bestc = c;
            }
        }
        agg[i] = best >= 0 ? best : na++;
    }
    return na;
}

// Modified Gram-Schmidt of the m x 6 matrix M (row-major) in place: Q in M,
// R (6 x 6, row-major).  Returns the mask of dropped (dependent) columns.
int mgs(std::vector<double>& M, int m, double* R) {
    int dead = 0;
    std::fill(R, R + 36, 0.0);
    double ref[6];
    for (int c = 0; c < 6; ++c) {
        double s = 0.0;
        for (int r = 0; r < m; ++r) s += M[6 * r + c] * M[6 * r + c];
        ref[c] = std::sqrt(s);
    }
    for (int c = 0; c < 6; ++c) {
        for (int q = 0; q < c; ++q) {
            if (dead & (1 << q)) continue;
            double s = 0.0;
            for (int r = 0; r < m; ++r) s += M[6 * r + q] * M[6 * r + c];
            R[6 * q + c] = s;
            for (int r = 0; r < m; ++r) M[6 * r + c] -= s * M[6 * r + q];
        }
        double s = 0.0;
        for (int r = 0; r < m; ++r) s += M[6 * r + c] * M[6 * r + c];
        const double nv = std::sqrt(s);
        if (!(nv > 1e-10 * ref[c]) || !(ref[c] > 0.0)) {
            dead |= 1 << c;
            for (int r = 0; r < m; ++r) M[6 * r + c] = 0.0;
            for (int q = 0; q < 6; ++q) R[6 * q + c] = 0.0;
            continue;
        }
        R[6 * c + c] = nv;
        for (int r = 0; r < m; ++r) M[6 * r + c] /= nv;
    }
    return dead;
}

template <class T>
tf_status up(T** dst, const std::vector<T>& v) {
    const size_t n = std::max<size_t>(v.size(), 1);
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(dst), n * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("device allocation failed in the multigrid set-up");
        return TF_OUT_OF_MEMORY;
    }
    if (!v.empty()) TF_CUDA(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return TF_OK;
}

template <class T>
tf_status zeros(T** dst, size_t n) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(dst), std::max<size_t>(n, 1) * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("device allocation failed in the multigrid set-up");
        return TF_OUT_OF_MEMORY;
    }
    TF_CUDA(cudaMemset(*dst, 0, std::max<size_t>(n, 1) * sizeof(T)));
    return TF_OK;
}

#define AMG_TRY(expr)               \
    do {                            \
        tf_status _s = (expr);      \
        if (_s != TF_OK) return _s; \
    } while (0)


}  // namespace

// Device view of one level: what the V-cycle reads and writes, all FP32
// (see the precision note above); the smoother weights are FP64 scalars.
struct AmgLevel {
    int n = 0, bs = 3;
    // matrix of levels >= 1: CSR of 6x6 row-major blocks
    int* rowptr = nullptr;
    int* colidx = nullptr;
    int* rowof = nullptr;
    int* diag = nullptr;  // block index of (i, i)
    float* val = nullptr;
    int64_t nnzb = 0;
    float* dinv = nullptr;   // [n][36] block inverses (levels >= 1)
    int* seg = nullptr;      // [n] instance of each node (levels >= 1)
    int* seg0 = nullptr;     // [nseg+1] node offsets per instance (levels >= 1)
    // prolongator to level + 1 (absent at the coarsest level): bs x 6
    // row-major blocks, once by fine row and once by coarse column
    int* prow = nullptr;     // [n+1] blocks of each fine node
    int* pcol = nullptr;     // [npb] coarse node of each block
    float* Pv = nullptr;     // [npb][bs*6]
    int* pcptr = nullptr;    // [n_{l+1}+1] blocks of each coarse node (column order)
    int* pcrow = nullptr;    // [npb] fine node of each block, column order
    float* Pc = nullptr;     // [npb][bs*6] the blocks in column order
    __half* Pvh = nullptr;   // level 0: FP16 copies of Pv and Pc for the V-cycle's transfers
    __half* Pch = nullptr;
    __half* valh = nullptr;  // levels >= 1: S = D^-1 A in FP16 [nnzb][36] for the V-cycle's sweeps
    int64_t npb = 0;
    uint8_t* dead = nullptr; // [n * bs] (levels >= 1) DOFs with a zero prolongator column
    // coarse image of the extra blocks outside the element pattern (levels >=
    // 1): X_l = P^T X_{l-1} P, CSR of 6x6 blocks (null: none)
    int* xrow = nullptr;
    int* xcol = nullptr;
    float* xval = nullptr;
    int64_t nx = 0;
    // vectors (levels >= 1: r input, e output; all levels: x, t work)
    float *r = nullptr, *x = nullptr, *t = nullptr, *e = nullptr;
    int ncoarse = 0;         // nodes of level + 1
    int* check = nullptr;    // checked build: failed index checks
};

// Lists of the numeric set-up of the transfer from level l to l + 1
// (device arrays, built once on the host from the block patterns).
struct AmgSetup {
    float* Pt = nullptr;     // [n][bs*6] tentative prolongator (one block per fine node)
    int* agg = nullptr;      // [n] aggregate of each fine node
    int* pbrow = nullptr;    // [npb] fine node of each prolongator block
    int* sptr = nullptr;     // [npb+1] fine-matrix blocks (i, j), agg(j) = column, per block (i, .)
    int* slist = nullptr;
    int* cperm = nullptr;    // [npb] row-order block at each column-order position
    int64_t nT = 0;          // blocks of T = A P (bs x 6)
    int* trow = nullptr;     // [nT] fine node of each T block
    int* tptr = nullptr;     // [nT+1] pairs (fine-matrix block, prolongator block) per T block
    int* ta = nullptr;
    int* tb = nullptr;
    float* T = nullptr;      // [nT][bs*6]
    int* gptr = nullptr;     // [nnzb_{l+1}+1] pairs (prolongator block, T block) per coarse block
    int* gp = nullptr;
    int* gt = nullptr;
    int* xptr = nullptr;     // [nx_{l+1}+1] triples (extra block (J, I), P block (J, K), P block (I, M))
    int* xtrip = nullptr;    // per coarse extra block (K, M)
};

struct Amg {
    int nlev = 0;
    bool smooth = true;        // smoothed (true) or plain (false) aggregation
    AmgLevel L[kAmgMaxLevels];
    AmgSetup S[kAmgMaxLevels];
    double* omega = nullptr;   // [nlev] smoother weights
    double* pscal = nullptr;   // [nlev][2] power-iteration scalars (scale, lambda)
    float* pv = nullptr;       // power-iteration vectors (max n*bs each)
    float* pw = nullptr;
    double* part = nullptr;    // per-CTA partial sums
    unsigned* ticket = nullptr;
    float* val32 = nullptr;    // FP32 copy of the level-0 values (sliced layout)
    // the smoother's level-0 operator S = D^-1 A in FP16, slot by slot in the
    // sliced order: entries 0-7 of a row's block as one 16-byte pack
    // ([slot][lane][8]), then entry 8 of every block ([slot][lane]) -- two
    // loads per block instead of nine
    __half* valh = nullptr;
    float* dinv32 = nullptr;   // FP32 copy of the level-0 block inverses
    float* diag32 = nullptr;   // FP32 copy of the level-0 diagonal blocks, [9 n] row-major
    int nseg = 1;
    int* cnode0 = nullptr;     // [nseg+1] coarsest-level node offsets per instance
    int* cinv0 = nullptr;      // [nseg+1] offsets of the dense inverses
    float* cinv = nullptr;     // coarsest inverses, m_g x m_g row-major
    bool coarse_exact = true;
    int max_cm = 0;
    int v0_smem = 0;           // shared memory of the level-0 prolongation (3 floats per block of a CTA)
    int tail = 0;              // levels tail..nlev-1 run in one kernel (one CTA per instance); 0: none
    int smooth_unroll = 4;     // slots in flight per lane in the level-0 smoother's row product (2, 4, 8)
    std::vector<int> h_n;      // nodes per level (host)
    std::vector<int> h_prow[kAmgMaxLevels], h_pcol[kAmgMaxLevels];  // prolongator patterns (host)
    int64_t x_version = -1;    // extra-block layout the coarse extra blocks were built for
    // what the next solve has to redo: 0 nothing, 1 the FP32 copies of the
    // level-0 matrix (new assembly, same time step), 2 the whole hierarchy
    int stale = 2;
    bool reused = false;       // the last numeric phase kept the coarse levels
    long rebuilds = 0;         // full numeric rebuilds so far
};

void amg_free(Amg* a) {
    if (!a) return;
    for (int l = 0; l < a->nlev; ++l) {
        AmgLevel& L = a->L[l];
        void* ptrs[] = {L.rowptr, L.colidx, L.rowof, L.diag, L.val, L.seg, L.seg0, L.prow, L.pcol, L.Pv,
                        L.pcptr, L.pcrow, L.Pc, L.dead, L.r, L.x, L.t, L.e, L.Pvh, L.Pch, L.valh};
        for (void* p : ptrs)
            if (p) cudaFree(p);
        if (l > 0 && L.dinv) cudaFree(L.dinv);
        AmgSetup& S = a->S[l];
        void* sptrs[] = {S.Pt, S.agg, S.pbrow, S.sptr, S.slist, S.cperm, S.trow, S.tptr, S.ta, S.tb, S.T,
                         S.gptr, S.gp, S.gt, S.xptr, S.xtrip, L.xrow, L.xcol, L.xval};
        for (void* p : sptrs)
            if (p) cudaFree(p);
    }
    void* ptrs[] = {a->omega, a->pscal, a->pv, a->pw, a->part, a->ticket, a->cnode0, a->cinv0, a->cinv,
                    a->val32, a->dinv32, a->valh, a->diag32};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete a;
}

// Symbolic set-up from the level-0 pattern, the reference positions and the
// fixed DOFs.  Level 0 uses the handle's own matrix, block inverses and
// sliced storage.
tf_status amg_build(tf_handle* h, const double* pos) {
    Device& d = h->d;
    Amg* a = new Amg;
    h->amg = a;
    a->nseg = d.nseg;
    a->smooth = h->opt.precond != 3;
    std::vector<HostLevel> H(1);
    H[0].n = d.nn;
    H[0].bs = 3;
    H[0].rowptr = h->h_rowptr;
    H[0].colidx = h->h_colidx;
    H[0].seg0 = h->h_seg_node0;
    int lev = 0;
    while (true) {
        HostLevel& F = H[lev];
        int maxn = 0;
        for (int g = 0; g < d.nseg; ++g) maxn = std::max(maxn, F.seg0[g + 1] - F.seg0[g]);
        if (maxn <= kCoarseNodes || lev + 1 >= kAmgMaxLevels) break;
        std::vector<int> agg;
        const int na = aggregate(F.rowptr, F.colidx, F.n, agg);
        if (na >= F.n) break;  // no coarsening possible
        // members per aggregate (node order)
        std::vector<int> mptr(na + 1, 0), mlist(F.n);
        for (int i = 0; i < F.n; ++i) mptr[agg[i] + 1]++;
        for (int c = 0; c < na; ++c) mptr[c + 1] += mptr[c];
        {
            std::vector<int> fill(mptr.begin(), mptr.end() - 1);
            for (int i = 0; i < F.n; ++i) mlist[fill[agg[i]]++] = i;
        }
        // tentative prolongator and the next near-null space
        const int bs = F.bs;
        std::vector<double> P((size_t)F.n * bs * 6, 0.0), Bc((size_t)na * 36, 0.0);
        std::vector<uint8_t> dead((size_t)na * 6, 0);
        std::vector<double> M;
        for (int c = 0; c < na; ++c) {
            const int m0 = mptr[c], m1 = mptr[c + 1];
            const int rows = (m1 - m0) * bs;
            M.assign((size_t)rows * 6, 0.0);
            if (lev == 0) {
                double cen[3] = {0, 0, 0};
                for (int q = m0; q < m1; ++q)
                    for (int k = 0; k < 3; ++k) cen[k] += pos[3 * (size_t)mlist[q] + k];
                for (int k = 0; k < 3; ++k) cen[k] /= (m1 - m0);
                for (int q = m0; q < m1; ++q) {
                    const int i = mlist[q];
                    const double rx = pos[3 * (size_t)i] - cen[0], ry = pos[3 * (size_t)i + 1] - cen[1],
                                 rz = pos[3 * (size_t)i + 2] - cen[2];
                    // rows x, y, z of [I | e_x x r, e_y x r, e_z x r]
                    const double rowsv[3][6] = {{1, 0, 0, 0, rz, -ry}, {0, 1, 0, -rz, 0, rx}, {0, 0, 1, ry, -rx, 0}};
                    for (int k = 0; k < 3; ++k) {
                        const bool fx = h->h_fixed[3 * (size_t)i + k] != 0;
                        for (int col = 0; col < 6; ++col)
                            M[(size_t)(bs * (q - m0) + k) * 6 + col] = fx ? 0.0 : rowsv[k][col];
                    }
                }
            } else {
                for (int q = m0; q < m1; ++q) {
                    const int i = mlist[q];
                    for (int k = 0; k < 6; ++k)
                        for (int col = 0; col < 6; ++col)
                            M[(size_t)(6 * (q - m0) + k) * 6 + col] = F.B[(size_t)i * 36 + 6 * k + col];
                }
            }
            double R[36];
            const int dm = mgs(M, rows, R);
            for (int k = 0; k < 6; ++k) dead[(size_t)c * 6 + k] = (dm >> k) & 1;
            std::copy(R, R + 36, Bc.begin() + (size_t)c * 36);
            for (int q = m0; q < m1; ++q) {
                const int i = mlist[q];
                for (int k = 0; k < bs; ++k)
                    for (int col = 0; col < 6; ++col)
                        P[((size_t)i * bs + k) * 6 + col] = M[(size_t)(bs * (q - m0) + k) * 6 + col];
            }
        }
        // prolongator pattern: block (i, J) for the aggregates J of node i's
        // neighbours (smoothed: P = (I - omega D^-1 A) P_tentative) or for
        // node i's own aggregate only (plain: P = P_tentative)
        std::vector<int> prow(F.n + 1, 0), pcol, mark(na, -1), cols;
        for (int i = 0; i < F.n; ++i) {
            cols.assign(1, agg[i]);
            mark[agg[i]] = i;
            if (a->smooth)
                for (int p = F.rowptr[i]; p < F.rowptr[i + 1]; ++p) {
                    const int J = agg[F.colidx[p]];
                    if (mark[J] != i) {
                        mark[J] = i;
                        cols.push_back(J);
                    }
                }
            std::sort(cols.begin(), cols.end());
            pcol.insert(pcol.end(), cols.begin(), cols.end());
            prow[i + 1] = static_cast<int>(pcol.size());
        }
        const int npb = static_cast<int>(pcol.size());
        std::vector<int> pbrow(npb);
        for (int i = 0; i < F.n; ++i)
            for (int b = prow[i]; b < prow[i + 1]; ++b) pbrow[b] = i;
        // smoothing lists: fine block (i, j) adds to prolongator block (i, agg(j))
        std::vector<int> sptr(npb + 1, 0), slist;
        if (a->smooth) {
            const int fnnzb = F.rowptr[F.n];
            std::vector<int> sb(fnnzb);
            for (int i = 0; i < F.n; ++i)
                for (int p = F.rowptr[i]; p < F.rowptr[i + 1]; ++p) {
                    const int J = agg[F.colidx[p]];
                    sb[p] = static_cast<int>(std::lower_bound(pcol.begin() + prow[i], pcol.begin() + prow[i + 1], J) -
                                             pcol.begin());
                    sptr[sb[p] + 1]++;
                }
            for (int b = 0; b < npb; ++b) sptr[b + 1] += sptr[b];
            slist.resize(fnnzb);
            std::vector<int> fill(sptr.begin(), sptr.end() - 1);
            for (int p = 0; p < fnnzb; ++p) slist[fill[sb[p]]++] = p;
        }
        // the same blocks by coarse column (fine nodes ascending within a column)
        std::vector<int> pcptr(na + 1, 0), cperm(npb), pcrow(npb);
        for (int b = 0; b < npb; ++b) pcptr[pcol[b] + 1]++;
        for (int c = 0; c < na; ++c) pcptr[c + 1] += pcptr[c];
        {
            std::vector<int> fill(pcptr.begin(), pcptr.end() - 1);
            for (int b = 0; b < npb; ++b) {
                const int q = fill[pcol[b]]++;
                cperm[q] = b;
                pcrow[q] = pbrow[b];
            }
        }
        // T = A P: pattern per fine row and, per T block, its pairs
        // (fine-matrix block (i, j), prolongator block (j, J))
        std::vector<int> trowptr(F.n + 1, 0), tcol;
        std::fill(mark.begin(), mark.end(), -1);
        for (int i = 0; i < F.n; ++i) {
            cols.clear();
            for (int p = F.rowptr[i]; p < F.rowptr[i + 1]; ++p) {
                const int j = F.colidx[p];
                for (int b = prow[j]; b < prow[j + 1]; ++b)
                    if (mark[pcol[b]] != i) {
                        mark[pcol[b]] = i;
                        cols.push_back(pcol[b]);
                    }
            }
            std::sort(cols.begin(), cols.end());
            tcol.insert(tcol.end(), cols.begin(), cols.end());
            trowptr[i + 1] = static_cast<int>(tcol.size());
        }
        const int64_t nT = (int64_t)tcol.size();
        std::vector<int> trow(nT), tptr(nT + 1, 0), posJ(na, -1);
        for (int i = 0; i < F.n; ++i) {
            for (int t = trowptr[i]; t < trowptr[i + 1]; ++t) {
                trow[t] = i;
                posJ[tcol[t]] = t;
            }
            for (int p = F.rowptr[i]; p < F.rowptr[i + 1]; ++p) {
                const int j = F.colidx[p];
                for (int b = prow[j]; b < prow[j + 1]; ++b) tptr[posJ[pcol[b]] + 1]++;
            }
        }
        for (int64_t t = 0; t < nT; ++t) tptr[t + 1] += tptr[t];
        std::vector<int> ta(tptr[nT]), tb(tptr[nT]);
        {
            std::vector<int> fill(tptr.begin(), tptr.end() - 1);
            for (int i = 0; i < F.n; ++i) {
                for (int t = trowptr[i]; t < trowptr[i + 1]; ++t) posJ[tcol[t]] = t;
                for (int p = F.rowptr[i]; p < F.rowptr[i + 1]; ++p) {
                    const int j = F.colidx[p];
                    for (int b = prow[j]; b < prow[j + 1]; ++b) {
                        const int k = fill[posJ[pcol[b]]]++;
                        ta[k] = p;
                        tb[k] = b;
                    }
                }
            }
        }
        // coarse pattern: row I joins the T rows of the fine nodes with a
        // block in column I
        HostLevel C;
        C.n = na;
        C.bs = 6;
        C.B = std::move(Bc);
        C.seg0.assign(d.nseg + 1, 0);
        // aggregates of an instance are contiguous and its first node is a
        // root: roots are created in node order, left-over nodes only join
        // aggregates of their own instance
        for (int g = 0; g <= d.nseg; ++g) C.seg0[g] = g < d.nseg ? (F.seg0[g] < F.n ? agg[F.seg0[g]] : na) : na;
        C.rowptr.assign(na + 1, 0);
        std::fill(mark.begin(), mark.end(), -1);
        for (int c = 0; c < na; ++c) {
            cols.clear();
            for (int q = pcptr[c]; q < pcptr[c + 1]; ++q) {
                const int i = pcrow[q];
                for (int t = trowptr[i]; t < trowptr[i + 1]; ++t)
                    if (mark[tcol[t]] != c) {
                        mark[tcol[t]] = c;
                        cols.push_back(tcol[t]);
                    }
            }
            std::sort(cols.begin(), cols.end());
            C.colidx.insert(C.colidx.end(), cols.begin(), cols.end());
            C.rowptr[c + 1] = static_cast<int>(C.colidx.size());
        }
        const int64_t cnnzb = (int64_t)C.colidx.size();
        // Galerkin pairs (prolongator block (i, I), T block (i, J)) per coarse block (I, J)
        std::vector<int> gptr(cnnzb + 1, 0);
        for (int c = 0; c < na; ++c) {
            for (int p = C.rowptr[c]; p < C.rowptr[c + 1]; ++p) posJ[C.colidx[p]] = p;
            for (int q = pcptr[c]; q < pcptr[c + 1]; ++q) {
                const int i = pcrow[q];
                for (int t = trowptr[i]; t < trowptr[i + 1]; ++t) gptr[posJ[tcol[t]] + 1]++;
            }
        }
        for (int64_t c = 0; c < cnnzb; ++c) gptr[c + 1] += gptr[c];
        std::vector<int> gp(gptr[cnnzb]), gt(gptr[cnnzb]);
        {
            std::vector<int> fill(gptr.begin(), gptr.end() - 1);
            for (int c = 0; c < na; ++c) {
                for (int p = C.rowptr[c]; p < C.rowptr[c + 1]; ++p) posJ[C.colidx[p]] = p;
                for (int q = pcptr[c]; q < pcptr[c + 1]; ++q) {
                    const int i = pcrow[q];
                    for (int t = trowptr[i]; t < trowptr[i + 1]; ++t) {
                        const int k = fill[posJ[tcol[t]]]++;
                        gp[k] = cperm[q];
                        gt[k] = t;
                    }
                }
            }
        }
        // device arrays of the fine level's transfer
        AmgLevel& DL = a->L[lev];
        DL.npb = npb;
        a->h_prow[lev] = prow;
        a->h_pcol[lev] = pcol;
        AMG_TRY(up(&DL.prow, prow));
        AMG_TRY(up(&DL.pcol, pcol));
        AMG_TRY(zeros(&DL.Pv, (size_t)npb * bs * 6));
        AMG_TRY(up(&DL.pcptr, pcptr));
        AMG_TRY(up(&DL.pcrow, pcrow));
        AMG_TRY(zeros(&DL.Pc, (size_t)npb * bs * 6));
        if (lev == 0) {
            AMG_TRY(zeros(&DL.Pvh, (size_t)npb * bs * 6));
            AMG_TRY(zeros(&DL.Pch, (size_t)npb * bs * 6));
        }
        AmgSetup& DS = a->S[lev];
        DS.nT = nT;
        AMG_TRY(up(&DS.Pt, std::vector<float>(P.begin(), P.end())));
        AMG_TRY(up(&DS.agg, agg));
        AMG_TRY(up(&DS.pbrow, pbrow));
        AMG_TRY(up(&DS.sptr, sptr));
        AMG_TRY(up(&DS.slist, slist));
        AMG_TRY(up(&DS.cperm, cperm));
        AMG_TRY(up(&DS.trow, trow));
        AMG_TRY(up(&DS.tptr, tptr));
        AMG_TRY(up(&DS.ta, ta));
        AMG_TRY(up(&DS.tb, tb));
        AMG_TRY(zeros(&DS.T, (size_t)nT * bs * 6));
        AMG_TRY(up(&DS.gptr, gptr));
        AMG_TRY(up(&DS.gp, gp));
        AMG_TRY(up(&DS.gt, gt));
        // the coarse level's own arrays
        AmgLevel& CL = a->L[lev + 1];
        CL.n = na;
        CL.bs = 6;
        CL.nnzb = cnnzb;
        std::vector<int> rowof(cnnzb), diag(na);
        std::vector<int> seg(na);
        for (int c = 0; c < na; ++c) {
            for (int p = C.rowptr[c]; p < C.rowptr[c + 1]; ++p) {
                rowof[p] = c;
                if (C.colidx[p] == c) diag[c] = p;
            }
        }
        for (int g = 0; g < d.nseg; ++g)
            for (int c = C.seg0[g]; c < C.seg0[g + 1]; ++c) seg[c] = g;
        AMG_TRY(up(&CL.rowptr, C.rowptr));
        AMG_TRY(up(&CL.colidx, C.colidx));
        AMG_TRY(up(&CL.rowof, rowof));
        AMG_TRY(up(&CL.diag, diag));
        AMG_TRY(up(&CL.seg, seg));
        AMG_TRY(up(&CL.seg0, C.seg0));
        AMG_TRY(up(&CL.dead, dead));
        AMG_TRY(zeros(&CL.val, (size_t)cnnzb * 36));  // float
        AMG_TRY(zeros(&CL.valh, (size_t)cnnzb * 36));
        AMG_TRY(zeros(&CL.dinv, (size_t)na * 36));
        H.push_back(std::move(C));
        ++lev;
    }
    a->nlev = lev + 1;
    if (a->nlev < 2) {  // nothing to coarsen: block-Jacobi is used instead
        amg_free(a);
        h->amg = nullptr;
        return TF_OK;
    }
    // level 0 device view: the handle's own arrays
    AmgLevel& L0 = a->L[0];
    L0.n = d.nn;
    L0.bs = 3;
    L0.nnzb = d.nnzb;
    {
        // blocks of the prolongator rows of each node-parallel CTA
        std::vector<int> c0(d.ncta), c1(d.ncta), prow0(d.nn + 1);
        TF_CUDA(cudaMemcpy(c0.data(), d.cta_node0, sizeof(int) * (size_t)d.ncta, cudaMemcpyDeviceToHost));
        TF_CUDA(cudaMemcpy(c1.data(), d.cta_node1, sizeof(int) * (size_t)d.ncta, cudaMemcpyDeviceToHost));
        TF_CUDA(cudaMemcpy(prow0.data(), L0.prow, sizeof(int) * (size_t)(d.nn + 1), cudaMemcpyDeviceToHost));
        int maxb = 1;
        for (int c = 0; c < d.ncta; ++c) maxb = std::max(maxb, prow0[c1[c]] - prow0[c0[c]]);
        a->v0_smem = static_cast<int>(3 * sizeof(float) * (size_t)maxb);
    }
    size_t maxv = 0;
    for (int l = 0; l < a->nlev; ++l) {
        AmgLevel& L = a->L[l];
        const size_t nv = (size_t)L.n * L.bs;
        maxv = std::max(maxv, nv);
        AMG_TRY(zeros(&L.x, nv));
        AMG_TRY(zeros(&L.t, nv));
        if (l > 0) {
            AMG_TRY(zeros(&L.r, nv));
            AMG_TRY(zeros(&L.e, nv));
        }
        a->h_n.push_back(L.n);
    }
    for (int l = 0; l < a->nlev; ++l) {
        a->L[l].ncoarse = l + 1 < a->nlev ? a->L[l + 1].n : 0;
        a->L[l].check = d.check;
    }
    AMG_TRY(zeros(&a->omega, (size_t)a->nlev));
    AMG_TRY(zeros(&a->val32, (size_t)d.nval));
    AMG_TRY(zeros(&a->valh, (size_t)d.nval));
    AMG_TRY(zeros(&a->dinv32, 9 * (size_t)d.nn));
    AMG_TRY(zeros(&a->diag32, 9 * (size_t)d.nn));
    AMG_TRY(zeros(&a->pscal, 2 * (size_t)a->nlev));
    AMG_TRY(zeros(&a->pv, maxv));
    AMG_TRY(zeros(&a->pw, maxv));
    int64_t maxc = 0;  // CTAs of the warp-per-row power iteration on the coarse levels
    for (int l = 1; l < a->nlev; ++l) maxc = std::max<int64_t>(maxc, cdiv(32 * (int64_t)a->L[l].n, kT));
    AMG_TRY(zeros(&a->part, (size_t)std::max<int64_t>({(int64_t)cdiv((int64_t)maxv, kT), (int64_t)d.ncta, maxc}) + 1));
    AMG_TRY(zeros(&a->ticket, 1));
    // coarsest level: dense inverse per instance
    const HostLevel& CH = H.back();
    std::vector<int> cinv0(d.nseg + 1, 0);
    a->max_cm = 0;
    for (int g = 0; g < d.nseg; ++g) {
        const int m = CH.bs * (CH.seg0[g + 1] - CH.seg0[g]);
        a->max_cm = std::max(a->max_cm, m);
        cinv0[g + 1] = cinv0[g] + m * m;
    }
    a->coarse_exact = a->max_cm <= kCoarseDofs;
    // the levels whose instances all have at most kTailNodes nodes run as
    // one kernel per V-cycle, one CTA per instance
    a->tail = a->coarse_exact ? a->nlev - 1 : 0;
    for (int l = a->nlev - 1; l >= 1 && a->coarse_exact; --l) {
        int maxn = 0;
        for (int g = 0; g < d.nseg; ++g) maxn = std::max(maxn, H[l].seg0[g + 1] - H[l].seg0[g]);
        if (maxn > kTailNodes) break;
        a->tail = l;
    }
    AMG_TRY(up(&a->cnode0, CH.seg0));
    AMG_TRY(up(&a->cinv0, cinv0));
    AMG_TRY(zeros(&a->cinv, (size_t)std::max(cinv0[d.nseg], 1)));
    return TF_OK;
}

// Patterns of the coarse images X_{l+1} = P_l^T X_l P_l of the extra blocks
// (packing couples, tf_add_K_triplets, DOF-binding merges), rebuilt on the
// host whenever the extra-block layout changes: per coarse extra block the
// list of triples (X_l block (J, I), P_l block (J, K), P_l block (I, M))
// whose products it sums.  The coarse operators then see the couplings the
// element graph does not have (e.g. between two surfaces pressed together).
tf_status amg_extra_symbolic(tf_handle* h) {
    Amg* a = h->amg;
    for (int l = 0; l < a->nlev; ++l) {
        AmgLevel& L = a->L[l];
        AmgSetup& S = a->S[l];
        void* ptrs[] = {S.xptr, S.xtrip, l > 0 ? L.xrow : nullptr, l > 0 ? L.xcol : nullptr,
                        l > 0 ? L.xval : nullptr};
        for (void* q : ptrs)
            if (q) cudaFree(q);
        S.xptr = S.xtrip = nullptr;
        if (l > 0) {
            L.xrow = L.xcol = nullptr;
            L.xval = nullptr;
            L.nx = 0;
        }
    }
    a->x_version = h->extra_version;
    if (h->d.nxb == 0 || h->h_xcols.empty()) return TF_OK;
    // level 0: (column, block index) per row, in the device layout
    std::vector<std::vector<std::pair<int, int>>> X(h->d.nn);
    for (int J = 0; J < h->d.nn; ++J)
        for (size_t q = 0; q < h->h_xcols[J].size(); ++q)
            X[J].emplace_back(h->h_xcols[J][q], h->h_xrow[J] + static_cast<int>(q));
    for (int l = 0; l + 1 < a->nlev; ++l) {
        const std::vector<int>& prow = a->h_prow[l];
        const std::vector<int>& pcol = a->h_pcol[l];
        const int nc = a->h_n[l + 1];
        struct Trip {
            int K, M, q, b1, b2;
        };
        std::vector<Trip> trips;
        for (size_t J = 0; J < X.size(); ++J)
            for (const auto& e : X[J])
                for (int b1 = prow[J]; b1 < prow[J + 1]; ++b1)
                    for (int b2 = prow[e.first]; b2 < prow[e.first + 1]; ++b2)
                        trips.push_back({pcol[b1], pcol[b2], e.second, b1, b2});
        if (trips.empty()) break;
        std::sort(trips.begin(), trips.end(), [](const Trip& u, const Trip& v) {
            return u.K != v.K ? u.K < v.K : (u.M != v.M ? u.M < v.M : u.q < v.q);
        });
        std::vector<int> xrow(nc + 1, 0), xcol, xptr(1, 0), xtrip;
        std::vector<std::vector<std::pair<int, int>>> Xn(nc);
        for (size_t t = 0; t < trips.size(); ++t) {
            const Trip& u = trips[t];
            if (t == 0 || u.K != trips[t - 1].K || u.M != trips[t - 1].M) {
                if (t > 0) xptr.push_back(static_cast<int>(xtrip.size() / 3));
                Xn[u.K].emplace_back(u.M, static_cast<int>(xcol.size()));
                xcol.push_back(u.M);
                xrow[u.K + 1]++;
            }
            xtrip.insert(xtrip.end(), {u.q, u.b1, u.b2});
        }
        xptr.push_back(static_cast<int>(xtrip.size() / 3));
        for (int K = 0; K < nc; ++K) xrow[K + 1] += xrow[K];
        AmgLevel& C = a->L[l + 1];
        AmgSetup& S = a->S[l];
        C.nx = static_cast<int64_t>(xcol.size());
        AMG_TRY(up(&C.xrow, xrow));
        AMG_TRY(up(&C.xcol, xcol));
        AMG_TRY(zeros(&C.xval, 36 * (size_t)C.nx));
        AMG_TRY(up(&S.xptr, xptr));
        AMG_TRY(up(&S.xtrip, xtrip));
        X.swap(Xn);
    }
    return TF_OK;
}

namespace {

__device__ __forceinline__ bool seg_stopped(const double* scal, int seg) {
    return __ldcg(&scal[(size_t)seg * S_COUNT + S_FLAG]) != 0.0;
}

// Sum of one value over the grid: partials per CTA, the last CTA to arrive
// folds them in a fixed order, all its threads at once (no waiting).  True in
// thread 0 of that CTA.
__device__ bool grid_sum(double v, double* part, unsigned* ticket, double* total) {
    __shared__ double sm[1][kT / 32 + 1];
    __shared__ bool last;
    double x[1] = {v};
    cta_sum<kT, 1>(x, sm);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = x[0];
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double t[1] = {0.0};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) t[0] += __ldcg(&part[b]);
    cta_sum<kT, 1>(t, sm);
    if (threadIdx.x != 0) return false;
    *total = t[0];
    *ticket = 0u;
    return true;
}

// Level-0 node of this thread (CTA tables of the node-parallel kernels).
struct Node0 {
    int i, seg;
    bool valid;
};
__device__ __forceinline__ Node0 node0(const Device& d) {
    Node0 q;
    q.seg = d.cta_seg[blockIdx.x];
    q.i = d.cta_node0[blockIdx.x] + threadIdx.x;
    q.valid = q.i < d.cta_node1[blockIdx.x];
    return q;
}

__device__ __forceinline__ void mul3(const float* __restrict__ D, const float r[3], float z[3]) {
    z[0] = fmaf(D[0], r[0], fmaf(D[1], r[1], D[2] * r[2]));
    z[1] = fmaf(D[3], r[0], fmaf(D[4], r[1], D[5] * r[2]));
    z[2] = fmaf(D[6], r[0], fmaf(D[7], r[1], D[8] * r[2]));
}

// Row of S = D^-1 A (FP16, sliced) times x, FP32 sums; the extra blocks X
// (FP64) enter as D^-1 (X x).
template <int U = 4>
__device__ __forceinline__ void row0s(const Device& d, const __half* __restrict__ valh,
                                      const float* __restrict__ dinv32, const float* __restrict__ x, int i,
                                      float y[3]) {
    const int lane = threadIdx.x & 31;
    const int wg = blockIdx.x * kWarps + (threadIdx.x >> 5);
    const int s0 = __ldg(&d.wslot0[wg]), s1 = __ldg(&d.wslot0[wg + 1]);
    float y0 = 0.f, y1 = 0.f, y2 = 0.f;
    const int* __restrict__ col = d.scol + lane;
    const uint4* __restrict__ p8 = reinterpret_cast<const uint4*>(valh) + lane;
    const __half* __restrict__ p1 = valh + (size_t)(d.nval / kSlotDoubles) * (kSlice * 8) + lane;
#pragma unroll U
    for (int s = s0; s < s1; ++s) {
        const int j = __ldg(&col[(size_t)s * kSlice]);
        if (!TF_IN(d.check, j, d.nn, CK_V0_COL)) continue;
        const uint4 pk = __ldg(&p8[(size_t)s * kSlice]);
        const float a8 = __half2float(p1[(size_t)s * kSlice]);
        // the low half of each word is the even entry
        const float2 a01 = make_float2(__half2float(__ushort_as_half((unsigned short)(pk.x & 0xffffu))),
                                       __half2float(__ushort_as_half((unsigned short)(pk.x >> 16))));
        const float2 a23 = make_float2(__half2float(__ushort_as_half((unsigned short)(pk.y & 0xffffu))),
                                       __half2float(__ushort_as_half((unsigned short)(pk.y >> 16))));
        const float2 a45 = make_float2(__half2float(__ushort_as_half((unsigned short)(pk.z & 0xffffu))),
                                       __half2float(__ushort_as_half((unsigned short)(pk.z >> 16))));
        const float2 a67 = make_float2(__half2float(__ushort_as_half((unsigned short)(pk.w & 0xffffu))),
                                       __half2float(__ushort_as_half((unsigned short)(pk.w >> 16))));
        const float x0 = x[3 * j], x1 = x[3 * j + 1], x2 = x[3 * j + 2];
        y0 = fmaf(a01.x, x0, fmaf(a01.y, x1, fmaf(a23.x, x2, y0)));
        y1 = fmaf(a23.y, x0, fmaf(a45.x, x1, fmaf(a45.y, x2, y1)));
        y2 = fmaf(a67.x, x0, fmaf(a67.y, x1, fmaf(a8, x2, y2)));
    }
    y[0] = y0;
    y[1] = y1;
    y[2] = y2;
    if (!d.xrow || d.xrow[i] == d.xrow[i + 1]) return;
    float e[3] = {0.f, 0.f, 0.f}, z[3];
    for (int q = d.xrow[i]; q < d.xrow[i + 1]; ++q) {
        const int j = d.xcol[q];
        if (!TF_IN(d.check, j, d.nn, CK_EXTRA_COL)) continue;
        const double* __restrict__ v = d.xval + 9 * (size_t)q;
#pragma unroll
        for (int r = 0; r < 3; ++r)
            e[r] = fmaf((float)v[3 * r], x[3 * j],
                        fmaf((float)v[3 * r + 1], x[3 * j + 1], fmaf((float)v[3 * r + 2], x[3 * j + 2], e[r])));
    }
    mul3(dinv32 + 9 * (size_t)i, e, z);
#pragma unroll
    for (int r = 0; r < 3; ++r) y[r] += z[r];
}

// Warp-cooperative product of row i of a 6x6-block CSR matrix with x.
// Lane 6 k + a (< 30) takes row a of blocks k, k + 5, k + 10, ... of the
// row: six FMAs per block row, every value used once (lane groups read
// 5 consecutive blocks); the five partial sums of each row a are then
// gathered by shuffles.  Every lane returns y.
__device__ __forceinline__ void row6_warp(const AmgLevel& L, int i, const float* __restrict__ x, float y[6]) {
    const int lane = threadIdx.x & 31;
    const int kb = lane / 6, a = lane - 6 * kb;
    float acc = 0.f;
    const int p0 = L.rowptr[i], p1 = L.rowptr[i + 1];
    if (lane < 30) {
#pragma unroll 2
        for (int p = p0 + kb; p < p1; p += 5) {
            const int j = __ldg(&L.colidx[p]);
            const float* __restrict__ v = L.val + 36 * (size_t)p + 6 * a;
            const float* __restrict__ xj = x + 6 * (size_t)j;
#pragma unroll
            for (int b2 = 0; b2 < 6; ++b2) acc = fmaf(__ldg(&v[b2]), xj[b2], acc);
        }
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        float s2 = 0.f;
#pragma unroll
        for (int g = 0; g < 5; ++g) s2 += __shfl_sync(0xffffffffu, acc, 6 * g + k);
        y[k] = s2;
    }
    if (L.xrow)  // coarse image of the extra blocks (few; every lane adds them)
        for (int q = L.xrow[i]; q < L.xrow[i + 1]; ++q) {
            const float* __restrict__ v = L.xval + 36 * (size_t)q;
            const float* __restrict__ xj = x + 6 * (size_t)L.xcol[q];
#pragma unroll
            for (int k = 0; k < 6; ++k)
#pragma unroll
                for (int m = 0; m < 6; ++m) y[k] = fmaf(v[6 * k + m], xj[m], y[k]);
        }
}

// y = S x for row i of a 6-DOF level, S = D^-1 A stored in FP16 (the
// element blocks only; extra6 adds the coarse image of the extra blocks).
__device__ __forceinline__ void row6_warp_h(const AmgLevel& L, int i, const float* __restrict__ x, float y[6]) {
    const int lane = threadIdx.x & 31;
    const int kb = lane / 6, a = lane - 6 * kb;
    float acc = 0.f;
    const int p0 = L.rowptr[i], p1 = L.rowptr[i + 1];
    if (lane < 30) {
#pragma unroll 2
        for (int p = p0 + kb; p < p1; p += 5) {
            const int j = __ldg(&L.colidx[p]);
            const __half2* __restrict__ v = reinterpret_cast<const __half2*>(L.valh + 36 * (size_t)p + 6 * a);
            const float* __restrict__ xj = x + 6 * (size_t)j;
#pragma unroll
            for (int b2 = 0; b2 < 3; ++b2) {
                const float2 f = __half22float2(__ldg(&v[b2]));
                acc = fmaf(f.x, xj[2 * b2], fmaf(f.y, xj[2 * b2 + 1], acc));
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        float s2 = 0.f;
#pragma unroll
        for (int g = 0; g < 5; ++g) s2 += __shfl_sync(0xffffffffu, acc, 6 * g + k);
        y[k] = s2;
    }
}

// e = X x for row i: the coarse image of the extra blocks (every lane)
__device__ __forceinline__ void extra6(const AmgLevel& L, int i, const float* __restrict__ x, float e[6]) {
#pragma unroll
    for (int k = 0; k < 6; ++k) e[k] = 0.f;
    if (!L.xrow) return;
    for (int q = L.xrow[i]; q < L.xrow[i + 1]; ++q) {
        const float* __restrict__ v = L.xval + 36 * (size_t)q;
        const float* __restrict__ xj = x + 6 * (size_t)L.xcol[q];
#pragma unroll
        for (int k = 0; k < 6; ++k)
#pragma unroll
            for (int m = 0; m < 6; ++m) e[k] = fmaf(v[6 * k + m], xj[m], e[k]);
    }
}

// r[a] without dynamic register indexing (which would go to local memory).
__device__ __forceinline__ float pick6(const float r[6], int a) {
    float v = 0.f;
#pragma unroll
    for (int k = 0; k < 6; ++k) v = (k == a) ? r[k] : v;
    return v;
}

// Lane a < 6 of the warp: (D r)_a for the 6x6 block D (r known to all lanes).
__device__ __forceinline__ float lane_mul6(const float* __restrict__ D, const float r[6], int a) {
    float s = 0.f;
#pragma unroll
    for (int b = 0; b < 6; ++b) s = fmaf(__ldg(&D[6 * a + b]), r[b], s);
    return s;
}

// ---- numeric phase -----------------------------------------------------------

__global__ void k_to_f32(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        b[k] = (float)a[k];
}

__global__ void k_f32_to_h(int64_t n, const float* __restrict__ a, __half* __restrict__ b) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        b[k] = __float2half_rn(a[k]);
}

// S = D^-1 A of a 6-DOF level in FP16, one thread per block row
__global__ void k_to_h6(AmgLevel L) {
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= L.nnzb * 6) return;
    const int64_t p = gid / 6;
    const int k = (int)(gid - 6 * p);
    const float* __restrict__ Di = L.dinv + 36 * (size_t)L.rowof[p] + 6 * k;
    const float* __restrict__ A = L.val + 36 * (size_t)p;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        float v = 0.f;
#pragma unroll
        for (int m = 0; m < 6; ++m) v = fmaf(Di[m], A[6 * m + c], v);
        L.valh[36 * (size_t)p + 6 * k + c] = __float2half_rn(v);
    }
}

// S = D^-1 A for the smoother, block by block in the sliced layout, FP16
// (its entries are O(1): the FP16 range and 11-bit mantissa suffice for a
// preconditioner; the Krylov operator itself stays FP64).
__global__ void k_to_h(Device d, const float* __restrict__ val32, const float* __restrict__ dinv32,
                       __half* __restrict__ valh, float* __restrict__ diag32) {
    const Node0 q = node0(d);
    const int lane = threadIdx.x & 31;
    const int wg = blockIdx.x * kWarps + (threadIdx.x >> 5);
    const int s0 = d.wslot0[wg], s1 = d.wslot0[wg + 1];
    float D[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) D[k] = q.valid ? dinv32[9 * (size_t)q.i + k] : 0.f;
    if (q.valid) {
        const float* __restrict__ Dg = val32 + d.diag[q.i];
#pragma unroll
        for (int k = 0; k < 9; ++k) diag32[9 * (size_t)q.i + k] = Dg[kSlice * k];
    }
    uint4* __restrict__ p8 = reinterpret_cast<uint4*>(valh) + lane;
    __half* __restrict__ p1 = valh + (size_t)(d.nval / kSlotDoubles) * (kSlice * 8) + lane;
    for (int s = s0; s < s1; ++s) {
        const size_t base = (size_t)s * kSlotDoubles + lane;
        float A[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) A[k] = val32[base + 32 * k];
        __half h[9];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c)
                h[3 * r + c] =
                    __float2half_rn(fmaf(D[3 * r], A[c], fmaf(D[3 * r + 1], A[3 + c], D[3 * r + 2] * A[6 + c])));
        uint4 pk;
        pk.x = (uint32_t)__half_as_ushort(h[0]) | ((uint32_t)__half_as_ushort(h[1]) << 16);
        pk.y = (uint32_t)__half_as_ushort(h[2]) | ((uint32_t)__half_as_ushort(h[3]) << 16);
        pk.z = (uint32_t)__half_as_ushort(h[4]) | ((uint32_t)__half_as_ushort(h[5]) << 16);
        pk.w = (uint32_t)__half_as_ushort(h[6]) | ((uint32_t)__half_as_ushort(h[7]) << 16);
        p8[(size_t)s * kSlice] = pk;
        p1[(size_t)s * kSlice] = h[8];
    }
}

// Element (r, c) of fine-matrix block b: level 0 reads the FP32 copy of the
// sliced storage, coarser levels their 6x6 CSR blocks.
template <int BS, bool L0>
__device__ __forceinline__ const float* fine_block(const AmgLevel& F, const int* __restrict__ bofs0,
                                                   const float* __restrict__ val0, int b) {
    return L0 ? val0 + __ldg(&bofs0[b]) : F.val + 36 * (size_t)b;
}
template <int BS, bool L0>
__device__ __forceinline__ float fine_at(const float* blk, int r, int c) {
    return L0 ? __ldg(&blk[kSlice * (3 * r + c)]) : __ldg(&blk[6 * r + c]);
}

// Prolongator block b = (i, J): P_t(i) [agg(i) = J] - omega D_i^-1 sum over
// the fine blocks (i, j) with agg(j) = J of A_ij P_t(j).  One thread per
// block; plain aggregation has empty lists and omega 0 (a copy of P_t).
template <int BS, bool L0>
__global__ void k_smooth_p(AmgLevel F, AmgSetup S, const double* __restrict__ omega, int smooth,
                           const int* __restrict__ colidx0, const int* __restrict__ bofs0,
                           const float* __restrict__ val0, const float* __restrict__ dinv0) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= F.npb) return;
    const int i = S.pbrow[b], J = F.pcol[b];
    float W[BS][6];
#pragma unroll
    for (int r = 0; r < BS; ++r)
#pragma unroll
        for (int c = 0; c < 6; ++c) W[r][c] = 0.f;
    for (int q = S.sptr[b]; q < S.sptr[b + 1]; ++q) {
        const int ab = __ldg(&S.slist[q]);
        const int j = L0 ? __ldg(&colidx0[ab]) : __ldg(&F.colidx[ab]);
        const float* blk = fine_block<BS, L0>(F, bofs0, val0, ab);
        const float* __restrict__ Pj = S.Pt + (size_t)j * BS * 6;
#pragma unroll
        for (int m = 0; m < BS; ++m) {
            float pm[6];
#pragma unroll
            for (int c = 0; c < 6; ++c) pm[c] = __ldg(&Pj[6 * m + c]);
#pragma unroll
            for (int r = 0; r < BS; ++r) {
                const float av = fine_at<BS, L0>(blk, r, m);
#pragma unroll
                for (int c = 0; c < 6; ++c) W[r][c] = fmaf(av, pm[c], W[r][c]);
            }
        }
    }
    const float om = smooth ? (float)__ldg(omega) : 0.f;
    const bool own = __ldg(&S.agg[i]) == J;
    const float* __restrict__ Di = L0 ? dinv0 + 9 * (size_t)i : F.dinv + 36 * (size_t)i;
    const float* __restrict__ Pi = S.Pt + (size_t)i * BS * 6;
    float* __restrict__ out = F.Pv + (size_t)b * BS * 6;
#pragma unroll
    for (int r = 0; r < BS; ++r)
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            float s = 0.f;
#pragma unroll
            for (int m = 0; m < BS; ++m) s = fmaf(__ldg(&Di[BS * r + m]), W[m][c], s);
            out[6 * r + c] = fmaf(-om, s, own ? __ldg(&Pi[6 * r + c]) : 0.f);
        }
}

// The prolongator blocks in coarse-column order (for the restriction).
__global__ void k_p_columns(AmgLevel F, AmgSetup S, int bsz) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= F.npb * bsz) return;
    const int64_t q = k / bsz;
    F.Pc[k] = F.Pv[(size_t)__ldg(&S.cperm[q]) * bsz + (k - q * bsz)];
}

// T = A P, row r of T block t = (i, J): sum over its pairs (A_ij, P_jJ).
template <int BS, bool L0>
__global__ void k_ap(AmgLevel F, AmgSetup S, const int* __restrict__ bofs0, const float* __restrict__ val0) {
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= S.nT * BS) return;
    const int64_t t = gid / BS;
    const int r = static_cast<int>(gid - BS * t);
    float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int q = S.tptr[t]; q < S.tptr[t + 1]; ++q) {
        const float* blk = fine_block<BS, L0>(F, bofs0, val0, __ldg(&S.ta[q]));
        const float* __restrict__ Pb = F.Pv + (size_t)__ldg(&S.tb[q]) * BS * 6;
#pragma unroll
        for (int m = 0; m < BS; ++m) {
            const float av = fine_at<BS, L0>(blk, r, m);
#pragma unroll
            for (int c = 0; c < 6; ++c) acc[c] = fmaf(av, __ldg(&Pb[6 * m + c]), acc[c]);
        }
    }
    float* out = S.T + (size_t)t * BS * 6 + 6 * r;
#pragma unroll
    for (int c = 0; c < 6; ++c) out[c] = acc[c];
}

// Coarse block c = (I, J), row p: sum over its pairs (P_iI, T_iJ) of
// (P_iI^T T_iJ)(p, :).
template <int BS>
__global__ void k_ptap(AmgLevel F, AmgSetup S, AmgLevel C) {
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= C.nnzb * 6) return;
    const int64_t c = gid / 6;
    const int p = static_cast<int>(gid - 6 * c);
    float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int q = S.gptr[c]; q < S.gptr[c + 1]; ++q) {
        const float* __restrict__ Pb = F.Pv + (size_t)__ldg(&S.gp[q]) * BS * 6;
        const float* __restrict__ Tb = S.T + (size_t)__ldg(&S.gt[q]) * BS * 6;
#pragma unroll
        for (int k = 0; k < BS; ++k) {
            const float pk = __ldg(&Pb[6 * k + p]);
#pragma unroll
            for (int c2 = 0; c2 < 6; ++c2) acc[c2] = fmaf(pk, __ldg(&Tb[6 * k + c2]), acc[c2]);
        }
    }
    const int I = C.rowof[c];
    if (C.colidx[c] == I && C.dead[6 * I + p]) acc[p] = 1.f;  // dropped coarse DOF: unit diagonal
    float* out = C.val + 36 * (size_t)c + 6 * p;
#pragma unroll
    for (int q2 = 0; q2 < 6; ++q2) out[q2] = acc[q2];
}

// Coarse extra block c = (K, M), row p: sum over its triples (X_JI, P_JK,
// P_IM) of (P_JK^T X_JI P_IM)(p, :).  Level 0's extra blocks are the FP64
// 3x3 blocks of the Krylov operator.
template <int BS, bool L0>
__global__ void k_xgal(AmgLevel F, AmgSetup S, AmgLevel C, const double* __restrict__ x0) {
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= C.nx * 6) return;
    const int64_t c = gid / 6;
    const int p = static_cast<int>(gid - 6 * c);
    float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int t = S.xptr[c]; t < S.xptr[c + 1]; ++t) {
        const int q = __ldg(&S.xtrip[3 * t]);
        const float* __restrict__ P1 = F.Pv + (size_t)__ldg(&S.xtrip[3 * t + 1]) * BS * 6;
        const float* __restrict__ P2 = F.Pv + (size_t)__ldg(&S.xtrip[3 * t + 2]) * BS * 6;
#pragma unroll
        for (int r = 0; r < BS; ++r) {
            const float pr = __ldg(&P1[6 * r + p]);
#pragma unroll
            for (int s2 = 0; s2 < BS; ++s2) {
                const float xv = L0 ? (float)__ldg(&x0[9 * (size_t)q + 3 * r + s2])
                                    : __ldg(&F.xval[36 * (size_t)q + 6 * r + s2]);
                const float px = pr * xv;
#pragma unroll
                for (int m = 0; m < 6; ++m) acc[m] = fmaf(px, __ldg(&P2[6 * s2 + m]), acc[m]);
            }
        }
    }
    float* out = C.xval + 36 * (size_t)c + 6 * p;
#pragma unroll
    for (int m = 0; m < 6; ++m) out[m] = acc[m];
}

// Inverse of a 6x6 block by Gauss-Jordan with partial pivoting (FP64 work).
__device__ void inv6(const float* __restrict__ A, float* __restrict__ out) {
    double M[6][12];
#pragma unroll
    for (int a = 0; a < 6; ++a)
#pragma unroll
        for (int b = 0; b < 6; ++b) {
            M[a][b] = A[6 * a + b];
            M[a][6 + b] = a == b ? 1.0 : 0.0;
        }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        int piv = k;
        double best = fabs(M[k][k]);
#pragma unroll
        for (int r = k + 1; r < 6; ++r)
            if (fabs(M[r][k]) > best) {
                best = fabs(M[r][k]);
                piv = r;
            }
        if (piv != k)
#pragma unroll
            for (int c = 0; c < 12; ++c) {
                const double tmp = M[k][c];
                M[k][c] = M[piv][c];
                M[piv][c] = tmp;
            }
        const double dk = M[k][k];
        const double rinv = dk != 0.0 ? 1.0 / dk : 1.0;
#pragma unroll
        for (int c = 0; c < 12; ++c) M[k][c] *= rinv;
#pragma unroll
        for (int r = 0; r < 6; ++r) {
            if (r == k) continue;
            const double f = M[r][k];
#pragma unroll
            for (int c = 0; c < 12; ++c) M[r][c] = fma(-f, M[k][c], M[r][c]);
        }
    }
#pragma unroll
    for (int a = 0; a < 6; ++a)
#pragma unroll
        for (int b = 0; b < 6; ++b) out[6 * a + b] = (float)M[a][6 + b];
}

__global__ void k_inv6(AmgLevel L) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= L.n) return;
    inv6(L.val + 36 * (size_t)L.diag[i], L.dinv + 36 * (size_t)i);
}

// power iteration for lambda_max(D^-1 A): v0 deterministic, scale = 1/|v0|
__global__ void k_pw_init(int64_t m, float* __restrict__ v, double* part, unsigned* ticket, double* scal) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double s = 0.0;
    if (k < m) {
        unsigned h = static_cast<unsigned>(k) * 2654435761u + 12345u;
        h ^= h >> 13;
        h *= 0x5bd1e995u;
        h ^= h >> 15;
        // zero-mean pseudo-random values: every mode, the rough ones included,
        // is present from the start (a positive vector barely excites the
        // largest eigenvalues, which would be underestimated)
        const float x = (h & 0xffffu) / 65536.0f - 0.5f;
        v[k] = x;
        s = (double)x * x;
    }
    double tot;
    if (grid_sum(s, part, ticket, &tot)) scal[0] = 1.0 / sqrt(tot);
}

__device__ __forceinline__ void pw_finish(double tot, double* scal, double* omega) {
    const double lam = sqrt(tot);
    scal[0] = lam > 0.0 ? 1.0 / lam : 1.0;
    scal[1] = lam;
    // 5 % margin: the power iteration approaches lambda_max from below
    *omega = lam > 0.0 ? (4.0 / 3.0) / (1.05 * lam) : 1.0;
}

__global__ void k_pw_step0(Device d, const __half* __restrict__ valh, const float* __restrict__ dinv32,
                           const float* __restrict__ v, float* __restrict__ w, double* part, unsigned* ticket,
                           double* scal, double* omega) {
    const Node0 q = node0(d);
    double s = 0.0;
    float y[3] = {0.f, 0.f, 0.f};
    if (q.valid) row0s(d, valh, dinv32, v, q.i, y);  // D^-1 A v = S v, the smoother's operator
    if (q.valid) {
        const float sc = (float)__ldcg(&scal[0]);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float z = sc * y[k];
            w[3 * q.i + k] = z;
            s += (double)z * z;
        }
    }
    double tot;
    if (grid_sum(s, part, ticket, &tot)) pw_finish(tot, scal, omega);
}

__global__ void k_pw_step6(AmgLevel L, const float* __restrict__ v, float* __restrict__ w, double* part,
                           unsigned* ticket, double* scal, double* omega) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // one warp per row
    const int lane = threadIdx.x & 31;
    double s = 0.0;
    if (i < L.n) {
        float y[6];
        row6_warp(L, i, v, y);
        const float sc = (float)__ldcg(&scal[0]);
#pragma unroll
        for (int k = 0; k < 6; ++k) y[k] *= sc;
        if (lane < 6) {
            const float z = lane_mul6(L.dinv + 36 * (size_t)i, y, lane);
            w[6 * i + lane] = z;
            s = (double)z * z;
        }
    }
    double tot;
    if (grid_sum(s, part, ticket, &tot)) pw_finish(tot, scal, omega);
}

// Gauss-Jordan inverse of the coarsest matrix of each instance (one CTA
// each, FP64 work, FP32 result)
__global__ void k_coarse_invert(AmgLevel L, const int* __restrict__ cnode0, const int* __restrict__ cinv0,
                                float* __restrict__ cinv) {
    extern __shared__ double M[];  // m x 2m
    __shared__ double f[kCoarseDofs];
    __shared__ int piv;
    __shared__ double tiny;
    const int g = blockIdx.x;
    const int n0 = cnode0[g], n1 = cnode0[g + 1];
    const int m = 6 * (n1 - n0), w = 2 * m;
    if (m == 0) return;
    for (int k = threadIdx.x; k < m * w; k += blockDim.x) {
        const int r = k / w, c = k - r * w;
        M[k] = (c - m == r) ? 1.0 : 0.0;
    }
    __syncthreads();
    for (int I = n0 + threadIdx.x; I < n1; I += blockDim.x) {
        for (int p = L.rowptr[I]; p < L.rowptr[I + 1]; ++p) {
            const int J = L.colidx[p] - n0;
            const float* v = L.val + 36 * (size_t)p;
            for (int a = 0; a < 6; ++a)
                for (int b = 0; b < 6; ++b) M[(6 * (I - n0) + a) * w + 6 * J + b] = (double)v[6 * a + b];
        }
        if (L.xrow)
            for (int q = L.xrow[I]; q < L.xrow[I + 1]; ++q) {
                const int J = L.xcol[q] - n0;
                if (J < 0 || J >= n1 - n0) continue;  // couples another instance: outside this inverse
                const float* v = L.xval + 36 * (size_t)q;
                for (int a = 0; a < 6; ++a)
                    for (int b = 0; b < 6; ++b) M[(6 * (I - n0) + a) * w + 6 * J + b] += (double)v[6 * a + b];
            }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double dmax = 0.0;
        for (int r = 0; r < m; ++r) dmax = fmax(dmax, fabs(M[r * w + r]));
        tiny = 1e-12 * dmax;
    }
    __syncthreads();
    for (int k = 0; k < m; ++k) {
        if (threadIdx.x == 0) {
            int best = k;
            double bv = fabs(M[k * w + k]);
            for (int r = k + 1; r < m; ++r)
                if (fabs(M[r * w + k]) > bv) {
                    bv = fabs(M[r * w + k]);
                    best = r;
                }
            piv = bv > tiny ? best : -1;
        }
        __syncthreads();
        if (piv < 0) {
            // (numerically) singular direction, e.g. a free rigid mode of an
            // unconstrained sheet: no coarse correction along it
            for (int c = threadIdx.x; c < w; c += blockDim.x) M[k * w + c] = 0.0;
            for (int r = threadIdx.x; r < m; r += blockDim.x) M[r * w + k] = 0.0;
            __syncthreads();
            continue;
        }
        const int pr = piv;
        if (pr != k)
            for (int c = threadIdx.x; c < w; c += blockDim.x) {
                const double tmp = M[k * w + c];
                M[k * w + c] = M[pr * w + c];
                M[pr * w + c] = tmp;
            }
        __syncthreads();
        const double dk = M[k * w + k];
        const double rinv = 1.0 / dk;
        __syncthreads();
        for (int c = threadIdx.x; c < w; c += blockDim.x) M[k * w + c] *= rinv;
        for (int r = threadIdx.x; r < m; r += blockDim.x) f[r] = M[r * w + k];
        __syncthreads();
        for (int q = threadIdx.x; q < m * w; q += blockDim.x) {
            const int r = q / w, c = q - r * w;
            if (r != k) M[q] = fma(-f[r], M[k * w + c], M[q]);
        }
        __syncthreads();
    }
    float* out = cinv + cinv0[g];
    for (int q = threadIdx.x; q < m * m; q += blockDim.x) {
        const int r = q / m, c = q - r * m;
        out[q] = (float)M[r * w + m + c];
    }
}

// ---- V-cycle (FP32) -------------------------------------------------------------

struct V0 {  // level-0 operands
    Device d;
    const double* omega;
    const float* dinv32;  // FP32 copy of the block inverses
    const __half* valh;   // S = D^-1 A, FP16
    const float* diag32;  // diagonal blocks D, FP32 [9 n]
};

// x = omega D^-1 r  (r is the Krylov method's FP64 vector)
__global__ void k_v0_pre(V0 a, const double* __restrict__ r, float* __restrict__ x) {
    pdl_enter();
    const Node0 q = node0(a.d);
    if (!q.valid || seg_stopped(a.d.scal, q.seg)) return;
    const float om = (float)__ldg(a.omega);
    float rr[3] = {(float)r[3 * q.i], (float)r[3 * q.i + 1], (float)r[3 * q.i + 2]}, z[3];
    mul3(a.dinv32 + 9 * (size_t)q.i, rr, z);
#pragma unroll
    for (int k = 0; k < 3; ++k) x[3 * q.i + k] = om * z[k];
}

// t = r - A x
template <int U>
__global__ void k_v0_resid(V0 a, const double* __restrict__ r, const float* __restrict__ x, float* __restrict__ t) {
    pdl_enter();
    const Node0 q = node0(a.d);
    if (seg_stopped(a.d.scal, q.seg)) return;
    float y[3];
    if (q.valid) row0s<U>(a.d, a.valh, a.dinv32, x, q.i, y);
    if (!q.valid) return;
    // A x = D (S x), D the diagonal block
    const float* __restrict__ Dg = a.diag32 + 9 * (size_t)q.i;
#pragma unroll
    for (int k = 0; k < 3; ++k)
        t[3 * q.i + k] = (float)r[3 * q.i + k] - fmaf(__ldg(&Dg[3 * k]), y[0],
                                                      fmaf(__ldg(&Dg[3 * k + 1]), y[1], __ldg(&Dg[3 * k + 2]) * y[2]));
}

// out = x + omega D^-1 (r - A x), written back as the FP64 preconditioned vector
template <int U>
__global__ void k_v0_post(V0 a, const double* __restrict__ r, const float* __restrict__ x, double* __restrict__ out) {
    pdl_enter();
    const Node0 q = node0(a.d);
    if (seg_stopped(a.d.scal, q.seg)) return;
    float y[3];
    if (q.valid) row0s<U>(a.d, a.valh, a.dinv32, x, q.i, y);
    if (!q.valid) return;
    // x + omega D^-1 (r - A x) = x + omega (D^-1 r - S x)
    const float om = (float)__ldg(a.omega);
    float rr[3] = {(float)r[3 * q.i], (float)r[3 * q.i + 1], (float)r[3 * q.i + 2]}, z[3];
    mul3(a.dinv32 + 9 * (size_t)q.i, rr, z);
#pragma unroll
    for (int k = 0; k < 3; ++k) out[3 * q.i + k] = (double)fmaf(om, z[k] - y[k], x[3 * q.i + k]);
}

// x_i += sum over the prolongator blocks (i, J) of P_iJ e_J.  The CTA's
// nodes own a contiguous range of blocks: consecutive threads take
// consecutive (block, row) pairs -- coalesced reads of the prolongator --
// into shared memory, then each node adds its blocks' rows in block order.
__global__ void k_v0_prolong(V0 a, AmgLevel F, const float* __restrict__ e, float* __restrict__ x) {
    extern __shared__ float part[];  // [3 * blocks of the CTA's nodes]
    pdl_enter();
    if (seg_stopped(a.d.scal, a.d.cta_seg[blockIdx.x])) return;
    const int n0 = a.d.cta_node0[blockIdx.x], n1 = a.d.cta_node1[blockIdx.x];
    const int b0 = __ldg(&F.prow[n0]);
    const int nitem = 3 * (__ldg(&F.prow[n1]) - b0);
    for (int q = threadIdx.x; q < nitem; q += blockDim.x) {
        const int bq = q / 3, k = q - 3 * bq;
        const int J = __ldg(&F.pcol[b0 + bq]);
        float s = 0.f;
        if (!TF_IN(F.check, J, F.ncoarse, CK_PROLONG_COL)) {
            part[q] = 0.f;
            continue;
        }
        const __half2* __restrict__ P2 = reinterpret_cast<const __half2*>(F.Pvh + 18 * (size_t)(b0 + bq) + 6 * k);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float2 f = __half22float2(__ldg(&P2[c]));
            s = fmaf(f.x, e[6 * J + 2 * c], fmaf(f.y, e[6 * J + 2 * c + 1], s));
        }
        part[q] = s;
    }
    __syncthreads();
    const int i = n0 + threadIdx.x;
    if (i >= n1) return;
    const int p0 = __ldg(&F.prow[i]) - b0, p1 = __ldg(&F.prow[i + 1]) - b0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float s = x[3 * i + k];
        for (int b = p0; b < p1; ++b) s += part[3 * b + k];
        x[3 * i + k] = s;
    }
}

// r_C(I) = sum over the prolongator blocks (i, I) of P_iI^T t_i;
// x_C = omega_C D_C^-1 r_C (pre-smoothing), by one warp: the lanes stride
// over the (block, row) pairs of column I, stored contiguously.
template <int BS>
__device__ __forceinline__ void restrict_node(const AmgLevel& F, const AmgLevel& C, const float* __restrict__ t,
                                              int I, const double* __restrict__ omegaC, int presmooth) {
    const int lane = threadIdx.x & 31;
    float rc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const int q0 = F.pcptr[I], np = BS * (F.pcptr[I + 1] - q0);
    constexpr bool kHalf = BS == 3;  // level 0: the FP16 copy of the prolongator
    const float* __restrict__ Pc = F.Pc + (size_t)q0 * BS * 6;
    const __half* __restrict__ Pch = kHalf ? F.Pch + (size_t)q0 * BS * 6 : nullptr;
    for (int qa = lane; qa < np; qa += 64) {
        // two (block, row) pairs per lane and pass: their loads overlap
        float tk[2] = {0.f, 0.f};
        int qq[2] = {0, 0};
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int q = qa + 32 * u;
            if (q < np) {
                const int m = q / BS, k = q - BS * m;
                const int i = __ldg(&F.pcrow[q0 + m]);
                if (!TF_IN(F.check, i, F.n, CK_RESTRICT_ROW)) continue;
                tk[u] = t[BS * (size_t)i + k];
                qq[u] = q;
            }
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            if constexpr (kHalf) {
                const __half2* __restrict__ P2 = reinterpret_cast<const __half2*>(Pch + 6 * (size_t)qq[u]);
#pragma unroll
                for (int b = 0; b < 3; ++b) {
                    const float2 f = __half22float2(__ldg(&P2[b]));
                    rc[2 * b] = fmaf(f.x, tk[u], rc[2 * b]);
                    rc[2 * b + 1] = fmaf(f.y, tk[u], rc[2 * b + 1]);
                }
            } else {
                const float* __restrict__ P = Pc + 6 * (size_t)qq[u];
#pragma unroll
                for (int b = 0; b < 6; ++b) rc[b] = fmaf(__ldg(&P[b]), tk[u], rc[b]);
            }
        }
    }
#pragma unroll
    for (int b = 0; b < 6; ++b)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) rc[b] += __shfl_xor_sync(0xffffffffu, rc[b], o);
    if (lane < 6) {
        C.r[6 * I + lane] = pick6(rc, lane);
        if (presmooth) C.x[6 * I + lane] = (float)__ldg(omegaC) * lane_mul6(C.dinv + 36 * (size_t)I, rc, lane);
    }
}

// Restriction, one warp per coarse node.
template <int BS>
__global__ void k_restrict(AmgLevel F, AmgLevel C, const float* __restrict__ t, const double* __restrict__ scal,
                           const double* __restrict__ omegaC, int presmooth) {
    pdl_enter();
    const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (I >= C.n || seg_stopped(scal, C.seg[I])) return;
    restrict_node<BS>(F, C, t, I, omegaC, presmooth);
}

// x_i += sum over the prolongator blocks (i, J) of P_iJ e_J (6-DOF level)
__device__ __forceinline__ void prolong_node(const AmgLevel& F, const float* __restrict__ e, int i, float* x) {
    float s[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) s[k] = x[6 * i + k];
    for (int b = __ldg(&F.prow[i]); b < __ldg(&F.prow[i + 1]); ++b) {
        const int J = __ldg(&F.pcol[b]);
        if (!TF_IN(F.check, J, F.ncoarse, CK_PROLONG_COL)) continue;
        const float* __restrict__ P = F.Pv + 36 * (size_t)b;
        float ec[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) ec[c] = e[6 * J + c];
#pragma unroll
        for (int k = 0; k < 6; ++k)
#pragma unroll
            for (int c = 0; c < 6; ++c) s[k] = fmaf(__ldg(&P[6 * k + c]), ec[c], s[k]);
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) x[6 * i + k] = s[k];
}

// out_i = x_i + omega D_i^-1 (r - A x)_i for row i, by one warp
__device__ __forceinline__ void post_row(const AmgLevel& L, const double* __restrict__ omega,
                                         const float* __restrict__ x, float* __restrict__ out, int i) {
    // x + omega (D^-1 (r - X x) - S x), S = D^-1 A in FP16, X the extra blocks
    const int lane = threadIdx.x & 31;
    float y[6], rr[6];
    row6_warp_h(L, i, x, y);
    extra6(L, i, x, rr);
#pragma unroll
    for (int k = 0; k < 6; ++k) rr[k] = L.r[6 * i + k] - rr[k];
    if (lane < 6)
        out[6 * i + lane] = fmaf((float)__ldg(omega), lane_mul6(L.dinv + 36 * (size_t)i, rr, lane) - pick6(y, lane),
                                 x[6 * i + lane]);
}

// t_i = r_i - (A x)_i with A x = D (S x) + X x, lane k < 6 writing component k
__device__ __forceinline__ void resid_row(const AmgLevel& L, const float* __restrict__ x, int i) {
    const int lane = threadIdx.x & 31;
    float y[6], e[6];
    row6_warp_h(L, i, x, y);
    extra6(L, i, x, e);
    if (lane < 6)
        L.t[6 * i + lane] = L.r[6 * i + lane] - lane_mul6(L.val + 36 * (size_t)L.diag[i], y, lane) - pick6(e, lane);
}

// t = r - A x  (one warp per row)
__global__ void k_v6_resid(AmgLevel L, const double* __restrict__ scal, const float* __restrict__ x) {
    pdl_enter();
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= L.n || seg_stopped(scal, L.seg[i])) return;
    resid_row(L, x, i);
}

// out = x + omega D^-1 (r - A x)  (one warp per row)
__global__ void k_v6_post(AmgLevel L, const double* __restrict__ scal, const double* __restrict__ omega,
                          const float* __restrict__ x, float* __restrict__ out) {
    pdl_enter();
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= L.n || seg_stopped(scal, L.seg[i])) return;
    post_row(L, omega, x, out, i);
}

// x_i += P_i e  (6-DOF fine level)
__global__ void k_v6_prolong(AmgLevel F, const double* __restrict__ scal, const float* __restrict__ e, float* x) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= F.n || seg_stopped(scal, F.seg[i])) return;
    prolong_node(F, e, i, x);
}

// Buffers of the damped-Jacobi sweeps of a coarse level (a sweep reads one
// vector and writes another): the pre-sweeps after the first (fused into the
// restriction, into x) alternate x and e; the post-sweeps alternate x and t
// and the last writes e, the level's output.
__host__ __device__ __forceinline__ float* pre_sweep_out(const AmgLevel& L, const float* cur) {
    return cur == L.x ? L.e : L.x;
}
__host__ __device__ __forceinline__ float* post_sweep_out(const AmgLevel& L, const float* cur, int s, int sweeps) {
    if (s == sweeps) return L.e;
    return cur == L.x ? L.t : L.x;
}

// e = C^-1 r on the coarsest level, one CTA per instance
__global__ void k_coarse_solve(AmgLevel L, const double* __restrict__ scal, const int* __restrict__ cnode0,
                               const int* __restrict__ cinv0, const float* __restrict__ cinv) {
    pdl_enter();
    const int g = blockIdx.x;
    if (seg_stopped(scal, g)) return;
    const int n0 = cnode0[g], m = 6 * (cnode0[g + 1] - n0);
    const float* __restrict__ Mi = cinv + cinv0[g];
    const float* __restrict__ r = L.r + 6 * (size_t)n0;
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
        float s = 0.f;
        for (int j = 0; j < m; ++j) s = fmaf(__ldg(&Mi[(size_t)k * m + j]), r[j], s);
        L.e[6 * (size_t)n0 + k] = s;
    }
}

// The coarse tail of a V-cycle: levels T.first .. T.last of one instance
// (one CTA each), block barriers instead of kernel boundaries.  Level
// T.first arrives restricted and pre-smoothed; its corrected x goes out in e.
struct Tail {
    AmgLevel L[kAmgMaxLevels];
    const double* omega;
    const double* scal;
    const int* cinv0;
    const float* cinv;
    int first, last;
    int sweeps;  // pre- and post-smoothing sweeps per level
};

__global__ void __launch_bounds__(kTailThreads) k_tail(Tail T) {
    pdl_enter();
    const int g = blockIdx.x;
    if (seg_stopped(T.scal, g)) return;
    const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    float* cur[kAmgMaxLevels];
    for (int l = T.first; l < T.last; ++l) {
        const AmgLevel& F = T.L[l];
        const AmgLevel& C = T.L[l + 1];
        float* x = F.x;
        for (int s = 2; s <= T.sweeps; ++s) {
            float* out = pre_sweep_out(F, x);
            for (int i = F.seg0[g] + warp; i < F.seg0[g + 1]; i += nw) post_row(F, T.omega + l, x, out, i);
            __syncthreads();
            x = out;
        }
        cur[l] = x;
        for (int i = F.seg0[g] + warp; i < F.seg0[g + 1]; i += nw) resid_row(F, x, i);
        __syncthreads();
        for (int I = C.seg0[g] + warp; I < C.seg0[g + 1]; I += nw)
            restrict_node<6>(F, C, F.t, I, T.omega + l + 1, l + 1 < T.last ? 1 : 0);
        __syncthreads();
    }
    {
        const AmgLevel& C = T.L[T.last];
        const int n0 = C.seg0[g], m = 6 * (C.seg0[g + 1] - n0);
        const float* __restrict__ Mi = T.cinv + T.cinv0[g];
        for (int k = threadIdx.x; k < m; k += blockDim.x) {
            float s2 = 0.f;
            for (int j = 0; j < m; ++j) s2 = fmaf(__ldg(&Mi[(size_t)k * m + j]), C.r[6 * (size_t)n0 + j], s2);
            C.e[6 * (size_t)n0 + k] = s2;
        }
    }
    __syncthreads();
    for (int l = T.last - 1; l >= T.first; --l) {
        const AmgLevel& F = T.L[l];
        float* x = cur[l];
        for (int i = F.seg0[g] + threadIdx.x; i < F.seg0[g + 1]; i += blockDim.x) prolong_node(F, T.L[l + 1].e, i, x);
        __syncthreads();
        for (int s = 1; s <= T.sweeps; ++s) {
            float* out = post_sweep_out(F, x, s, T.sweeps);
            for (int i = F.seg0[g] + warp; i < F.seg0[g + 1]; i += nw) post_row(F, T.omega + l, x, out, i);
            __syncthreads();
            x = out;
        }
    }
}

}  // namespace

void amg_mark_stale(tf_handle* h, int level) {
    if (h->amg) h->amg->stale = std::max(h->amg->stale, level);
}

bool amg_reused(const tf_handle* h) { return h->amg && h->amg->reused; }

long amg_rebuilds(const tf_handle* h) { return h->amg ? h->amg->rebuilds : 0; }

bool use_multigrid(const tf_handle* h) { return h->amg != nullptr; }

// Numeric phase for the current matrix.  Within a time step the matrix of
// a later Newton iteration differs little from the first one's, so a new
// assembly only refreshes the FP32 copies the level-0 smoother reads; the
// coarse operators, block inverses and smoother weights are rebuilt at the
// first solve of each time step (and whenever a solve with reused coarse
// levels fails, see krylov_solve).
// The level-0 copies the smoother reads, from the current assembly: FP32
// values and block inverses, the FP16 operator S = D^-1 A and the diagonal
// blocks (kernels only: also captured into the device Newton loop).
void amg_refresh(tf_handle* h) {
    Amg* a = h->amg;
    Device& d = h->d;
    cudaStream_t st = h->stream;
    k_to_f32<<<4 * 152, kT, 0, st>>>(d.nval, d.val, a->val32);
    h->launches++;
    k_to_f32<<<4 * 152, kT, 0, st>>>(9 * (int64_t)d.nn, d.dinv, a->dinv32);
    h->launches++;
    k_to_h<<<d.ncta, kNodeThreads, 0, st>>>(d, a->val32, a->dinv32, a->valh, a->diag32);
    h->launches++;
}

// The refresh above has run for the current assembly (inside the device
// Newton loop): nothing is stale, the coarse levels are the reused ones.
void amg_refreshed(tf_handle* h) {
    if (!h->amg) return;
    h->amg->stale = 0;
    h->amg->reused = true;
}

tf_status amg_numeric(tf_handle* h) {
    NvtxRange nvtx_range("tf multigrid numeric");
    Amg* a = h->amg;
    if (a->stale == 0) return TF_OK;
    if (a->v0_smem > 48 * 1024)  // outside any stream capture: the V-cycles launched later need it
        TF_CUDA(cudaFuncSetAttribute(k_v0_prolong, cudaFuncAttributeMaxDynamicSharedMemorySize, a->v0_smem));
    Device& d = h->d;
    cudaStream_t st = h->stream;
    amg_refresh(h);
    a->reused = a->stale == 1;
    if (a->reused) {
        a->stale = 0;
        return TF_OK;
    }
    ++a->rebuilds;
    if (a->x_version != h->extra_version) AMG_TRY(amg_extra_symbolic(h));
    // level by level: smoother weight from lambda_max(D^-1 A) (the
    // prolongator smoothing uses it too), prolongator, Galerkin product
    // A_{l+1} = P^T (A P) and the next level's block inverses
    const int last = a->coarse_exact ? a->nlev - 1 : a->nlev;  // levels with a smoother
    for (int l = 0; l < a->nlev; ++l) {
        AmgLevel& L = a->L[l];
        if (l < last) {
            const int64_t m = (int64_t)L.n * L.bs;
            double* scal = a->pscal + 2 * l;
            float *v = a->pv, *w = a->pw;
            k_pw_init<<<cdiv(m, kT), kT, 0, st>>>(m, v, a->part, a->ticket, scal);
            TF_LAUNCH_CHECK(h);
            for (int it = 0; it < kPowerIters; ++it) {
                if (l == 0)
                    k_pw_step0<<<d.ncta, kNodeThreads, 0, st>>>(d, a->valh, a->dinv32, v, w, a->part, a->ticket,
                                                                scal, a->omega);
                else
                    k_pw_step6<<<cdiv(32 * (int64_t)L.n, kT), kT, 0, st>>>(L, v, w, a->part, a->ticket, scal,
                                                                            a->omega + l);
                TF_LAUNCH_CHECK(h);
                std::swap(v, w);
            }
        }
        if (l + 1 == a->nlev) break;
        AmgSetup& S = a->S[l];
        AmgLevel& C = a->L[l + 1];
        const int sm = a->smooth ? 1 : 0;
        if (l == 0) {
            k_smooth_p<3, true><<<cdiv(L.npb, kT), kT, 0, st>>>(L, S, a->omega, sm, d.colidx, d.bofs, a->val32,
                                                                a->dinv32);
            TF_LAUNCH_CHECK(h);
            k_ap<3, true><<<cdiv(S.nT * 3, kT), kT, 0, st>>>(L, S, d.bofs, a->val32);
        } else {
            k_smooth_p<6, false><<<cdiv(L.npb, kT), kT, 0, st>>>(L, S, a->omega + l, sm, nullptr, nullptr,
                                                                 nullptr, nullptr);
            TF_LAUNCH_CHECK(h);
            k_ap<6, false><<<cdiv(S.nT * 6, kT), kT, 0, st>>>(L, S, nullptr, nullptr);
        }
        TF_LAUNCH_CHECK(h);
        k_p_columns<<<cdiv(L.npb * L.bs * 6, kT), kT, 0, st>>>(L, S, L.bs * 6);
        TF_LAUNCH_CHECK(h);
        if (l == 0) {
            k_f32_to_h<<<4 * 152, kT, 0, st>>>(L.npb * L.bs * 6, L.Pv, L.Pvh);
            TF_LAUNCH_CHECK(h);
            k_f32_to_h<<<4 * 152, kT, 0, st>>>(L.npb * L.bs * 6, L.Pc, L.Pch);
            TF_LAUNCH_CHECK(h);
        }
        if (l == 0) k_ptap<3><<<cdiv(C.nnzb * 6, kT), kT, 0, st>>>(L, S, C);
        else k_ptap<6><<<cdiv(C.nnzb * 6, kT), kT, 0, st>>>(L, S, C);
        TF_LAUNCH_CHECK(h);
        if (C.nx > 0) {
            if (l == 0) k_xgal<3, true><<<cdiv(C.nx * 6, kT), kT, 0, st>>>(L, S, C, d.xval);
            else k_xgal<6, false><<<cdiv(C.nx * 6, kT), kT, 0, st>>>(L, S, C, nullptr);
            TF_LAUNCH_CHECK(h);
        }
        k_inv6<<<cdiv(C.n, kT), kT, 0, st>>>(C);
        TF_LAUNCH_CHECK(h);
        k_to_h6<<<cdiv(C.nnzb * 6, kT), kT, 0, st>>>(C);
        TF_LAUNCH_CHECK(h);
    }
    if (a->coarse_exact) {
        AmgLevel& L = a->L[a->nlev - 1];
        const size_t smem = sizeof(double) * (size_t)a->max_cm * 2 * a->max_cm;
        static bool configured = false;
        if (!configured) {
            TF_CUDA(cudaFuncSetAttribute(k_coarse_invert, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(sizeof(double) * 2 * kCoarseDofs * kCoarseDofs)));
            configured = true;
        }
        k_coarse_invert<<<a->nseg, kT, smem, st>>>(L, a->cnode0, a->cinv0, a->cinv);
        TF_LAUNCH_CHECK(h);
    }
    a->stale = 0;
    return TF_OK;
}

// The level-0 smoother's row product with 2, 4 or 8 slots in flight per
// lane, timed on the handle's own matrix (k_v0_resid: one residual of the
// current smoother operator into the level's work vector); called once per
// handle by the solve autotuner.
tf_status amg_autotune(tf_handle* h) {
    Amg* a = h->amg;
    Device& d = h->d;
    cudaStream_t st = h->stream;
    AmgLevel& L0 = a->L[0];
    V0 v0{d, a->omega, a->dinv32, a->valh, a->diag32};
    float best = 1e30f;
    for (int u : {2, 4, 8}) {
        for (int r = 0; r < 4; ++r) {  // one warm-up, three timed
            if (r == 1) TF_CUDA(cudaEventRecord(h->ev[4], st));
            if (u == 2) k_v0_resid<2><<<d.ncta, kNodeThreads, 0, st>>>(v0, d.g, L0.x, L0.t);
            else if (u == 4) k_v0_resid<4><<<d.ncta, kNodeThreads, 0, st>>>(v0, d.g, L0.x, L0.t);
            else k_v0_resid<8><<<d.ncta, kNodeThreads, 0, st>>>(v0, d.g, L0.x, L0.t);
            TF_LAUNCH_CHECK(h);
        }
        TF_CUDA(cudaEventRecord(h->ev[5], st));
        TF_CUDA(cudaEventSynchronize(h->ev[5]));
        float ms = 0.f;
        TF_CUDA(cudaEventElapsedTime(&ms, h->ev[4], h->ev[5]));
        if (ms < best) {
            best = ms;
            a->smooth_unroll = u;
        }
    }
    return TF_OK;
}

int amg_smoother_unroll(const tf_handle* h) { return h->amg ? h->amg->smooth_unroll : 0; }

int amg_vcycle_kernels(const tf_handle* h) {
    const Amg* a = h->amg;
    const int per = 2 * kCoarseSweeps + 2;  // kernels of a coarse level run kernel by kernel
    if (a->tail > 0) return 5 + per * (a->tail - 1) + 1;
    return 5 + per * (a->nlev - 2) + (a->coarse_exact ? 1 : 3);
}

// out = M^-1 r: one V-cycle (all launches on h->stream, no host work).
// Levels below `tail` run kernel by kernel over all instances; the tail runs
// as one kernel with a CTA per instance.
void amg_vcycle(tf_handle* h, const double* r, double* out) {
    Amg* a = h->amg;
    Device& d = h->d;
    cudaStream_t st = h->stream;
    const int nl = a->nlev;
    const int stop = a->tail > 0 ? a->tail : nl - 1;  // first level not handled kernel by kernel
    V0 v0{d, a->omega, a->dinv32, a->valh, a->diag32};
    AmgLevel& L0 = a->L[0];
    auto presmooth = [&](int l) { return (l < nl - 1 || !a->coarse_exact) ? 1 : 0; };
    launch_pdl(k_v0_pre, d.ncta, kNodeThreads, st, v0, r, L0.x);
    switch (a->smooth_unroll) {
        case 2: launch_pdl(k_v0_resid<2>, d.ncta, kNodeThreads, st, v0, r, L0.x, L0.t); break;
        case 8: launch_pdl(k_v0_resid<8>, d.ncta, kNodeThreads, st, v0, r, L0.x, L0.t); break;
        default: launch_pdl(k_v0_resid<4>, d.ncta, kNodeThreads, st, v0, r, L0.x, L0.t); break;
    }
    launch_pdl(k_restrict<3>, cdiv(32 * (int64_t)a->L[1].n, kT), kT, st, L0, a->L[1], (const float*)L0.t,
               (const double*)d.scal, (const double*)(a->omega + 1), presmooth(1));
    float* cur[kAmgMaxLevels] = {};
    for (int l = 1; l < stop; ++l) {
        AmgLevel& L = a->L[l];
        const int nb = cdiv(32 * (int64_t)L.n, kT);
        float* x = L.x;  // first pre-sweep: fused into the restriction
        for (int s = 2; s <= kCoarseSweeps; ++s) {
            float* o = pre_sweep_out(L, x);
            launch_pdl(k_v6_post, nb, kT, st, L, (const double*)d.scal, (const double*)(a->omega + l),
                       (const float*)x, o);
            x = o;
        }
        cur[l] = x;
        launch_pdl(k_v6_resid, nb, kT, st, L, (const double*)d.scal, (const float*)x);
        launch_pdl(k_restrict<6>, cdiv(32 * (int64_t)a->L[l + 1].n, kT), kT, st, L, a->L[l + 1], (const float*)L.t,
                   (const double*)d.scal, (const double*)(a->omega + l + 1), presmooth(l + 1));
    }
    if (a->tail > 0) {
        Tail T;
        for (int l = 0; l < nl; ++l) T.L[l] = a->L[l];
        T.omega = a->omega;
        T.scal = d.scal;
        T.cinv0 = a->cinv0;
        T.cinv = a->cinv;
        T.first = a->tail;
        T.last = nl - 1;
        T.sweeps = kCoarseSweeps;
        launch_pdl(k_tail, a->nseg, kTailThreads, st, T);
    } else {
        AmgLevel& LC = a->L[nl - 1];
        if (a->coarse_exact) {
            launch_pdl(k_coarse_solve, a->nseg, 128, st, LC, d.scal, a->cnode0, a->cinv0, a->cinv);
        } else {
            // x from the restriction's pre-smoothing; three more sweeps into e
            const int nbc = cdiv(32 * (int64_t)LC.n, kT);
            launch_pdl(k_v6_post, nbc, kT, st, LC, d.scal, a->omega + nl - 1, LC.x, LC.e);
            launch_pdl(k_v6_post, nbc, kT, st, LC, d.scal, a->omega + nl - 1, LC.e, LC.t);
            launch_pdl(k_v6_post, nbc, kT, st, LC, d.scal, a->omega + nl - 1, LC.t, LC.e);
        }
    }
    for (int l = stop - 1; l >= 1; --l) {
        AmgLevel& L = a->L[l];
        float* x = cur[l];
        launch_pdl(k_v6_prolong, cdiv(L.n, kT), kT, st, L, d.scal, (const float*)a->L[l + 1].e, x);
        for (int s = 1; s <= kCoarseSweeps; ++s) {
            float* o = post_sweep_out(L, x, s, kCoarseSweeps);
            launch_pdl(k_v6_post, cdiv(32 * (int64_t)L.n, kT), kT, st, L, (const double*)d.scal,
                       (const double*)(a->omega + l), (const float*)x, o);
            x = o;
        }
    }
    launch_pdl_smem(k_v0_prolong, d.ncta, kNodeThreads, (size_t)a->v0_smem, st, v0, L0, (const float*)a->L[1].e,
                    L0.x);
    switch (a->smooth_unroll) {
        case 2: launch_pdl(k_v0_post<2>, d.ncta, kNodeThreads, st, v0, r, L0.x, out); break;
        case 8: launch_pdl(k_v0_post<8>, d.ncta, kNodeThreads, st, v0, r, L0.x, out); break;
        default: launch_pdl(k_v0_post<4>, d.ncta, kNodeThreads, st, v0, r, L0.x, out); break;
    }
}

}  // namespace tf

extern "C" TF_API tf_status tf_multigrid_blocks(tf_handle* h, int64_t* blocks, int64_t* prolongator_blocks) {
    if (!h || !blocks || !prolongator_blocks) {
        tf::set_error("tf_multigrid_blocks: bad arguments");
        return TF_BAD_INPUT;
    }
    tf::Amg* a = h->amg;
    for (int l = 0; l < (a ? a->nlev : 0); ++l) {
        blocks[l] = a->L[l].nnzb;
        prolongator_blocks[l] = a->L[l].npb;
    }
    return TF_OK;
}

extern "C" TF_API tf_status tf_multigrid_info(tf_handle* h, int32_t* levels, int32_t* nodes, double* weights) {
    if (!h || !levels) {
        tf::set_error("tf_multigrid_info: bad arguments");
        return TF_BAD_INPUT;
    }
    tf::Amg* a = h->amg;
    *levels = a ? a->nlev : 0;
    if (!a) return TF_OK;
    if (nodes)
        for (int l = 0; l < a->nlev; ++l) nodes[l] = a->h_n[l];
    if (weights) {
        TF_CUDA(cudaSetDevice(h->device));
        TF_CUDA(cudaStreamSynchronize(h->stream));
        TF_CUDA(cudaMemcpy(weights, a->omega, sizeof(double) * a->nlev, cudaMemcpyDeviceToHost));
    }
    return TF_OK;
}
