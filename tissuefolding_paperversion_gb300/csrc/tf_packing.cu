// Implicit packing between tissue surfaces on the device: the couple
// detection the reference runs once per time step and the packing forces and
// Jacobian it adds in every Newton iteration.
//
// Reference (TissueFolding/TissueFolding/SourceCode/):
//   * Simulation::detectPacingNodes (Simulation.cpp:8167-8440), an O(N^2)
//     scan over node pairs: couples of packing-eligible nodes
//     (Node::checkIfNodeHasPacking, Node.cpp:133-150: mass > 0, apical or
//     basal) on the same surface, not element neighbours
//     (Node::isMyNeig), closer than the detection distance of the first
//     node's cell in a 10 x 5 grid over the bounding box; the couple keeps
//     the unit vector from the second node to the first (initialWeightPoint).
//     The grid holds 0.4 x the mean side length of the prisms whose centres
//     fall in each cell (Simulation::getAverageSideLength, :3205-3265); the
//     centres are bounding-box fractions in [0, 1), so only cell [0][0] is
//     populated and a node whose x or y reaches the box's maximum finds none.
//     The force threshold is 0.4 x the mean of the apical and basal side
//     lengths.  The reference's merge of its 16 node segments (:8426) leaves
//     out the couples found from the last segment (flag bit 0 here).
//   * node masses: Simulation::updateNodeMasses (:7552-7561) from
//     ShapeBase::growShapeByFg's volume per node det(Fg) V_ref / 6
//     (ShapeBase.cpp:1243-1245), V_ref from Prism::calculateReferenceVolume
//     (Prism.cpp:876-908);
//   * Simulation::calculatePackingForcesImplicit3D (:7149-7203),
//     calculatePackingJacobian3D (:7205-7300) and addPackingForces
//     (:8869-8900): per couple and axis a sigmoid force
//     F = 5000 m / (1 + exp(-(5 / threshold) d)) w and its derivative on the
//     4 K entries of the axis.
//
// Here the O(N^2) scan becomes a hashed cell list (cell size = the detection
// distance): count per first node, exclusive scan, fill, each first node's
// couples sorted by the second node -- the reference's couple order.  The
// K entries of a couple's off-diagonal blocks live in the extra-block CSR the
// Krylov products include (the element pattern never holds them: couples are
// not neighbours); the diagonal entries and the forces are added node by node
// in couple order, so the assembly stays reproducible.
#include <algorithm>
#include <cmath>
#include <vector>

#include "tf_internal.cuh"

namespace tf {

namespace {

constexpr double kMultiplier = 5000.0;  // packingMultiplier (Simulation.cpp:8187)
constexpr double kSaturation = 5.0;     // sigmoidSaturationForPacking (:8188)
constexpr int kT = 256;
enum Par { P_THR = 0, P_DET, P_T2, P_BB0X, P_BB0Y, P_BBSX, P_BBSY, P_CELL, P_COUNT = 8 };

#define PK_TRY(expr)                \
    do {                            \
        tf_status _s = (expr);      \
        if (_s != TF_OK) return _s; \
    } while (0)

template <class T>
tf_status alloc(T** p, size_t n) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(n, 1) * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("device allocation failed in the packing set-up");
        return TF_OUT_OF_MEMORY;
    }
    return TF_OK;
}

template <class T>
tf_status put(T** p, const std::vector<T>& v) {
    PK_TRY(alloc(p, v.size()));
    if (!v.empty()) TF_CUDA(cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return TF_OK;
}

}  // namespace

struct Packing {
    int flags = 1;
    int nn = 0, ne = 0;
    // per handle
    int8_t* place = nullptr;   // [nn] node placement
    double* vref = nullptr;    // [ne] reference prism volumes
    uint8_t* ebasal = nullptr; // [ne] 1: the prism has a basal node (basal placement or spans the tissue)
    int* nptr = nullptr;       // [nn+1] prisms of each node, in prism order
    int* nelem = nullptr;
    double* mass = nullptr;    // [nn] node masses of the step
    double* vpn = nullptr;     // [ne] volume per node of each prism
    float* posf = nullptr;     // [3 nn] positions rounded to FP32 (the scan's cheap rejection)
    unsigned* posmax = nullptr;  // bits of the largest |FP32 coordinate|
    double* par = nullptr;     // [P_COUNT] parameters of the detection
    double* part = nullptr;    // per-CTA partials of the parameter reduction
    unsigned* ticket = nullptr;
    int T = 0;                 // hash table size (power of two)
    int* hoff = nullptr;       // [T+1] counts, then offsets
    int* hcur = nullptr;       // [T] fill cursors
    int* hids = nullptr;       // [nn] node ids by bucket
    int* ccount = nullptr;     // [nn+1] couples per first node, then offsets
    int* scan_tmp = nullptr;   // block sums of the scans
    // couples of the step
    int64_t n = 0, cap = 0;
    int* c0 = nullptr;
    int* c1 = nullptr;
    double* w = nullptr;       // [3n]
    double* mbar = nullptr;    // [n]
    int* x01 = nullptr;        // [n] extra block (c1, c0) of A
    int* x10 = nullptr;        // [n] extra block (c0, c1) of A
    // per-node incidence for the assembly: the couples of each node in order
    int nnodes = 0;
    int* pnode = nullptr;
    int* pptr = nullptr;
    int* plist = nullptr;      // couple * 2 + role (0: first node, 1: second)
    double h_par[P_COUNT] = {};
    std::vector<int> h_c0, h_c1;
    std::vector<std::pair<int, int>> h_blocks;  // extra blocks (J, I) of the current couples
    bool linked = false;       // incidence tables and block positions match h_c0 / h_c1
};

void packing_free(Packing* p) {
    if (!p) return;
    void* ptrs[] = {p->place, p->vref, p->ebasal, p->nptr, p->nelem, p->mass, p->vpn, p->posf, p->posmax, p->par, p->part, p->ticket,
                    p->hoff, p->hcur, p->hids,
                    p->ccount, p->scan_tmp, p->c0, p->c1, p->w, p->mbar, p->x01, p->x10, p->pnode, p->pptr,
                    p->plist};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    delete p;
}

namespace {

// ---- exclusive scan of n ints (in place, out[n] = total) ----------------------

constexpr int kScan = 1024;

__global__ void k_scan_local(int n, int* __restrict__ a, int* __restrict__ bsum) {
    __shared__ int s[kScan];
    const int i = blockIdx.x * kScan + threadIdx.x;
    const int v = i < n ? a[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < kScan; o <<= 1) {
        const int t = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
        __syncthreads();
        s[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) a[i] = s[threadIdx.x] - v;  // exclusive
    if (threadIdx.x == kScan - 1) bsum[blockIdx.x] = s[kScan - 1];
}

// One CTA: exclusive scan of the block sums (nb of them), total into a[n].
__global__ void k_scan_top(int nb, int* __restrict__ bsum, int* __restrict__ total) {
    __shared__ int s[kScan];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += kScan) {
        const int i = base + threadIdx.x;
        const int v = i < nb ? bsum[i] : 0;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < kScan; o <<= 1) {
            const int t = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
            __syncthreads();
            s[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < nb) bsum[i] = carry + s[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == kScan - 1) carry += s[kScan - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_add(int n, int* __restrict__ a, const int* __restrict__ bsum) {
    const int i = blockIdx.x * kScan + threadIdx.x;
    if (i < n) a[i] += bsum[blockIdx.x];
}

tf_status scan_exclusive(tf_handle* h, int* a, int n, int* tmp) {
    const int nb = cdiv(n, kScan);
    k_scan_local<<<nb, kScan, 0, h->stream>>>(n, a, tmp);
    TF_LAUNCH_CHECK(h);
    k_scan_top<<<1, kScan, 0, h->stream>>>(nb, tmp, a + n);
    TF_LAUNCH_CHECK(h);
    k_scan_add<<<nb, kScan, 0, h->stream>>>(n, a, tmp);
    TF_LAUNCH_CHECK(h);
    return TF_OK;
}

// ---- detection ---------------------------------------------------------------

// ShapeBase::determinant3by3Matrix (ShapeBase.cpp:2050-2056), Fg stored [9][ne]
__device__ __forceinline__ double det_fg(const double* __restrict__ Fg, int ne, int e) {
    auto f = [&](int r, int c) { return Fg[(size_t)(3 * r + c) * ne + e]; };
    double d = f(0, 0) * __dsub_rn(__dmul_rn(f(1, 1), f(2, 2)), __dmul_rn(f(1, 2), f(2, 1)));
    d = __dsub_rn(d, f(0, 1) * __dsub_rn(__dmul_rn(f(1, 0), f(2, 2)), __dmul_rn(f(1, 2), f(2, 0))));
    d = __dadd_rn(d, f(0, 2) * __dsub_rn(__dmul_rn(f(1, 0), f(2, 1)), __dmul_rn(f(1, 1), f(2, 0))));
    return d;
}

// node masses in prism order (updateNodeMasses)
// The volume per node of each prism, (det(Fg) V_ref) / 6, once per prism
// (ShapeBase::growShapeByFg, ShapeBase.cpp:1243-1245) ...
__global__ void k_pk_vpn(int ne, const double* __restrict__ Fg, const double* __restrict__ vref,
                         double* __restrict__ vpn) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    vpn[e] = (det_fg(Fg, ne, e) * vref[e]) / 6;
}

// ... and each node's sum over its prisms in prism order (updateNodeMasses).
__global__ void k_pk_mass(int nn, const double* __restrict__ vpn, const int* __restrict__ nptr,
                          const int* __restrict__ nelem, double* __restrict__ mass) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    double m = 0.0;
    for (int q = nptr[i]; q < nptr[i + 1]; ++q) m += vpn[nelem[q]];
    mass[i] = m;
}

__device__ __forceinline__ double dist2(const double* __restrict__ p, int a, int b) {
    const double dx = p[3 * a] - p[3 * b], dy = p[3 * a + 1] - p[3 * b + 1], dz = p[3 * a + 2] - p[3 * b + 2];
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// Prism::getApicalSideLengthAverage / getBasalSideLengthAverage (Prism.cpp:1443-1490)
__device__ __forceinline__ double side_avg(const double* __restrict__ p, const int* __restrict__ conn, int ne, int e,
                                           int o) {
    const int n0 = conn[(size_t)(o + 0) * ne + e], n1 = conn[(size_t)(o + 1) * ne + e],
              n2 = conn[(size_t)(o + 2) * ne + e];
    const int pa[3] = {n0, n0, n1}, pb[3] = {n1, n2, n2};
    double s = 0.0;
    int c = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double d2 = dist2(p, pa[k], pb[k]);
        if (d2 > 0) {
            s += sqrt(d2);
            ++c;
        }
    }
    return c > 0 ? s / c : s;
}

// Side-length sums and the bounding box over the whole grid: per-CTA
// partials, folded in a fixed order by the last CTA to arrive (no waiting),
// which writes the detection parameters.
constexpr int kParCtas = 2 * 152;
constexpr int kPart = 7;  // dsum, count, grid sum, min x, min y, max x, max y

__global__ void __launch_bounds__(kT) k_pk_params(int nn, int ne, const double* __restrict__ pos,
                                                  const int* __restrict__ conn, const uint8_t* __restrict__ ebasal,
                                                  double* __restrict__ part, unsigned* __restrict__ ticket,
                                                  double* __restrict__ par) {
    __shared__ double sm[kPart][kT / 32 + 1];
    __shared__ bool last;
    double ds = 0.0, dn = 0.0, gs = 0.0;
    const int stride = gridDim.x * blockDim.x;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += stride) {
        double v = side_avg(pos, conn, ne, e, 3);
        if (v > 0) {
            ds += v;
            dn += 1.0;
        }
        if (ebasal[e]) {
            v = side_avg(pos, conn, ne, e, 0);
            if (v > 0) {
                ds += v;
                dn += 1.0;
            }
        }
        gs += v;
    }
    // the box's maximum over nodes 1.. (node 0 is settled in the fold)
    double mn[2] = {INFINITY, INFINITY}, mx[2] = {-INFINITY, -INFINITY};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += stride)
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            mn[k] = fmin(mn[k], pos[3 * i + k]);
            if (i > 0) mx[k] = fmax(mx[k], pos[3 * i + k]);
        }
    constexpr int kind[kPart] = {0, 0, 0, 1, 1, 2, 2};
    double v[kPart] = {ds, dn, gs, mn[0], mn[1], mx[0], mx[1]};
    cta_combine<kT, kPart>(v, kind, sm);
    if (threadIdx.x == 0) {
        for (int q = 0; q < kPart; ++q) part[(size_t)kPart * blockIdx.x + q] = v[q];
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __shared__ double scan[kT];
    __threadfence();
    // fold: each thread its CTAs in order, then the fixed-order CTA combine
    double fold[kPart] = {0.0, 0.0, 0.0, INFINITY, INFINITY, -INFINITY, -INFINITY};
    for (int c = threadIdx.x; c < (int)gridDim.x; c += blockDim.x)
#pragma unroll
        for (int q = 0; q < kPart; ++q) fold[q] = combine_as(kind[q], fold[q], __ldcg(&part[(size_t)kPart * c + q]));
    cta_combine<kT, kPart>(fold, kind, sm);
    if (threadIdx.x == 0) *ticket = 0u;
    fold[3] = fmin(fold[3], kBoxCorner);  // calculateBoundingBox's corners
    fold[4] = fmin(fold[4], kBoxCorner);
    const double hx = reference_box_max<kT>(nn, pos, 0, fold[5], scan);
    const double hy = reference_box_max<kT>(nn, pos, 1, fold[6], scan);
    if (threadIdx.x != 0) return;
    const double col = fold[0] / fold[1];
    const double g00 = 0.4 * (fold[2] / ne);
    par[P_THR] = 0.4 * col;
    par[P_DET] = g00;
    par[P_T2] = g00 * g00;
    par[P_BB0X] = fold[3];
    par[P_BB0Y] = fold[4];
    par[P_BBSX] = hx - fold[3];
    par[P_BBSY] = hy - fold[4];
    par[P_CELL] = g00 * (1.0 + 1e-9);  // cells a hair wider than the distance: no pair is missed by rounding
}

__device__ __forceinline__ bool eligible(const double* __restrict__ mass, const int8_t* __restrict__ place, int i) {
    const int8_t pl = place[i];
    return mass[i] != 0 && (pl == 0 || pl == 1);
}

__device__ __forceinline__ long long cell_of(double x, double h) { return (long long)floor(x / h); }

__device__ __forceinline__ unsigned bucket(long long cx, long long cy, long long cz, int T) {
    unsigned long long k = (unsigned long long)cx * 0x9E3779B97F4A7C15ull;
    k ^= (unsigned long long)cy * 0xC2B2AE3D27D4EB4Full + (k << 6) + (k >> 2);
    k ^= (unsigned long long)cz * 0x165667B19E3779F9ull + (k << 6) + (k >> 2);
    k ^= k >> 31;
    return (unsigned)(k & (unsigned long long)(T - 1));
}

__global__ void k_pk_hcount(int nn, const double* __restrict__ pos, const double* __restrict__ mass,
                            const int8_t* __restrict__ place, const double* __restrict__ par, int T,
                            int* __restrict__ hoff) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn || !eligible(mass, place, i)) return;
    const double h = par[P_CELL];
    if (!(h > 0)) return;
    atomicAdd(&hoff[bucket(cell_of(pos[3 * i], h), cell_of(pos[3 * i + 1], h), cell_of(pos[3 * i + 2], h), T)], 1);
}

__global__ void k_pk_hfill(int nn, const double* __restrict__ pos, const double* __restrict__ mass,
                           const int8_t* __restrict__ place, const double* __restrict__ par, int T,
                           int* __restrict__ hcur, int* __restrict__ hids) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn || !eligible(mass, place, i)) return;
    const double h = par[P_CELL];
    if (!(h > 0)) return;
    const unsigned b = bucket(cell_of(pos[3 * i], h), cell_of(pos[3 * i + 1], h), cell_of(pos[3 * i + 2], h), T);
    hids[atomicAdd(&hcur[b], 1)] = i;
}

struct Scan {
    int nn, T, last_start;
    const double* pos;
    const float* posf;
    const unsigned* posmax;
    const double* mass;
    const int8_t* place;
    const double* par;
    const int* hoff;
    const int* hids;
    const int* rowptr;
    const int* colidx;
};

__device__ __forceinline__ bool neighbours(const Scan& S, int i, int j) {
    int lo = S.rowptr[i], hi = S.rowptr[i + 1];
    while (lo < hi) {
        const int m = (lo + hi) >> 1;
        const int c = S.colidx[m];
        if (c == j) return true;
        if (c < j) lo = m + 1;
        else hi = m;
    }
    return false;
}

// FP32 copies of the positions and the largest |coordinate| among them.
__global__ void k_pk_posf(int nn, const double* __restrict__ pos, float* __restrict__ posf,
                          unsigned* __restrict__ posmax) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float m = 0.f;
    if (i < nn)
        for (int k = 0; k < 3; ++k) {
            const float v = (float)pos[3 * (size_t)i + k];
            posf[3 * (size_t)i + k] = v;
            m = fmaxf(m, fabsf(v));
        }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(posmax, __float_as_uint(m));  // non-negative floats order as their bits
}

// Calls f(j, d2) for every couple (i, j) of first node i, in bucket order.
template <class F>
__device__ void for_each_partner(const Scan& S, int i, F f) {
    if (!eligible(S.mass, S.place, i) || i >= S.last_start) return;
    const double* p = S.pos;
    // grid cell of the first node (Simulation.cpp:8240-8242): only cell [0][0] holds a distance
    const double fx = floor((p[3 * i] - S.par[P_BB0X]) / S.par[P_BBSX]);
    const double fy = floor((p[3 * i + 1] - S.par[P_BB0Y]) / S.par[P_BBSY]);
    if (fx != 0.0 || fy != 0.0) return;
    const double t2 = S.par[P_T2], h = S.par[P_CELL];
    if (!(t2 > 0)) return;
    const long long cx = cell_of(p[3 * i], h), cy = cell_of(p[3 * i + 1], h), cz = cell_of(p[3 * i + 2], h);
    const int8_t pl = S.place[i];
    // Cheap rejection in FP32: with M the largest |coordinate| and u = 2^-24,
    // each FP32 difference is within 2.1 u M + 1.1 u r of the exact one for a
    // pair closer than r, so a pair whose FP32 squared distance exceeds
    // (r + sqrt(3)(2.1 u M + 1.1 u r))^2 (1 + 5u) is farther than r; only the
    // others take the exact FP64 test below.
    const double u = 5.9604644775390625e-08;
    const double r = sqrt(t2), M = (double)__uint_as_float(*S.posmax) * (1.0 + 4.0 * u);
    const double del = 1.7320508075688772 * (2.1 * u * M + 1.1 * u * r);
    const float t2f = __double2float_ru((r + del) * (r + del) * (1.0 + 5.0 * u));
    const float xi = S.posf[3 * (size_t)i], yi = S.posf[3 * (size_t)i + 1], zi = S.posf[3 * (size_t)i + 2];
    unsigned seen[27];
    int nseen = 0;
    for (int a = -1; a <= 1; ++a)
        for (int b = -1; b <= 1; ++b)
            for (int c = -1; c <= 1; ++c) {
                const unsigned bk = bucket(cx + a, cy + b, cz + c, S.T);
                bool dup = false;
                for (int k = 0; k < nseen; ++k) dup |= seen[k] == bk;
                if (dup) continue;
                seen[nseen++] = bk;
                for (int q = S.hoff[bk]; q < S.hoff[bk + 1]; ++q) {
                    const int j = S.hids[q];
                    if (j <= i || S.place[j] != pl) continue;
                    const float dxf = xi - S.posf[3 * (size_t)j], dyf = yi - S.posf[3 * (size_t)j + 1],
                                dzf = zi - S.posf[3 * (size_t)j + 2];
                    if (dxf * dxf + dyf * dyf + dzf * dzf > t2f) continue;
                    const double d2 = dist2(p, i, j);
                    if (!(d2 < t2) || neighbours(S, i, j)) continue;
                    f(j, d2);
                }
            }
}

__global__ void k_pk_count(Scan S, int* __restrict__ count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.nn) return;
    int n = 0;
    for_each_partner(S, i, [&](int, double) { ++n; });
    count[i] = n;
}

__global__ void k_pk_fill(Scan S, const int* __restrict__ off, int* __restrict__ c0, int* __restrict__ c1,
                          double* __restrict__ w, double* __restrict__ mbar) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.nn) return;
    const int o0 = off[i];
    int k = o0;
    for_each_partner(S, i, [&](int j, double d2) {
        c0[k] = i;
        c1[k] = j;
        const double d = sqrt(d2);
#pragma unroll
        for (int a = 0; a < 3; ++a) w[3 * (size_t)k + a] = (S.pos[3 * i + a] - S.pos[3 * j + a]) / d;
        mbar[k] = 0.5 * (S.mass[i] + S.mass[j]);
        ++k;
    });
    // the reference finds the partners of i in node order
    for (int a = o0 + 1; a < k; ++a)
        for (int b = a; b > o0 && c1[b - 1] > c1[b]; --b) {
            const int t = c1[b];
            c1[b] = c1[b - 1];
            c1[b - 1] = t;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const double u = w[3 * (size_t)b + q];
                w[3 * (size_t)b + q] = w[3 * (size_t)(b - 1) + q];
                w[3 * (size_t)(b - 1) + q] = u;
            }
            const double u = mbar[b];
            mbar[b] = mbar[b - 1];
            mbar[b - 1] = u;
        }
}

// ---- assembly -----------------------------------------------------------------

struct Axis {
    double F, d0, d1;
};

// Force on the first node and the derivatives of the couple along axis a
// (calculatePackingForcesImplicit3D / calculatePackingJacobian3D).
__device__ __forceinline__ Axis axis_terms(const double* __restrict__ uk, int i, int j, double w, double mb, double k,
                                           int a) {
    double dd = uk[3 * i + a] - uk[3 * j + a];
    if (w > 0) dd *= -1.0;
    const double ex = exp(__dmul_rn(k, -1.0 * dd));
    Axis t;
    t.F = __dmul_rn(__ddiv_rn(__dmul_rn(kMultiplier, mb), __dadd_rn(1.0, ex)), w);
    const double sig = __ddiv_rn(1.0, __dadd_rn(1.0, ex));
    t.d0 = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(sig, __dsub_rn(1.0, sig)), kMultiplier), mb), w), k);
    t.d1 = -1.0 * t.d0;
    if (w > 0) {
        t.d0 *= -1.0;
        t.d1 *= -1.0;
    }
    return t;
}

struct Asm {
    const double* uk;
    const int* c0;
    const int* c1;
    const double* w;
    const double* mbar;
    const double* par;
    const uint8_t* fixed;
    int nn;
    int64_t nxb;
    int* check;  // checked build: failed index checks
};

// Forces and diagonal K entries, node by node in couple order.
__global__ void k_pk_nodes(Asm A, int nnodes, const int* __restrict__ pnode, const int* __restrict__ pptr,
                           const int* __restrict__ plist, const int* __restrict__ diag, double* __restrict__ val,
                           double* __restrict__ g) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nnodes) return;
    const int i = pnode[t];
    const double k = __ddiv_rn(kSaturation, A.par[P_THR]);
    double P[3] = {0.0, 0.0, 0.0}, v[3];
    double* D = val + diag[i];
#pragma unroll
    for (int a = 0; a < 3; ++a) v[a] = D[kSlice * 4 * a];
    for (int q = pptr[t]; q < pptr[t + 1]; ++q) {
        const int c = plist[q] >> 1, role = plist[q] & 1;
        const int n0 = A.c0[c], n1 = A.c1[c];
        if (!TF_IN(A.check, n0, A.nn, CK_PACK_NODE) || !TF_IN(A.check, n1, A.nn, CK_PACK_NODE)) continue;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const Axis x = axis_terms(A.uk, n0, n1, A.w[3 * (size_t)c + a], A.mbar[c], k, a);
            P[a] = role == 0 ? __dadd_rn(P[a], x.F) : __dsub_rn(P[a], x.F);
            v[a] = __dsub_rn(v[a], x.d0);
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (A.fixed[3 * i + a]) continue;  // calcutateFixedK runs after the packing writers
        g[3 * i + a] = __dadd_rn(g[3 * i + a], P[a]);
        D[kSlice * 4 * a] = v[a];
    }
}

// Off-diagonal K entries of each couple (extra blocks of A: K(r, c) is entry
// (c % 3, r % 3) of block (c / 3, r / 3)).
__global__ void k_pk_pairs(Asm A, int n, const int* __restrict__ x01, const int* __restrict__ x10,
                           double* __restrict__ xval) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const double k = __ddiv_rn(kSaturation, A.par[P_THR]);
    const int n0 = A.c0[c], n1 = A.c1[c];
    if (!TF_IN(A.check, n0, A.nn, CK_PACK_NODE) || !TF_IN(A.check, n1, A.nn, CK_PACK_NODE) ||
        !TF_IN(A.check, x01[c], A.nxb, CK_PACK_BLOCK) || !TF_IN(A.check, x10[c], A.nxb, CK_PACK_BLOCK))
        return;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const Axis x = axis_terms(A.uk, n0, n1, A.w[3 * (size_t)c + a], A.mbar[c], k, a);
        if (A.fixed[3 * n0 + a] || A.fixed[3 * n1 + a]) continue;
        double* b01 = xval + 9 * (size_t)x01[c] + 4 * a;  // K(3 n0 + a, 3 n1 + a)
        double* b10 = xval + 9 * (size_t)x10[c] + 4 * a;  // K(3 n1 + a, 3 n0 + a)
        *b01 = __dsub_rn(*b01, x.d1);
        *b10 = __dsub_rn(*b10, x.d1);
    }
}

}  // namespace

// Host-side set-up when packing is switched on.
tf_status packing_setup(tf_handle* h, int flags) {
    Device& d = h->d;
    Packing* p = new Packing;
    p->flags = flags;
    p->nn = d.nn;
    p->ne = d.ne;
    h->pk = p;
    std::vector<int8_t> place(h->h_place.begin(), h->h_place.end());
    std::vector<uint8_t> ebasal(d.ne, 0);
    std::vector<int> nptr(d.nn + 1, 0), nelem(6 * (size_t)d.ne);
    for (int e = 0; e < d.ne; ++e)
        for (int a = 0; a < 6; ++a) {
            const int i = h->h_conn[6 * (size_t)e + a];
            nptr[i + 1]++;
            if (h->h_place[i] == 0) ebasal[e] = 1;
        }
    for (int i = 0; i < d.nn; ++i) nptr[i + 1] += nptr[i];
    {
        std::vector<int> fill(nptr.begin(), nptr.end() - 1);
        for (int e = 0; e < d.ne; ++e)
            for (int a = 0; a < 6; ++a) nelem[fill[h->h_conn[6 * (size_t)e + a]]++] = e;
    }
    int T = 1024;
    while (T < 2 * d.nn) T <<= 1;
    p->T = T;
    PK_TRY(put(&p->place, place));
    PK_TRY(put(&p->vref, h->h_vref));
    PK_TRY(put(&p->ebasal, ebasal));
    PK_TRY(put(&p->nptr, nptr));
    PK_TRY(put(&p->nelem, nelem));
    PK_TRY(alloc(&p->mass, d.nn));
    PK_TRY(alloc(&p->vpn, d.ne));
    PK_TRY(alloc(&p->posf, 3 * (size_t)d.nn));
    PK_TRY(alloc(&p->posmax, 1));
    PK_TRY(alloc(&p->par, P_COUNT));
    PK_TRY(alloc(&p->part, (size_t)kPart * kParCtas));
    PK_TRY(alloc(&p->ticket, 1));
    TF_CUDA(cudaMemset(p->ticket, 0, sizeof(unsigned)));
    PK_TRY(alloc(&p->hoff, (size_t)T + 1));
    PK_TRY(alloc(&p->hcur, (size_t)T));
    PK_TRY(alloc(&p->hids, d.nn));
    PK_TRY(alloc(&p->ccount, (size_t)d.nn + 1));
    PK_TRY(alloc(&p->scan_tmp, (size_t)cdiv(std::max(T, d.nn), kScan) + 1));
    return TF_OK;
}

// Couples at the current positions (the step's start shape) and their
// extra blocks.
tf_status packing_detect(tf_handle* h) {
    NvtxRange nvtx_range("tf packing detection");
    Packing* p = h->pk;
    Device& d = h->d;
    cudaStream_t st = h->stream;
    const int nn = d.nn;
    k_pk_vpn<<<cdiv(d.ne, kT), kT, 0, st>>>(d.ne, d.Fg, p->vref, p->vpn);
    TF_LAUNCH_CHECK(h);
    k_pk_mass<<<cdiv(nn, kT), kT, 0, st>>>(nn, p->vpn, p->nptr, p->nelem, p->mass);
    TF_LAUNCH_CHECK(h);
    k_pk_params<<<kParCtas, kT, 0, st>>>(nn, d.ne, d.uk, d.conn, p->ebasal, p->part, p->ticket, p->par);
    TF_LAUNCH_CHECK(h);
    TF_CUDA(cudaMemsetAsync(p->posmax, 0, sizeof(unsigned), st));
    k_pk_posf<<<cdiv(nn, kT), kT, 0, st>>>(nn, d.uk, p->posf, p->posmax);
    TF_LAUNCH_CHECK(h);
    TF_CUDA(cudaMemsetAsync(p->hoff, 0, sizeof(int) * ((size_t)p->T + 1), st));
    k_pk_hcount<<<cdiv(nn, kT), kT, 0, st>>>(nn, d.uk, p->mass, p->place, p->par, p->T, p->hoff);
    TF_LAUNCH_CHECK(h);
    PK_TRY(scan_exclusive(h, p->hoff, p->T, p->scan_tmp));
    TF_CUDA(cudaMemcpyAsync(p->hcur, p->hoff, sizeof(int) * (size_t)p->T, cudaMemcpyDeviceToDevice, st));
    k_pk_hfill<<<cdiv(nn, kT), kT, 0, st>>>(nn, d.uk, p->mass, p->place, p->par, p->T, p->hcur, p->hids);
    TF_LAUNCH_CHECK(h);
    int seg = nn / 16;
    if (seg < 1) seg = 1;
    const int last = (p->flags & 1) ? (nn / seg - 1) * seg : nn;
    Scan S{nn, p->T, last, d.uk, p->posf, p->posmax, p->mass, p->place, p->par, p->hoff, p->hids, d.rowptr, d.colidx};
    k_pk_count<<<cdiv(nn, kT), kT, 0, st>>>(S, p->ccount);
    TF_LAUNCH_CHECK(h);
    PK_TRY(scan_exclusive(h, p->ccount, nn, p->scan_tmp));
    int total = 0;
    TF_CUDA(cudaMemcpyAsync(&total, p->ccount + nn, sizeof(int), cudaMemcpyDeviceToHost, st));
    TF_CUDA(cudaMemcpyAsync(p->h_par, p->par, sizeof(double) * P_COUNT, cudaMemcpyDeviceToHost, st));
    TF_CUDA(cudaStreamSynchronize(st));
    if (total > p->cap) {
        void* old[] = {p->c0, p->c1, p->w, p->mbar, p->x01, p->x10};
        for (void* q : old)
            if (q) cudaFree(q);
        p->cap = std::max<int64_t>(total, 2 * p->cap);
        PK_TRY(alloc(&p->c0, p->cap));
        PK_TRY(alloc(&p->c1, p->cap));
        PK_TRY(alloc(&p->w, 3 * p->cap));
        PK_TRY(alloc(&p->mbar, p->cap));
        PK_TRY(alloc(&p->x01, p->cap));
        PK_TRY(alloc(&p->x10, p->cap));
    }
    p->n = total;
    if (total > 0) {
        k_pk_fill<<<cdiv(nn, kT), kT, 0, st>>>(S, p->ccount, p->c0, p->c1, p->w, p->mbar);
        TF_LAUNCH_CHECK(h);
    }
    std::vector<int> c0(total), c1(total);
    if (total > 0) {
        TF_CUDA(cudaMemcpyAsync(c0.data(), p->c0, sizeof(int) * (size_t)total, cudaMemcpyDeviceToHost, st));
        TF_CUDA(cudaMemcpyAsync(c1.data(), p->c1, sizeof(int) * (size_t)total, cudaMemcpyDeviceToHost, st));
    }
    TF_CUDA(cudaStreamSynchronize(st));
    if (p->linked && c0 == p->h_c0 && c1 == p->h_c1) return TF_OK;  // same couples: tables still valid
    p->h_c0.swap(c0);
    p->h_c1.swap(c1);
    p->linked = true;
    // per-node incidence in couple order
    {
        std::vector<int> cnt(nn, 0);
        for (int c = 0; c < total; ++c) {
            cnt[p->h_c0[c]]++;
            cnt[p->h_c1[c]]++;
        }
        std::vector<int> pnode, pptr(1, 0), pos(nn, -1);
        for (int i = 0; i < nn; ++i)
            if (cnt[i]) {
                pos[i] = static_cast<int>(pnode.size());
                pnode.push_back(i);
                pptr.push_back(pptr.back() + cnt[i]);
            }
        std::vector<int> plist(2 * (size_t)total), fill(pptr.begin(), pptr.end() - 1);
        for (int c = 0; c < total; ++c) {
            plist[fill[pos[p->h_c0[c]]]++] = 2 * c;
            plist[fill[pos[p->h_c1[c]]]++] = 2 * c + 1;
        }
        void* old[] = {p->pnode, p->pptr, p->plist};
        for (void* q : old)
            if (q) cudaFree(q);
        p->pnode = p->pptr = p->plist = nullptr;
        p->nnodes = static_cast<int>(pnode.size());
        PK_TRY(put(&p->pnode, pnode));
        PK_TRY(put(&p->pptr, pptr));
        PK_TRY(put(&p->plist, plist));
    }
    // extra blocks: the user's (triplets, bindings) plus both blocks of every couple
    std::vector<std::pair<int, int>> blocks;
    blocks.reserve(2 * (size_t)total);
    for (int c = 0; c < total; ++c) {
        blocks.emplace_back(p->h_c1[c], p->h_c0[c]);
        blocks.emplace_back(p->h_c0[c], p->h_c1[c]);
    }
    std::sort(blocks.begin(), blocks.end());
    if (blocks != p->h_blocks || h->h_xcols.empty() != (blocks.empty() && h->h_xuser.empty())) {
        p->h_blocks = blocks;
        if (h->h_xuser.empty()) h->h_xuser.resize(nn);
        h->h_xcols = h->h_xuser;
        for (const auto& b : blocks) {
            std::vector<int>& xc = h->h_xcols[b.first];
            auto it = std::lower_bound(xc.begin(), xc.end(), b.second);
            if (it == xc.end() || *it != b.second) xc.insert(it, b.second);
        }
        int64_t nxb = 0;
        for (const auto& xc : h->h_xcols) nxb += (int64_t)xc.size();
        h->h_xval.assign(9 * (size_t)nxb, 0.0);
        h->h_xcol_prev.clear();
        for (const auto& xc : h->h_xcols) h->h_xcol_prev.insert(h->h_xcol_prev.end(), xc.begin(), xc.end());
        if (nxb > 0 || d.nxb > 0) PK_TRY(upload_extra(h, true));
    }
    return packing_relink(h);
}

// Positions of the couples' blocks in the current extra-block layout (after
// every change of that layout: a new detection, new user blocks).
tf_status packing_relink(tf_handle* h) {
    Packing* p = h->pk;
    if (!p || p->n == 0) return TF_OK;
    const int nn = h->d.nn;
    const int64_t total = p->n;
    std::vector<int> row(nn + 1, 0);
    for (int i = 0; i < nn; ++i) row[i + 1] = row[i] + static_cast<int>(h->h_xcols[i].size());
    auto slot = [&](int J, int I) {
        const auto& xc = h->h_xcols[J];
        return row[J] + static_cast<int>(std::lower_bound(xc.begin(), xc.end(), I) - xc.begin());
    };
    std::vector<int> x01(total), x10(total);
    for (int64_t c = 0; c < total; ++c) {
        x01[c] = slot(p->h_c1[c], p->h_c0[c]);
        x10[c] = slot(p->h_c0[c], p->h_c1[c]);
    }
    TF_CUDA(cudaMemcpy(p->x01, x01.data(), sizeof(int) * (size_t)total, cudaMemcpyHostToDevice));
    TF_CUDA(cudaMemcpy(p->x10, x10.data(), sizeof(int) * (size_t)total, cudaMemcpyHostToDevice));
    return TF_OK;
}

tf_status packing_assemble(tf_handle* h) {
    Packing* p = h->pk;
    if (!p || p->n == 0) return TF_OK;
    Device& d = h->d;
    Asm A{d.uk, p->c0, p->c1, p->w, p->mbar, p->par, d.fixed, d.nn, d.nxb, d.check};
    k_pk_nodes<<<cdiv(p->nnodes, 128), 128, 0, h->stream>>>(A, p->nnodes, p->pnode, p->pptr, p->plist, d.diag, d.val,
                                                            d.g);
    TF_LAUNCH_CHECK(h);
    k_pk_pairs<<<cdiv(p->n, 128), 128, 0, h->stream>>>(A, static_cast<int>(p->n), p->x01, p->x10, d.xval);
    TF_LAUNCH_CHECK(h);
    return TF_OK;
}

tf_status packing_get(tf_handle* h, int64_t* n, int32_t* nodes, double* w, double* mbar, double* threshold,
                      double* detect) {
    Packing* p = h->pk;
    if (n) *n = p ? p->n : 0;
    if (!p) {
        if (threshold) *threshold = 0.0;
        if (detect) *detect = 0.0;
        return TF_OK;
    }
    TF_CUDA(cudaStreamSynchronize(h->stream));
    if (threshold) *threshold = p->h_par[P_THR];
    if (detect) *detect = p->h_par[P_DET];
    if (p->n == 0) return TF_OK;
    if (nodes)
        for (int64_t c = 0; c < p->n; ++c) {
            nodes[2 * c] = p->h_c0[c];
            nodes[2 * c + 1] = p->h_c1[c];
        }
    if (w) TF_CUDA(cudaMemcpy(w, p->w, sizeof(double) * 3 * (size_t)p->n, cudaMemcpyDeviceToHost));
    if (mbar) TF_CUDA(cudaMemcpy(mbar, p->mbar, sizeof(double) * (size_t)p->n, cudaMemcpyDeviceToHost));
    return TF_OK;
}

tf_status packing_masses(tf_handle* h, double* mass) {
    if (!h->pk) return set_error("packing is off"), TF_BAD_INPUT;
    TF_CUDA(cudaStreamSynchronize(h->stream));
    TF_CUDA(cudaMemcpy(mass, h->pk->mass, sizeof(double) * (size_t)h->d.nn, cudaMemcpyDeviceToHost));
    return TF_OK;
}

}  // namespace tf
