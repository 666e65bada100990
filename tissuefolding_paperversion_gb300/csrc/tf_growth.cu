// Growth functions on the device: the reference's GrowthFunctionBase types
// 1 (uniform), 2 (ring) and 3 (grid-based), GrowthFunctionTypes.h, applied in
// the order they were added, each in its time window and z range, by one
// kernel per step that multiplies every prism's growth increment by theirs
// (Simulation::calculateGrowth, Simulation.cpp:9651-9666, with
// calculateGrowthUniform :9757-9799, calculateGrowthRing :9801-9885 and
// calculateGrowthGridBased :10065-10114; ShapeBase::calculateFgFromRates
// ShapeBase.cpp:396-421, calculateFgFromGridCorners :432-562,
// updateGrowthIncrement :567-586, growShapeByFg :1215-1251).  The handle's
// per-element rates (tf_set_growth_rates) act as a uniform function first in
// the list.
//
// Uniform: diag(exp(rate dt)) turned by the function's xy angle.  Ring: the
// same with the rates scaled by 1 - (d - r_in)/(r_out - r_in) for prisms
// whose centre lies at a distance d in (r_in, r_out) from the ring's centre
// (the reference keeps centre, radii and d in single precision).  Grid:
// a function holds an nx x ny grid of growth rates (x, y, z; 1/s) and xy
// angles (degrees).  Once, on the host (the GridBasedGrowthFunction
// constructor and preCalculateAnglesForCompatibleAveraging): grid points whose
// in-plane aspect ratio |rx/ry| (or its inverse) is below 1.1 carry no angle;
// in each grid cell the angles of the 4 corners are brought to [0, pi] and
// next to the first corner that carries one, a corner turned by about 90 (or
// 270) degrees from it swapping its x and y rates.  Every step, per prism in
// the function's time window whose initial relative z is within [zmin, zmax]:
// its position in the tissue's bounding box -- pinned on the initial mesh or
// the current one -- gives a cell and fractions
// (ShapeBase::convertRelativePosToGridIndex, ShapeBase.cpp:633-660); the rates
// are the nearest corner's (interpolation 0) or the bilinear mean of the 4
// (interpolation 1, the angle averaged over the corners that carry one); the
// increment diag(exp(rate dt)), turned by that angle about z, multiplies Fg
// from the left after the per-element rates' increment
// (ShapeBase::updateGrowthIncrement :567-586, growShapeByFg :1215-1251).
//
// Bounding-box positions (Simulation.cpp:5833-5843, 630-645): prism centres
// relative to the nodes' box (Simulation::calculateBoundingBox :9148-9185,
// whose running "else if" never tests a node that lowers the minimum for the
// maximum -- reproduced exactly); the prisms of a column take the apical
// prism's position except the two top ones
// (Simulation::updateRelativePositionsToApicalPositioning :5987-6003, columns
// of Prism::constructElementStackList, Prism.cpp:2542-2584).
#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <vector>

#include "tf_internal.cuh"

namespace tf {

namespace {

constexpr int kT = 256;
constexpr int kBoxCtas = 2 * 152;        // k_box: two CTAs per SM
constexpr int kMaxFns = kMaxGrowthFunctions;
constexpr double kPi = 3.14159265358979323846;

#define GR_TRY(expr)                \
    do {                            \
        tf_status _s = (expr);      \
        if (_s != TF_OK) return _s; \
    } while (0)

template <class T>
tf_status put(T** p, const std::vector<T>& v) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(v.size(), 1) * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        set_error("device allocation failed for a growth function");
        return TF_OUT_OF_MEMORY;
    }
    if (!v.empty()) TF_CUDA(cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return TF_OK;
}

}  // namespace

enum GrowthType { kUniform = 1, kRing = 2, kGrid = 3 };  // GrowthFunctionBase::Type

struct GrowthFn {
    int type = kGrid;
    double t0 = 0, t1 = 0, zmin = 0, zmax = 1;
    // uniform and ring: maximum rates (1/s) and the rotation of the xy angle
    double rate[3] = {0.0, 0.0, 0.0};
    double R[9] = {1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0};
    // ring, in single precision as Simulation::calculateGrowthRing reads them
    float cx = 0.f, cy = 0.f, rin = 0.f, rout = 0.f;
    // grid
    int nx = 0, ny = 0;
    double* cg = nullptr;    // [(nx-1)*(ny-1)][4][3] compatible corner rates
    double* ca = nullptr;    // [(nx-1)*(ny-1)][4] compatible corner angles (rad)
    uint8_t* ce = nullptr;   // [(nx-1)*(ny-1)][4] 1: the corner carries no angle
};

struct Growth {
    std::vector<GrowthFn> fns;
    bool setup = false;       // grid positions set up (first grid function)
    int interp = 1;           // gridGrowthsInterpolationType (Simulation.cpp:146)
    int pinned = 0;           // GridGrowthsPinnedOnInitialMesh (Simulation.cpp:144)
    int layers = 0;           // TissueHeightDiscretisationLayers
    double height = 0;        // TissueHeight
    double* relz = nullptr;   // [ne] initial relative z (0 apical, 1 basal)
    double* rel0 = nullptr;   // [2][ne] pinned bounding-box positions
    double* rel = nullptr;    // [2][ne] positions at the current step's start
    int* colsrc = nullptr;    // [ne] the prism whose position a prism takes
    double* box = nullptr;    // [4] min x, min y, size x, size y
    double* part = nullptr;   // [kBoxCtas][4] k_box's per-CTA partials
    double* gbar = nullptr;   // [18][ne] Gauss-weighted dN/dX (growth rotation)
    unsigned* ticket = nullptr;  // k_box's arrival counter (0 between launches)
};

namespace {

void free_fn(GrowthFn& f) {
    cudaFree(f.cg);
    cudaFree(f.ca);
    cudaFree(f.ce);
    f.cg = f.ca = nullptr;
    f.ce = nullptr;
}

// ShapeBase::setTissuePlacement (ShapeBase.cpp:705-770): 3 lateral, 1 apical,
// 0 basal, 2 mid-line or spanning the tissue.
int element_placement(const tf_handle* h, int e) {
    bool ap = false, ba = false, la = false;
    for (int a = 0; a < 6; ++a) {
        const int p = h->h_place[h->h_conn[6 * (size_t)e + a]];
        if (p == 1) ap = true;
        else if (p == 0) ba = true;
        else if (p == 3) la = true;
    }
    if (la) return 3;
    if (ap) return ba ? 2 : 1;
    return ba ? 0 : 2;
}

// Simulation::calculateBoundingBox over every node, no y symmetry.
void host_box(const double* pos, int nn, double lo[3], double size[3]) {
    double hi[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = kBoxCorner;
        hi[k] = -kBoxCorner;
    }
    for (int i = 0; i < nn; ++i)
        for (int k = 0; k < 3; ++k) {
            const double p = pos[3 * (size_t)i + k];
            if (p < lo[k]) lo[k] = p;
            else if (p > hi[k]) hi[k] = p;
        }
    for (int k = 0; k < 3; ++k) size[k] = hi[k] - lo[k];
}

// Simulation::calculateTissueHeight (Simulation.cpp:3280-3330) for a
// columnar tissue: from the first basal node, prism by prism up to an apical
// node, summing Prism::getElementHeight (Prism.cpp:1526-1531).
void tissue_height(const tf_handle* h, const double* pos, int* layers, double* height) {
    const int nn = h->d.nn, ne = h->d.ne;
    *layers = 0;
    *height = 0.0;
    int cur = -1;
    for (int i = 0; i < nn && cur < 0; ++i)
        if (h->h_place[i] == 0) cur = i;
    if (cur < 0) return;
    for (int guard = 0; h->h_place[cur] != 1 && guard <= ne; ++guard) {
        int found = -1, slot = -1;
        for (int e = 0; e < ne && found < 0; ++e)
            for (int a = 0; a < 3; ++a)
                if (h->h_conn[6 * (size_t)e + a] == cur) {
                    found = e;
                    slot = a;
                    break;
                }
        if (found < 0) return;
        const int* c = &h->h_conn[6 * (size_t)found];
        double s = 0.0;
        for (int k = 0; k < 3; ++k) {
            const double dd = pos[3 * (size_t)c[0] + k] - pos[3 * (size_t)c[3] + k];
            s += dd * dd;
        }
        *height += std::pow(s, 0.5);
        ++*layers;
        cur = c[slot + 3];
    }
}

// Corner values of every cell, made compatible (GridBasedGrowthFunction's
// constructor, GrowthFunctionTypes.h:281-351, and
// preCalculateAnglesForCompatibleAveraging, :427-579).
void compatible_corners(int nx, int ny, const double* rates, const double* angles_deg, std::vector<double>& cg,
                        std::vector<double>& ca, std::vector<uint8_t>& ce) {
    const size_t ncell = (size_t)(nx - 1) * (ny - 1);
    cg.assign(12 * ncell, 0.0);
    ca.assign(4 * ncell, 0.0);
    ce.assign(4 * ncell, 0);
    auto rate = [&](int i, int j, int k) { return rates[3 * ((size_t)i * ny + j) + k]; };
    auto angle = [&](int i, int j) { return angles_deg ? angles_deg[(size_t)i * ny + j] * kPi / 180.0 : 0.0; };
    auto carries_angle = [&](int i, int j) {
        double ar = rate(i, j, 0) / rate(i, j, 1);
        if (ar < 0) ar *= -1.0;
        if (ar < 1.0) ar = 1 / ar;
        return !(ar < 1.1);
    };
    for (int ix = 0; ix < nx - 1; ++ix)
        for (int iy = 0; iy < ny - 1; ++iy) {
            const int ci[4] = {ix, ix + 1, ix, ix + 1}, cj[4] = {iy, iy, iy + 1, iy + 1};
            double g[4][3], a[4] = {0.0, 0.0, 0.0, 0.0};
            bool elim[4] = {false, false, false, false};
            for (int c = 0; c < 4; ++c) {
                for (int k = 0; k < 3; ++k) g[c][k] = rate(ci[c], cj[c], k);
                if (carries_angle(ci[c], cj[c])) a[c] = angle(ci[c], cj[c]);
                else elim[c] = true;
            }
            for (int c = 0; c < 4; ++c) {
                while (a[c] < 0) a[c] += kPi;
                while (a[c] > kPi) a[c] -= kPi;
            }
            // the base angle: the first corner that carries one (else corner 3, angle 0)
            int base = 3;
            double tet = 0;
            for (int c = 0; c < 4; ++c)
                if (!elim[c]) {
                    tet = a[c];
                    base = c;
                    break;
                }
            bool flip[4] = {false, false, false, false};
            for (int c = base; c < 4; ++c) {
                const double dt = a[c] - tet;
                if (dt > 0) {
                    if (dt >= kPi / 4.0 && dt < 3.0 * kPi / 4.0) {
                        a[c] = a[c] - kPi / 2.0;
                        flip[c] = true;
                    } else if (dt >= 3.0 * kPi / 4.0 && dt < 5.0 * kPi / 4.0) {
                        a[c] = a[c] - kPi;
                    } else if (dt >= 5.0 * kPi / 4.0 && dt < 7.0 * kPi / 4.0) {
                        a[c] = a[c] - 6.0 * kPi / 4.0;
                        flip[c] = true;
                    } else if (dt >= 7.0 * kPi / 4.0) {
                        a[c] = a[c] - 2.0 * kPi;
                    }
                } else if (dt < 0) {
                    if (dt <= -kPi / 4.0 && dt > -3.0 * kPi / 4.0) {
                        a[c] = a[c] + kPi / 2.0;
                        flip[c] = true;
                    } else if (dt <= -3.0 * kPi / 4.0 && dt > -5.0 * kPi / 4.0) {
                        a[c] = a[c] + kPi;
                    } else if (dt <= -5.0 * kPi / 4.0 && dt > -7.0 * kPi / 4.0) {
                        a[c] = a[c] + 6.0 * kPi / 4.0;
                        flip[c] = true;
                    } else if (dt <= -7.0 * kPi / 4.0) {
                        a[c] = a[c] + 2.0 * kPi;
                    }
                }
            }
            const size_t cell = (size_t)ix * (ny - 1) + iy;
            for (int c = 0; c < 4; ++c) {
                if (flip[c]) std::swap(g[c][0], g[c][1]);
                for (int k = 0; k < 3; ++k) cg[12 * cell + 3 * c + k] = g[c][k];
                ca[4 * cell + c] = a[c];
                ce[4 * cell + c] = elim[c] ? 1 : 0;
            }
        }
}

// ---- device ---------------------------------------------------------------

// calculateBoundingBox in x and y on the device, bit for bit: per-CTA
// minima over all nodes and maxima over nodes 1.., folded in CTA order by the
// last CTA to arrive (no waiting), which settles node 0
// (reference_box_max) and writes min x, min y, size x, size y.
__global__ void __launch_bounds__(kT) k_box(int nn, const double* __restrict__ pos, double* __restrict__ part,
                                            unsigned* __restrict__ ticket, double* __restrict__ box) {
    constexpr int kind[4] = {1, 1, 2, 2};
    __shared__ double sm[4][kT / 32 + 1];
    __shared__ double scan[kT];
    __shared__ bool last;
    double v[4] = {INFINITY, INFINITY, -INFINITY, -INFINITY};  // min x, min y, max x, max y (nodes 1..)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        const double x = pos[3 * (size_t)i], y = pos[3 * (size_t)i + 1];
        v[0] = fmin(v[0], x);
        v[1] = fmin(v[1], y);
        if (i > 0) {
            v[2] = fmax(v[2], x);
            v[3] = fmax(v[3], y);
        }
    }
    cta_combine<kT, 4>(v, kind, sm);
    if (threadIdx.x == 0) {
        for (int q = 0; q < 4; ++q) part[4 * (size_t)blockIdx.x + q] = v[q];
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double f[4] = {INFINITY, INFINITY, -INFINITY, -INFINITY};
    for (int c = threadIdx.x; c < (int)gridDim.x; c += blockDim.x)
#pragma unroll
        for (int q = 0; q < 4; ++q) f[q] = combine_as(kind[q], f[q], __ldcg(&part[4 * (size_t)c + q]));
    cta_combine<kT, 4>(f, kind, sm);
    if (threadIdx.x == 0) *ticket = 0u;
    const double lox = fmin(f[0], kBoxCorner), loy = fmin(f[1], kBoxCorner);  // calculateBoundingBox's corners
    const double hx = reference_box_max<kT>(nn, pos, 0, f[2], scan);
    const double hy = reference_box_max<kT>(nn, pos, 1, f[3], scan);
    if (threadIdx.x == 0) {
        box[0] = lox;
        box[1] = loy;
        box[2] = hx - lox;
        box[3] = hy - loy;
    }
}

// ShapeBase::calculateRelativePosInBoundingBox (ShapeBase.cpp:1842-1848) of
// the prism colsrc[e], whose position prism e takes.
__global__ void k_relpos(int ne, const int* __restrict__ conn, const double* __restrict__ pos,
                         const double* __restrict__ box, const int* __restrict__ colsrc, double* __restrict__ rel) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int s = colsrc[e];
    double c[2] = {0.0, 0.0};
    for (int a = 0; a < 6; ++a) {
        const int n = conn[(size_t)a * ne + s];
        c[0] += pos[3 * (size_t)n];
        c[1] += pos[3 * (size_t)n + 1];
    }
    rel[e] = (c[0] / 6 - box[0]) / box[2];
    rel[ne + e] = (c[1] / 6 - box[1]) / box[3];
}

struct FnArgs {
    int type, nx, ny;
    double zmin, zmax;
    double rate[3];
    double R[9];
    float cx, cy, rin, rout;
    const double* cg;
    const double* ca;
    const uint8_t* ce;
};

struct GrowArgs {
    int ne, nfn, interp;
    double dt;
    const double* rates;  // [3][ne] per-element rates, or null
    const int* conn;      // [6][ne]
    const double* pos;    // node positions of the step's start shape
    const double* relz;   // [ne] initial relative z
    const double* rel;    // [2][ne] pinned bounding-box positions, or null: from box and colsrc
    const double* box;    // [4] this step's box (grid functions, current positions)
    const int* colsrc;    // [ne] the prism whose position a prism takes
    const double* gbar;   // [18][ne] Gauss-weighted dN_a/dX_k (growth rotation)
    int nn;
    int* check;           // checked build: failed index tests
    FnArgs fn[kMaxFns];
};

// Products and sums written out with explicit rounding, in the reference's
// order of operations (left to right; its 3x3 products accumulating over k
// from 0), so that no multiply-add is contracted into an FMA.  Where almost all of
// a cell's corners carry no angle the interpolated angle is divided by a
// small 1 - fe, which magnifies any rounding difference.
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }

// Every growth increment here turns about z only, so increments and their
// products keep the form [[a, b, 0], [c, d, 0], [0, 0, e]]; the reference's
// 3x3 products of such matrices add exact zero products, left out here.
__device__ __forceinline__ void mul_xy_z(const double* A, const double* B, double* C) {
    C[0] = add(mul(A[0], B[0]), mul(A[1], B[3]));
    C[1] = add(mul(A[0], B[1]), mul(A[1], B[4]));
    C[3] = add(mul(A[3], B[0]), mul(A[4], B[3]));
    C[4] = add(mul(A[3], B[1]), mul(A[4], B[4]));
    C[8] = mul(A[8], B[8]);
    C[2] = C[5] = C[6] = C[7] = 0.0;
}

// M Fg for an increment M of that form and a general Fg.
__device__ __forceinline__ void mul_xy_z_full(const double* M, const double* F, double* C) {
    for (int j = 0; j < 3; ++j) {
        C[j] = add(mul(M[0], F[j]), mul(M[1], F[3 + j]));
        C[3 + j] = add(mul(M[3], F[j]), mul(M[4], F[3 + j]));
        C[6 + j] = mul(M[8], F[6 + j]);
    }
}

// R diag(d0, d1, d2) R^T for R = [[c, -s, 0], [s, c, 0], [0, 0, 1]], the two
// 3x3 products of the reference with their exact zero terms left out (adding
// a zero product changes no sum): T = R D has one product per entry, and each
// in-plane entry of T R^T is one sum of two products.
__device__ __forceinline__ void rotate_diag(double c, double s, double d0, double d1, double d2, double* inc) {
    const double ms = -1.0 * s;
    const double t00 = mul(c, d0), t01 = mul(ms, d1), t10 = mul(s, d0), t11 = mul(c, d1);
    inc[0] = add(mul(t00, c), mul(t01, ms));
    inc[1] = add(mul(t00, s), mul(t01, c));
    inc[3] = add(mul(t10, c), mul(t11, ms));
    inc[4] = add(mul(t10, s), mul(t11, c));
    inc[2] = inc[5] = inc[6] = inc[7] = 0.0;
    inc[8] = d2;
}

// ShapeBase::calculateFgFromRates with tissue weight 1: R diag(exp(r dt)) R^T,
// R the function's rotation about z (R[0] = cos, R[3] = sin).
__device__ __forceinline__ void rates_increment(const double* r, const double* R, double dt, double* inc) {
    rotate_diag(R[0], R[3], exp(r[0] * 1.0 * dt), exp(r[1] * 1.0 * dt), exp(r[2] * 1.0 * dt), inc);
}

// ShapeBase::calculateFgFromGridCorners for a columnar prism (tissue weight 1).
__device__ void grid_increment(const FnArgs& F, int interp, double rel_x, double rel_y, double dt, double* inc) {
    // ShapeBase::convertRelativePosToGridIndex
    const double rx = rel_x * (float)(F.nx - 1), ry = rel_y * (float)(F.ny - 1);
    int ix = (int)floor(rx), iy = (int)floor(ry);
    double fx = rx - ix, fy = ry - iy;
    if (ix >= F.nx - 1) {
        ix = F.nx - 2;
        fx = 1.0;
    } else if (ix < 0) {
        ix = 0;
        fx = 0.0;
    }
    if (iy >= F.ny - 1) {
        iy = F.ny - 2;
        fy = 1.0;
    } else if (iy < 0) {
        iy = 0;
        fy = 0.0;
    }
    const size_t cell = (size_t)ix * (F.ny - 1) + iy;
    const double* g = F.cg + 12 * cell;  // corner c, axis k at g[3c + k]
    const double* an = F.ca + 4 * cell;
    const uint8_t* el = F.ce + 4 * cell;
    const double ux = 1.0 - fx, uy = 1.0 - fy;
    double growth[3];
    double angle = 0;
    if (interp == 0) {
        const int c = fx > 0.5 ? (fy > 0.5 ? 3 : 1) : (fy > 0.5 ? 2 : 0);
        for (int k = 0; k < 3; ++k) growth[k] = g[3 * c + k];
    } else {
        double fe = 0.0;
        if (el[0]) fe = add(fe, mul(ux, uy));
        if (el[1]) fe = add(fe, mul(fx, uy));
        if (el[2]) fe = add(fe, mul(ux, fy));
        if (el[3]) fe = add(fe, mul(fx, fy));
        angle = add(add(add(mul(mul(an[0], ux), uy), mul(mul(an[1], fx), uy)), mul(mul(an[2], ux), fy)),
                    mul(mul(an[3], fx), fy));
        if (fe > 0) {
            if (fe >= 0.9999999) angle = 0.0;
            else angle /= (1.0 - fe);
        }
        for (int k = 0; k < 3; ++k)
            growth[k] = add(add(add(mul(mul(g[k], ux), uy), mul(mul(g[3 + k], fx), uy)), mul(mul(g[6 + k], ux), fy)),
                            mul(mul(g[9 + k], fx), fy));
    }
    const double d0 = exp(growth[0] * dt), d1 = exp(growth[1] * dt), d2 = exp(growth[2] * dt);
    if (angle != 0.0) {  // R inc R^T, R the rotation by the angle about z
        rotate_diag(cos(angle), sin(angle), d0, d1, d2, inc);
    } else {
        for (int k = 0; k < 9; ++k) inc[k] = 0.0;
        inc[0] = d0;
        inc[4] = d1;
        inc[8] = d2;
    }
}

// The rotation factor of the polar decomposition F = R U (R = U_svd V_svd^T
// of the reference's singular value decomposition) by Higham's scaled Newton
// iteration X <- (z X + X^-T / z) / 2, z = |det X|^(-1/3) (scaled for the first
// three iterations, plain Newton after).
__device__ void polar_rotation(const double* F, double* R) {
    double X[9];
    for (int k = 0; k < 9; ++k) X[k] = F[k];
    for (int it = 0; it < 40; ++it) {
        double inv[9];
        inv3_cof(X, inv);
        const double det = X[0] * (X[4] * X[8] - X[5] * X[7]) - X[1] * (X[3] * X[8] - X[5] * X[6]) +
                           X[2] * (X[3] * X[7] - X[4] * X[6]);
        const double zi = it < 3 ? cbrt(fabs(det)) : 1.0;  // 1 / z
        const double z = it < 3 ? 1.0 / zi : 1.0;
        double d = 0.0;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                const double y = 0.5 * (z * X[3 * i + j] + inv[3 * j + i] * zi);
                d += (y - X[3 * i + j]) * (y - X[3 * i + j]);
                X[3 * i + j] = y;
            }
        if (!(d > 1e-30)) break;
    }
    for (int k = 0; k < 9; ++k) R[k] = X[k];
}

// ShapeBase::CalculateGrowthRotationByF for prism e: the Gauss-weighted
// deformation gradient of the current shape (calculateTriPointFForRatation,
// :1674-1687), its rotation (calculate3DRotMatFromF, :1731-1810: rotated if an
// off-diagonal entry exceeds 0.017), the rotation's angle about z
// (disassembleRotationMatrixForZ, :1690-1721: atan2(R01, R00), used beyond
// 0.017 rad).  True with Rz = [[c, -s, 0], [s, c, 0], [0, 0, 1]].
__device__ bool growth_rotation(const GrowArgs& G, int e, double* Rz) {
    if (!G.gbar) return false;
    const int ne = G.ne;
    double F[9] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int a = 0; a < 6; ++a) {
        const int n = G.conn[(size_t)a * ne + e];
        if (!TF_IN(G.check, n, G.nn, CK_GROW_NODE)) continue;
        double x[3], g[3];
        for (int i = 0; i < 3; ++i) x[i] = G.pos[3 * (size_t)n + i];
        for (int k = 0; k < 3; ++k) g[k] = G.gbar[(size_t)(3 * a + k) * ne + e];
        for (int i = 0; i < 3; ++i)
            for (int k = 0; k < 3; ++k) F[3 * i + k] += x[i] * g[k];
    }
    // R is the orthogonal matrix nearest to F, so |R - I| <= |R - F| + |F - I|
    // <= 2 |F - I| (Frobenius): within 0.017 no off-diagonal entry of R can
    // exceed the reference's threshold and the iteration is not needed
    double dev = 0.0;
    for (int k = 0; k < 9; ++k) {
        const double v = F[k] - ((k & 3) == 0 ? 1.0 : 0.0);
        dev += v * v;
    }
    if (4.0 * dev <= 0.017 * 0.017 * (1.0 - 1e-9)) return false;
    double R[9];
    polar_rotation(F, R);
    bool off = false;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            if (i != j && (R[3 * i + j] > 0.017 || R[3 * i + j] < -0.017)) off = true;
    if (!off) return false;
    const double tz = atan2(R[1], R[0]);
    if (!(tz > 0.017 || tz < -0.017)) return false;
    const double c = cos(tz), s = sin(tz);
    const double r[9] = {c, -1.0 * s, 0.0, s, c, 0.0, 0.0, 0.0, 1.0};
    for (int k = 0; k < 9; ++k) Rz[k] = r[k];
    return true;
}

// Gauss-weighted shape-function gradients: gbar[3a + k] = sum over the 6
// Gauss points of (1/6) dN_a/dX_k.
__global__ void k_gbar(int ne, const double* __restrict__ gx, double* __restrict__ gbar) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    for (int r = 0; r < 18; ++r) {
        double s = 0.0;
        for (int gp = 0; gp < 6; ++gp) s += gx[(size_t)r * (6 * (size_t)ne) + 6 * (size_t)e + gp] * (1.0 / 6.0);
        gbar[(size_t)r * ne + e] = s;
    }
}

// Per prism: the growth increment of the step -- diag(exp(rate dt)) of the
// per-element rates, then each active function's increment multiplied on
// the left (updateGrowthIncrement) -- and Fg <- increment Fg (growShapeByFg).
__global__ void k_grow(GrowArgs G, double* __restrict__ Fg, double* __restrict__ invFg) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= G.ne) return;
    const int ne = G.ne;
    double M[9] = {1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0};
    if (G.rates)
        for (int k = 0; k < 3; ++k) M[4 * k] = exp(G.rates[(size_t)k * ne + e] * 1.0 * G.dt);
    bool centred = false, have_rel = false;
    double cx = 0.0, cy = 0.0, rel_x = 0.0, rel_y = 0.0;
    for (int f = 0; f < G.nfn; ++f) {
        const FnArgs& F = G.fn[f];
        double inc[9];
        if (F.type == kGrid) {
            const double rz = G.relz[e];
            if (rz < F.zmin || rz > F.zmax) continue;  // isGrowthRateApplicable (ShapeBase.cpp:277-300): identity
            if (!have_rel) {
                if (G.rel) {
                    rel_x = G.rel[e];
                    rel_y = G.rel[ne + e];
                } else {  // as k_relpos computes it
                    const int sp = TF_IN(G.check, G.colsrc[e], ne, CK_GROW_PRISM) ? G.colsrc[e] : e;
                    double c[2] = {0.0, 0.0};
                    for (int a = 0; a < 6; ++a) {
                        const int n = G.conn[(size_t)a * ne + sp];
                        if (!TF_IN(G.check, n, G.nn, CK_GROW_NODE)) continue;
                        c[0] += G.pos[3 * (size_t)n];
                        c[1] += G.pos[3 * (size_t)n + 1];
                    }
                    rel_x = (c[0] / 6 - G.box[0]) / G.box[2];
                    rel_y = (c[1] / 6 - G.box[1]) / G.box[3];
                }
                have_rel = true;
            }
            grid_increment(F, G.interp, rel_x, rel_y, G.dt, inc);
        } else {
            const double rz = G.relz[e];
            if (rz < F.zmin || rz > F.zmax) continue;
            double r[3] = {F.rate[0], F.rate[1], F.rate[2]};
            if (F.type == kRing) {
                if (!centred) {  // ShapeBase::getCentre (ShapeBase.cpp:240-250)
                    for (int a = 0; a < 6; ++a) {
                        const int n = G.conn[(size_t)a * ne + e];
                        if (!TF_IN(G.check, n, G.nn, CK_GROW_NODE)) continue;
                        cx = add(cx, G.pos[3 * (size_t)n]);
                        cy = add(cy, G.pos[3 * (size_t)n + 1]);
                    }
                    cx /= 6;
                    cy /= 6;
                    centred = true;
                }
                const double dx = (double)F.cx - cx, dy = (double)F.cy - cy;
                const double d2 = add(mul(dx, dx), mul(dy, dy));
                const float rin2 = __fmul_rn(F.rin, F.rin), rout2 = __fmul_rn(F.rout, F.rout);
                if (!(d2 > (double)rin2 && d2 < (double)rout2)) continue;
                const float dist = __double2float_rn(sqrt(d2));
                const double sf = 1.0 - (double)__fdiv_rn(__fsub_rn(dist, F.rin), __fsub_rn(F.rout, F.rin));
                for (int k = 0; k < 3; ++k) r[k] = mul(r[k], sf);
            }
            rates_increment(r, F.R, G.dt, inc);
        }
        double P[9];
        mul_xy_z(inc, M, P);
        for (int k = 0; k < 9; ++k) M[k] = P[k];
    }
    // ShapeBase::CalculateGrowthRotationByF (ShapeBase.cpp:1656-1672), then
    // the rotated increment of growShapeByFg (:1216-1225): Rz M Rz^T
    double Rz[9];
    if (growth_rotation(G, e, Rz)) {
        const double RzT[9] = {Rz[0], Rz[3], 0.0, Rz[1], Rz[4], 0.0, 0.0, 0.0, 1.0};
        double T[9];
        mul_xy_z(Rz, M, T);
        mul_xy_z(T, RzT, M);
    }
    double F0[9], out[9], inv[9];
    for (int k = 0; k < 9; ++k) F0[k] = Fg[(size_t)k * ne + e];
    mul_xy_z_full(M, F0, out);
    inv3_cof(out, inv);
    for (int k = 0; k < 9; ++k) {
        Fg[(size_t)k * ne + e] = out[k];
        invFg[(size_t)k * ne + e] = inv[k];
    }
}

// Box and bounding-box positions of the current positions into rel_out.
tf_status launch_relpos(tf_handle* h, double* rel_out) {
    Growth* g = h->growth;
    Device& d = h->d;
    k_box<<<kBoxCtas, kT, 0, h->stream>>>(d.nn, d.uk, g->part, g->ticket, g->box);
    TF_LAUNCH_CHECK(h);
    k_relpos<<<cdiv(d.ne, kT), kT, 0, h->stream>>>(d.ne, d.conn, d.uk, g->box, g->colsrc, rel_out);
    TF_LAUNCH_CHECK(h);
    return TF_OK;
}

}  // namespace

void growth_free(Growth* g) {
    if (!g) return;
    for (auto& f : g->fns) free_fn(f);
    void* ptrs[] = {g->relz, g->rel0, g->rel, g->colsrc, g->box, g->part, g->ticket, g->gbar};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete g;
}

// Tissue height, initial relative z (assignInitialZPositions, Simulation.cpp
// :3367-3371, after calculateBoundingBox), the columns and the pinned
// positions (Simulation.cpp:630-645), from the mesh's positions at creation.
tf_status growth_setup(tf_handle* h) {
    Growth* g = new Growth;
    h->growth = g;
    const int ne = h->d.ne, nn = h->d.nn;
    const double* pos0 = h->h_pos0.data();
    tissue_height(h, pos0, &g->layers, &g->height);
    double lo[3], size[3];
    host_box(pos0, nn, lo, size);
    // ShapeBase::setInitialZPosition (ShapeBase.cpp:612-627)
    std::vector<double> relz(ne), rel(2 * (size_t)ne), rel0(2 * (size_t)ne);
    for (int e = 0; e < ne; ++e) {
        double c[3] = {0.0, 0.0, 0.0};
        for (int a = 0; a < 6; ++a)
            for (int k = 0; k < 3; ++k) c[k] += pos0[3 * (size_t)h->h_conn[6 * (size_t)e + a] + k];
        for (int k = 0; k < 3; ++k) c[k] /= 6;
        double r = 1.0 - ((c[2] - lo[2]) / g->height);
        if (r < 0) r = 0;
        if (r > 1.0) r = 1.0;
        relz[e] = r;
        rel[e] = (c[0] - lo[0]) / size[0];
        rel[ne + e] = (c[1] - lo[1]) / size[1];
    }
    // Columns: from each basal prism up, the first prism (in element order)
    // whose basal triangle is the current apical one.
    std::map<std::array<int, 3>, int> by_basal;
    auto tri = [&](int e, int o) {
        std::array<int, 3> k = {h->h_conn[6 * (size_t)e + o], h->h_conn[6 * (size_t)e + o + 1],
                                h->h_conn[6 * (size_t)e + o + 2]};
        std::sort(k.begin(), k.end());
        return k;
    };
    for (int e = 0; e < ne; ++e) by_basal.emplace(tri(e, 0), e);
    std::vector<int> colsrc(ne);
    for (int e = 0; e < ne; ++e) colsrc[e] = e;
    const int L = g->layers;
    std::vector<int> col;
    for (int e = 0; e < ne; ++e) {
        if (element_placement(h, e) != 0 || L < 3) continue;
        col.assign(1, e);
        for (int i = 1; i < L; ++i) {
            auto it = by_basal.find(tri(col.back(), 3));
            if (it == by_basal.end() || it->second == col.back()) break;
            col.push_back(it->second);
        }
        if ((int)col.size() != L) continue;
        const int top = col.back();
        if (element_placement(h, top) != 1) continue;
        for (int i = 0; i < L - 2; ++i) colsrc[col[i]] = top;
    }
    for (int e = 0; e < ne; ++e) {
        rel0[e] = rel[colsrc[e]];
        rel0[ne + e] = rel[ne + colsrc[e]];
    }
    GR_TRY(put(&g->relz, relz));
    GR_TRY(put(&g->rel0, rel0));
    GR_TRY(put(&g->rel, std::vector<double>(2 * (size_t)ne, 0.0)));
    GR_TRY(put(&g->colsrc, colsrc));
    GR_TRY(put(&g->box, std::vector<double>(4, 0.0)));
    GR_TRY(put(&g->part, std::vector<double>(4 * (size_t)kBoxCtas, 0.0)));
    {
        cudaError_t err = cudaMalloc(reinterpret_cast<void**>(&g->gbar), 18 * sizeof(double) * (size_t)ne);
        if (err != cudaSuccess) {
            cudaGetLastError();
            g->gbar = nullptr;
            set_error("device allocation failed for a growth function");
            return TF_OUT_OF_MEMORY;
        }
        k_gbar<<<cdiv(ne, kT), kT, 0, h->stream>>>(ne, h->d.gx, g->gbar);
        TF_LAUNCH_CHECK(h);
        TF_CUDA(cudaStreamSynchronize(h->stream));
    }
    GR_TRY(put(&g->ticket, std::vector<unsigned>(1, 0u)));
    return TF_OK;
}

namespace {

// The rotation of GrowthFunctionBase's xy angle (UniformGrowthFunction /
// RingGrowthFunction constructors, GrowthFunctionTypes.h:37-52, :196-211).
void angle_rotation(double angle, double* R) {
    const double c = std::cos(angle), s = std::sin(angle);
    const double r[9] = {c, -1.0 * s, 0.0, s, c, 0.0, 0.0, 0.0, 1.0};
    for (int k = 0; k < 9; ++k) R[k] = r[k];
}

GrowthFn window(double t0, double t1, double zmin, double zmax) {
    GrowthFn f;
    f.t0 = static_cast<float>(t0);  // GrowthFunctionBase keeps its times as float
    f.t1 = static_cast<float>(t1);
    f.zmin = zmin;
    f.zmax = zmax;
    return f;
}

}  // namespace

tf_status growth_add_uniform(tf_handle* h, const double* rates, double angle, double t0, double t1, double zmin,
                             double zmax) {
    GrowthFn f = window(t0, t1, zmin, zmax);
    f.type = kUniform;
    for (int k = 0; k < 3; ++k) f.rate[k] = rates[k];
    angle_rotation(angle, f.R);
    h->growth->fns.push_back(f);
    return TF_OK;
}

tf_status growth_add_ring(tf_handle* h, double cx, double cy, double r_in, double r_out, const double* rates,
                          double angle, double t0, double t1, double zmin, double zmax) {
    GrowthFn f = window(t0, t1, zmin, zmax);
    f.type = kRing;
    for (int k = 0; k < 3; ++k) f.rate[k] = rates[k];
    angle_rotation(angle, f.R);
    f.cx = static_cast<float>(cx);  // RingGrowthFunction::getCentre / getInnerRadius / getOuterRadius
    f.cy = static_cast<float>(cy);
    f.rin = static_cast<float>(r_in);
    f.rout = static_cast<float>(r_out);
    h->growth->fns.push_back(f);
    return TF_OK;
}

tf_status growth_add_grid(tf_handle* h, int nx, int ny, const double* rates, const double* angles_deg, double t0,
                          double t1, double zmin, double zmax) {
    GrowthFn f = window(t0, t1, zmin, zmax);
    f.type = kGrid;
    f.nx = nx;
    f.ny = ny;
    std::vector<double> cg, ca;
    std::vector<uint8_t> ce;
    compatible_corners(nx, ny, rates, angles_deg, cg, ca, ce);
    tf_status s = put(&f.cg, cg);
    if (s == TF_OK) s = put(&f.ca, ca);
    if (s == TF_OK) s = put(&f.ce, ce);
    if (s != TF_OK) {
        free_fn(f);
        return s;
    }
    h->growth->fns.push_back(f);
    return TF_OK;
}

void growth_clear(tf_handle* h) {
    if (!h->growth) return;
    for (auto& f : h->growth->fns) free_fn(f);
    h->growth->fns.clear();
}

void growth_set_mode(tf_handle* h, int interp, int pinned) {
    h->growth->interp = interp;
    h->growth->pinned = pinned;
}

// Simulation::updatePinningPositions (Simulation.cpp:6018-6023): the current
// bounding-box positions become the pinned ones.
tf_status growth_repin(tf_handle* h) { return launch_relpos(h, h->growth->rel0); }

int growth_count(const tf_handle* h) { return h->growth ? static_cast<int>(h->growth->fns.size()) : 0; }

// The growth of a step when growth functions are active at the handle's time
// (each in init_time <= t < end_time): the per-element rates and the active
// functions in one increment per prism.  *done = false: none is active, the
// per-element rates alone apply.
tf_status launch_growth_functions(tf_handle* h, bool* done) {
    *done = false;
    Growth* g = h->growth;
    if (!g || g->fns.empty()) return TF_OK;
    Device& d = h->d;
    const double t = h->time;
    GrowArgs A{};
    A.ne = d.ne;
    A.interp = g->interp;
    A.dt = h->dt;
    A.rates = h->have_rates ? d.rates : nullptr;
    A.conn = d.conn;
    A.pos = d.uk;
    A.relz = g->relz;
    A.rel = g->pinned ? g->rel0 : nullptr;
    A.box = g->box;
    A.colsrc = g->colsrc;
    bool grid = false;
    for (const auto& f : g->fns) {
        if (!(t >= f.t0 && t < f.t1)) continue;
        FnArgs& F = A.fn[A.nfn++];
        F.type = f.type;
        F.nx = f.nx;
        F.ny = f.ny;
        F.zmin = f.zmin;
        F.zmax = f.zmax;
        for (int k = 0; k < 3; ++k) F.rate[k] = f.rate[k];
        for (int k = 0; k < 9; ++k) F.R[k] = f.R[k];
        F.cx = f.cx;
        F.cy = f.cy;
        F.rin = f.rin;
        F.rout = f.rout;
        F.cg = f.cg;
        F.ca = f.ca;
        F.ce = f.ce;
        grid |= f.type == kGrid;
    }
    A.nn = d.nn;
    A.check = d.check;
    A.gbar = g->gbar;  // the reference turns the growth with the prism whenever functions exist (Simulation.cpp:5872-5876)
    if (grid && !g->pinned) {  // this step's box; k_grow forms the positions
        k_box<<<kBoxCtas, kT, 0, h->stream>>>(d.nn, d.uk, g->part, g->ticket, g->box);
        TF_LAUNCH_CHECK(h);
    }
    k_grow<<<cdiv(d.ne, kT), kT, 0, h->stream>>>(A, d.Fg, d.invFg);
    TF_LAUNCH_CHECK(h);
    *done = true;
    return TF_OK;
}

// Host copies for the tests: relative z, pinned positions, and the positions
// of the current shape.
tf_status growth_positions(tf_handle* h, double* relz, double* rel0, double* rel) {
    Growth* g = h->growth;
    const size_t ne = h->d.ne;
    if (relz) TF_CUDA(cudaMemcpyAsync(relz, g->relz, ne * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (rel0) TF_CUDA(cudaMemcpyAsync(rel0, g->rel0, 2 * ne * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (rel) {
        GR_TRY(launch_relpos(h, g->rel));
        TF_CUDA(cudaMemcpyAsync(rel, g->rel, 2 * ne * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    }
    TF_CUDA(cudaStreamSynchronize(h->stream));
    return TF_OK;
}

}  // namespace tf
