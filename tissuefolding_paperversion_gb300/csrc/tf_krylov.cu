// FP64 Krylov solve of A du = g with A = K^T: the replacement for the
// reference's Pardiso phases 11/22/33 (NewtonRaphsonSolver.cpp:418-683,
// transposed solve iparm[11] = 1 at :639).
//
//   * block-Jacobi preconditioner on the 3x3 diagonal blocks;
//   * CG when every element has zero internal viscosity (A symmetric),
//     BiCGStab otherwise (the viscous tangent is not symmetric);
//   * a batch of independent instances is one block-diagonal system, solved
//     with separate Krylov scalars, tolerance and stop flag per instance:
//     every CTA of the node-parallel kernels covers nodes of one instance,
//     reductions are per instance, and an instance whose flag is set is
//     skipped by all later kernels (a single mesh is a batch of one);
//   * all scalars stay on the device: each reduction kernel writes per-CTA
//     partial sums and the last CTA of the instance to finish (atomic ticket,
//     no waiting) folds them in a fixed order, so results are bitwise
//     reproducible;
//   * iterations run in chunks of 8-64 replayed from CUDA graphs; the host
//     reads the flags once per chunk.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "tf_internal.cuh"

namespace tf {

namespace {

constexpr int kThreads = kNodeThreads;

enum Flag { F_RUNNING = 0, F_CONVERGED = 1, F_BREAKDOWN = 2, F_NAN = 3 };
// Cause of a breakdown (S_WHY): which denominator vanished.
enum Why { W_NONE = 0, W_CG_PAP = 1, W_CG_RZ = 2, W_BI_RV = 3, W_BI_OMEGA = 4, W_BI_RHO = 5 };
const char* const kWhy[] = {"", "(p, Ap) <= 0", "(r, M^-1 r) <= 0", "(rhat, A phat) = 0", "omega = 0",
                            "(rhat, r) = 0"};

struct Ctx {
    const int* __restrict__ wslot0;
    const int* __restrict__ scol;
    const double* __restrict__ val;
    const double* __restrict__ dinv;
    double* scal;               // [nseg][S_COUNT]
    double* part;               // [3][ncta]
    unsigned* tickets;          // [nseg]
    int ncta;
    const int* __restrict__ cta_seg;
    const int* __restrict__ cta_node0;
    const int* __restrict__ cta_node1;
    const int* __restrict__ seg_cta0;
    const int* __restrict__ seg_solve;
    const int* __restrict__ xrow;     // extra blocks (tf_add_K_triplets), null: none
    const int* __restrict__ xcol;
    const double* __restrict__ xval;
    int nn;
    int* check;                       // checked build: failed index checks
};

struct Where {
    int node;    // node of this thread
    bool valid;  // node inside this CTA's range
    int seg;     // instance of this CTA
    double* s;   // its scalars
};

__device__ __forceinline__ Where where(const Ctx& c) {
    Where w;
    w.seg = c.cta_seg[blockIdx.x];
    w.node = c.cta_node0[blockIdx.x] + threadIdx.x;
    w.valid = w.node < c.cta_node1[blockIdx.x];
    w.s = c.scal + (size_t)w.seg * S_COUNT;
    return w;
}

template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double (*sm)[kThreads / 32]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double x = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sm[k][warp] = x;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double x = lane < kThreads / 32 ? sm[k][lane] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            v[k] = x;  // valid in thread 0
        }
    }
    __syncthreads();
}

// Writes this CTA's partial sums; returns true in the CTA of the instance
// that arrives last, whose thread 0 then holds the fixed-order totals.
template <int NV>
__device__ bool reduce_seg(const Ctx& c, int seg, double (&v)[NV], double (&tot)[NV]) {
    __shared__ double sm[NV][kThreads / 32];
    __shared__ bool last;
    block_sum<NV>(v, sm);
    const int b0 = c.seg_cta0[seg], b1 = c.seg_cta0[seg + 1];
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) c.part[(size_t)k * c.ncta + blockIdx.x] = v[k];
        __threadfence();
        const unsigned ticket = atomicAdd(&c.tickets[seg], 1u);
        last = (ticket == (unsigned)(b1 - b0 - 1));
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        acc[k] = 0.0;
        for (int b = b0 + threadIdx.x; b < b1; b += kThreads) acc[k] += __ldcg(&c.part[(size_t)k * c.ncta + b]);
    }
    block_sum<NV>(acc, sm);
#pragma unroll
    for (int k = 0; k < NV; ++k) tot[k] = acc[k];
    if (threadIdx.x == 0) c.tickets[seg] = 0u;
    return true;
}

__device__ __forceinline__ bool stopped(const Where& w) { return __ldcg(&w.s[S_FLAG]) != 0.0; }

__device__ __forceinline__ void apply_dinv(const double* __restrict__ D, const double r[3], double z[3]) {
    z[0] = fma(D[0], r[0], fma(D[1], r[1], D[2] * r[2]));
    z[1] = fma(D[3], r[0], fma(D[4], r[1], D[5] * r[2]));
    z[2] = fma(D[6], r[0], fma(D[7], r[1], D[8] * r[2]));
}

template <int U = 2>
__device__ __forceinline__ void bsr_row(const Ctx& c, int i, const double* __restrict__ x, double y[3]) {
    sliced_row<double, U>(c.wslot0, c.scol, c.val, x, y, c.nn, c.check);
    if (c.xrow) {
        for (int p = c.xrow[i]; p < c.xrow[i + 1]; ++p) {
            const int j = c.xcol[p];
            if (!TF_IN(c.check, j, c.nn, CK_EXTRA_COL)) continue;
            const double* __restrict__ a = c.xval + 9 * (size_t)p;
            const double x0 = x[3 * j], x1 = x[3 * j + 1], x2 = x[3 * j + 2];
            y[0] = fma(a[0], x0, fma(a[1], x1, fma(a[2], x2, y[0])));
            y[1] = fma(a[3], x0, fma(a[4], x1, fma(a[5], x2, y[1])));
            y[2] = fma(a[6], x0, fma(a[7], x1, fma(a[8], x2, y[2])));
        }
    }
}

// Sets an instance's stop flag from its first scalars (bb = |b|^2).  With an
// absolute update accuracy atol > 0, the relative tolerance is loosened to
// the residual |r| <= atol / sinv (sinv = the largest |du| / |g| of the
// instance's earlier solves, which bounds |A^-1 r| / |r| along the
// directions the step has produced), at most to a relative 0.1.
__device__ __forceinline__ void start_flags(double* s, double bb, double tol2, double atol, double rr) {
    s[S_BB] = bb;
    s[S_RR] = rr;
    s[S_RR0] = rr;
    s[S_ITER] = 0.0;
    const double sinv = s[S_SINV];
    if (atol > 0.0 && sinv > 0.0 && bb > 0.0) {
        const double r = atol / sinv;
        tol2 = fmax(tol2, fmin(r * r / bb, 1e-2));
    }
    s[S_TOL2] = tol2;
    s[S_WHY] = W_NONE;
    s[S_FLAG] = (bb == 0.0 || rr <= tol2 * bb) ? F_CONVERGED : (isfinite(bb) && isfinite(rr) ? F_RUNNING : F_NAN);
}

// ---- CG -------------------------------------------------------------------

// r = b, z = M^-1 r, p = z, x = 0;  rz = (r,z), bb = (b,b).  Instances left
// out of this solve (seg_solve = 0) either keep their x (keep != 0, a retry of
// other instances) or solve with b = 0, which sets x = 0 (an instance whose
// Newton loop has stopped); both are flagged done at once.
__global__ void k_cg_init(Ctx c, const double* __restrict__ b, double* __restrict__ x, double* __restrict__ r,
                          double* __restrict__ z, double* __restrict__ p, double tol2, double atol, int keep,
                          int jac, const double* __restrict__ x0) {
    const Where w = where(c);
    const bool active = c.seg_solve[w.seg] != 0;
    if (!active && keep) {
        if (threadIdx.x == 0) w.s[S_FLAG] = F_CONVERGED;
        return;
    }
    double v[3] = {0.0, 0.0, 0.0};  // (r, z), |r|^2, |b|^2
    if (w.valid) {
        const int i = w.node;
        double rr[3], zz[3], ax[3] = {0.0, 0.0, 0.0};
        if (x0 && active) bsr_row(c, i, x0, ax);  // start from x0: r = b - A x0
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double bk = active ? b[3 * i + d] : 0.0;
            rr[d] = bk - ax[d];
            r[3 * i + d] = rr[d];
            x[3 * i + d] = (x0 && active) ? x0[3 * i + d] : 0.0;
            v[2] = fma(bk, bk, v[2]);
        }
        if (jac) {
            apply_dinv(c.dinv + 9 * (size_t)i, rr, zz);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if (!active) zz[d] = 0.0;
                z[3 * i + d] = zz[d];
                p[3 * i + d] = zz[d];
                v[0] = fma(rr[d], zz[d], v[0]);
            }
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) v[1] = fma(rr[d], rr[d], v[1]);
    }
    double tot[3];
    if (reduce_seg<3>(c, w.seg, v, tot) && threadIdx.x == 0) {
        if (jac) w.s[S_RZ] = tot[0];
        start_flags(w.s, tot[2], tol2, atol, tot[1]);
    }
}

// q = A p; alpha = rz / (p, q)
template <int U>
__global__ void k_cg_spmv(Ctx c, const double* __restrict__ p, double* __restrict__ q) {
    pdl_enter();
    const Where w = where(c);
    if (stopped(w)) return;
    double v[1] = {0.0};
    if (w.valid) {
        double y[3];
        bsr_row<U>(c, w.node, p, y);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            q[3 * w.node + d] = y[d];
            v[0] = fma(p[3 * w.node + d], y[d], v[0]);
        }
    }
    double tot[1];
    if (reduce_seg<1>(c, w.seg, v, tot) && threadIdx.x == 0) {
        const double pq = tot[0];
        if (!(pq > 0.0) || !isfinite(pq)) {
            w.s[S_FLAG] = isfinite(pq) ? F_BREAKDOWN : F_NAN;
            w.s[S_WHY] = W_CG_PAP;
        } else {
            w.s[S_PQ] = pq;
            w.s[S_ALPHA] = w.s[S_RZ] / pq;
        }
    }
}

// x += alpha p; r -= alpha q; z = M^-1 r;  beta = (r,z)_new / (r,z)
__global__ void k_cg_update(Ctx c, double* __restrict__ x, double* __restrict__ r, double* __restrict__ z,
                            const double* __restrict__ p, const double* __restrict__ q, int jac) {
    pdl_enter();
    const Where w = where(c);
    if (stopped(w)) return;
    const double alpha = __ldcg(&w.s[S_ALPHA]);
    double v[2] = {0.0, 0.0};
    if (w.valid) {
        const int i = w.node;
        double rr[3], zz[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int k = 3 * i + d;
            x[k] = fma(alpha, p[k], x[k]);
            rr[d] = fma(-alpha, q[k], r[k]);
            r[k] = rr[d];
        }
        if (jac) {
            apply_dinv(c.dinv + 9 * (size_t)i, rr, zz);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                z[3 * i + d] = zz[d];
                v[0] = fma(rr[d], zz[d], v[0]);
            }
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) v[1] = fma(rr[d], rr[d], v[1]);
    }
    double tot[2];
    if (reduce_seg<2>(c, w.seg, v, tot) && threadIdx.x == 0) {
        double* s = w.s;
        const double rz = tot[0], rr = tot[1];
        if (jac) {
            s[S_BETA] = rz / s[S_RZ];
            s[S_RZ] = rz;
        }
        s[S_RR] = rr;
        s[S_ITER] += 1.0;
        if (!isfinite(rr)) s[S_FLAG] = F_NAN;
        else if (rr <= s[S_TOL2] * s[S_BB]) s[S_FLAG] = F_CONVERGED;
        else if (jac && !(rz > 0.0)) {
            s[S_FLAG] = F_BREAKDOWN;
            s[S_WHY] = W_CG_RZ;
        }
    }
}

// With the multigrid preconditioner (z = M^-1 r computed between kernels):
// rz = (r, z), beta = rz / rz_old; start != 0 also sets p = z (first step).
__global__ void k_cg_rz(Ctx c, const double* __restrict__ r, const double* __restrict__ z, double* __restrict__ p,
                        int start) {
    pdl_enter();
    const Where w = where(c);
    if (stopped(w)) return;
    double v[1] = {0.0};
    if (w.valid)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int k = 3 * w.node + d;
            v[0] = fma(r[k], z[k], v[0]);
            if (start) p[k] = z[k];
        }
    double tot[1];
    if (reduce_seg<1>(c, w.seg, v, tot) && threadIdx.x == 0) {
        double* s = w.s;
        const double rz = tot[0];
        if (!start) s[S_BETA] = rz / s[S_RZ];
        s[S_RZ] = rz;
        if (!isfinite(rz)) {
            s[S_FLAG] = F_NAN;
        } else if (!(rz > 0.0)) {
            s[S_FLAG] = F_BREAKDOWN;
            s[S_WHY] = W_CG_RZ;
        }
    }
}

// p = z + beta p
__global__ void k_cg_direction(Ctx c, const double* __restrict__ z, double* __restrict__ p) {
    pdl_enter();
    const Where w = where(c);
    if (stopped(w) || !w.valid) return;
    const double beta = __ldcg(&w.s[S_BETA]);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int k = 3 * w.node + d;
        p[k] = fma(beta, p[k], z[k]);
    }
}

// ---- BiCGStab ---------------------------------------------------------------

// r = rhat = b, p = v = 0, x = 0; rho = (rhat, r)
__global__ void k_bi_init(Ctx c, const double* __restrict__ b, double* __restrict__ x, double* __restrict__ r,
                          double* __restrict__ rhat, double* __restrict__ p, double* __restrict__ v, double tol2,
                          double atol, int keep, const double* __restrict__ x0) {
    const Where w = where(c);
    const bool active = c.seg_solve[w.seg] != 0;
    if (!active && keep) {
        if (threadIdx.x == 0) w.s[S_FLAG] = F_CONVERGED;
        return;
    }
    double s[2] = {0.0, 0.0};  // |r|^2, |b|^2
    if (w.valid) {
        double ax[3] = {0.0, 0.0, 0.0};
        if (x0 && active) bsr_row(c, w.node, x0, ax);  // start from x0: r = b - A x0
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int k = 3 * w.node + d;
            const double bk = active ? b[k] : 0.0;
            const double rk = bk - ax[d];
            r[k] = rk;
            rhat[k] = rk;
            p[k] = 0.0;
            v[k] = 0.0;
            x[k] = (x0 && active) ? x0[k] : 0.0;
            s[0] = fma(rk, rk, s[0]);
            s[1] = fma(bk, bk, s[1]);
        }
    }
    double tot[2];
    if (reduce_seg<2>(c, w.seg, s, tot) && threadIdx.x == 0) {
        w.s[S_RHO] = tot[0];
        w.s[S_ALPHA] = 1.0;
        w.s[S_OMEGA] = 1.0;
        w.s[S_BETA] = 0.0;
        start_flags(w.s, tot[1], tol2, atol, tot[0]);
    }
}

// p = r + beta (p - omega v); phat = M^-1 p
__global__ void k_bi_dir(Ctx c, const double* __restrict__ r, const double* __restrict__ v, double* __restrict__ p,
                         double* __restrict__ phat, int jac) {
    pdl_enter();
    const Where w = where(c);
    if (stopped(w) || !w.valid) return;
    const double beta = __ldcg(&w.s[S_BETA]), omega = __ldcg(&w.s[S_OMEGA]);
    const int i = w.node;
    double pp[3], z[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int k = 3 * i + d;
        pp[d] = fma(beta, fma(-omega, v[k], p[k]), r[k]);
        p[k] = pp[d];
    }
    if (!jac) return;
    apply_dinv(c.dinv + 9 * (size_t)i, pp, z);
#pragma unroll
    for (int d = 0; d < 3; ++d) phat[3 * i + d] = z[d];
}

// v = A phat; alpha = rho / (rhat, v)
template <int U>
__global__ void k_bi_spmv1(Ctx c, const double* __restrict__ phat, const double* __restrict__ rhat,
                           double* __restrict__ v) {
    pdl_enter();
    const Where w = where(c);
    if (stopped(w)) return;
    double s[1] = {0.0};
    if (w.valid) {
        double y[3];
        bsr_row<U>(c, w.node, phat, y);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            v[3 * w.node + d] = y[d];
            s[0] = fma(rhat[3 * w.node + d], y[d], s[0]);
        }
    }
    double tot[1];
    if (reduce_seg<1>(c, w.seg, s, tot) && threadIdx.x == 0) {
        const double rv = tot[0];
        if (rv == 0.0 || !isfinite(rv)) {
            w.s[S_FLAG] = isfinite(rv) ? F_BREAKDOWN : F_NAN;
            w.s[S_WHY] = W_BI_RV;
        } else {
            w.s[S_ALPHA] = w.s[S_RHO] / rv;
        }
    }
}

// s = r - alpha v; shat = M^-1 s; |s|^2.  When |s| already meets the
// tolerance the half step is the solution: x += alpha phat and stop (t and
// omega would otherwise be formed from a vanishing s).
__global__ void k_bi_s(Ctx c, const double* __restrict__ r, const double* __restrict__ v, double* __restrict__ s,
                       double* __restrict__ shat, double* __restrict__ x, const double* __restrict__ phat, int jac) {
    pdl_enter();
    const Where w = where(c);
    if (stopped(w)) return;
    const double alpha = __ldcg(&w.s[S_ALPHA]);
    double acc[1] = {0.0};
    if (w.valid) {
        const int i = w.node;
        double ss[3], z[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int k = 3 * i + d;
            ss[d] = fma(-alpha, v[k], r[k]);
            s[k] = ss[d];
            acc[0] = fma(ss[d], ss[d], acc[0]);
        }
        if (jac) {
            apply_dinv(c.dinv + 9 * (size_t)i, ss, z);
#pragma unroll
            for (int d = 0; d < 3; ++d) shat[3 * i + d] = z[d];
        }
    }
    double tot[1];
    if (reduce_seg<1>(c, w.seg, acc, tot) && threadIdx.x == 0) {
        if (!isfinite(tot[0])) w.s[S_FLAG] = F_NAN;
        else if (tot[0] <= w.s[S_TOL2] * w.s[S_BB]) {
            w.s[S_RR] = tot[0];  // the residual of x + alpha phat is s
            w.s[S_FLAG] = -1.0;  // half step converged
        }
    }
}

// Applies the half step x += alpha phat of instances flagged -1 by k_bi_s
// and marks them converged.
__global__ void k_bi_half(Ctx c, double* __restrict__ x, const double* __restrict__ phat) {
    pdl_enter();
    const Where w = where(c);
    if (__ldcg(&w.s[S_FLAG]) != -1.0) return;
    const double alpha = __ldcg(&w.s[S_ALPHA]);
    if (w.valid)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int k = 3 * w.node + d;
            x[k] = fma(alpha, phat[k], x[k]);
        }
    double tot[1] = {0.0}, v[1] = {0.0};
    if (reduce_seg<1>(c, w.seg, v, tot) && threadIdx.x == 0) {
        w.s[S_ITER] += 1.0;
        w.s[S_FLAG] = F_CONVERGED;
    }
}

// t = A shat; omega = (t, s) / (t, t)
template <int U>
__global__ void k_bi_spmv2(Ctx c, const double* __restrict__ shat, const double* __restrict__ s,
                           double* __restrict__ t) {
    pdl_enter();
    const Where w = where(c);
    if (stopped(w)) return;
    double acc[2] = {0.0, 0.0};
    if (w.valid) {
        double y[3];
        bsr_row<U>(c, w.node, shat, y);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            t[3 * w.node + d] = y[d];
            acc[0] = fma(y[d], s[3 * w.node + d], acc[0]);
            acc[1] = fma(y[d], y[d], acc[1]);
        }
    }
    double tot[2];
    if (reduce_seg<2>(c, w.seg, acc, tot) && threadIdx.x == 0) {
        const double ts = tot[0], tt = tot[1];
        if (!isfinite(ts) || !isfinite(tt)) w.s[S_FLAG] = F_NAN;
        else w.s[S_OMEGA] = (tt > 0.0) ? ts / tt : 0.0;
    }
}

// x += alpha phat + omega shat; r = s - omega t; rho' = (rhat, r)
__global__ void k_bi_x(Ctx c, double* __restrict__ x, double* __restrict__ r, const double* __restrict__ rhat,
                       const double* __restrict__ phat, const double* __restrict__ shat, const double* __restrict__ s,
                       const double* __restrict__ t) {
    pdl_enter();
    const Where w = where(c);
    if (stopped(w)) return;
    const double alpha = __ldcg(&w.s[S_ALPHA]), omega = __ldcg(&w.s[S_OMEGA]);
    double acc[2] = {0.0, 0.0};
    if (w.valid) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int k = 3 * w.node + d;
            x[k] = fma(omega, shat[k], fma(alpha, phat[k], x[k]));
            const double rk = fma(-omega, t[k], s[k]);
            r[k] = rk;
            acc[0] = fma(rhat[k], rk, acc[0]);
            acc[1] = fma(rk, rk, acc[1]);
        }
    }
    double tot[2];
    if (reduce_seg<2>(c, w.seg, acc, tot) && threadIdx.x == 0) {
        double* q = w.s;
        const double rho = tot[0], rr = tot[1];
        const double om = q[S_OMEGA];
        q[S_BETA] = (rho / q[S_RHO]) * (q[S_ALPHA] / om);
        q[S_RHO] = rho;
        q[S_RR] = rr;
        q[S_ITER] += 1.0;
        if (!isfinite(rr)) q[S_FLAG] = F_NAN;
        else if (rr <= q[S_TOL2] * q[S_BB]) q[S_FLAG] = F_CONVERGED;
        else if (om == 0.0 || rho == 0.0) {
            q[S_FLAG] = F_BREAKDOWN;
            q[S_WHY] = om == 0.0 ? W_BI_OMEGA : W_BI_RHO;
        }
    }
}

// Restart of BiCGStab from the current iterate after a breakdown: x and its
// residual r are kept, the shadow residual becomes rhat = r and the search
// directions start again.  |b|, the tolerance and the iteration count carry
// over.  Instances outside seg_solve keep their result and are flagged done.
__global__ void k_bi_restart(Ctx c, const double* __restrict__ r, double* __restrict__ rhat, double* __restrict__ p,
                             double* __restrict__ v) {
    const Where w = where(c);
    const bool active = c.seg_solve[w.seg] != 0;
    if (!active) {
        if (threadIdx.x == 0) w.s[S_FLAG] = F_CONVERGED;
        return;
    }
    double s[1] = {0.0};
    if (w.valid) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int k = 3 * w.node + d;
            const double rk = r[k];
            rhat[k] = rk;
            p[k] = 0.0;
            v[k] = 0.0;
            s[0] = fma(rk, rk, s[0]);
        }
    }
    double tot[1];
    if (reduce_seg<1>(c, w.seg, s, tot) && threadIdx.x == 0) {
        double* q = w.s;
        q[S_RHO] = tot[0];
        q[S_RR] = tot[0];
        q[S_ALPHA] = 1.0;
        q[S_OMEGA] = 1.0;
        q[S_BETA] = 0.0;
        q[S_WHY] = W_NONE;
        if (!isfinite(tot[0])) q[S_FLAG] = F_NAN;
        else q[S_FLAG] = (tot[0] <= q[S_TOL2] * q[S_BB]) ? F_CONVERGED : F_RUNNING;
    }
}

// ---- Newton update ------------------------------------------------------------

// uk += du; |du|^2 per instance  (NewtonRaphsonSolver::updateUkInIteration
// :755-761, checkConvergenceViaDeltaU :727-740)
// APPLY = false: |du|^2 only (the same sum, uk untouched), for the Newton
// test before the update is applied.
template <bool APPLY>
__global__ void k_update(Ctx c, double* __restrict__ uk, const double* __restrict__ du,
                         const int* __restrict__ skip = nullptr) {
    if (skip && __ldcg(skip)) return;  // the device Newton loop handed this update to the host
    const Where w = where(c);
    double v[1] = {0.0};
    if (w.valid) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int k = 3 * w.node + d;
            const double dk = du[k];
            if (APPLY) uk[k] = uk[k] + dk;
            v[0] = fma(dk, dk, v[0]);
        }
    }
    double tot[1];
    if (reduce_seg<1>(c, w.seg, v, tot) && threadIdx.x == 0) {
        w.s[S_DU2] = tot[0];
        if (!APPLY) return;
        // |du| / |g| of this solve: the scale that turns a residual into an update error
        const double bb = w.s[S_BB];
        if (bb > 0.0 && isfinite(tot[0])) w.s[S_SINV] = fmax(w.s[S_SINV], sqrt(tot[0] / bb));
    }
}

Ctx make_ctx(tf_handle* h) {
    Device& d = h->d;
    Ctx c;
    c.wslot0 = d.wslot0;
    c.scol = d.scol;
    c.val = d.val;
    c.dinv = d.dinv;
    c.scal = d.scal;
    c.part = d.part;
    c.tickets = d.tickets;
    c.ncta = d.ncta;
    c.cta_seg = d.cta_seg;
    c.cta_node0 = d.cta_node0;
    c.cta_node1 = d.cta_node1;
    c.seg_cta0 = d.seg_cta0;
    c.seg_solve = d.seg_solve;
    c.xrow = d.nxb > 0 ? d.xrow : nullptr;
    c.xcol = d.xcol;
    c.xval = d.xval;
    c.nn = d.nn;
    c.check = d.check;
    return c;
}

// Issues n iterations of `method` on the stream (no host interaction).
template <int U>
void issue_iterations_u(tf_handle* h, const Ctx& c, int method, int n) {
    Device& d = h->d;
    cudaStream_t st = h->stream;
    const int nb = d.ncta;
    const int jac = use_multigrid(h) ? 0 : 1;
    for (int it = 0; it < n; ++it) {
        if (method == 1) {
            launch_pdl(k_cg_spmv<U>, nb, kThreads, st, c, d.p, d.q);
            launch_pdl(k_cg_update, nb, kThreads, st, c, d.du, d.r, d.z, d.p, d.q, jac);
            if (!jac) {
                amg_vcycle(h, d.r, d.z);
                launch_pdl(k_cg_rz, nb, kThreads, st, c, d.r, d.z, d.p, 0);
            }
            launch_pdl(k_cg_direction, nb, kThreads, st, c, d.z, d.p);
        } else {
            launch_pdl(k_bi_dir, nb, kThreads, st, c, d.r, d.q, d.p, d.z, jac);
            if (!jac) amg_vcycle(h, d.p, d.z);
            launch_pdl(k_bi_spmv1<U>, nb, kThreads, st, c, d.z, d.rhat, d.q);
            launch_pdl(k_bi_s, nb, kThreads, st, c, d.r, d.q, d.s, d.sh, d.du, d.z, jac);
            if (!jac) amg_vcycle(h, d.s, d.sh);
            launch_pdl(k_bi_half, nb, kThreads, st, c, d.du, d.z);
            launch_pdl(k_bi_spmv2<U>, nb, kThreads, st, c, d.sh, d.s, d.t);
            launch_pdl(k_bi_x, nb, kThreads, st, c, d.du, d.r, d.rhat, d.z, d.sh, d.s, d.t);
        }
    }
}

void issue_iterations(tf_handle* h, const Ctx& c, int method, int n) {
    switch (h->spmv_unroll) {
        case 1: issue_iterations_u<1>(h, c, method, n); break;
        case 4: issue_iterations_u<4>(h, c, method, n); break;
        default: issue_iterations_u<2>(h, c, method, n); break;
    }
}

// y = A x alone (no dot, no flags): the SpMV variants the solve autotuner times
template <int U>
__global__ void k_spmv_probe(Ctx c, const double* __restrict__ x, double* __restrict__ y) {
    const Where w = where(c);
    if (!w.valid) return;
    double v[3];
    bsr_row<U>(c, w.node, x, v);
#pragma unroll
    for (int d = 0; d < 3; ++d) y[3 * w.node + d] = v[d];
}

// Picks the solve's kernel variants by timing them on the handle's own
// matrix, once per handle before its first solve builds any graph: the
// FP64 block SpMV with 1, 2 or 4 slots in flight per lane, and (multigrid)
// the level-0 smoother's row product with 2, 4 or 8.  Results do not depend
// on the choice (the same products in the same order).
tf_status autotune_solve(tf_handle* h) {
    if (h->solve_tuned) return TF_OK;
    h->solve_tuned = true;
    if (h->opt.autotune_off) return TF_OK;
    Device& d = h->d;
    const Ctx c = make_ctx(h);
    cudaStream_t st = h->stream;
    // every instance "running" while the variants are timed (the solver's
    // start writes all the scalars afterwards; nothing is kept across solves
    // before the first one)
    TF_CUDA(cudaMemsetAsync(d.scal, 0, sizeof(double) * (size_t)d.nseg * S_COUNT, st));
    float best = 1e30f;
    for (int u : {1, 2, 4}) {
        for (int r = 0; r < 4; ++r) {  // one warm-up, three timed
            if (r == 1) TF_CUDA(cudaEventRecord(h->ev[4], st));
            if (u == 1) k_spmv_probe<1><<<d.ncta, kThreads, 0, st>>>(c, d.du, d.q);
            else if (u == 2) k_spmv_probe<2><<<d.ncta, kThreads, 0, st>>>(c, d.du, d.q);
            else k_spmv_probe<4><<<d.ncta, kThreads, 0, st>>>(c, d.du, d.q);
            TF_LAUNCH_CHECK(h);
        }
        TF_CUDA(cudaEventRecord(h->ev[5], st));
        TF_CUDA(cudaEventSynchronize(h->ev[5]));
        float ms = 0.f;
        TF_CUDA(cudaEventElapsedTime(&ms, h->ev[4], h->ev[5]));
        if (ms < best) {
            best = ms;
            h->spmv_unroll = u;
        }
    }
    if (use_multigrid(h)) return amg_autotune(h);
    return TF_OK;
}

int kernels_per_iteration(const tf_handle* h, int method) {
    if (!use_multigrid(h)) return method == 1 ? 3 : 6;
    const int v = amg_vcycle_kernels(h);
    return method == 1 ? 4 + v : 6 + 2 * v;
}

constexpr int kChunk0 = 4;  // iterations of the smallest graph chunk
constexpr int kChunks = 5;  // chunks of 4, 8, 16, 32 and 64 iterations

// A chunk of `kChunk0 << ci` iterations, captured once into a CUDA graph.
tf_status run_chunk(tf_handle* h, const Ctx& c, int method, int ci) {
    const int n = kChunk0 << ci;
    cudaGraphExec_t& ex = h->graph[method - 1][ci];
    if (!ex) {
        cudaGraph_t g = nullptr;
        TF_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        issue_iterations(h, c, method, n);
        const cudaError_t e = cudaStreamEndCapture(h->stream, &g);
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
        const cudaError_t e2 = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        if (e2 != cudaSuccess) {
            ex = nullptr;
            return cuda_fail(e2, "cudaGraphInstantiate");
        }
        h->graph_kernels[method - 1][ci] = (int64_t)n * kernels_per_iteration(h, method);
    }
    TF_CUDA(cudaGraphLaunch(ex, h->stream));
    h->launches += h->graph_kernels[method - 1][ci];
    return TF_OK;
}

// Loop control of the device-side Krylov loop (one warp): counts the
// iteration and keeps the loop going while an instance is still running and
// the iteration cap is not reached, so the loop always ends.
__global__ void k_krylov_ctl(const double* __restrict__ scal, int nseg, int* __restrict__ ctl,
                             cudaGraphConditionalHandle loop) {
    bool running = false;
    for (int g = threadIdx.x; g < nseg; g += 32) running |= __ldcg(&scal[(size_t)g * S_COUNT + S_FLAG]) == F_RUNNING;
    running = __any_sync(0xffffffffu, running);
    if (threadIdx.x == 0) {
        const int it = ctl[0] + 1;
        ctl[0] = it;
        cudaGraphSetConditional(loop, (running && it < ctl[1]) ? 1u : 0u);
    }
}

// Resets the iteration count of a device-side Krylov loop (and, inside an
// enclosing loop, opens the Krylov loop's condition again).
__global__ void k_krylov_arm(int* __restrict__ ctl, int cap, cudaGraphConditionalHandle loop, int open) {
    ctl[0] = 0;
    ctl[1] = cap;
    if (open) cudaGraphSetConditional(loop, 1u);
}

// A whole solve's iterations as one graph: a conditional while node whose
// body is one iteration followed by k_krylov_ctl; no host round trip and no
// iteration past convergence.  Returns false when the graph cannot be built
// (the caller then runs host-checked chunks).
bool build_krylov_loop(tf_handle* h, const Ctx& c, int method) {
    cudaGraph_t g = nullptr;
    if (cudaGraphCreate(&g, 0) != cudaSuccess) return false;
    cudaGraphConditionalHandle hc = 0;
    bool ok = cudaGraphConditionalHandleCreate(&hc, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
    cudaGraphNodeParams p = {};
    cudaGraphNode_t node = nullptr;
    if (ok) {
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = hc;
        p.conditional.type = cudaGraphCondTypeWhile;
        p.conditional.size = 1;
        ok = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &p) == cudaSuccess;
    }
    if (ok) {
        cudaGraph_t body = p.conditional.phGraph_out[0];
        ok = cudaStreamBeginCaptureToGraph(h->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
             cudaSuccess;
        if (ok) {
            issue_iterations(h, c, method, 1);
            k_krylov_ctl<<<1, 32, 0, h->stream>>>(h->d.scal, h->d.nseg, h->kloop_ctl, hc);
            cudaGraph_t out = nullptr;
            ok = cudaStreamEndCapture(h->stream, &out) == cudaSuccess;
        }
    }
    if (ok) ok = cudaGraphInstantiate(&h->kloop[method - 1], g, 0) == cudaSuccess;
    cudaGraphDestroy(g);
    if (!ok) {
        h->kloop[method - 1] = nullptr;
        (void)cudaGetLastError();
    }
    return ok;
}

tf_status krylov_run(tf_handle* h, int method, int keep, int* iters, double* relres) {
    Device& d = h->d;
    const Ctx c = make_ctx(h);
    cudaStream_t st = h->stream;
    const double tol2 = h->opt.krylov_rtol * h->opt.krylov_rtol;
    const int jac = use_multigrid(h) ? 0 : 1;
    // The first solve of a time step starts from the previous step's first
    // update (the steps differ little: on the 320,000-prism sheet |du| of the
    // first Newton iteration changes by ~0.1 % from step to step); the stop
    // test stays relative to |g|, so the accuracy is that of a zero start.
    const double* x0 = (keep == 0 && h->newton_index == 0 && h->have_du0) ? h->du0 : nullptr;
    if (keep == 2) {  // BiCGStab restart: block inverse and x are kept
        k_bi_restart<<<d.ncta, kThreads, 0, st>>>(c, d.r, d.rhat, d.p, d.q);
    } else {
        const tf_status sb = launch_block_inverse(h);
        if (sb != TF_OK) return sb;
        if (use_multigrid(h)) {
            const tf_status sa = amg_numeric(h);
            if (sa != TF_OK) return sa;
        }
        {
            const tf_status su = autotune_solve(h);  // once per handle, before any graph captures the choice
            if (su != TF_OK) return su;
        }
        if (method == 1) {
            k_cg_init<<<d.ncta, kThreads, 0, st>>>(c, d.g, d.du, d.r, d.z, d.p, tol2, h->solve_atol, keep, jac, x0);
            if (!jac) {
                TF_LAUNCH_CHECK(h);
                amg_vcycle(h, d.r, d.z);
                h->launches += amg_vcycle_kernels(h);
                k_cg_rz<<<d.ncta, kThreads, 0, st>>>(c, d.r, d.z, d.p, 1);
            }
        } else {
            k_bi_init<<<d.ncta, kThreads, 0, st>>>(c, d.g, d.du, d.r, d.rhat, d.p, d.q, tol2, h->solve_atol, keep, x0);
        }
    }
    TF_LAUNCH_CHECK(h);
    const int maxit = h->opt.krylov_max_iter;
    const size_t nscal = (size_t)d.nseg * S_COUNT;
    // Iterations run in graph chunks of 4/8/16/32/64 with a flag check after
    // each batch.  The solve of a step's k-th Newton iteration needs about as
    // many iterations as the k-th one of the previous step (later Newton
    // iterations, solved to an absolute update accuracy, need far fewer than
    // the first), so the first batch covers 7/8 of that count (largest chunks
    // first, no check in between) and the rest goes in chunks of 4: at most 4
    // iterations run past convergence.  Outside a Newton step the previous
    // solve's count is used; without a previous count the chunks double from 8.
    const int slot = h->newton_index >= 0 ? std::min(h->newton_index, 7) : -1;
    const int prev = slot >= 0 ? h->plan_iters[method - 1][slot] : h->last_iters[method - 1];
    int launched = 0, ci = 1;
    int planned = (keep == 0) ? (prev * 7) / 8 : 0;
    bool done = false, fixed = planned > 0;
    if (h->opt.host_loops) h->kloop_off = true;
    if (!h->kloop_off && !h->kloop_ctl) {
        TF_CUDA(cudaMalloc(&h->kloop_ctl, 2 * sizeof(int)));
        TF_CUDA(cudaMallocHost(&h->kloop_host, sizeof(int)));
    }
    if (!h->kloop_off && !h->kloop[method - 1] && !build_krylov_loop(h, c, method)) h->kloop_off = true;
    if (!h->kloop_off) {
        // the device-side loop: every iteration until convergence (or the cap)
        k_krylov_arm<<<1, 1, 0, st>>>(h->kloop_ctl, maxit, 0, 0);
        TF_LAUNCH_CHECK(h);
        TF_CUDA(cudaGraphLaunch(h->kloop[method - 1], st));
        TF_CUDA(cudaMemcpyAsync(h->kloop_host, h->kloop_ctl, sizeof(int), cudaMemcpyDeviceToHost, st));
        TF_CUDA(cudaMemcpyAsync(d.host_scal, d.scal, sizeof(double) * nscal, cudaMemcpyDeviceToHost, st));
        TF_CUDA(cudaStreamSynchronize(st));
        launched = *h->kloop_host;
        h->launches += (int64_t)launched * (kernels_per_iteration(h, method) + 1);
        done = true;
    }
    while (launched < maxit && !done) {
        int target = planned > 0 ? planned : (fixed ? kChunk0 : (kChunk0 << ci));
        planned = 0;
        target = std::min(target, maxit - launched);
        int issued = 0;
        for (int cj = kChunks - 1; cj >= 0 && issued < target; --cj)
            while (target - issued >= (kChunk0 << cj)) {
                const tf_status s = run_chunk(h, c, method, cj);
                if (s != TF_OK) return s;
                issued += kChunk0 << cj;
            }
        if (issued < target) {  // fewer than 4 left before maxit or in the plan
            const int rest = target - issued;
            issue_iterations(h, c, method, rest);
            TF_LAUNCH_CHECK(h);
            h->launches += (int64_t)rest * kernels_per_iteration(h, method) - 1;
            issued = target;
        }
        launched += issued;
        TF_CUDA(cudaMemcpyAsync(d.host_scal, d.scal, sizeof(double) * nscal, cudaMemcpyDeviceToHost, st));
        TF_CUDA(cudaStreamSynchronize(st));
        done = true;
        for (int g = 0; g < d.nseg && done; ++g)
            if (d.host_scal[(size_t)g * S_COUNT + S_FLAG] == F_RUNNING) done = false;
        if (ci < kChunks - 1) ++ci;
    }
    int worst = F_CONVERGED, itmax = 0, bad = -1, bad_it = 0, why = 0;
    double rmax = 0.0, bad_rel = 0.0;
    for (int g = 0; g < d.nseg; ++g) {
        const double* s = d.host_scal + (size_t)g * S_COUNT;
        const int f = static_cast<int>(s[S_FLAG]);
        if ((f == F_BREAKDOWN || f == F_NAN) && bad < 0) {
            bad = g;
            bad_it = static_cast<int>(s[S_ITER]);
            why = static_cast<int>(s[S_WHY]);
            bad_rel = s[S_BB] > 0.0 ? std::sqrt(s[S_RR] / s[S_BB]) : 0.0;
        }
        itmax = std::max(itmax, static_cast<int>(s[S_ITER]));
        if (s[S_BB] > 0.0) rmax = std::max(rmax, std::sqrt(s[S_RR] / s[S_BB]));
        if (f == F_NAN) worst = F_NAN;
        else if (f == F_BREAKDOWN && worst != F_NAN) worst = F_BREAKDOWN;
        else if (f == F_RUNNING && worst == F_CONVERGED) worst = F_RUNNING;
    }
    *iters = itmax;
    *relres = rmax;
    if (keep == 0) {
        h->last_iters[method - 1] = itmax;
        if (slot >= 0) h->plan_iters[method - 1][slot] = itmax;
    }
    if (worst == F_CONVERGED) return TF_OK;
    char rel[32];
    std::snprintf(rel, sizeof(rel), "%.3g", bad_rel);
    const std::string where = " (instance " + std::to_string(bad) + ", iteration " + std::to_string(bad_it) +
                              (method == 1 ? ", CG, " : ", BiCGStab, ") + kWhy[why < 0 || why > 5 ? 0 : why] +
                              ", relative residual " + rel + ")";
    if (worst == F_NAN) {
        set_error("non-finite value in the linear solve" + where);
        return TF_NAN_DETECTED;
    }
    if (worst == F_BREAKDOWN) {
        set_error("Krylov breakdown" + where);
        return TF_KRYLOV_BREAKDOWN;
    }
    set_error("linear solve reached its iteration cap");
    return TF_KRYLOV_NOT_CONVERGED;
}

}  // namespace

// Auto mode picks CG when the tangent is symmetric; CG needs a positive
// definite operator, which large compressive growth can take away (the
// geometric stiffness term), so the instances whose CG breaks down are solved
// again with BiCGStab -- the others keep their CG result -- as the
// reference's direct LU would not care.
tf_status krylov_solve(tf_handle* h, int* iters, double* relres) {
    Device& d = h->d;
    TF_CUDA(cudaMemcpyAsync(d.seg_solve, d.seg_active, sizeof(int) * (size_t)d.nseg, cudaMemcpyDeviceToDevice,
                            h->stream));
    tf_status s = krylov_run(h, h->method, 0, iters, relres);
    if (s != TF_OK && use_multigrid(h) && amg_reused(h)) {
        // the coarse levels came from an earlier Newton iteration: rebuild
        // them for this matrix and solve again
        amg_mark_stale(h, 2);
        TF_CUDA(cudaMemcpyAsync(d.seg_solve, d.seg_active, sizeof(int) * (size_t)d.nseg, cudaMemcpyDeviceToDevice,
                                h->stream));
        int it2 = 0;
        s = krylov_run(h, h->method, 0, &it2, relres);
        *iters += it2;
    }
    if (s == TF_KRYLOV_BREAKDOWN && h->method == 1 && h->opt.krylov_method == 0) {
        std::vector<int> redo(d.nseg, 0);
        for (int g = 0; g < d.nseg; ++g)
            redo[g] = d.host_scal[(size_t)g * S_COUNT + S_FLAG] == F_BREAKDOWN ? 1 : 0;
        TF_CUDA(cudaMemcpyAsync(d.seg_solve, redo.data(), sizeof(int) * (size_t)d.nseg, cudaMemcpyHostToDevice,
                                h->stream));
        int it2 = 0;
        s = krylov_run(h, 2, 1, &it2, relres);
        *iters += it2;
    }
    // BiCGStab breakdowns: restart the instances concerned from their
    // current iterate with a fresh shadow residual
    const bool bicg = h->method == 2 || h->opt.krylov_method == 0;
    for (int restart = 0; restart < 3 && s == TF_KRYLOV_BREAKDOWN && bicg; ++restart) {
        std::vector<int> redo(d.nseg, 0);
        for (int g = 0; g < d.nseg; ++g)
            redo[g] = d.host_scal[(size_t)g * S_COUNT + S_FLAG] == F_BREAKDOWN ? 1 : 0;
        TF_CUDA(cudaMemcpyAsync(d.seg_solve, redo.data(), sizeof(int) * (size_t)d.nseg, cudaMemcpyHostToDevice,
                                h->stream));
        int it2 = 0;
        s = krylov_run(h, 2, 2, &it2, relres);
        *iters += it2;
    }
    return s;
}

tf_status launch_update(tf_handle* h) {
    Device& d = h->d;
    const Ctx c = make_ctx(h);
    k_update<true><<<d.ncta, kThreads, 0, h->stream>>>(c, d.uk, d.du);
    TF_LAUNCH_CHECK(h);
    return TF_OK;
}

tf_status launch_update_norm(tf_handle* h) {
    Device& d = h->d;
    const Ctx c = make_ctx(h);
    k_update<false><<<d.ncta, kThreads, 0, h->stream>>>(c, d.uk, d.du);
    TF_LAUNCH_CHECK(h);
    return TF_OK;
}

// ---- the Newton loop on the device -----------------------------------------
// Iterations 2, 3, ... of a time step (the first, with the multigrid rebuild
// and any retries, runs host-driven) as one graph: a conditional while node
// whose body is a whole Newton iteration -- assembly, the level-0 refresh of
// the multigrid, the Krylov solve as a nested while node, |du|, the Newton
// test of every instance (k_newton_ctl) and the update -- so a step needs one
// host wait after its first iteration.  Anything the device does not decide
// (a solve that did not converge, a non-finite update, a loosened solve whose
// |du| lands near newton_tol) stops the loop before the update is applied and
// hands the iteration back to the host path.

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__global__ void k_stamp_begin(NewtonDev* nd) { nd->t0 = global_ns(); }
__global__ void k_stamp_end(NewtonDev* nd) { nd->t_asm += global_ns() - nd->t0; }

// The Newton test of every instance after a solve (one CTA): the reference's
// |du| <= tol (NewtonRaphsonSolver.cpp:727-752) and the iteration cap, the
// instance mask of the next iteration, and the loop condition.
__global__ void __launch_bounds__(256) k_newton_ctl(const double* __restrict__ scal, int nseg,
                                                    int* __restrict__ active, int* __restrict__ it,
                                                    int* __restrict__ cv, int* __restrict__ capped, NewtonDev* nd,
                                                    double tol, double rtol2, int max_iter, double atol,
                                                    cudaGraphConditionalHandle loop) {
    __shared__ int exc, any;
    __shared__ double dmax;
    __shared__ int kmax;
    if (threadIdx.x == 0) {
        exc = 0;
        any = 0;
        dmax = 0.0;
        kmax = 0;
    }
    __syncthreads();
    for (int g = threadIdx.x; g < nseg; g += blockDim.x) {
        if (!active[g]) continue;
        const double* s = scal + (size_t)g * S_COUNT;
        const double dn = sqrt(__ldcg(&s[S_DU2]));
        const bool near = atol > 0.0 && __ldcg(&s[S_TOL2]) > rtol2 && near_newton_tol(dn, tol, atol);
        // reason: 1 a loosened solve near newton_tol, 2 a solve that did not
        // converge (flag 2 + the solver's flag), 3 a non-finite update
        const double fl = __ldcg(&s[S_FLAG]);
        const int why = !isfinite(dn) ? 3 : (fl != F_CONVERGED ? 2 : (near ? 1 : 0));
        if (why) atomicMax(&exc, why == 2 ? 10 + (int)fl : why);
        atomicMax(&kmax, (int)__ldcg(&s[S_ITER]));
    }
    __syncthreads();
    if (exc) {
        if (threadIdx.x == 0) {
            nd->krylov_total += kmax;  // the handed-back iteration's solve ran too
            nd->krylov_max = max(nd->krylov_max, kmax);
            nd->exc = exc;
            cudaGraphSetConditional(loop, 0u);
        }
        return;
    }
    for (int g = threadIdx.x; g < nseg; g += blockDim.x) {
        if (!active[g]) continue;
        const double* s = scal + (size_t)g * S_COUNT;
        const double dn = sqrt(__ldcg(&s[S_DU2]));
        // dn >= 0: the bit patterns of non-negative doubles order like the values
        atomicMax(reinterpret_cast<unsigned long long*>(&dmax), (unsigned long long)__double_as_longlong(dn));
        it[g] += 1;
        if (!(dn > tol)) {
            cv[g] = 1;
            active[g] = 0;
        } else if (it[g] > max_iter) {
            capped[g] = 1;
            active[g] = 0;
        } else {
            any = 1;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int k = nd->k;
        if (k < 32) nd->dunorm[k] = dmax;
        nd->k = k + 1;
        nd->krylov_total += kmax;
        nd->krylov_max = max(nd->krylov_max, kmax);
        cudaGraphSetConditional(loop, any ? 1u : 0u);
    }
}

namespace {

// A conditional handle of the graph being captured on h->stream (its value is
// set by a kernel before the node that uses it: nothing resets it when an
// enclosing loop runs the node again).
bool capture_handle(tf_handle* h, cudaGraphConditionalHandle* hc) {
    cudaStreamCaptureStatus stat;
    cudaGraph_t g = nullptr;
    if (cudaStreamGetCaptureInfo(h->stream, &stat, nullptr, &g, nullptr, nullptr, nullptr) != cudaSuccess ||
        stat != cudaStreamCaptureStatusActive)
        return false;
    return cudaGraphConditionalHandleCreate(hc, g, 0, 0) == cudaSuccess;
}

// Adds a while node on handle hc to the graph being captured on h->stream and
// captures its body (one call of `body` on h->stream, swapped for the capture
// stream); later work captured on h->stream follows the node.
template <class Body>
bool capture_while(tf_handle* h, cudaGraphConditionalHandle hc, Body body) {
    cudaStreamCaptureStatus stat;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    const cudaGraphEdgeData* edges = nullptr;
    size_t ndeps = 0;
    if (cudaStreamGetCaptureInfo(h->stream, &stat, nullptr, &g, &deps, &edges, &ndeps) != cudaSuccess ||
        stat != cudaStreamCaptureStatusActive)
        return false;
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = hc;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    if (cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &p) != cudaSuccess) return false;
    if (cudaStreamUpdateCaptureDependencies(h->stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies) !=
        cudaSuccess)
        return false;
    cudaGraph_t bg = p.conditional.phGraph_out[0];
    if (cudaStreamBeginCaptureToGraph(h->cap_stream, bg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) !=
        cudaSuccess)
        return false;
    std::swap(h->stream, h->cap_stream);
    body();
    std::swap(h->stream, h->cap_stream);
    cudaGraph_t out = nullptr;
    return cudaStreamEndCapture(h->cap_stream, &out) == cudaSuccess;
}

// One Newton iteration on h->stream (being captured): see above.
bool issue_newton_iteration(tf_handle* h, cudaGraphConditionalHandle newton) {
    Device& d = h->d;
    const Ctx c = make_ctx(h);
    cudaStream_t st = h->stream;
    const int method = h->method;
    const bool mg = use_multigrid(h);
    k_stamp_begin<<<1, 1, 0, st>>>(h->nd);
    if (launch_prepare(h) != TF_OK || launch_element(h) != TF_OK) return false;
    if (h->opt.deterministic && launch_deterministic_gather(h) != TF_OK) return false;
    k_stamp_end<<<1, 1, 0, st>>>(h->nd);
    if (cudaMemcpyAsync(d.seg_solve, d.seg_active, sizeof(int) * (size_t)d.nseg, cudaMemcpyDeviceToDevice, st) !=
        cudaSuccess)
        return false;
    if (launch_block_inverse(h) != TF_OK) return false;
    if (mg) amg_refresh(h);
    const double tol2 = h->opt.krylov_rtol * h->opt.krylov_rtol;
    const int jac = mg ? 0 : 1;
    if (method == 1) {
        k_cg_init<<<d.ncta, kThreads, 0, st>>>(c, d.g, d.du, d.r, d.z, d.p, tol2, h->opt.update_atol, 0, jac,
                                                nullptr);
        if (mg) {
            amg_vcycle(h, d.r, d.z);
            k_cg_rz<<<d.ncta, kThreads, 0, st>>>(c, d.r, d.z, d.p, 1);
        }
    } else {
        k_bi_init<<<d.ncta, kThreads, 0, st>>>(c, d.g, d.du, d.r, d.rhat, d.p, d.q, tol2, h->opt.update_atol, 0,
                                                nullptr);
    }
    cudaGraphConditionalHandle kc = 0;
    if (!capture_handle(h, &kc)) return false;
    k_krylov_arm<<<1, 1, 0, st>>>(h->kloop_ctl, h->opt.krylov_max_iter, kc, 1);
    bool ok = capture_while(h, kc, [&] {
        issue_iterations(h, c, method, 1);
        k_krylov_ctl<<<1, 32, 0, h->stream>>>(d.scal, d.nseg, h->kloop_ctl, kc);
    });
    if (!ok) return false;
    k_update<false><<<d.ncta, kThreads, 0, st>>>(c, d.uk, d.du);
    int* seg = h->nd_seg;
    k_newton_ctl<<<1, 256, 0, st>>>(d.scal, d.nseg, d.seg_active, seg, seg + d.nseg, seg + 2 * d.nseg, h->nd,
                                     h->opt.newton_tol, tol2, h->opt.newton_max_iter, h->opt.update_atol, newton);
    k_update<true><<<d.ncta, kThreads, 0, st>>>(c, d.uk, d.du, &h->nd->exc);
    return cudaGetLastError() == cudaSuccess;
}

bool build_newton_loop(tf_handle* h) {
    cudaGraph_t g = nullptr;
    if (cudaGraphCreate(&g, 0) != cudaSuccess) return false;
    cudaGraphConditionalHandle hc = 0;
    bool ok = cudaGraphConditionalHandleCreate(&hc, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
    cudaGraphNodeParams p = {};
    cudaGraphNode_t node = nullptr;
    if (ok) {
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = hc;
        p.conditional.type = cudaGraphCondTypeWhile;
        p.conditional.size = 1;
        ok = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &p) == cudaSuccess;
    }
    if (ok) {
        ok = cudaStreamBeginCaptureToGraph(h->stream, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (ok) {
            const int64_t l0 = h->launches;
            ok = issue_newton_iteration(h, hc);
            h->launches = l0;
            // kernels of one iteration outside the Krylov loop: two time
            // stamps, prepare, element (+2 order-fixed gathers), block
            // inverse, the multigrid refresh (3), the solver's start (CG with
            // multigrid: init, a V-cycle, rz), the loop arm, |du|, the Newton
            // test and the update
            const bool mg = use_multigrid(h);
            h->nloop_kernels = 2 + 2 + (h->opt.deterministic ? 2 : 0) + 1 + (mg ? 3 : 0) +
                               (h->method == 1 && mg ? 2 + amg_vcycle_kernels(h) : 1) + 1 + 3;
            cudaGraph_t out = nullptr;
            ok = (cudaStreamEndCapture(h->stream, &out) == cudaSuccess) && ok;
        }
    }
    if (ok) ok = cudaGraphInstantiate(&h->nloop, g, 0) == cudaSuccess;
    cudaGraphDestroy(g);
    if (!ok) {
        h->nloop = nullptr;
        (void)cudaGetLastError();
    }
    return ok;
}

}  // namespace

tf_status newton_device_loop(tf_handle* h, int* it, int* cv, int* capped, int* k, tf_step_stats* st, float* ms_asm,
                             bool* ran, bool* exc) {
    Device& d = h->d;
    *ran = false;
    *exc = false;
    // the device loop covers the plain path: no packing, no bound DOFs, no
    // checked build (those keep host work between the iterations)
#ifdef TF_CHECKED
    return TF_OK;
#endif
    if (h->nloop_off || h->pk || !h->bind_slave.empty() || h->kloop_off || h->opt.host_loops) return TF_OK;
    if (!h->kloop_ctl) {
        TF_CUDA(cudaMalloc(&h->kloop_ctl, 2 * sizeof(int)));
        TF_CUDA(cudaMallocHost(&h->kloop_host, sizeof(int)));
    }
    if (!h->nd) {
        TF_CUDA(cudaMalloc(&h->nd, sizeof(NewtonDev)));
        TF_CUDA(cudaMallocHost(&h->nd_host, sizeof(NewtonDev)));
        TF_CUDA(cudaMalloc(&h->nd_seg, 3 * sizeof(int) * (size_t)d.nseg));
        TF_CUDA(cudaMallocHost(&h->nd_seg_host, 3 * sizeof(int) * (size_t)d.nseg));
    }
    if (!h->cap_stream) TF_CUDA(cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking));
    if (h->nloop && h->nloop_dt != h->dt) {
        cudaGraphExecDestroy(h->nloop);
        h->nloop = nullptr;
    }
    if (!h->nloop) {
        if (!build_newton_loop(h)) {
            h->nloop_off = true;
            return TF_OK;
        }
        h->nloop_dt = h->dt;
    }
    // state in: the host's per-instance bookkeeping and mask
    NewtonDev& nh = *h->nd_host;
    std::memset(&nh, 0, sizeof(NewtonDev));
    nh.k = *k;
    int* sh = h->nd_seg_host;
    for (int g = 0; g < d.nseg; ++g) {
        sh[g] = it[g];
        sh[d.nseg + g] = cv[g];
        sh[2 * d.nseg + g] = capped[g];
    }
    TF_CUDA(cudaMemcpyAsync(h->nd, h->nd_host, sizeof(NewtonDev), cudaMemcpyHostToDevice, h->stream));
    TF_CUDA(cudaMemcpyAsync(h->nd_seg, sh, 3 * sizeof(int) * (size_t)d.nseg, cudaMemcpyHostToDevice, h->stream));
    TF_CUDA(cudaMemcpyAsync(d.seg_active, h->h_active.data(), sizeof(int) * (size_t)d.nseg, cudaMemcpyHostToDevice,
                            h->stream));
    TF_CUDA(cudaGraphLaunch(h->nloop, h->stream));
    TF_CUDA(cudaMemcpyAsync(h->nd_host, h->nd, sizeof(NewtonDev), cudaMemcpyDeviceToHost, h->stream));
    TF_CUDA(cudaMemcpyAsync(sh, h->nd_seg, 3 * sizeof(int) * (size_t)d.nseg, cudaMemcpyDeviceToHost, h->stream));
    TF_CUDA(cudaMemcpyAsync(h->h_active.data(), d.seg_active, sizeof(int) * (size_t)d.nseg, cudaMemcpyDeviceToHost,
                            h->stream));
    TF_CUDA(cudaStreamSynchronize(h->stream));
    // state out
    *ran = true;
    *exc = nh.exc != 0;
    st->device_handback = nh.exc;
    for (int g = 0; g < d.nseg; ++g) {
        it[g] = sh[g];
        cv[g] = sh[d.nseg + g];
        capped[g] = sh[2 * d.nseg + g];
    }
    for (int j = *k; j < std::min(nh.k, 32); ++j) st->dunorm[j] = nh.dunorm[j];
    const int done = nh.k - *k;
    *k = nh.k;
    st->device_iters += done;
    st->krylov_iters_total += nh.krylov_total;
    st->krylov_iters_max = std::max(st->krylov_iters_max, nh.krylov_max);
    *ms_asm += (float)(nh.t_asm * 1e-6);
    // kernels the graph ran: the fixed ones of each Newton iteration (an
    // iteration handed back ran all but the update) and one control kernel
    // more than the solver's own per Krylov iteration
    h->launches += (int64_t)(done + (*exc ? 1 : 0)) * h->nloop_kernels +
                   (int64_t)nh.krylov_total * (kernels_per_iteration(h, h->method) + 1);
    if (use_multigrid(h)) amg_refreshed(h);
    h->assembled = true;
    return TF_OK;
}

void destroy_graphs(tf_handle* h) {
    for (auto& row : h->graph)
        for (auto& g : row)
            if (g) {
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
    for (auto& g : h->kloop)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    if (h->nloop) {
        cudaGraphExecDestroy(h->nloop);
        h->nloop = nullptr;
    }
}

}  // namespace tf
