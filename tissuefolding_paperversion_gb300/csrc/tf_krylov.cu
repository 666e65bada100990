// FP64 Krylov solve of A du = g with A = K^T: the replacement for the
// reference's Pardiso phases 11/22/33 (NewtonRaphsonSolver.cpp:418-683,
// transposed solve iparm[11] = 1 at :639).
//
//   * block-Jacobi preconditioner on the 3x3 diagonal blocks;
//   * CG when every element has zero internal viscosity (A symmetric),
//     BiCGStab otherwise (the viscous tangent is not symmetric);
//   * all scalars stay on the device: each reduction kernel writes per-CTA
//     partial sums and the last CTA to finish (atomic ticket, no waiting)
//     folds them in a fixed order, so results are bitwise reproducible;
//   * the host checks convergence once per chunk of iterations; kernels of
//     a chunk that run after convergence or breakdown return immediately.
#include "tf_internal.cuh"

namespace tf {

namespace {

constexpr int kThreads = 256;

enum Flag { F_RUNNING = 0, F_CONVERGED = 1, F_BREAKDOWN = 2, F_NAN = 3 };
enum Extra { S_ITER = 20, S_TOL2 = 21, S_RHAT_V = 22 };

struct Ctx {
    int nn;
    const int* __restrict__ rowptr;
    const int* __restrict__ colidx;
    const double* __restrict__ val;
    const double* __restrict__ dinv;
    double* scal;
    double* part;         // [3][gridDim.x]
    unsigned* counter;
};

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
}

// Writes this CTA's partial sums and returns true in the CTA that arrives
// last; that CTA then holds the fixed-order totals in `tot` (thread 0).
template <int NV>
__device__ bool reduce_grid(const Ctx& c, double (&v)[NV], double (&tot)[NV]) {
    __shared__ double sm[NV][kThreads / 32];
    __shared__ bool last;
    block_sum<NV>(v, sm);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) c.part[k * gridDim.x + blockIdx.x] = v[k];
        __threadfence();
        const unsigned ticket = atomicAdd(c.counter, 1u);
        last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        acc[k] = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += kThreads) acc[k] += __ldcg(&c.part[k * gridDim.x + b]);
    }
    __syncthreads();
    block_sum<NV>(acc, sm);
#pragma unroll
    for (int k = 0; k < NV; ++k) tot[k] = acc[k];
    if (threadIdx.x == 0) *c.counter = 0u;
    return true;
}

__device__ __forceinline__ bool stopped(const Ctx& c) { return __ldcg(&c.scal[S_FLAG]) != 0.0; }

__device__ __forceinline__ void apply_dinv(const double* __restrict__ D, const double r[3], double z[3]) {
    z[0] = fma(D[0], r[0], fma(D[1], r[1], D[2] * r[2]));
    z[1] = fma(D[3], r[0], fma(D[4], r[1], D[5] * r[2]));
    z[2] = fma(D[6], r[0], fma(D[7], r[1], D[8] * r[2]));
}

__device__ __forceinline__ void bsr_row(const Ctx& c, int i, const double* __restrict__ x, double y[3]) {
    double y0 = 0.0, y1 = 0.0, y2 = 0.0;
    const int b0 = c.rowptr[i], b1 = c.rowptr[i + 1];
    for (int b = b0; b < b1; ++b) {
        const int j = __ldg(&c.colidx[b]);
        const double* __restrict__ a = c.val + 9 * (size_t)b;
        const double x0 = x[3 * j], x1 = x[3 * j + 1], x2 = x[3 * j + 2];
        y0 = fma(a[0], x0, fma(a[1], x1, fma(a[2], x2, y0)));
        y1 = fma(a[3], x0, fma(a[4], x1, fma(a[5], x2, y1)));
        y2 = fma(a[6], x0, fma(a[7], x1, fma(a[8], x2, y2)));
    }
    y[0] = y0;
    y[1] = y1;
    y[2] = y2;
}

// ---- CG -------------------------------------------------------------------

// r = b, z = M^-1 r, p = z, x = 0;  rz = (r,z), bb = (b,b)
__global__ void k_cg_init(Ctx c, const double* __restrict__ b, double* __restrict__ x, double* __restrict__ r,
                          double* __restrict__ z, double* __restrict__ p) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    double v[2] = {0.0, 0.0};
    if (i < c.nn) {
        double rr[3], zz[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            rr[d] = b[3 * i + d];
            r[3 * i + d] = rr[d];
            x[3 * i + d] = 0.0;
        }
        apply_dinv(c.dinv + 9 * (size_t)i, rr, zz);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            z[3 * i + d] = zz[d];
            p[3 * i + d] = zz[d];
            v[0] = fma(rr[d], zz[d], v[0]);
            v[1] = fma(rr[d], rr[d], v[1]);
        }
    }
    double tot[2];
    if (reduce_grid<2>(c, v, tot) && threadIdx.x == 0) {
        c.scal[S_RZ] = tot[0];
        c.scal[S_BB] = tot[1];
        c.scal[S_RR] = tot[1];
        c.scal[S_RR0] = tot[1];
        c.scal[S_ITER] = 0.0;
        c.scal[S_FLAG] = (tot[1] == 0.0) ? F_CONVERGED : (isfinite(tot[1]) ? F_RUNNING : F_NAN);
    }
}

// q = A p; alpha = rz / (p, q)
__global__ void k_cg_spmv(Ctx c, const double* __restrict__ p, double* __restrict__ q) {
    if (stopped(c)) return;
    const int i = blockIdx.x * kThreads + threadIdx.x;
    double v[1] = {0.0};
    if (i < c.nn) {
        double y[3];
        bsr_row(c, i, p, y);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            q[3 * i + d] = y[d];
            v[0] = fma(p[3 * i + d], y[d], v[0]);
        }
    }
    double tot[1];
    if (reduce_grid<1>(c, v, tot) && threadIdx.x == 0) {
        const double pq = tot[0];
        if (!(pq > 0.0) || !isfinite(pq)) {
            c.scal[S_FLAG] = isfinite(pq) ? F_BREAKDOWN : F_NAN;
        } else {
            c.scal[S_PQ] = pq;
            c.scal[S_ALPHA] = c.scal[S_RZ] / pq;
        }
    }
}

// x += alpha p; r -= alpha q; z = M^-1 r;  beta = (r,z)_new / (r,z)
__global__ void k_cg_update(Ctx c, double* __restrict__ x, double* __restrict__ r, double* __restrict__ z,
                            const double* __restrict__ p, const double* __restrict__ q) {
    if (stopped(c)) return;
    const double alpha = __ldcg(&c.scal[S_ALPHA]);
    const int i = blockIdx.x * kThreads + threadIdx.x;
    double v[2] = {0.0, 0.0};
    if (i < c.nn) {
        double rr[3], zz[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int k = 3 * i + d;
            x[k] = fma(alpha, p[k], x[k]);
            rr[d] = fma(-alpha, q[k], r[k]);
            r[k] = rr[d];
        }
        apply_dinv(c.dinv + 9 * (size_t)i, rr, zz);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            z[3 * i + d] = zz[d];
            v[0] = fma(rr[d], zz[d], v[0]);
            v[1] = fma(rr[d], rr[d], v[1]);
        }
    }
    double tot[2];
    if (reduce_grid<2>(c, v, tot) && threadIdx.x == 0) {
        const double rz = tot[0], rr = tot[1];
        c.scal[S_BETA] = rz / c.scal[S_RZ];
        c.scal[S_RZ] = rz;
        c.scal[S_RR] = rr;
        c.scal[S_ITER] += 1.0;
        if (!isfinite(rr)) c.scal[S_FLAG] = F_NAN;
        else if (rr <= c.scal[S_TOL2] * c.scal[S_BB]) c.scal[S_FLAG] = F_CONVERGED;
        else if (!(rz > 0.0)) c.scal[S_FLAG] = F_BREAKDOWN;
    }
}

// p = z + beta p
__global__ void k_cg_direction(Ctx c, const double* __restrict__ z, double* __restrict__ p) {
    if (stopped(c)) return;
    const double beta = __ldcg(&c.scal[S_BETA]);
    const int k = blockIdx.x * kThreads + threadIdx.x;
    if (k < 3 * c.nn) p[k] = fma(beta, p[k], z[k]);
}

// ---- BiCGStab ---------------------------------------------------------------

// r = rhat = b, p = v = 0, x = 0; rho = (rhat, r)
__global__ void k_bi_init(Ctx c, const double* __restrict__ b, double* __restrict__ x, double* __restrict__ r,
                          double* __restrict__ rhat, double* __restrict__ p, double* __restrict__ v) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    double s[1] = {0.0};
    if (i < c.nn) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int k = 3 * i + d;
            const double bk = b[k];
            r[k] = bk;
            rhat[k] = bk;
            p[k] = 0.0;
            v[k] = 0.0;
            x[k] = 0.0;
            s[0] = fma(bk, bk, s[0]);
        }
    }
    double tot[1];
    if (reduce_grid<1>(c, s, tot) && threadIdx.x == 0) {
        c.scal[S_RHO] = tot[0];
        c.scal[S_BB] = tot[0];
        c.scal[S_RR] = tot[0];
        c.scal[S_RR0] = tot[0];
        c.scal[S_ALPHA] = 1.0;
        c.scal[S_OMEGA] = 1.0;
        c.scal[S_BETA] = 0.0;
        c.scal[S_ITER] = 0.0;
        c.scal[S_FLAG] = (tot[0] == 0.0) ? F_CONVERGED : (isfinite(tot[0]) ? F_RUNNING : F_NAN);
    }
}

// p = r + beta (p - omega v); phat = M^-1 p
__global__ void k_bi_dir(Ctx c, const double* __restrict__ r, const double* __restrict__ v, double* __restrict__ p,
                         double* __restrict__ phat) {
    if (stopped(c)) return;
    const double beta = __ldcg(&c.scal[S_BETA]), omega = __ldcg(&c.scal[S_OMEGA]);
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= c.nn) return;
    double pp[3], z[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int k = 3 * i + d;
        pp[d] = fma(beta, fma(-omega, v[k], p[k]), r[k]);
        p[k] = pp[d];
    }
    apply_dinv(c.dinv + 9 * (size_t)i, pp, z);
#pragma unroll
    for (int d = 0; d < 3; ++d) phat[3 * i + d] = z[d];
}

// v = A phat; alpha = rho / (rhat, v)
__global__ void k_bi_spmv1(Ctx c, const double* __restrict__ phat, const double* __restrict__ rhat,
                           double* __restrict__ v) {
    if (stopped(c)) return;
    const int i = blockIdx.x * kThreads + threadIdx.x;
    double s[1] = {0.0};
    if (i < c.nn) {
        double y[3];
        bsr_row(c, i, phat, y);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            v[3 * i + d] = y[d];
            s[0] = fma(rhat[3 * i + d], y[d], s[0]);
        }
    }
    double tot[1];
    if (reduce_grid<1>(c, s, tot) && threadIdx.x == 0) {
        const double rv = tot[0];
        if (rv == 0.0 || !isfinite(rv)) c.scal[S_FLAG] = isfinite(rv) ? F_BREAKDOWN : F_NAN;
        else c.scal[S_ALPHA] = c.scal[S_RHO] / rv;
    }
}

// s = r - alpha v; shat = M^-1 s
__global__ void k_bi_s(Ctx c, const double* __restrict__ r, const double* __restrict__ v, double* __restrict__ s,
                       double* __restrict__ shat) {
    if (stopped(c)) return;
    const double alpha = __ldcg(&c.scal[S_ALPHA]);
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= c.nn) return;
    double ss[3], z[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int k = 3 * i + d;
        ss[d] = fma(-alpha, v[k], r[k]);
        s[k] = ss[d];
    }
    apply_dinv(c.dinv + 9 * (size_t)i, ss, z);
#pragma unroll
    for (int d = 0; d < 3; ++d) shat[3 * i + d] = z[d];
}

// t = A shat; omega = (t, s) / (t, t)
__global__ void k_bi_spmv2(Ctx c, const double* __restrict__ shat, const double* __restrict__ s,
                           double* __restrict__ t) {
    if (stopped(c)) return;
    const int i = blockIdx.x * kThreads + threadIdx.x;
    double w[2] = {0.0, 0.0};
    if (i < c.nn) {
        double y[3];
        bsr_row(c, i, shat, y);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            t[3 * i + d] = y[d];
            w[0] = fma(y[d], s[3 * i + d], w[0]);
            w[1] = fma(y[d], y[d], w[1]);
        }
    }
    double tot[2];
    if (reduce_grid<2>(c, w, tot) && threadIdx.x == 0) {
        const double ts = tot[0], tt = tot[1];
        if (!isfinite(ts) || !isfinite(tt)) c.scal[S_FLAG] = F_NAN;
        else c.scal[S_OMEGA] = (tt > 0.0) ? ts / tt : 0.0;
    }
}

// x += alpha phat + omega shat; r = s - omega t; rho' = (rhat, r)
__global__ void k_bi_x(Ctx c, double* __restrict__ x, double* __restrict__ r, const double* __restrict__ rhat,
                       const double* __restrict__ phat, const double* __restrict__ shat, const double* __restrict__ s,
                       const double* __restrict__ t) {
    if (stopped(c)) return;
    const double alpha = __ldcg(&c.scal[S_ALPHA]), omega = __ldcg(&c.scal[S_OMEGA]);
    const int i = blockIdx.x * kThreads + threadIdx.x;
    double w[2] = {0.0, 0.0};
    if (i < c.nn) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int k = 3 * i + d;
            x[k] = fma(omega, shat[k], fma(alpha, phat[k], x[k]));
            const double rk = fma(-omega, t[k], s[k]);
            r[k] = rk;
            w[0] = fma(rhat[k], rk, w[0]);
            w[1] = fma(rk, rk, w[1]);
        }
    }
    double tot[2];
    if (reduce_grid<2>(c, w, tot) && threadIdx.x == 0) {
        const double rho = tot[0], rr = tot[1];
        const double omega_ = c.scal[S_OMEGA];
        c.scal[S_BETA] = (rho / c.scal[S_RHO]) * (c.scal[S_ALPHA] / omega_);
        c.scal[S_RHO] = rho;
        c.scal[S_RR] = rr;
        c.scal[S_ITER] += 1.0;
        if (!isfinite(rr)) c.scal[S_FLAG] = F_NAN;
        else if (rr <= c.scal[S_TOL2] * c.scal[S_BB]) c.scal[S_FLAG] = F_CONVERGED;
        else if (omega_ == 0.0 || rho == 0.0) c.scal[S_FLAG] = F_BREAKDOWN;
    }
}

// ---- Newton update ------------------------------------------------------------

// uk += du; |du|^2  (NewtonRaphsonSolver::updateUkInIteration :755-761,
// checkConvergenceViaDeltaU :727-740)
__global__ void k_update(Ctx c, double* __restrict__ uk, const double* __restrict__ du) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    double v[1] = {0.0};
    if (i < c.nn) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int k = 3 * i + d;
            const double dk = du[k];
            uk[k] = uk[k] + dk;
            v[0] = fma(dk, dk, v[0]);
        }
    }
    double tot[1];
    if (reduce_grid<1>(c, v, tot) && threadIdx.x == 0) c.scal[S_DU2] = tot[0];
}

Ctx make_ctx(tf_handle* h) {
    Device& d = h->d;
    Ctx c;
    c.nn = d.nn;
    c.rowptr = d.rowptr;
    c.colidx = d.colidx;
    c.val = d.val;
    c.dinv = d.dinv;
    c.scal = d.scal;
    c.part = d.part;
    c.counter = reinterpret_cast<unsigned*>(d.scal + S_COUNT);
    return c;
}

}  // namespace

namespace {
tf_status krylov_run(tf_handle* h, int method, int* iters, double* relres);
}

// Auto mode picks CG when the tangent is symmetric; CG needs a positive
// definite operator, which large compressive growth can take away (the
// geometric stiffness term), so a CG breakdown there falls back to
// BiCGStab, as the reference's direct LU would not care.
tf_status krylov_solve(tf_handle* h, int* iters, double* relres) {
    tf_status s = krylov_run(h, h->method, iters, relres);
    if (s == TF_KRYLOV_BREAKDOWN && h->method == 1 && h->opt.krylov_method == 0) {
        int it2 = 0;
        s = krylov_run(h, 2, &it2, relres);
        *iters += it2;
    }
    return s;
}

namespace {
tf_status krylov_run(tf_handle* h, int method, int* iters, double* relres) {
    Device& d = h->d;
    Ctx c = make_ctx(h);
    const int nb = cdiv(d.nn, kThreads);
    const int nbv = cdiv(3 * (int64_t)d.nn, kThreads);
    cudaStream_t st = h->stream;
    const tf_status sb = launch_block_inverse(h);
    if (sb != TF_OK) return sb;
    const double tol = h->opt.krylov_rtol;
    const double tol2 = tol * tol;
    TF_CUDA(cudaMemcpyAsync(d.scal + S_TOL2, &tol2, sizeof(double), cudaMemcpyHostToDevice, st));
    if (method == 1) {
        k_cg_init<<<nb, kThreads, 0, st>>>(c, d.g, d.du, d.r, d.z, d.p);
    } else {
        k_bi_init<<<nb, kThreads, 0, st>>>(c, d.g, d.du, d.r, d.rhat, d.p, d.q);
    }
    TF_LAUNCH_CHECK(h);
    const int maxit = h->opt.krylov_max_iter;
    int launched = 0, chunk = 8;
    double flag = 0.0;
    while (launched < maxit) {
        const int n = chunk < maxit - launched ? chunk : maxit - launched;
        for (int it = 0; it < n; ++it) {
            if (method == 1) {
                k_cg_spmv<<<nb, kThreads, 0, st>>>(c, d.p, d.q);
                TF_LAUNCH_CHECK(h);
                k_cg_update<<<nb, kThreads, 0, st>>>(c, d.du, d.r, d.z, d.p, d.q);
                TF_LAUNCH_CHECK(h);
                k_cg_direction<<<nbv, kThreads, 0, st>>>(c, d.z, d.p);
                TF_LAUNCH_CHECK(h);
            } else {
                k_bi_dir<<<nb, kThreads, 0, st>>>(c, d.r, d.q, d.p, d.z);
                TF_LAUNCH_CHECK(h);
                k_bi_spmv1<<<nb, kThreads, 0, st>>>(c, d.z, d.rhat, d.q);
                TF_LAUNCH_CHECK(h);
                k_bi_s<<<nb, kThreads, 0, st>>>(c, d.r, d.q, d.s, d.sh);
                TF_LAUNCH_CHECK(h);
                k_bi_spmv2<<<nb, kThreads, 0, st>>>(c, d.sh, d.s, d.t);
                TF_LAUNCH_CHECK(h);
                k_bi_x<<<nb, kThreads, 0, st>>>(c, d.du, d.r, d.rhat, d.z, d.sh, d.s, d.t);
                TF_LAUNCH_CHECK(h);
            }
        }
        launched += n;
        TF_CUDA(cudaMemcpyAsync(d.host_scal, d.scal, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, st));
        TF_CUDA(cudaStreamSynchronize(st));
        flag = d.host_scal[S_FLAG];
        if (flag != 0.0) break;
        if (chunk < 64) chunk *= 2;
    }
    const double bb = d.host_scal[S_BB], rr = d.host_scal[S_RR];
    *iters = static_cast<int>(d.host_scal[S_ITER]);
    *relres = bb > 0.0 ? sqrt(rr / bb) : 0.0;
    if (flag == F_CONVERGED) return TF_OK;
    if (flag == F_NAN) {
        set_error("non-finite value in the linear solve");
        return TF_NAN_DETECTED;
    }
    if (flag == F_BREAKDOWN) {
        set_error("Krylov breakdown");
        return TF_KRYLOV_BREAKDOWN;
    }
    set_error("linear solve reached its iteration cap");
    return TF_KRYLOV_NOT_CONVERGED;
}
}  // namespace

tf_status launch_update(tf_handle* h) {
    Device& d = h->d;
    Ctx c = make_ctx(h);
    k_update<<<cdiv(d.nn, kThreads), kThreads, 0, h->stream>>>(c, d.uk, d.du);
    TF_LAUNCH_CHECK(h);
    return TF_OK;
}

}  // namespace tf
