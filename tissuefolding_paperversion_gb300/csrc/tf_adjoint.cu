// Discrete adjoint of n implicit time steps, for gradients of a shape loss
// with respect to per-element in-plane growth rates and log Young's moduli.
// No counterpart in the reference.
//
// Forward (tf_adj_forward): from the handle's current positions with Fg = I,
// run n steps of updateStepNR with growth rates (r_e, r_e, 0) and
// E_e = exp(logE_e), storing the state every `every` steps; evaluate
//   L = sum over apical nodes (z - amp exp(-((x-cx)^2 + (y-cy)^2) / (2 w^2)))^2.
// Backward (tf_adj_backward): segments last to first; each segment is
// recomputed from its checkpoint, then for step n = N..1
//   A_n^T lambda_n = -dL/du_n [n = N] + (dg_{n+1}/du_n)^T lambda_{n+1}
// with A_n = -dg_n/du_n the assembled Jacobian (K^T of the reference), and
//   dL/dtheta = -sum_n lambda_n^T dg_n/dtheta
// contracted element by element (k_adjoint_element).  The step-to-step
// coupling (dg_{n+1}/du_n) is the velocity part of the viscous terms and the
// dependence of the external-viscosity surfaces on the step's start shape.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "tf_internal.cuh"

namespace tf {
namespace {

constexpr int kT = 256;

__global__ void k_set_material(int ne, const double* __restrict__ logE, const double* __restrict__ nu,
                               double* __restrict__ lam, double* __restrict__ mu) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const double E = exp(logE[e]);
    const double v = nu[e];
    lam[e] = E * v / (1 + v) / (1 - 2.0 * v);  // Prism::setElasticProperties, Prism.cpp:510-511
    mu[e] = E / 2.0 / (1 + v);
}

__global__ void k_set_rates(int ne, const double* __restrict__ r, double* __restrict__ rates) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    rates[e] = r[e];
    rates[ne + e] = r[e];
    rates[2 * ne + e] = 0.0;
}

__global__ void k_reset_Fg(int ne, double* __restrict__ Fg, double* __restrict__ invFg) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const double v = (k % 4 == 0) ? 1.0 : 0.0;
        Fg[k * ne + e] = v;
        invFg[k * ne + e] = v;
    }
}

// loss partials per CTA and dL/du (apical nodes only)
__global__ void k_loss(int nn, const double* __restrict__ x, const int* __restrict__ apical, double cx, double cy,
                       double amp, double w, double* __restrict__ dl, double* __restrict__ part) {
    __shared__ double sm[kT];
    const int i = blockIdx.x * kT + threadIdx.x;
    double l = 0.0;
    if (i < nn) {
        dl[3 * i] = dl[3 * i + 1] = dl[3 * i + 2] = 0.0;
        if (apical[i]) {
            const double dx = x[3 * i] - cx, dy = x[3 * i + 1] - cy;
            const double f = amp * exp(-(dx * dx + dy * dy) / (2.0 * w * w));
            const double res = x[3 * i + 2] - f;
            l = res * res;
            dl[3 * i] = 2.0 * res * f * dx / (w * w);
            dl[3 * i + 1] = 2.0 * res * f * dy / (w * w);
            dl[3 * i + 2] = 2.0 * res;
        }
    }
    sm[threadIdx.x] = l;
    __syncthreads();
    for (int s = kT / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}

// rhs = scale * src + carry, zero on fixed DOFs
__global__ void k_rhs(int n3, const double* __restrict__ src, double scale, const double* __restrict__ carry,
                      const uint8_t* __restrict__ fixed, double* __restrict__ rhs) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n3) return;
    const double v = (src ? scale * src[k] : 0.0) + carry[k];
    rhs[k] = fixed[k] ? 0.0 : v;
}

// transposed copy of the block values: blocks (i,j) <- (j,i)^T
__global__ void k_transpose_blocks(int64_t nnzb, const int* __restrict__ tblk, const int* __restrict__ bofs,
                                   const double* __restrict__ val, double* __restrict__ valT) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nnzb) return;
    const double* src = val + bofs[tblk[b]];
    double* dst = valT + bofs[b];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) dst[kSlice * (3 * i + k)] = src[kSlice * (3 * k + i)];
}

// node terms of the carry to step n-1: external viscosity
// g_i = -A_i eta_i (u_n - u_{n-1})_i / dt  gives  +A_i eta_i / dt lambda_i
__global__ void k_carry_nodes(int nn, const double* __restrict__ area, const double* __restrict__ ext_visc,
                              double idt, const double* __restrict__ lamv, double* __restrict__ carry) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int k = 3 * i + d;
        carry[k] += area[i] * ext_visc[k] * idt * lamv[k];
    }
}

// face terms of the carry: A_i depends on u_{n-1} through the exposed face
// areas (Prism.cpp:2424-2503); d g_i / d A_i = -eta_i v_i.
__device__ void face_carry(const double* __restrict__ xp, const double* __restrict__ xn, double idt,
                           const double* __restrict__ ext_visc, const double* __restrict__ lamv, int n0, int n1,
                           int n2, double* __restrict__ carry) {
    const int ids[3] = {n0, n1, n2};
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < 3; ++q)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int k = 3 * ids[q] + d;
            const double v = (xn[k] - xp[k]) * idt;
            s -= ext_visc[k] * v * lamv[k];
        }
    s /= 3.0;
    double e1[3], e2[3], nrm[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        e1[d] = xp[3 * n1 + d] - xp[3 * n0 + d];
        e2[d] = xp[3 * n2 + d] - xp[3 * n0 + d];
    }
    nrm[0] = e1[1] * e2[2] - e1[2] * e2[1];
    nrm[1] = e1[2] * e2[0] - e1[0] * e2[2];
    nrm[2] = e1[0] * e2[1] - e1[1] * e2[0];
    const double len = sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
    if (!(len > 0.0)) return;
    const double nh[3] = {nrm[0] / len, nrm[1] / len, nrm[2] / len};
    // d area / d p1 = 0.5 (e2 x nh), d area / d p2 = 0.5 (nh x e1), p0 = -(sum)
    double g1[3], g2[3];
    g1[0] = 0.5 * (e2[1] * nh[2] - e2[2] * nh[1]);
    g1[1] = 0.5 * (e2[2] * nh[0] - e2[0] * nh[2]);
    g1[2] = 0.5 * (e2[0] * nh[1] - e2[1] * nh[0]);
    g2[0] = 0.5 * (nh[1] * e1[2] - nh[2] * e1[1]);
    g2[1] = 0.5 * (nh[2] * e1[0] - nh[0] * e1[2]);
    g2[2] = 0.5 * (nh[0] * e1[1] - nh[1] * e1[0]);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        atomicAdd(&carry[3 * n0 + d], -s * (g1[d] + g2[d]));
        atomicAdd(&carry[3 * n1 + d], s * g1[d]);
        atomicAdd(&carry[3 * n2 + d], s * g2[d]);
    }
}

__global__ void k_carry_faces(int ne, const int* __restrict__ conn, const int* __restrict__ exposure,
                              const double* __restrict__ xp, const double* __restrict__ xn, double idt,
                              const double* __restrict__ ext_visc, const double* __restrict__ lamv,
                              double* __restrict__ carry) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int ex = exposure[e];
    if (ex & 1) face_carry(xp, xn, idt, ext_visc, lamv, conn[3 * ne + e], conn[4 * ne + e], conn[5 * ne + e], carry);
    if (ex & 2) face_carry(xp, xn, idt, ext_visc, lamv, conn[0 * ne + e], conn[1 * ne + e], conn[2 * ne + e], carry);
}

}  // namespace
}  // namespace tf

struct tf_adjoint {
    int n_steps = 0, every = 1;
    double dt = 0.0;
    double params[4] = {0, 0, 0, 0};
    double loss = 0.0;
    std::vector<double*> ck_u, ck_Fg, ck_iFg;  // states at steps 0, every, 2 every, ...
    double* final_u = nullptr;                 // state after the last step
    double* final_Fg = nullptr;
    double* final_iFg = nullptr;
    double* rate = nullptr;  // [E]
    double* logE = nullptr;  // [E]
    int device = 0;
};

using namespace tf;

namespace {

tf_status dalloc(double** p, size_t n) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(n, 1) * sizeof(double));
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("device allocation failed in the adjoint");
        return TF_OUT_OF_MEMORY;
    }
    return TF_OK;
}

#define TFA_TRY(expr)               \
    do {                            \
        tf_status _s = (expr);      \
        if (_s != TF_OK) return _s; \
    } while (0)

tf_status ialloc(int** p, size_t n) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(n, 1) * sizeof(int));
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("device allocation failed in the adjoint");
        return TF_OUT_OF_MEMORY;
    }
    return TF_OK;
}

tf_status ensure_adjoint_buffers(tf_handle* h) {
    Device& d = h->d;
    if (d.valT) return TF_OK;
    // the block pattern is structurally symmetric: (i,j) is present iff (j,i) is
    std::vector<int> tblk(d.nnzb);
    for (int i = 0; i < d.nn; ++i)
        for (int p = h->h_rowptr[i]; p < h->h_rowptr[i + 1]; ++p) {
            const int j = h->h_colidx[p];
            auto b = h->h_colidx.begin() + h->h_rowptr[j], en = h->h_colidx.begin() + h->h_rowptr[j + 1];
            tblk[p] = static_cast<int>(std::lower_bound(b, en, i) - h->h_colidx.begin());
        }
    const size_t n3 = 3 * (size_t)d.nn;
    TFA_TRY(ialloc(&d.tblk, d.nnzb));
    TFA_TRY(ialloc(&d.apical, d.nn));
    TFA_TRY(dalloc(&d.valT, (size_t)d.nval));
    TF_CUDA(cudaMemset(d.valT, 0, sizeof(double) * (size_t)d.nval));  // padding stays zero
    TFA_TRY(dalloc(&d.lamv, n3));
    TFA_TRY(dalloc(&d.carry, n3));
    TFA_TRY(dalloc(&d.dldu, n3));
    TFA_TRY(dalloc(&d.gr, d.ne));
    TFA_TRY(dalloc(&d.ge, d.ne));
    TFA_TRY(dalloc(&d.nu, d.ne));
    TF_CUDA(cudaMemcpy(d.tblk, tblk.data(), sizeof(int) * (size_t)d.nnzb, cudaMemcpyHostToDevice));
    TF_CUDA(cudaMemcpy(d.apical, h->h_apical.data(), sizeof(int) * (size_t)d.nn, cudaMemcpyHostToDevice));
    TF_CUDA(cudaMemcpy(d.nu, h->h_nu.data(), sizeof(double) * (size_t)d.ne, cudaMemcpyHostToDevice));
    return TF_OK;
}

tf_status loss_value(tf_handle* h, const double* params, double* loss) {
    Device& d = h->d;
    const int nb = cdiv(d.nn, kT);
    std::vector<double> part(nb);
    static_assert(kT == kNodeThreads, "one partial sum per node CTA");
    double* dpart = d.part;  // 3 * ncta doubles, ncta = nb for a single mesh
    k_loss<<<nb, kT, 0, h->stream>>>(d.nn, d.uk, d.apical, params[0], params[1], params[2], params[3], d.dldu, dpart);
    TF_LAUNCH_CHECK(h);
    TF_CUDA(cudaMemcpyAsync(part.data(), dpart, sizeof(double) * nb, cudaMemcpyDeviceToHost, h->stream));
    TF_CUDA(cudaStreamSynchronize(h->stream));
    double s = 0.0;
    for (double v : part) s += v;
    *loss = s;
    return TF_OK;
}

// Linear solve with the transposed block values, A^T lambda = rhs (rhs in
// g, lambda in du).  The values are transposed in place, so the captured
// Krylov graphs (which hold the value pointer) stay valid.
// Relative residual of the adjoint's transposed solves: their errors are
// carried through every earlier step of the backward pass (measured on the
// 320,000-prism sheet, 50 steps: gradients within 2e-5 of central
// differences at 1e-8, within 3e-7 at 1e-12-1e-13).
constexpr double kAdjointRtol = 1e-12;

tf_status solve_transposed(tf_handle* h, int* iters) {
    Device& d = h->d;
    k_transpose_blocks<<<cdiv(d.nnzb, kT), kT, 0, h->stream>>>(d.nnzb, d.tblk, d.bofs, d.val, d.valT);
    TF_LAUNCH_CHECK(h);
    TF_CUDA(cudaMemcpyAsync(d.val, d.valT, sizeof(double) * (size_t)d.nval, cudaMemcpyDeviceToDevice,
                            h->stream));
    amg_mark_stale(h, 2);  // the multigrid hierarchy follows the transposed matrix
    double rr = 0.0;
    const double rtol = h->opt.krylov_rtol;
    h->opt.krylov_rtol = std::min(rtol, kAdjointRtol);
    const tf_status s = krylov_solve(h, iters, &rr);
    h->opt.krylov_rtol = rtol;
    TFA_TRY(take_check(h));
    return s == TF_KRYLOV_NOT_CONVERGED ? TF_OK : s;
}

// Device buffers freed on scope exit.
struct Scratch {
    std::vector<void*> p;
    ~Scratch() {
        for (void* q : p) cudaFree(q);
    }
    tf_status get(double** out, size_t n) {
        TFA_TRY(dalloc(out, n));
        p.push_back(*out);
        return TF_OK;
    }
};

tf_status copy_state(tf_handle* h, double* u, double* F, double* iF, const double* su, const double* sF,
                     const double* siF) {
    const Device& d = h->d;
    const size_t n3 = 3 * (size_t)d.nn, n9 = 9 * (size_t)d.ne;
    TF_CUDA(cudaMemcpyAsync(u, su, n3 * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    TF_CUDA(cudaMemcpyAsync(F, sF, n9 * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    TF_CUDA(cudaMemcpyAsync(iF, siF, n9 * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    return TF_OK;
}

tf_status adj_forward(tf_handle* h, tf_adjoint* a, const double* rate, const double* logE) {
    NvtxRange nvtx_range("tf adjoint forward");
    Device& d = h->d;
    const int ne = d.ne;
    const size_t n3 = 3 * (size_t)d.nn, n9 = 9 * (size_t)ne;
    TFA_TRY(dalloc(&a->rate, ne));
    TFA_TRY(dalloc(&a->logE, ne));
    TFA_TRY(dalloc(&a->final_u, n3));
    TFA_TRY(dalloc(&a->final_Fg, n9));
    TFA_TRY(dalloc(&a->final_iFg, n9));
    TF_CUDA(cudaMemcpy(a->rate, rate, sizeof(double) * ne, cudaMemcpyHostToDevice));
    TF_CUDA(cudaMemcpy(a->logE, logE, sizeof(double) * ne, cudaMemcpyHostToDevice));
    k_set_material<<<cdiv(ne, kT), kT, 0, h->stream>>>(ne, a->logE, d.nu, d.lam, d.mu);
    TF_LAUNCH_CHECK(h);
    k_set_rates<<<cdiv(ne, kT), kT, 0, h->stream>>>(ne, a->rate, d.rates);
    TF_LAUNCH_CHECK(h);
    k_reset_Fg<<<cdiv(ne, kT), kT, 0, h->stream>>>(ne, d.Fg, d.invFg);
    TF_LAUNCH_CHECK(h);
    h->have_rates = true;
    tf_status status = TF_OK;
    for (int n = 0; n < a->n_steps; ++n) {
        if (n % a->every == 0) {
            a->ck_u.push_back(nullptr);
            a->ck_Fg.push_back(nullptr);
            a->ck_iFg.push_back(nullptr);
            TFA_TRY(dalloc(&a->ck_u.back(), n3));
            TFA_TRY(dalloc(&a->ck_Fg.back(), n9));
            TFA_TRY(dalloc(&a->ck_iFg.back(), n9));
            TFA_TRY(copy_state(h, a->ck_u.back(), a->ck_Fg.back(), a->ck_iFg.back(), d.uk, d.Fg, d.invFg));
        }
        tf_step_stats st;
        const tf_status s = tf_newton_step(h, a->dt, &st);
        if (s != TF_OK && s != TF_NOT_CONVERGED) return s;
        if (s == TF_NOT_CONVERGED) status = s;
    }
    TFA_TRY(copy_state(h, a->final_u, a->final_Fg, a->final_iFg, d.uk, d.Fg, d.invFg));
    TFA_TRY(loss_value(h, a->params, &a->loss));
    return status;
}

tf_status adj_backward(tf_handle* h, tf_adjoint* a, double dloss, double* grad_rate, double* grad_logE) {
    NvtxRange nvtx_range("tf adjoint backward");
    Device& d = h->d;
    const int ne = d.ne;
    const size_t n3 = 3 * (size_t)d.nn, n9 = 9 * (size_t)ne;
    const int N = a->n_steps, every = a->every;
    cudaStream_t st = h->stream;
    h->dt = a->dt;
    // dL/du at the final state
    TF_CUDA(cudaMemcpyAsync(d.uk, a->final_u, n3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
    double lossv = 0.0;
    TFA_TRY(loss_value(h, a->params, &lossv));
    TF_CUDA(cudaMemsetAsync(d.carry, 0, n3 * sizeof(double), st));
    TF_CUDA(cudaMemsetAsync(d.gr, 0, ne * sizeof(double), st));
    TF_CUDA(cudaMemsetAsync(d.ge, 0, ne * sizeof(double), st));
    k_set_material<<<cdiv(ne, kT), kT, 0, st>>>(ne, a->logE, d.nu, d.lam, d.mu);
    TF_LAUNCH_CHECK(h);
    k_set_rates<<<cdiv(ne, kT), kT, 0, st>>>(ne, a->rate, d.rates);
    TF_LAUNCH_CHECK(h);
    h->have_rates = true;
    // states of one span: su[k] = u_{n0+k}, sF/siF[k] = Fg after the growth of step n0+k
    Scratch sc;
    std::vector<double*> su(every + 1), sF(every + 1), siF(every + 1);
    for (int k = 0; k <= every; ++k) {
        TFA_TRY(sc.get(&su[k], n3));
        TFA_TRY(sc.get(&sF[k], n9));
        TFA_TRY(sc.get(&siF[k], n9));
    }
    const int nspan = (N + every - 1) / every;
    for (int s = nspan - 1; s >= 0; --s) {
        const int n0 = s * every, n1 = std::min(N, n0 + every);
        // recompute steps n0+1 .. n1-1 from the saved state; u_{n1} is saved
        TFA_TRY(copy_state(h, d.uk, d.Fg, d.invFg, a->ck_u[s], a->ck_Fg[s], a->ck_iFg[s]));
        TFA_TRY(copy_state(h, su[0], sF[0], siF[0], a->ck_u[s], a->ck_Fg[s], a->ck_iFg[s]));
        for (int n = n0 + 1; n < n1; ++n) {
            tf_step_stats ss;
            const tf_status t = tf_newton_step(h, a->dt, &ss);
            if (t != TF_OK && t != TF_NOT_CONVERGED) return t;
            const int k = n - n0;
            TFA_TRY(copy_state(h, su[k], sF[k], siF[k], d.uk, d.Fg, d.invFg));
        }
        if (s + 1 < nspan)
            TFA_TRY(copy_state(h, su[n1 - n0], sF[n1 - n0], siF[n1 - n0], a->ck_u[s + 1], a->ck_Fg[s + 1],
                               a->ck_iFg[s + 1]));
        else
            TFA_TRY(copy_state(h, su[n1 - n0], sF[n1 - n0], siF[n1 - n0], a->final_u, a->final_Fg, a->final_iFg));
        for (int n = n1; n > n0; --n) {
            const int k = n - n0;
            // step n: viscosity surfaces from the start shape u_{n-1}, then
            // the Jacobian at u_n with velocity (u_n - u_{n-1}) / dt
            TF_CUDA(cudaMemcpyAsync(d.uk, su[k - 1], n3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
            TFA_TRY(launch_viscosity_surfaces(h));
            TF_CUDA(cudaMemcpyAsync(d.un, su[k - 1], n3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
            TFA_TRY(copy_state(h, d.uk, d.Fg, d.invFg, su[k], sF[k], siF[k]));
            TFA_TRY(tf_assemble(h));
            // rhs = -dloss dL/du_N (last step only) + carry from step n+1
            k_rhs<<<cdiv((int64_t)n3, kT), kT, 0, st>>>((int)n3, n == N ? d.dldu : nullptr, -dloss, d.carry,
                                                         d.fixed, d.g);
            TF_LAUNCH_CHECK(h);
            int it = 0;
            TFA_TRY(solve_transposed(h, &it));
            // contract lambda with the parameter derivatives; carry to step n-1
            TF_CUDA(cudaMemcpyAsync(d.lamv, d.du, n3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
            TF_CUDA(cudaMemsetAsync(d.carry, 0, n3 * sizeof(double), st));
            TFA_TRY(launch_adjoint_element(h, d.lamv, d.carry, d.gr, d.ge, (double)n * a->dt));
            k_carry_nodes<<<cdiv(d.nn, kT), kT, 0, st>>>(d.nn, d.area, d.ext_visc, 1.0 / a->dt, d.lamv, d.carry);
            TF_LAUNCH_CHECK(h);
            k_carry_faces<<<cdiv(ne, kT), kT, 0, st>>>(ne, d.conn, d.exposure, su[k - 1], su[k], 1.0 / a->dt,
                                                      d.ext_visc, d.lamv, d.carry);
            TF_LAUNCH_CHECK(h);
        }
    }
    // leave the handle at the final state
    TFA_TRY(copy_state(h, d.uk, d.Fg, d.invFg, a->final_u, a->final_Fg, a->final_iFg));
    TF_CUDA(cudaMemcpyAsync(grad_rate, d.gr, ne * sizeof(double), cudaMemcpyDeviceToHost, st));
    TF_CUDA(cudaMemcpyAsync(grad_logE, d.ge, ne * sizeof(double), cudaMemcpyDeviceToHost, st));
    TF_CUDA(cudaStreamSynchronize(st));
    return TF_OK;
}

// The adjoint's forward runs, and the steps its backward pass recomputes,
// rebuild the multigrid's coarse levels at every time step (as a handle with
// multigrid_reuse_steps < 0 does) for the scope of the call.
struct CoarseRebuiltEachStep {
    tf_handle* h;
    int keep;
    explicit CoarseRebuiltEachStep(tf_handle* hh) : h(hh), keep(hh->opt.multigrid_reuse_steps) {
        h->opt.multigrid_reuse_steps = 0;
    }
    ~CoarseRebuiltEachStep() { h->opt.multigrid_reuse_steps = keep; }
};

}  // namespace

extern "C" {

TF_API tf_status tf_adj_forward(tf_handle* h, const double* rate, const double* logE, int32_t n_steps, double dt,
                                int32_t every, const double* loss_params, double* loss, tf_adjoint** saved) {
    if (saved) *saved = nullptr;
    if (!h || !rate || !logE || n_steps <= 0 || !(dt > 0.0) || !std::isfinite(dt) || every <= 0 || !loss_params ||
        !loss || !saved) {
        set_error("tf_adj_forward: bad arguments");
        return TF_BAD_INPUT;
    }
    if (h->d.nseg != 1) {
        set_error("tf_adj_forward: the adjoint works on single-mesh handles");
        return TF_BAD_INPUT;
    }
    if (h->d.nxb > 0 || !h->bind_slave.empty() || h->pk || growth_count(h) > 0) {
        set_error("tf_adj_forward: added K entries, packing, bound DOFs and growth functions are not differentiated");
        return TF_BAD_INPUT;
    }
    if (!(loss_params[3] > 0.0)) {
        set_error("tf_adj_forward: the loss width loss_params[3] must be positive");
        return TF_BAD_INPUT;
    }
    TF_CUDA(cudaSetDevice(h->device));
    TFA_TRY(ensure_adjoint_buffers(h));
    tf_adjoint* a = new tf_adjoint;
    a->n_steps = n_steps;
    a->every = every;
    a->dt = dt;
    a->device = h->device;
    std::memcpy(a->params, loss_params, sizeof(a->params));
    CoarseRebuiltEachStep rebuilt(h);
    const tf_status s = adj_forward(h, a, rate, logE);
    if (s != TF_OK && s != TF_NOT_CONVERGED) {
        tf_adj_free(a);
        return s;
    }
    *loss = a->loss;
    *saved = a;
    return s;
}

TF_API tf_status tf_adj_backward(tf_handle* h, tf_adjoint* a, double dloss, double* grad_rate, double* grad_logE) {
    if (!h || !a || !grad_rate || !grad_logE || !std::isfinite(dloss)) {
        set_error("tf_adj_backward: bad arguments");
        return TF_BAD_INPUT;
    }
    if (a->device != h->device || !h->d.valT) {
        set_error("tf_adj_backward: saved state does not belong to this handle");
        return TF_BAD_INPUT;
    }
    TF_CUDA(cudaSetDevice(h->device));
    CoarseRebuiltEachStep rebuilt(h);
    return adj_backward(h, a, dloss, grad_rate, grad_logE);
}

TF_API tf_status tf_adj_free(tf_adjoint* a) {
    if (!a) return TF_OK;
    cudaSetDevice(a->device);
    for (double* p : a->ck_u) cudaFree(p);
    for (double* p : a->ck_Fg) cudaFree(p);
    for (double* p : a->ck_iFg) cudaFree(p);
    cudaFree(a->final_u);
    cudaFree(a->final_Fg);
    cudaFree(a->final_iFg);
    cudaFree(a->rate);
    cudaFree(a->logE);
    delete a;
    return TF_OK;
}

}  // extern "C"
