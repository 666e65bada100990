// Prism element kernel: residual and 18x18 tangent of every prism, fused
// with the scatter into the block-sparse Jacobian.
//
// Maths follows the reference's element routines (paths relative to
// TissueFolding/TissueFolding/SourceCode/):
//   Prism::calculateCurrNodalForces      Prism.cpp:749-874
//   ShapeBase::calculateForces3D         ShapeBase.cpp:2184-2235
//   neo-Hookean S, D81, Cauchy stress    ShapeBase.cpp:2284-2341
//   calculateImplicitKElastic            ShapeBase.cpp:2619-2639, :2786-2890
//   calculateImplicitKViscous            ShapeBase.cpp:2641-2705, :2892-3053
//   write*ToMainKatrix / ge, gv scatter  ShapeBase.cpp:2148-2180, :2707-2758
// with two exact identities used to cut FP64 work:
//   * Fe C^-1 Fe^T = I, so sigma = (mu (b - I) + lambda lnJ I) / J with
//     b = Fe Fe^T, and the 3^6 contraction of integral 1 collapses to
//     lambda a_i b_k + (mu - lambda lnJ)(delta_ik a.b + a_k b_i);
//   * dN_x = F^-T dN_X with dN_X = InvdXde^T dN precomputed per element.
//
// Layout: one CTA handles kElemPerCta prisms.  Phase A: one thread per
// (prism, Gauss point) builds the per-point quantities in shared memory.
// Phase B: each thread owns 3x3 node-pair blocks, sums the six Gauss points
// and scatters the block.  The matrix assembled is A = K^T, the system the
// reference solves (Pardiso iparm[11] = 1, NewtonRaphsonSolver.cpp:639); in
// that orientation every element block (a, b) lands at block
// (conn[a], conn[b]) without a transpose.  Fixed DOFs are masked here, which
// is calcutateFixedK (NewtonRaphsonSolver.cpp:237-255) without a second pass.
#include "tf_internal.cuh"

namespace tf {

namespace {

enum Mode { kAtomic = 0, kEval = 1, kStore = 2 };

struct ElemArgs {
    int ne;
    const int* __restrict__ conn;
    const double* __restrict__ gx;
    const double* __restrict__ wdet;
    const double* __restrict__ invFg;
    const double* __restrict__ lam;
    const double* __restrict__ mu;
    const double* __restrict__ eta;
    const uint8_t* __restrict__ fixed;
    const int* __restrict__ slot;
    const double* __restrict__ uk;
    const double* __restrict__ vel;
    double dt;
    double* __restrict__ val;  // kAtomic: block values
    double* __restrict__ g;    // kAtomic: right-hand side
    // kEval outputs (reference orientation), element-relative
    int e0, count;
    double* __restrict__ Ke;
    double* __restrict__ Kv;
    double* __restrict__ fe;
    double* __restrict__ fv;
    // kStore outputs
    double* __restrict__ eblk;  // [9][36*ne]
    double* __restrict__ ef;    // [18][ne]
};

struct Gp {
    double dn[18];
    double c1, c2;
    double sdn[18];
    double pv[9];
    double pdn[18];
    double svdn[18];
    double fe[18];
    double fv[18];
};

template <int NE>
__device__ __forceinline__ int elem_index(const ElemArgs& A, int el, int mode) {
    int e = blockIdx.x * NE + el;
    return mode == kEval ? A.e0 + e : e;
}

template <int NE, int MODE>
__global__ void __launch_bounds__(NE * kGauss) k_element(ElemArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Gp* sh = reinterpret_cast<Gp*>(smem_raw);  // [NE][6]
    const int tid = threadIdx.x;
    const int limit = (MODE == kEval) ? A.e0 + A.count : A.ne;

    // ---------------- phase A: one thread per (prism, Gauss point) -------
    {
        const int el = tid / kGauss;
        const int gp = tid - el * kGauss;
        const int e = elem_index<NE>(A, el, MODE);
        Gp& S = sh[el * kGauss + gp];
        if (e < limit) {
            const int ne = A.ne;
            int nd[6];
#pragma unroll
            for (int a = 0; a < 6; ++a) nd[a] = __ldg(&A.conn[a * ne + e]);
            double gX[18];
            const int q = 6 * e + gp;
#pragma unroll
            for (int k = 0; k < 18; ++k) gX[k] = __ldg(&A.gx[(size_t)k * (6 * (size_t)ne) + q]);
            // F = sum_a x_a (x) dN_X,a.  The gradients sum to zero, so the
            // positions are taken relative to node 0: that removes the
            // cancellation of ~|x| / h between the products at coordinates far
            // from the origin (the result is unchanged in exact arithmetic).
            double F[9];
#pragma unroll
            for (int k = 0; k < 9; ++k) F[k] = 0.0;
            const double o0 = A.uk[3 * nd[0]], o1 = A.uk[3 * nd[0] + 1], o2 = A.uk[3 * nd[0] + 2];
#pragma unroll
            for (int a = 1; a < 6; ++a) {
                const double x0 = A.uk[3 * nd[a]] - o0, x1 = A.uk[3 * nd[a] + 1] - o1, x2 = A.uk[3 * nd[a] + 2] - o2;
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    F[j] = fma(x0, gX[3 * a + j], F[j]);
                    F[3 + j] = fma(x1, gX[3 * a + j], F[3 + j]);
                    F[6 + j] = fma(x2, gX[3 * a + j], F[6 + j]);
                }
            }
            double iFg[9];
#pragma unroll
            for (int k = 0; k < 9; ++k) iFg[k] = __ldg(&A.invFg[k * ne + e]);
            double Fe[9];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    Fe[3 * i + j] = fma(F[3 * i], iFg[j], fma(F[3 * i + 1], iFg[3 + j], F[3 * i + 2] * iFg[6 + j]));
            // J = det Fe, b = Fe Fe^T
            const double J = Fe[0] * (Fe[4] * Fe[8] - Fe[5] * Fe[7]) - Fe[1] * (Fe[3] * Fe[8] - Fe[5] * Fe[6]) +
                             Fe[2] * (Fe[3] * Fe[7] - Fe[4] * Fe[6]);
            const double lnJ = log(J);
            const double rJ = 1.0 / J;
            const double lam = __ldg(&A.lam[e]), mu = __ldg(&A.mu[e]);
            double b[6];  // 00 11 22 01 02 12
            b[0] = fma(Fe[0], Fe[0], fma(Fe[1], Fe[1], Fe[2] * Fe[2]));
            b[1] = fma(Fe[3], Fe[3], fma(Fe[4], Fe[4], Fe[5] * Fe[5]));
            b[2] = fma(Fe[6], Fe[6], fma(Fe[7], Fe[7], Fe[8] * Fe[8]));
            b[3] = fma(Fe[0], Fe[3], fma(Fe[1], Fe[4], Fe[2] * Fe[5]));
            b[4] = fma(Fe[0], Fe[6], fma(Fe[1], Fe[7], Fe[2] * Fe[8]));
            b[5] = fma(Fe[3], Fe[6], fma(Fe[4], Fe[7], Fe[5] * Fe[8]));
            // cofactors of F: F^-T = cof / detF
            double cf[9];
            cf[0] = F[4] * F[8] - F[5] * F[7];
            cf[1] = F[5] * F[6] - F[3] * F[8];
            cf[2] = F[3] * F[7] - F[4] * F[6];
            cf[3] = F[2] * F[7] - F[1] * F[8];
            cf[4] = F[0] * F[8] - F[2] * F[6];
            cf[5] = F[1] * F[6] - F[0] * F[7];
            cf[6] = F[1] * F[5] - F[2] * F[4];
            cf[7] = F[2] * F[3] - F[0] * F[5];
            cf[8] = F[0] * F[4] - F[1] * F[3];
            const double detF = fma(F[0], cf[0], fma(F[1], cf[1], F[2] * cf[2]));
            const double rdF = 1.0 / detF;
            const double wdV = __ldg(&A.wdet[q]) * detF;
            // sigma' = w dV sigma = (w dV / J) (mu (b - I) + lambda lnJ I)
            const double sc = wdV * rJ;
            const double dterm = fma(lam, lnJ, -mu);
            double sg[6];
            sg[0] = sc * fma(mu, b[0], dterm);
            sg[1] = sc * fma(mu, b[1], dterm);
            sg[2] = sc * fma(mu, b[2], dterm);
            sg[3] = sc * mu * b[3];
            sg[4] = sc * mu * b[4];
            sg[5] = sc * mu * b[5];
            S.c1 = sc * lam;
            S.c2 = sc * (mu - lam * lnJ);
            double dn[18];
#pragma unroll
            for (int a = 0; a < 6; ++a) {
                const double g0 = gX[3 * a], g1 = gX[3 * a + 1], g2 = gX[3 * a + 2];
                dn[3 * a] = rdF * fma(cf[0], g0, fma(cf[1], g1, cf[2] * g2));
                dn[3 * a + 1] = rdF * fma(cf[3], g0, fma(cf[4], g1, cf[5] * g2));
                dn[3 * a + 2] = rdF * fma(cf[6], g0, fma(cf[7], g1, cf[8] * g2));
            }
#pragma unroll
            for (int k = 0; k < 18; ++k) S.dn[k] = dn[k];
#pragma unroll
            for (int a = 0; a < 6; ++a) {
                const double d0 = dn[3 * a], d1 = dn[3 * a + 1], d2 = dn[3 * a + 2];
                const double s0 = fma(sg[0], d0, fma(sg[3], d1, sg[4] * d2));
                const double s1 = fma(sg[3], d0, fma(sg[1], d1, sg[5] * d2));
                const double s2 = fma(sg[4], d0, fma(sg[5], d1, sg[2] * d2));
                S.sdn[3 * a] = s0;
                S.sdn[3 * a + 1] = s1;
                S.sdn[3 * a + 2] = s2;
                S.fe[3 * a] = -s0;
                S.fe[3 * a + 1] = -s1;
                S.fe[3 * a + 2] = -s2;
            }
            const double eta = __ldg(&A.eta[e]);
            if (eta != 0.0) {
                // grad v = sum_c v_c (x) dn_c  (ShapeBase.cpp:2892-2919)
                double L[9];
#pragma unroll
                for (int k = 0; k < 9; ++k) L[k] = 0.0;
                const double w0 = A.vel[3 * nd[0]], w1 = A.vel[3 * nd[0] + 1], w2 = A.vel[3 * nd[0] + 2];
#pragma unroll
                for (int c = 1; c < 6; ++c) {
                    const double v0 = A.vel[3 * nd[c]] - w0, v1 = A.vel[3 * nd[c] + 1] - w1, v2 = A.vel[3 * nd[c] + 2] - w2;
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        L[j] = fma(v0, dn[3 * c + j], L[j]);
                        L[3 + j] = fma(v1, dn[3 * c + j], L[3 + j]);
                        L[6 + j] = fma(v2, dn[3 * c + j], L[6 + j]);
                    }
                }
                // sigma_v' = w dV eta sym(L);  pv = 0.5 eta w dV (I/dt - L)
                const double ew = eta * wdV;
                const double hw = 0.5 * ew;
                double sv[6];
                sv[0] = ew * L[0];
                sv[1] = ew * L[4];
                sv[2] = ew * L[8];
                sv[3] = hw * (L[1] + L[3]);
                sv[4] = hw * (L[2] + L[6]);
                sv[5] = hw * (L[5] + L[7]);
                const double idt = 1.0 / A.dt;
                double pv[9];
#pragma unroll
                for (int k = 0; k < 9; ++k) pv[k] = -hw * L[k];
                pv[0] = fma(hw, idt, pv[0]);
                pv[4] = fma(hw, idt, pv[4]);
                pv[8] = fma(hw, idt, pv[8]);
#pragma unroll
                for (int k = 0; k < 9; ++k) S.pv[k] = pv[k];
#pragma unroll
                for (int a = 0; a < 6; ++a) {
                    const double d0 = dn[3 * a], d1 = dn[3 * a + 1], d2 = dn[3 * a + 2];
                    S.pdn[3 * a] = fma(pv[0], d0, fma(pv[3], d1, pv[6] * d2));
                    S.pdn[3 * a + 1] = fma(pv[1], d0, fma(pv[4], d1, pv[7] * d2));
                    S.pdn[3 * a + 2] = fma(pv[2], d0, fma(pv[5], d1, pv[8] * d2));
                    const double s0 = fma(sv[0], d0, fma(sv[3], d1, sv[4] * d2));
                    const double s1 = fma(sv[3], d0, fma(sv[1], d1, sv[5] * d2));
                    const double s2 = fma(sv[4], d0, fma(sv[5], d1, sv[2] * d2));
                    S.svdn[3 * a] = s0;
                    S.svdn[3 * a + 1] = s1;
                    S.svdn[3 * a + 2] = s2;
                    S.fv[3 * a] = -s0;
                    S.fv[3 * a + 1] = -s1;
                    S.fv[3 * a + 2] = -s2;
                }
            }
        }
    }
    __syncthreads();

    // ---------------- element forces: Gauss sum, fixed mask, scatter ------
    for (int task = tid; task < NE * 18; task += NE * kGauss) {
        const int el = task / 18;
        const int k = task - el * 18;
        const int e = elem_index<NE>(A, el, MODE);
        if (e >= limit) continue;
        const bool visc = __ldg(&A.eta[e]) != 0.0;
        double se = 0.0, sv = 0.0;
#pragma unroll
        for (int gp = 0; gp < kGauss; ++gp) {
            se += sh[el * kGauss + gp].fe[k];
            if (visc) sv += sh[el * kGauss + gp].fv[k];
        }
        const int a = k / 3, d = k - 3 * (k / 3);
        const int node = __ldg(&A.conn[a * A.ne + e]);
        const bool fx = A.fixed[3 * node + d] != 0;
        if (MODE == kEval) {
            const int r = e - A.e0;
            if (A.fe) A.fe[18 * (size_t)r + k] = fx ? 0.0 : se;
            if (A.fv) A.fv[18 * (size_t)r + k] = fx ? 0.0 : sv;
        } else if (MODE == kStore) {
            A.ef[(size_t)k * A.ne + e] = fx ? 0.0 : se + sv;
        } else {
            if (!fx) atomicAdd(&A.g[3 * node + d], se + sv);
        }
    }

    // ---------------- phase B: 3x3 node-pair blocks ------------------------
    for (int task = tid; task < NE * 36; task += NE * kGauss) {
        const int el = task / 36;
        const int pr = task - el * 36;
        const int e = elem_index<NE>(A, el, MODE);
        if (e >= limit) continue;
        const int a = pr / 6, bq = pr - 6 * (pr / 6);
        const bool visc = __ldg(&A.eta[e]) != 0.0;
        double ke[9], kv[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            ke[k] = 0.0;
            kv[k] = 0.0;
        }
#pragma unroll
        for (int gp = 0; gp < kGauss; ++gp) {
            const Gp& S = sh[el * kGauss + gp];
            const double a0 = S.dn[3 * a], a1 = S.dn[3 * a + 1], a2 = S.dn[3 * a + 2];
            const double b0 = S.dn[3 * bq], b1 = S.dn[3 * bq + 1], b2 = S.dn[3 * bq + 2];
            const double c1 = S.c1, c2 = S.c2;
            const double s = fma(a0, b0, fma(a1, b1, a2 * b2));
            const double t = fma(a0, S.sdn[3 * bq], fma(a1, S.sdn[3 * bq + 1], a2 * S.sdn[3 * bq + 2]));
            const double dg = fma(c2, s, t);
            const double ca[3] = {c1 * a0, c1 * a1, c1 * a2};
            const double da[3] = {c2 * a0, c2 * a1, c2 * a2};
            const double bb[3] = {b0, b1, b2};
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    double v = fma(ca[i], bb[k], fma(da[k], bb[i], ke[3 * i + k]));
                    if (i == k) v += dg;
                    ke[3 * i + k] = v;
                }
            if (visc) {
                const double pa[3] = {S.pdn[3 * a], S.pdn[3 * a + 1], S.pdn[3 * a + 2]};
                const double sva[3] = {S.svdn[3 * a], S.svdn[3 * a + 1], S.svdn[3 * a + 2]};
                const double svb[3] = {S.svdn[3 * bq], S.svdn[3 * bq + 1], S.svdn[3 * bq + 2]};
                const double aa[3] = {a0, a1, a2};
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int k = 0; k < 3; ++k)
                        kv[3 * i + k] = fma(s, S.pv[3 * i + k],
                                            fma(bb[i], pa[k], fma(sva[i], bb[k], fma(-svb[i], aa[k], kv[3 * i + k]))));
            }
        }
        if (MODE == kEval) {
            // reference orientation: TriPointKe[3a+i][3b+k] = ke(i,k);
            // TriPointKv[3b+k][3a+i] = kv(i,k)  (ShapeBase.cpp:2968-2975)
            const size_t r = (size_t)(e - A.e0);
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    if (A.Ke) A.Ke[324 * r + (3 * a + i) * 18 + 3 * bq + k] = ke[3 * i + k];
                    if (A.Kv) A.Kv[324 * r + (3 * bq + k) * 18 + 3 * a + i] = visc ? kv[3 * i + k] : 0.0;
                }
        } else {
            const int na = __ldg(&A.conn[a * A.ne + e]);
            const int nb = __ldg(&A.conn[bq * A.ne + e]);
            bool fr[3], fc[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                fr[i] = A.fixed[3 * na + i] != 0;
                fc[i] = A.fixed[3 * nb + i] != 0;
            }
            if (MODE == kStore) {
                const size_t base = (size_t)pr * A.ne + e;
                const size_t stride = (size_t)36 * A.ne;
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int k = 0; k < 3; ++k)
                        A.eblk[(3 * i + k) * stride + base] = (fr[i] || fc[k]) ? 0.0 : ke[3 * i + k] + kv[3 * i + k];
            } else {
                const int blk = __ldg(&A.slot[pr * A.ne + e]);
                double* dst = A.val + 9 * (size_t)blk;
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int k = 0; k < 3; ++k)
                        if (!fr[i] && !fc[k]) atomicAdd(dst + 3 * i + k, ke[3 * i + k] + kv[3 * i + k]);
            }
        }
    }
}

ElemArgs make_args(tf_handle* h) {
    const Device& d = h->d;
    ElemArgs A{};
    A.ne = d.ne;
    A.conn = d.conn;
    A.gx = d.gx;
    A.wdet = d.wdet;
    A.invFg = d.invFg;
    A.lam = d.lam;
    A.mu = d.mu;
    A.eta = d.eta;
    A.fixed = d.fixed;
    A.slot = d.slot;
    A.uk = d.uk;
    A.vel = d.vel;
    A.dt = h->dt;
    A.val = d.val;
    A.g = d.g;
    A.eblk = d.eblk;
    A.ef = d.ef;
    return A;
}

template <int NE, int MODE>
tf_status launch_mode(tf_handle* h, ElemArgs A, int n) {
    if (n <= 0) return TF_OK;
    const size_t smem = sizeof(Gp) * NE * kGauss;
    static bool configured = false;
    if (!configured) {
        TF_CUDA(cudaFuncSetAttribute(k_element<NE, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        configured = true;
    }
    k_element<NE, MODE><<<cdiv(n, NE), NE * kGauss, smem, h->stream>>>(A);
    TF_LAUNCH_CHECK(h);
    return TF_OK;
}

}  // namespace

tf_status launch_element(tf_handle* h) {
    ElemArgs A = make_args(h);
    if (h->opt.deterministic) return launch_mode<kElemPerCta, kStore>(h, A, h->d.ne);
    return launch_mode<kElemPerCta, kAtomic>(h, A, h->d.ne);
}

tf_status launch_element_eval(tf_handle* h, int e0, int count, double* Ke, double* Kv, double* fe, double* fv) {
    ElemArgs A = make_args(h);
    A.e0 = e0;
    A.count = count;
    A.Ke = Ke;
    A.Kv = Kv;
    A.fe = fe;
    A.fv = fv;
    return launch_mode<8, kEval>(h, A, count);
}

}  // namespace tf
