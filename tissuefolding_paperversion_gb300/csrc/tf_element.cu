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
// with exact identities that cut FP64 work:
//   * Fe C^-1 Fe^T = I, so sigma = (mu (b - I) + lambda lnJ I) / J with
//     b = Fe Fe^T, and the 3^6 contraction of integral 1 collapses to
//     lambda a_i b_k + (mu - lambda lnJ)(delta_ik a.b + a_k b_i);
//   * dN_x = F^-T dN_X with dN_X = InvdXde^T dN precomputed per element;
//   * with a = dN_a, b = dN_b, s = a.b and t = a.(sigma' b) the whole 3x3
//     block (elastic + both viscous integrals) of one Gauss point is
//       K_ab = u_a b^T + b w_a^T - v_b a^T + s Q + t I
//     where per node c:  u_c = c1 dN_c + sigma_v' dN_c,
//                        w_c = c2 dN_c + P^T dN_c,   v_c = sigma_v' dN_c,
//     and Q = c2 I + P, P = 0.5 eta w dV (I/dt - grad v) (primes: times
//     w dV).  That is 45 multiply-adds per block and Gauss point instead of
//     64; without viscosity K_ab = K_ba^T and only the 21 pairs a <= b are
//     formed.
//
// Precision split.  GB300 issues FP32 FMAs at about 64 times its FP64 rate,
// and the tangent's block sums are ~85 % of the kernel's FP64 work.  Phase A
// (deformation gradient, stress, shape gradients, forces) stays FP64.  The
// per-Gauss-point vectors the blocks are built from are split into
// double-float pairs x = hi + lo (two FP32 values, ~48 significant bits) and
// the block sums run in double-float arithmetic on the FP32 pipe: products by
// Dekker's exact product (hi*hi and its rounding error by one FMA, plus the
// cross terms), sums by Knuth's two-sum, the low parts gathered in a second
// FP32 accumulator and renormalised once per Gauss point (Dekker, "A
// floating-point technique for extending the available precision", 1971;
// Knuth, TAOCP vol. 2, 4.2.2).  A block entry carries a relative error of
// ~1e-13 of its largest term, far inside the 1e-11 parity bound and far
// below what moves a Newton iterate; the forces and everything the residual
// depends on stay FP64 (with viscosity the forces use one FP64 stress
// sigma' + sigma_v', and the tangent's sigma' dN and sigma_v' dN come from
// the double-float splits of the two stresses).
//
// Layout: one CTA of 2 x 6 x NE threads handles NE prisms.  Phase A: one
// thread per (prism, Gauss point) -- the first half of the CTA -- builds the
// per-point vectors in shared memory.  Phase B: every thread owns 3x3
// node-pair blocks, sums the six Gauss points and scatters the block.  The matrix assembled is A = K^T, the system the reference
// solves (Pardiso iparm[11] = 1, NewtonRaphsonSolver.cpp:639); in that
// orientation every element block (a, b) lands at block (conn[a], conn[b])
// without a transpose.  Fixed DOFs are masked here, which is calcutateFixedK
// (NewtonRaphsonSolver.cpp:237-255) without a second pass.
#include "tf_internal.cuh"

namespace tf {

namespace {

enum Mode { kAtomic = 0, kStore = 2 };

// Threads per Gauss point: phase A runs on the first NE x 6 threads of the
// CTA, the pair phase and the force sums on all of them.  Twice the threads
// of phase A give the pair phase (FP32 pipe) more warps to hide its latency
// while other CTAs on the SM run phase A (FP64 pipe): 3.65 against 4.68 ms
// per 320,000-prism assembly with the merged force stress below and the
// Gauss loop of the pair phase kept rolled (unrolled it overflows the
// instruction cache); three threads per Gauss point were slower (registers
// then allow one CTA per SM).
constexpr int kTpg = 2;

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
    double idt;                 // 1 / dt
    double* __restrict__ val;   // kAtomic: block values
    double* __restrict__ g;     // kAtomic: right-hand side
    double* __restrict__ eblk;  // kStore: [9][36*ne]
    double* __restrict__ ef;    // kStore: [18][ne]
    // batches: elements of instances whose Newton loop has stopped are skipped
    const int* __restrict__ elem_seg;
    const int* __restrict__ seg_active;
    int masked;
    // parity evaluation (reference orientation), element-relative
    int e0, count;
    double* __restrict__ Ke;
    double* __restrict__ Kv;
    double* __restrict__ fe;
    double* __restrict__ fv;
    // checked build
    int nn;
    int64_t nval;
    int* check;
};

// Per-Gauss-point values in registers.
struct GaussPoint {
    double dn[18];   // current shape gradients dN_c (node-major)
    double sg[6];    // sigma' = w dV sigma     (00 11 22 01 02 12)
    double c1, c2;   // w dV lambda / J, w dV (mu - lambda lnJ) / J
    double sv[6];    // sigma_v' = w dV eta sym(grad v)
    double pv[9];    // P = 0.5 eta w dV (I/dt - grad v)
    double fe[9];    // Fe (row-major), kept for the adjoint
    double wdv;      // w dV
    double sc;       // w dV / J
};

__device__ __forceinline__ void sym_apply(const double* s, double d0, double d1, double d2, double* o) {
    o[0] = fma(s[0], d0, fma(s[3], d1, s[4] * d2));
    o[1] = fma(s[3], d0, fma(s[1], d1, s[5] * d2));
    o[2] = fma(s[4], d0, fma(s[5], d1, s[2] * d2));
}

// Prism::calculateCurrNodalForces (Prism.cpp:749-874) for Gauss point gp of
// element e, in closed form.
__device__ __forceinline__ void gauss_point(const ElemArgs& A, int e, int gp, bool visc, GaussPoint& G) {
    const int ne = A.ne;
    int nd[6];
#pragma unroll
    for (int a = 0; a < 6; ++a) {
        nd[a] = __ldg(&A.conn[a * ne + e]);
        if (!TF_IN(A.check, nd[a], A.nn, CK_ELEM_NODE)) nd[a] = 0;
    }
    double gX[18];
    const size_t q = 6 * (size_t)e + gp;
#pragma unroll
    for (int k = 0; k < 18; ++k) gX[k] = __ldg(&A.gx[(size_t)k * (6 * (size_t)ne) + q]);
    // F = sum_a x_a (x) dN_X,a.  The gradients sum to zero, so positions are
    // taken relative to node 0, which removes the cancellation of ~|x|/h
    // between the products far from the origin (exact arithmetic: no change).
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
    // Every multiply-add below is an explicit fma, so the rounding does not
    // depend on how the compiler contracts expressions in each instantiation
    // of the kernel (the order-fixed assembly stays bitwise reproducible
    // whatever tile the autotuner picks).
    const double J = fma(Fe[0], fma(Fe[4], Fe[8], -(Fe[5] * Fe[7])),
                         fma(-Fe[1], fma(Fe[3], Fe[8], -(Fe[5] * Fe[6])), Fe[2] * fma(Fe[3], Fe[7], -(Fe[4] * Fe[6]))));
    const double lnJ = log(J);
    const double rJ = 1.0 / J;
    const double lam = __ldg(&A.lam[e]), mu = __ldg(&A.mu[e]);
    double b[6];
    b[0] = fma(Fe[0], Fe[0], fma(Fe[1], Fe[1], Fe[2] * Fe[2]));
    b[1] = fma(Fe[3], Fe[3], fma(Fe[4], Fe[4], Fe[5] * Fe[5]));
    b[2] = fma(Fe[6], Fe[6], fma(Fe[7], Fe[7], Fe[8] * Fe[8]));
    b[3] = fma(Fe[0], Fe[3], fma(Fe[1], Fe[4], Fe[2] * Fe[5]));
    b[4] = fma(Fe[0], Fe[6], fma(Fe[1], Fe[7], Fe[2] * Fe[8]));
    b[5] = fma(Fe[3], Fe[6], fma(Fe[4], Fe[7], Fe[5] * Fe[8]));
    double cf[9];  // cofactors: F^-T = cf / det F
    cf[0] = fma(F[4], F[8], -(F[5] * F[7]));
    cf[1] = fma(F[5], F[6], -(F[3] * F[8]));
    cf[2] = fma(F[3], F[7], -(F[4] * F[6]));
    cf[3] = fma(F[2], F[7], -(F[1] * F[8]));
    cf[4] = fma(F[0], F[8], -(F[2] * F[6]));
    cf[5] = fma(F[1], F[6], -(F[0] * F[7]));
    cf[6] = fma(F[1], F[5], -(F[2] * F[4]));
    cf[7] = fma(F[2], F[3], -(F[0] * F[5]));
    cf[8] = fma(F[0], F[4], -(F[1] * F[3]));
    const double detF = fma(F[0], cf[0], fma(F[1], cf[1], F[2] * cf[2]));
    const double rdF = 1.0 / detF;
    const double wdV = __ldg(&A.wdet[q]) * detF;
    G.wdv = wdV;
#pragma unroll
    for (int k = 0; k < 9; ++k) G.fe[k] = Fe[k];
    const double sc = wdV * rJ;
    G.sc = sc;
    const double dterm = fma(lam, lnJ, -mu);
    G.sg[0] = sc * fma(mu, b[0], dterm);
    G.sg[1] = sc * fma(mu, b[1], dterm);
    G.sg[2] = sc * fma(mu, b[2], dterm);
    G.sg[3] = sc * mu * b[3];
    G.sg[4] = sc * mu * b[4];
    G.sg[5] = sc * mu * b[5];
    G.c1 = sc * lam;
    G.c2 = sc * fma(-lam, lnJ, mu);
#pragma unroll
    for (int a = 0; a < 6; ++a) {
        const double g0 = gX[3 * a], g1 = gX[3 * a + 1], g2 = gX[3 * a + 2];
        G.dn[3 * a] = rdF * fma(cf[0], g0, fma(cf[1], g1, cf[2] * g2));
        G.dn[3 * a + 1] = rdF * fma(cf[3], g0, fma(cf[4], g1, cf[5] * g2));
        G.dn[3 * a + 2] = rdF * fma(cf[6], g0, fma(cf[7], g1, cf[8] * g2));
    }
    if (visc) {
        // grad v = sum_c v_c (x) dN_c (ShapeBase.cpp:2892-2919), velocities
        // relative to node 0 for the same reason as the positions
        double L[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) L[k] = 0.0;
        const double w0 = A.vel[3 * nd[0]], w1 = A.vel[3 * nd[0] + 1], w2 = A.vel[3 * nd[0] + 2];
#pragma unroll
        for (int c = 1; c < 6; ++c) {
            const double v0 = A.vel[3 * nd[c]] - w0, v1 = A.vel[3 * nd[c] + 1] - w1, v2 = A.vel[3 * nd[c] + 2] - w2;
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                L[j] = fma(v0, G.dn[3 * c + j], L[j]);
                L[3 + j] = fma(v1, G.dn[3 * c + j], L[3 + j]);
                L[6 + j] = fma(v2, G.dn[3 * c + j], L[6 + j]);
            }
        }
        const double eta = __ldg(&A.eta[e]);
        const double ew = eta * wdV;
        const double hw = 0.5 * ew;
        G.sv[0] = ew * L[0];
        G.sv[1] = ew * L[4];
        G.sv[2] = ew * L[8];
        G.sv[3] = hw * (L[1] + L[3]);
        G.sv[4] = hw * (L[2] + L[6]);
        G.sv[5] = hw * (L[5] + L[7]);
#pragma unroll
        for (int k = 0; k < 9; ++k) G.pv[k] = -hw * L[k];
        G.pv[0] = fma(hw, A.idt, G.pv[0]);
        G.pv[4] = fma(hw, A.idt, G.pv[4]);
        G.pv[8] = fma(hw, A.idt, G.pv[8]);
    }
}

// ---- double-float arithmetic (phase B) ----------------------------------
// A value is hi + lo with hi, lo FP32.  Every operation is an explicit
// rounding intrinsic, so no instantiation of the kernel contracts or
// reassociates differently (the order-fixed assembly stays bitwise
// reproducible whatever tile the autotuner picks).

// The FP64 <-> FP32 conversion instructions run on GB300's slow FP64 path,
// so the split and the join work on the bit patterns (integer pipe) with one
// FP64 subtraction or addition each.

// float with x's value rounded to 24 significant bits; x must be a double
// whose low 29 mantissa bits are zero (then the result is exact): sign,
// exponent rebased 1023 -> 127, the top 23 mantissa bits.  Magnitudes below
// FP32's normal range become a signed zero; NaN and infinity stay NaN and
// infinity.
__device__ __forceinline__ float f32_of_trunc(unsigned hi, unsigned lo) {
    const unsigned sgn = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ffu);
    const int fe = e - 896;
    unsigned f = sgn | ((unsigned)fe << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
    f = (fe > 0) ? f : sgn;
    f = (e == 0x7ff) ? (sgn | 0x7f800000u | ((hi & 0xfffffu) ? 0x400000u : 0u)) : f;
    return __uint_as_float(f);
}

// x rounded to 24 significant bits (round half away from zero on the bit
// pattern; the carry runs into the exponent), as a double and as a float.
__device__ __forceinline__ double round24(double x, float* f) {
    const unsigned lo = __double2loint(x), hi = __double2hiint(x);
    const unsigned lo2 = lo + (1u << 28);
    const unsigned hi2 = hi + (lo2 < lo ? 1u : 0u);
    const unsigned lo3 = lo2 & ~((1u << 29) - 1u);
    const bool special = ((hi >> 20) & 0x7ffu) == 0x7ffu;
    *f = f32_of_trunc(special ? hi : hi2, special ? lo : lo3);
    return special ? x : __hiloint2double(hi2, lo3);
}

// x = hi + lo, hi and lo FP32 (~48 significant bits in all)
__device__ __forceinline__ float2 df_split(double x) {
    float h, l;
    const double hd = round24(x, &h);
    round24(x - hd, &l);
    return make_float2(h, l);
}

// float -> double, exact, on the bit pattern (subnormal floats become zero)
__device__ __forceinline__ double f64_of(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned sgn = u & 0x80000000u;
    unsigned hi = sgn | ((e + 896u) << 20) | ((u & 0x7fffffu) >> 3);
    hi = (e == 0u) ? sgn : hi;
    hi = (e == 0xffu) ? (sgn | 0x7ff00000u | ((u & 0x7fffffu) ? 0x80000u : 0u)) : hi;
    const unsigned lo = (e == 0u || e == 0xffu) ? 0u : (u << 29);
    return __hiloint2double(hi, lo);
}

__device__ __forceinline__ double df_join(float h, float l) { return f64_of(h) + f64_of(l); }

// (H, L) += x * y: Dekker's product (the rounding error of hi*hi by one FMA,
// the cross terms into the low word; lo*lo is below the format's precision),
// Knuth's two-sum of the high words, the error into the low word.
__device__ __forceinline__ void df_mac(float& H, float& L, float2 x, float2 y) {
    const float p = __fmul_rn(x.x, y.x);
    float e = __fmaf_rn(x.x, y.x, -p);
    e = __fmaf_rn(x.x, y.y, e);
    e = __fmaf_rn(x.y, y.x, e);
    const float s = __fadd_rn(H, p);
    const float bb = __fsub_rn(s, H);
    const float err = __fadd_rn(__fsub_rn(H, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    L = __fadd_rn(L, __fadd_rn(err, e));
    H = s;
}

// (H, L) += x
__device__ __forceinline__ void df_add(float& H, float& L, float2 x) {
    const float s = __fadd_rn(H, x.x);
    const float bb = __fsub_rn(s, H);
    const float err = __fadd_rn(__fsub_rn(H, __fsub_rn(s, bb)), __fsub_rn(x.x, bb));
    L = __fadd_rn(L, __fadd_rn(err, x.y));
    H = s;
}

// Fast two-sum: the low word brought back under half an ulp of the high word.
__device__ __forceinline__ void df_norm(float& H, float& L) {
    const float s = __fadd_rn(H, L);
    L = __fsub_rn(L, __fsub_rn(s, H));
    H = s;
}

__device__ __forceinline__ float2 df_neg(float2 x) { return make_float2(-x.x, -x.y); }

// Shared per-Gauss-point vectors of the fast kernel: the tangent's inputs as
// double-float pairs, the force terms in FP64.
template <bool VISC>
struct GpFast;
template <>
struct GpFast<false> {
    float2 dn[18], sdn[18], u[18], w[18];
    float2 c2;
    double fs[18];   // sigma' dN (forces)
};
template <>
struct GpFast<true> {
    float2 dn[18], sdn[18], u[18], w[18], v[18], Q[9];
    double fs[18];           // (sigma' + sigma_v') dN (forces)
};

// o = s d for a symmetric s (00 11 22 01 02 12), in double-float
__device__ __forceinline__ void df_sym_apply(const float2* s, const float2* d, float2* o) {
    const int ix[9] = {0, 3, 4, 3, 1, 5, 4, 5, 2};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float H = 0.0f, L = 0.0f;
#pragma unroll
        for (int j = 0; j < 3; ++j) df_mac(H, L, s[ix[3 * i + j]], d[j]);
        df_norm(H, L);
        o[i] = make_float2(H, L);
    }
}

// Node pairs a <= b of the symmetric (inviscid) case.
__constant__ int8_t kPairA[21] = {0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 4, 4, 5};
__constant__ int8_t kPairB[21] = {0, 1, 2, 3, 4, 5, 1, 2, 3, 4, 5, 2, 3, 4, 5, 3, 4, 5, 4, 5, 5};

__device__ __forceinline__ bool element_live(const ElemArgs& A, int e) {
    return e < A.ne && (!A.masked || A.seg_active[A.elem_seg[e]] != 0);
}

template <int NE, int MODE, bool VISC>
__global__ void __launch_bounds__(NE * kGauss * kTpg) k_element(ElemArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using Gp = GpFast<VISC>;
    Gp* sh = reinterpret_cast<Gp*>(smem_raw);  // [NE][6]
    const int tid = threadIdx.x;
    constexpr int NT = NE * kGauss * kTpg;

    // ---------------- phase A ----------------------------------------------
    if (tid < NE * kGauss) {
        const int el = tid / kGauss;
        const int gp = tid - el * kGauss;
        const int e = blockIdx.x * NE + el;
        if (element_live(A, e)) {
            const bool visc = VISC && (__ldg(&A.eta[e]) != 0.0);
            GaussPoint G;
            gauss_point(A, e, gp, visc, G);
            Gp& S = sh[el * kGauss + gp];
            // scalars and matrices the per-node vectors are formed from
            const float2 c1 = df_split(G.c1), c2 = df_split(G.c2);
            float2 Pm[9];
            if constexpr (VISC) {
#pragma unroll
                for (int k = 0; k < 9; ++k) Pm[k] = df_split(visc ? G.pv[k] : 0.0);
            }
            // VISC: one FP64 stress sigma' + sigma_v' for the forces; the
            // tangent's sigma' dN and sigma_v' dN in double-float from the
            // splits of the two stresses (54 FP64 multiply-adds and 36 splits
            // fewer per Gauss point than forming both products in FP64)
            double st[6];
            float2 sgs[6], svs[6];
            if constexpr (VISC) {
#pragma unroll
                for (int k = 0; k < 6; ++k) {
                    st[k] = visc ? G.sg[k] + G.sv[k] : G.sg[k];
                    sgs[k] = df_split(G.sg[k]);
                    svs[k] = df_split(visc ? G.sv[k] : 0.0);
                }
            }
#pragma unroll
            for (int a = 0; a < 6; ++a) {
                const double d0 = G.dn[3 * a], d1 = G.dn[3 * a + 1], d2 = G.dn[3 * a + 2];
                const float2 dn[3] = {df_split(d0), df_split(d1), df_split(d2)};
                if constexpr (VISC) {
                    double s3[3];
                    sym_apply(st, d0, d1, d2, s3);
                    float2 sd[3];
                    df_sym_apply(sgs, dn, sd);
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        S.dn[3 * a + i] = dn[i];
                        S.fs[3 * a + i] = s3[i];
                        S.sdn[3 * a + i] = sd[i];
                    }
                } else {
                    double s3[3];
                    sym_apply(G.sg, d0, d1, d2, s3);
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        S.dn[3 * a + i] = dn[i];
                        S.fs[3 * a + i] = s3[i];
                        S.sdn[3 * a + i] = df_split(s3[i]);
                    }
                }
                if constexpr (VISC) {
                    float2 vs[3];
                    df_sym_apply(svs, dn, vs);
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        const float2 vv = vs[i];
                        S.v[3 * a + i] = vv;
                        // u = c1 dN + sigma_v' dN
                        float uH = 0.0f, uL = 0.0f;
                        df_mac(uH, uL, c1, dn[i]);
                        df_add(uH, uL, vv);
                        df_norm(uH, uL);
                        S.u[3 * a + i] = make_float2(uH, uL);
                        // w = c2 dN + P^T dN
                        float wH = 0.0f, wL = 0.0f;
                        df_mac(wH, wL, c2, dn[i]);
#pragma unroll
                        for (int j = 0; j < 3; ++j) df_mac(wH, wL, Pm[3 * j + i], dn[j]);
                        df_norm(wH, wL);
                        S.w[3 * a + i] = make_float2(wH, wL);
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        float uH = 0.0f, uL = 0.0f, wH = 0.0f, wL = 0.0f;
                        df_mac(uH, uL, c1, dn[i]);
                        df_mac(wH, wL, c2, dn[i]);
                        S.u[3 * a + i] = make_float2(uH, uL);
                        S.w[3 * a + i] = make_float2(wH, wL);
                    }
                }
            }
            if constexpr (VISC) {
                // Q = c2 I + P
#pragma unroll
                for (int k = 0; k < 9; ++k) {
                    float qH = Pm[k].x, qL = Pm[k].y;
                    if (k == 0 || k == 4 || k == 8) {
                        df_add(qH, qL, c2);
                        df_norm(qH, qL);
                    }
                    S.Q[k] = make_float2(qH, qL);
                }
            } else {
                S.c2 = c2;
            }
        }
    }
    __syncthreads();

    // ---------------- element forces: Gauss sum, fixed mask, scatter ------
    // f_a = - sum_g (sigma' + sigma_v') dN_a  (ShapeBase.cpp:2203-2227)
    for (int task = tid; task < NE * 18; task += NT) {
        const int el = task / 18;
        const int k = task - el * 18;
        const int e = blockIdx.x * NE + el;
        if (!element_live(A, e)) continue;
        double f = 0.0;
#pragma unroll
        for (int gp = 0; gp < kGauss; ++gp) {
            f -= sh[el * kGauss + gp].fs[k];
        }
        const int a = k / 3, d = k - 3 * (k / 3);
        const int node = __ldg(&A.conn[a * A.ne + e]);
        if (!TF_IN(A.check, node, A.nn, CK_ELEM_NODE)) continue;
        const bool fx = A.fixed[3 * node + d] != 0;
        if (MODE == kStore) A.ef[(size_t)k * A.ne + e] = fx ? 0.0 : f;
        else if (!fx) atomicAdd(&A.g[3 * node + d], f);
    }

    // ---------------- phase B: 3x3 node-pair blocks ------------------------
    constexpr int kPairs = VISC ? 36 : 21;
    for (int task = tid; task < NE * kPairs; task += NT) {
        const int el = task / kPairs;
        const int pr = task - el * kPairs;
        const int e = blockIdx.x * NE + el;
        if (!element_live(A, e)) continue;
        const int a = VISC ? pr / 6 : kPairA[pr];
        const int bq = VISC ? pr - 6 * (pr / 6) : kPairB[pr];
        float aH[9], aL[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) aH[k] = aL[k] = 0.0f;
#pragma unroll 1
        for (int gp = 0; gp < kGauss; ++gp) {
            const Gp& S = sh[el * kGauss + gp];
            const float2 a3[3] = {S.dn[3 * a], S.dn[3 * a + 1], S.dn[3 * a + 2]};
            const float2 b3[3] = {S.dn[3 * bq], S.dn[3 * bq + 1], S.dn[3 * bq + 2]};
            float sH = 0.0f, sL = 0.0f, tH = 0.0f, tL = 0.0f;
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                df_mac(sH, sL, a3[j], b3[j]);
                df_mac(tH, tL, a3[j], S.sdn[3 * bq + j]);
            }
            const float2 ua[3] = {S.u[3 * a], S.u[3 * a + 1], S.u[3 * a + 2]};
            const float2 wa[3] = {S.w[3 * a], S.w[3 * a + 1], S.w[3 * a + 2]};
            if constexpr (VISC) {
                const float2 s2 = make_float2(sH, sL), t2 = make_float2(tH, tL);
                const float2 vb[3] = {df_neg(S.v[3 * bq]), df_neg(S.v[3 * bq + 1]), df_neg(S.v[3 * bq + 2])};
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        float& H = aH[3 * i + k];
                        float& L = aL[3 * i + k];
                        df_mac(H, L, ua[i], b3[k]);
                        df_mac(H, L, b3[i], wa[k]);
                        df_mac(H, L, vb[i], a3[k]);
                        df_mac(H, L, s2, S.Q[3 * i + k]);
                        if (i == k) df_add(H, L, t2);
                        df_norm(H, L);
                    }
            } else {
                // c2 s + t on the diagonal
                float dH = tH, dL = tL;
                df_mac(dH, dL, S.c2, make_float2(sH, sL));
                const float2 dg = make_float2(dH, dL);
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        float& H = aH[3 * i + k];
                        float& L = aL[3 * i + k];
                        df_mac(H, L, ua[i], b3[k]);
                        df_mac(H, L, b3[i], wa[k]);
                        if (i == k) df_add(H, L, dg);
                        df_norm(H, L);
                    }
            }
        }
        double acc[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) acc[k] = df_join(aH[k], aL[k]);
        const int na = __ldg(&A.conn[a * A.ne + e]);
        const int nb = __ldg(&A.conn[bq * A.ne + e]);
        if (!TF_IN(A.check, na, A.nn, CK_ELEM_NODE) || !TF_IN(A.check, nb, A.nn, CK_ELEM_NODE)) continue;
        bool fr[3], fc[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            fr[i] = A.fixed[3 * na + i] != 0;
            fc[i] = A.fixed[3 * nb + i] != 0;
        }
        const bool mirror = !VISC && (a != bq);
        if (MODE == kStore) {
            const size_t stride = (size_t)36 * A.ne;
            const size_t base = (size_t)(6 * a + bq) * A.ne + e;
            const size_t baseT = (size_t)(6 * bq + a) * A.ne + e;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const double v = (fr[i] || fc[k]) ? 0.0 : acc[3 * i + k];
                    A.eblk[(3 * i + k) * stride + base] = v;
                    if (mirror) A.eblk[(3 * k + i) * stride + baseT] = v;
                }
        } else {
            const int off = __ldg(&A.slot[(6 * a + bq) * A.ne + e]);
            if (!TF_IN(A.check, off, A.nval - 8 * kSlice, CK_ELEM_SLOT)) continue;
            double* dst = A.val + off;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 3; ++k)
                    if (!fr[i] && !fc[k]) atomicAdd(dst + kSlice * (3 * i + k), acc[3 * i + k]);
            if (mirror) {
                const int offT = __ldg(&A.slot[(6 * bq + a) * A.ne + e]);
                if (!TF_IN(A.check, offT, A.nval - 8 * kSlice, CK_ELEM_SLOT)) continue;
                double* dt = A.val + offT;
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int k = 0; k < 3; ++k)
                        if (!fr[i] && !fc[k]) atomicAdd(dt + kSlice * (3 * k + i), acc[3 * i + k]);
            }
        }
    }
}

// ---- parity evaluation: separate elastic / viscous outputs ----------------

struct GpEval {
    double dn[18];
    double c1, c2;
    double sdn[18];
    double pv[9];
    double pdn[18];
    double svdn[18];
};

template <int NE>
__global__ void __launch_bounds__(NE * kGauss) k_element_eval(ElemArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    GpEval* sh = reinterpret_cast<GpEval*>(smem_raw);
    const int tid = threadIdx.x;
    const int limit = A.e0 + A.count;
    {
        const int el = tid / kGauss;
        const int gp = tid - el * kGauss;
        const int e = A.e0 + blockIdx.x * NE + el;
        if (e < limit) {
            const bool visc = __ldg(&A.eta[e]) != 0.0;
            GaussPoint G;
            gauss_point(A, e, gp, visc, G);
            GpEval& S = sh[el * kGauss + gp];
            S.c1 = G.c1;
            S.c2 = G.c2;
#pragma unroll
            for (int a = 0; a < 6; ++a) {
                const double d0 = G.dn[3 * a], d1 = G.dn[3 * a + 1], d2 = G.dn[3 * a + 2];
                S.dn[3 * a] = d0;
                S.dn[3 * a + 1] = d1;
                S.dn[3 * a + 2] = d2;
                sym_apply(G.sg, d0, d1, d2, &S.sdn[3 * a]);
                if (visc) {
                    sym_apply(G.sv, d0, d1, d2, &S.svdn[3 * a]);
                    S.pdn[3 * a] = fma(G.pv[0], d0, fma(G.pv[3], d1, G.pv[6] * d2));
                    S.pdn[3 * a + 1] = fma(G.pv[1], d0, fma(G.pv[4], d1, G.pv[7] * d2));
                    S.pdn[3 * a + 2] = fma(G.pv[2], d0, fma(G.pv[5], d1, G.pv[8] * d2));
                } else {
                    S.svdn[3 * a] = S.svdn[3 * a + 1] = S.svdn[3 * a + 2] = 0.0;
                    S.pdn[3 * a] = S.pdn[3 * a + 1] = S.pdn[3 * a + 2] = 0.0;
                }
            }
#pragma unroll
            for (int k = 0; k < 9; ++k) S.pv[k] = visc ? G.pv[k] : 0.0;
        }
    }
    __syncthreads();
    for (int task = tid; task < NE * 18; task += NE * kGauss) {
        const int el = task / 18;
        const int k = task - el * 18;
        const int e = A.e0 + blockIdx.x * NE + el;
        if (e >= limit) continue;
        double se = 0.0, sv = 0.0;
#pragma unroll
        for (int gp = 0; gp < kGauss; ++gp) {
            se -= sh[el * kGauss + gp].sdn[k];
            sv -= sh[el * kGauss + gp].svdn[k];
        }
        const int a = k / 3, d = k - 3 * (k / 3);
        const bool fx = A.fixed[3 * __ldg(&A.conn[a * A.ne + e]) + d] != 0;
        const size_t r = (size_t)(e - A.e0);
        if (A.fe) A.fe[18 * r + k] = fx ? 0.0 : se;
        if (A.fv) A.fv[18 * r + k] = fx ? 0.0 : sv;
    }
    for (int task = tid; task < NE * 36; task += NE * kGauss) {
        const int el = task / 36;
        const int pr = task - el * 36;
        const int e = A.e0 + blockIdx.x * NE + el;
        if (e >= limit) continue;
        const int a = pr / 6, bq = pr - 6 * (pr / 6);
        const bool visc = __ldg(&A.eta[e]) != 0.0;
        double ke[9], kv[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) ke[k] = kv[k] = 0.0;
#pragma unroll
        for (int gp = 0; gp < kGauss; ++gp) {
            const GpEval& S = sh[el * kGauss + gp];
            const double aa[3] = {S.dn[3 * a], S.dn[3 * a + 1], S.dn[3 * a + 2]};
            const double bb[3] = {S.dn[3 * bq], S.dn[3 * bq + 1], S.dn[3 * bq + 2]};
            const double s = fma(aa[0], bb[0], fma(aa[1], bb[1], aa[2] * bb[2]));
            const double t = fma(aa[0], S.sdn[3 * bq], fma(aa[1], S.sdn[3 * bq + 1], aa[2] * S.sdn[3 * bq + 2]));
            const double dg = fma(S.c2, s, t);
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    double v = fma(S.c1 * aa[i], bb[k], fma(S.c2 * aa[k], bb[i], ke[3 * i + k]));
                    if (i == k) v += dg;
                    ke[3 * i + k] = v;
                }
            if (visc) {
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int k = 0; k < 3; ++k)
                        kv[3 * i + k] = fma(s, S.pv[3 * i + k],
                                            fma(bb[i], S.pdn[3 * a + k],
                                                fma(S.svdn[3 * a + i], bb[k], fma(-S.svdn[3 * bq + i], aa[k], kv[3 * i + k]))));
            }
        }
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
    }
}

// ---- adjoint contractions of one converged step --------------------------
//
// With lambda the adjoint of step n (A^T lambda = rhs) and
// Lam = sum_a lambda_a (x) dN_a per Gauss point:
//   dL/dlogE_e += sum_gp w dV <sigma, Lam>                 (forces are linear in E)
//   dL/dr_e    += n dt sum_{j=x,y} sum_gp w dV [<sigma,Lam> - (2 mu c_j.Lam c_j
//                  + lambda tr Lam) / J]                   (c_j = column j of Fe,
//                  d Fe / d ln Fg_jj = -Fe e_j e_j^T, ln Fg_jj = n r dt)
//   carry to step n-1 (velocity terms, d v / d u_{n-1} = -1/dt):
//     w_b += sum_gp 0.5 eta w dV / dt (Lam + Lam^T) dN_b
// Element-relative outputs: gr[e], ge[e] (no atomics), carry via atomics.
struct AdjArgs {
    const double* __restrict__ lamv;  // adjoint vector lambda [3N]
    double* __restrict__ carry;       // [3N] accumulates the carry to step n-1
    double* __restrict__ gr;          // [E] growth-rate gradient (accumulated)
    double* __restrict__ ge;          // [E] log E gradient (accumulated)
    double ndt;                       // n * dt
    double idt;
};

template <int NE>
__global__ void __launch_bounds__(NE * kGauss) k_adjoint_element(ElemArgs A, AdjArgs D) {
    __shared__ double s_gr[NE][kGauss], s_ge[NE][kGauss];
    __shared__ double s_w[NE][kGauss][18];
    const int el = threadIdx.x / kGauss, gp = threadIdx.x - (threadIdx.x / kGauss) * kGauss;
    const int e = blockIdx.x * NE + el;
    double tr = 0.0, te = 0.0;
    double w18[18];
#pragma unroll
    for (int k = 0; k < 18; ++k) w18[k] = 0.0;
    if (e < A.ne) {
        const bool visc = __ldg(&A.eta[e]) != 0.0;
        GaussPoint G;
        gauss_point(A, e, gp, visc, G);
        double Lm[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) Lm[k] = 0.0;
#pragma unroll
        for (int a = 0; a < 6; ++a) {
            const int nd = __ldg(&A.conn[a * A.ne + e]);
            const double l0 = D.lamv[3 * nd], l1 = D.lamv[3 * nd + 1], l2 = D.lamv[3 * nd + 2];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                Lm[j] = fma(l0, G.dn[3 * a + j], Lm[j]);
                Lm[3 + j] = fma(l1, G.dn[3 * a + j], Lm[3 + j]);
                Lm[6 + j] = fma(l2, G.dn[3 * a + j], Lm[6 + j]);
            }
        }
        // <sigma', Lam> with sigma' symmetric (00 11 22 01 02 12)
        const double sl = fma(G.sg[0], Lm[0], fma(G.sg[1], Lm[4], fma(G.sg[2], Lm[8],
                          fma(G.sg[3], Lm[1] + Lm[3], fma(G.sg[4], Lm[2] + Lm[6], G.sg[5] * (Lm[5] + Lm[7]))))));
        te = sl;
        // Fe columns, 1/J and the material, recomputed as in gauss_point
        const double lam = __ldg(&A.lam[e]), mu = __ldg(&A.mu[e]);
        const double trL = Lm[0] + Lm[4] + Lm[8];
        // w dV (2 mu c.Lam c + lambda tr Lam) / J = 2 mu sc c.Lam c + c1 tr Lam
        const double sc = G.sc;
        (void)lam;
        double t = 0.0;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const double c0 = G.fe[j], c1v = G.fe[3 + j], c2v = G.fe[6 + j];
            const double Lc0 = fma(Lm[0], c0, fma(Lm[1], c1v, Lm[2] * c2v));
            const double Lc1 = fma(Lm[3], c0, fma(Lm[4], c1v, Lm[5] * c2v));
            const double Lc2 = fma(Lm[6], c0, fma(Lm[7], c1v, Lm[8] * c2v));
            const double cLc = fma(c0, Lc0, fma(c1v, Lc1, c2v * Lc2));
            t += sl - fma(2.0 * mu * sc, cLc, G.c1 * trL);
        }
        tr = D.ndt * t;
        if (visc) {
            const double hw = 0.5 * __ldg(&A.eta[e]) * G.wdv * D.idt;
            double S[9];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 3; ++k) S[3 * i + k] = hw * (Lm[3 * i + k] + Lm[3 * k + i]);
#pragma unroll
            for (int b = 0; b < 6; ++b) {
                const double d0 = G.dn[3 * b], d1 = G.dn[3 * b + 1], d2 = G.dn[3 * b + 2];
                w18[3 * b] = fma(S[0], d0, fma(S[1], d1, S[2] * d2));
                w18[3 * b + 1] = fma(S[3], d0, fma(S[4], d1, S[5] * d2));
                w18[3 * b + 2] = fma(S[6], d0, fma(S[7], d1, S[8] * d2));
            }
        }
    }
    s_gr[el][gp] = tr;
    s_ge[el][gp] = te;
#pragma unroll
    for (int k = 0; k < 18; ++k) s_w[el][gp][k] = w18[k];
    __syncthreads();
    if (e < A.ne && gp == 0) {
        double a = 0.0, b = 0.0;
#pragma unroll
        for (int q = 0; q < kGauss; ++q) {
            a += s_gr[el][q];
            b += s_ge[el][q];
        }
        D.gr[e] += a;
        D.ge[e] += b;
    }
    for (int task = threadIdx.x; task < NE * 18; task += NE * kGauss) {
        const int l = task / 18, k = task - 18 * (task / 18);
        const int ee = blockIdx.x * NE + l;
        if (ee >= A.ne || __ldg(&A.eta[ee]) == 0.0) continue;
        double v = 0.0;
#pragma unroll
        for (int q = 0; q < kGauss; ++q) v += s_w[l][q][k];
        const int nd = __ldg(&A.conn[(k / 3) * A.ne + ee]);
        atomicAdd(&D.carry[3 * nd + (k % 3)], v);
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
    A.idt = 1.0 / h->dt;
    A.val = d.val;
    A.g = d.g;
    A.eblk = d.eblk;
    A.ef = d.ef;
    A.elem_seg = d.elem_seg;
    A.seg_active = d.seg_active;
    A.masked = d.nseg > 1 ? 1 : 0;
    A.nn = d.nn;
    A.nval = d.nval;
    A.check = d.check;
    return A;
}

template <int NE, int MODE, bool VISC>
tf_status launch_fast(tf_handle* h, const ElemArgs& A) {
    const size_t smem = sizeof(GpFast<VISC>) * NE * kGauss;
    static int configured_device = -1;
    if (configured_device != h->device) {
        TF_CUDA(cudaFuncSetAttribute(k_element<NE, MODE, VISC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        configured_device = h->device;
    }
    k_element<NE, MODE, VISC><<<cdiv(A.ne, NE), NE * kGauss * kTpg, smem, h->stream>>>(A);
    TF_LAUNCH_CHECK(h);
    return TF_OK;
}

template <int NE>
tf_status launch_ne(tf_handle* h, const ElemArgs& A) {
    const bool visc = h->d.any_visc;
    if (h->opt.deterministic) return visc ? launch_fast<NE, kStore, true>(h, A) : launch_fast<NE, kStore, false>(h, A);
    return visc ? launch_fast<NE, kAtomic, true>(h, A) : launch_fast<NE, kAtomic, false>(h, A);
}

tf_status launch_with(tf_handle* h, const ElemArgs& A, int ne_per_cta) {
    switch (ne_per_cta) {
        case 8: return launch_ne<8>(h, A);
        case 32: return launch_ne<32>(h, A);
        default: return launch_ne<16>(h, A);
    }
}

}  // namespace

tf_status launch_element(tf_handle* h) {
    const ElemArgs A = make_args(h);
    if (A.ne <= 0) return TF_OK;
    return launch_with(h, A, h->elem_cta);
}

// Picks the prisms-per-CTA tile (8, 16 or 32 prisms x 6 Gauss points) by
// timing each candidate on the handle's own mesh; run once per handle before
// the first assembly.  Results do not depend on the choice.
tf_status autotune_element(tf_handle* h) {
    if (h->tuned || h->d.ne <= 0) return TF_OK;
    h->tuned = true;
    if (h->opt.autotune_off) return TF_OK;
    const ElemArgs A = make_args(h);
    const int cand[3] = {8, 16, 32};
    float best = 1e30f;
    for (int c : cand) {
        if (launch_with(h, A, c) != TF_OK) continue;  // warm-up (and smem attribute)
        TF_CUDA(cudaEventRecord(h->ev[4], h->stream));
        for (int r = 0; r < 2; ++r) {
            const tf_status s = launch_with(h, A, c);
            if (s != TF_OK) return s;
        }
        TF_CUDA(cudaEventRecord(h->ev[5], h->stream));
        TF_CUDA(cudaEventSynchronize(h->ev[5]));
        float ms = 0.f;
        TF_CUDA(cudaEventElapsedTime(&ms, h->ev[4], h->ev[5]));
        if (ms < best) {
            best = ms;
            h->elem_cta = c;
        }
    }
    return TF_OK;
}

tf_status launch_adjoint_element(tf_handle* h, const double* lamv, double* carry, double* gr, double* ge,
                                 double ndt) {
    ElemArgs A = make_args(h);
    if (A.ne <= 0) return TF_OK;
    AdjArgs D{lamv, carry, gr, ge, ndt, 1.0 / h->dt};
    constexpr int NE = 16;
    k_adjoint_element<NE><<<cdiv(A.ne, NE), NE * kGauss, 0, h->stream>>>(A, D);
    TF_LAUNCH_CHECK(h);
    return TF_OK;
}

tf_status launch_element_eval(tf_handle* h, int e0, int count, double* Ke, double* Kv, double* fe, double* fv) {
    ElemArgs A = make_args(h);
    A.e0 = e0;
    A.count = count;
    A.Ke = Ke;
    A.Kv = Kv;
    A.fe = fe;
    A.fv = fv;
    if (count <= 0) return TF_OK;
    constexpr int NE = 8;
    const size_t smem = sizeof(GpEval) * NE * kGauss;
    static bool configured = false;
    if (!configured) {
        TF_CUDA(cudaFuncSetAttribute(k_element_eval<NE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        configured = true;
    }
    k_element_eval<NE><<<cdiv(count, NE), NE * kGauss, smem, h->stream>>>(A);
    TF_LAUNCH_CHECK(h);
    return TF_OK;
}

}  // namespace tf
