// Node-level kernels of the Newton assembly and the per-step set-up.
//
//   k_prepare          calculateDisplacementMatrix (NewtonRaphsonSolver.cpp:148-152),
//                      calculateExternalViscousForcesForNR (:297-324),
//                      addImplicitKViscousExternalToJacobian (:326-348),
//                      the diagonal of calcutateFixedK (:237-255)
//   k_gather_*         order-fixed assembly: every block / DOF sums its element
//                      contributions in element order, as the reference's serial
//                      scatter does (:273-295)
//   k_growth           ShapeBase::calculateFgFromRates (ShapeBase.cpp:396-421)
//                      and growShapeByFg (:1215-1251)
//   k_face_area,       Prism::calculateApicalArea / calculateBasalArea
//   k_node_area        (Prism.cpp:2424-2503) and
//                      Simulation::updateNodeViscositySurfaces (Simulation.cpp:7563-7581)
//   k_block_inverse    3x3 diagonal blocks for the block-Jacobi preconditioner
//   k_update           updateUkInIteration (:755-761) with |du|^2
#include "tf_internal.cuh"

namespace tf {

namespace {

__global__ void k_prepare(int nn, const double* __restrict__ uk, const double* __restrict__ un, double dt,
                          const double* __restrict__ area, const double* __restrict__ ext_visc,
                          const uint8_t* __restrict__ fixed, const int* __restrict__ diag, double* __restrict__ vel,
                          double* __restrict__ g, double* __restrict__ val, int write_diag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    const double idt = 1.0 / dt;
    const double A = area[i];
    const double Adt = A / dt;
    double* D = val + diag[i];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int k = 3 * i + d;
        const double v = (uk[k] - un[k]) * idt;
        vel[k] = v;
        const bool fx = fixed[k] != 0;
        g[k] = fx ? 0.0 : (A * ext_visc[k] * v) * -1.0;
        if (write_diag) D[kSlice * 4 * d] = fx ? 1.0 : Adt * ext_visc[k];
    }
}

// Deterministic assembly: block values.  glist holds element-slot ids
// (p * ne + e) sorted by (block, e), so each block adds its contributions in
// element order.
__global__ void k_gather_blocks(int64_t nnzb, int ne, const int* __restrict__ gptr, const int* __restrict__ glist,
                                const double* __restrict__ eblk, const int* __restrict__ rowof,
                                const int* __restrict__ colidx, const int* __restrict__ bofs,
                                const double* __restrict__ area,
                                const double* __restrict__ ext_visc, const uint8_t* __restrict__ fixed, double dt,
                                double* __restrict__ val) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nnzb) return;
    const size_t stride = (size_t)36 * ne;
    double acc[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) acc[k] = 0.0;
    for (int p = gptr[b]; p < gptr[b + 1]; ++p) {
        const size_t id = (size_t)glist[p];
#pragma unroll
        for (int k = 0; k < 9; ++k) acc[k] += eblk[k * stride + id];
    }
    const int row = rowof[b];
    if (colidx[b] == row) {
        const double Adt = area[row] / dt;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int k = 3 * row + d;
            acc[4 * d] = fixed[k] ? 1.0 : Adt * ext_visc[k] + acc[4 * d];
        }
    }
    double* dst = val + bofs[b];
#pragma unroll
    for (int k = 0; k < 9; ++k) dst[kSlice * k] = acc[k];
}

// Deterministic assembly: forces.  flist holds (a * ne + e) sorted by
// (node, e).
__global__ void k_gather_forces(int nn, int ne, const int* __restrict__ fptr, const int* __restrict__ flist,
                                const double* __restrict__ ef, const uint8_t* __restrict__ fixed,
                                double* __restrict__ g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    double s[3] = {0.0, 0.0, 0.0};
    for (int p = fptr[i]; p < fptr[i + 1]; ++p) {
        const int id = flist[p];
        const int a = id / ne, e = id - a * ne;
#pragma unroll
        for (int d = 0; d < 3; ++d) s[d] += ef[(size_t)(3 * a + d) * ne + e];
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int k = 3 * i + d;
        g[k] = fixed[k] ? 0.0 : s[d] + g[k];
    }
}

__global__ void k_growth(int ne, double dt, const double* __restrict__ rates, double* __restrict__ Fg,
                         double* __restrict__ invFg) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    double inc[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) inc[d] = exp(rates[d * ne + e] * 1.0 * dt);
    double F[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) F[3 * i + j] = inc[i] * Fg[(3 * i + j) * ne + e];
    double inv[9];
    inv3_cof(F, inv);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        Fg[k * ne + e] = F[k];
        invFg[k * ne + e] = inv[k];
    }
}

__device__ __forceinline__ double face_area(const double* __restrict__ x, int n0, int n1, int n2) {
    const double Threshold = 1E-5;
    double s1[3], s2[3], Side1 = 0.0, Side2 = 0.0, costet = 0.0, Area = 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        s1[i] = x[3 * n1 + i] - x[3 * n0 + i];
        s2[i] = x[3 * n2 + i] - x[3 * n0 + i];
        costet += s1[i] * s2[i];
        Side1 += s1[i] * s1[i];
        Side2 += s2[i] * s2[i];
    }
    if (Side1 > Threshold && Side2 > Threshold) {
        Side1 = sqrt(Side1);
        Side2 = sqrt(Side2);
        costet /= (Side1 * Side2);
        const double sinTetSq = 1 - costet * costet;
        double sintet = 0;
        if (sinTetSq > Threshold) sintet = sqrt(sinTetSq);
        Area = Side1 * Side2 * sintet / 2.0;
    }
    return Area;
}

// farea[2][ne]: apical face (nodes 3,4,5), basal face (nodes 0,1,2)
__global__ void k_face_area(int ne, const int* __restrict__ conn, const int* __restrict__ exposure,
                            const double* __restrict__ x, double* __restrict__ farea) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int ex = exposure[e];
    double ap = 0.0, ba = 0.0;
    if (ex & 1) ap = face_area(x, conn[3 * ne + e], conn[4 * ne + e], conn[5 * ne + e]);
    if (ex & 2) ba = face_area(x, conn[0 * ne + e], conn[1 * ne + e], conn[2 * ne + e]);
    farea[e] = ap;
    farea[ne + e] = ba;
}

// alist holds (face * ne + e), sorted by (node, e, face): the summation order
// of ShapeBase::assignViscositySurfaceAreaToNodes called in element order.
__global__ void k_node_area(int nn, const int* __restrict__ aptr, const int* __restrict__ alist,
                            const double* __restrict__ farea, double* __restrict__ area) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    double s = 0.0;
    for (int p = aptr[i]; p < aptr[i + 1]; ++p) s += farea[alist[p]] / 3;
    area[i] = s;
}

__global__ void k_block_inverse(int nn, const int* __restrict__ diag, const double* __restrict__ val,
                                double* __restrict__ dinv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    double M[9], inv[9];
    const double* D = val + diag[i];
#pragma unroll
    for (int k = 0; k < 9; ++k) M[k] = D[kSlice * k];
    inv3_cof(M, inv);
#pragma unroll
    for (int k = 0; k < 9; ++k) dinv[9 * (size_t)i + k] = inv[k];
}

}  // namespace

tf_status launch_prepare(tf_handle* h) {
    Device& d = h->d;
    if (!h->opt.deterministic) TF_CUDA(cudaMemsetAsync(d.val, 0, sizeof(double) * (size_t)d.nval, h->stream));
    k_prepare<<<cdiv(d.nn, 256), 256, 0, h->stream>>>(d.nn, d.uk, d.un, h->dt, d.area, d.ext_visc, d.fixed, d.diag,
                                                       d.vel, d.g, d.val, h->opt.deterministic ? 0 : 1);
    TF_LAUNCH_CHECK(h);
    return TF_OK;
}

tf_status launch_deterministic_gather(tf_handle* h) {
    Device& d = h->d;
    k_gather_blocks<<<cdiv(d.nnzb, 256), 256, 0, h->stream>>>(d.nnzb, d.ne, d.gptr, d.glist, d.eblk, d.rowof, d.colidx, d.bofs,
                                                              d.area, d.ext_visc, d.fixed, h->dt, d.val);
    TF_LAUNCH_CHECK(h);
    k_gather_forces<<<cdiv(d.nn, 256), 256, 0, h->stream>>>(d.nn, d.ne, d.fptr, d.flist, d.ef, d.fixed, d.g);
    TF_LAUNCH_CHECK(h);
    return TF_OK;
}

tf_status launch_growth(tf_handle* h) {
    Device& d = h->d;
    k_growth<<<cdiv(d.ne, 256), 256, 0, h->stream>>>(d.ne, h->dt, d.rates, d.Fg, d.invFg);
    TF_LAUNCH_CHECK(h);
    return TF_OK;
}

tf_status launch_viscosity_surfaces(tf_handle* h) {
    Device& d = h->d;
    k_face_area<<<cdiv(d.ne, 256), 256, 0, h->stream>>>(d.ne, d.conn, d.exposure, d.uk, d.farea);
    TF_LAUNCH_CHECK(h);
    k_node_area<<<cdiv(d.nn, 256), 256, 0, h->stream>>>(d.nn, d.aptr, d.alist, d.farea, d.area);
    TF_LAUNCH_CHECK(h);
    return TF_OK;
}

tf_status launch_block_inverse(tf_handle* h) {
    Device& d = h->d;
    k_block_inverse<<<cdiv(d.nn, 256), 256, 0, h->stream>>>(d.nn, d.diag, d.val, d.dinv);
    TF_LAUNCH_CHECK(h);
    return TF_OK;
}

}  // namespace tf
