// Internal declarations shared by the CUDA translation units of libtfgpu.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tf_gpu.h"

namespace tf {

// Element-kernel tiling: NE prisms per CTA, one thread per Gauss point.
constexpr int kGauss = 6;
constexpr int kElemPerCta = 16;
constexpr int kCtaThreads = kElemPerCta * kGauss;  // 96

struct Device {
    // sizes
    int nn = 0, ne = 0;
    int64_t nnzb = 0;
    bool any_visc = false;
    // mesh / material (SoA)
    int* conn = nullptr;        // [6][ne]
    double* gx = nullptr;       // [18][6*ne] reference shape gradients
    double* wdet = nullptr;     // [6*ne] w * det(dX/dxi)
    double* detdxde = nullptr;  // [6*ne]
    double* Fg = nullptr;       // [9][ne]
    double* invFg = nullptr;    // [9][ne]
    double* rates = nullptr;    // [3][ne] growth rates (1/s)
    double* lam = nullptr;      // [ne]
    double* mu = nullptr;       // [ne]
    double* eta = nullptr;      // [ne]
    int* exposure = nullptr;    // [ne] bit0 apical face exposed, bit1 basal face exposed
    int* aptr = nullptr;        // [nn+1] exposed faces touching each node
    int* alist = nullptr;       // face ids (face*ne + e) sorted by (node, e, face)
    double* farea = nullptr;    // [2][ne] apical / basal face areas
    uint8_t* fixed = nullptr;   // [3nn]
    double* ext_visc = nullptr; // [3nn]
    double* area = nullptr;     // [nn]
    // block sparse A = K^T (3x3 blocks, row-major inside a block)
    int* rowptr = nullptr;      // [nn+1]
    int* colidx = nullptr;      // [nnzb]
    int* diag = nullptr;        // [nn] block index of (i,i)
    int* rowof = nullptr;       // [nnzb] block row of each block
    int* slot = nullptr;        // [36][ne] block index of pair (a,b)
    double* val = nullptr;      // [9*nnzb]
    // deterministic assembly: per-element blocks and the gather lists
    double* eblk = nullptr;     // [9][36*ne] element blocks (A orientation)
    double* ef = nullptr;       // [18][ne] element forces
    int* gptr = nullptr;        // [nnzb+1] contributions per block
    int* glist = nullptr;       // [36*ne] (element-slot ids p*ne+e, ordered)
    int* fptr = nullptr;        // [nn+1] contributions per node
    int* flist = nullptr;       // [6*ne]
    // Newton state
    double* uk = nullptr;
    double* un = nullptr;
    double* vel = nullptr;
    double* g = nullptr;        // rhs gSum
    double* du = nullptr;
    double* dinv = nullptr;     // [9nn] inverse diagonal blocks
    // Krylov work vectors
    double *r = nullptr, *p = nullptr, *z = nullptr, *q = nullptr, *rhat = nullptr, *s = nullptr, *t = nullptr, *sh = nullptr;
    double* scal = nullptr;     // device scalars, S_COUNT per instance
    double* part = nullptr;     // per-CTA partial sums [3][ncta]
    double* host_scal = nullptr; // pinned mirror of scal
    unsigned* tickets = nullptr; // per-instance reduction tickets
    // instances (a batch is one block-diagonal system; a single mesh is a
    // batch of one)
    int nseg = 1;
    int ncta = 0;               // CTAs of the node-parallel kernels
    int* seg_node0 = nullptr;   // [nseg+1] node offsets
    int* elem_seg = nullptr;    // [ne] instance of each element
    int* cta_seg = nullptr;     // [ncta] instance of each CTA
    int* cta_node0 = nullptr;   // [ncta] first node of each CTA
    int* cta_node1 = nullptr;   // [ncta] end node of each CTA
    int* seg_cta0 = nullptr;    // [nseg+1] CTA ranges per instance
    int* seg_active = nullptr;  // [nseg] 1 while the instance's Newton loop runs
    int* seg_solve = nullptr;   // [nseg] instances a linear solve works on
    // adjoint (allocated by the first tf_adj_forward)
    int* tblk = nullptr;        // [nnzb] block index of the transposed block
    double* valT = nullptr;     // [9*nnzb] transposed block values
    double* lamv = nullptr;     // [3nn] adjoint of the current step
    double* carry = nullptr;    // [3nn] carry to the previous step
    double* dldu = nullptr;     // [3nn] dL/du at the final state
    double* gr = nullptr;       // [ne] dL/d growth rate
    double* ge = nullptr;       // [ne] dL/d log E
    double* nu = nullptr;       // [ne] Poisson ratios (clamped to [0, 0.5])
    int* apical = nullptr;      // [nn] 1 for apical nodes
};

// Indices into Device::scal (device-resident Krylov scalars).
enum Scal {
    S_RZ = 0, S_RZ_OLD, S_PQ, S_ALPHA, S_BETA, S_OMEGA, S_RHO, S_RHO_OLD,
    S_TS, S_TT, S_RR, S_BB, S_RR0, S_DU2, S_FLAG, S_ITER, S_TOL2, S_WHY, S_COUNT = 32
};

constexpr int kNodeThreads = 256;    // nodes per CTA of the node-parallel kernels

}  // namespace tf

struct tf_handle {
    tf::Device d;
    tf_options opt{};
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[8] = {};
    double dt = 60.0;
    bool have_rates = false;
    bool assembled = false;
    int64_t launches = 0;
    int method = 1;  // 1 CG, 2 BiCGStab
    std::vector<int> h_conn;
    std::vector<int> h_rowptr, h_colidx;
    std::vector<uint8_t> h_fixed;
    std::vector<double> h_nu;                   // Poisson ratios, clamped as the material setup does
    std::vector<int> h_apical;                  // 1 for apical nodes (tissue placement 1)
    std::vector<int> h_seg_node0, h_seg_elem0;  // host copies of the instance offsets
    std::vector<int> h_active;                  // host mirror of seg_active
    int elem_cta = 16;                          // prisms per CTA of the element kernel (autotuned)
    bool tuned = false;
    cudaGraphExec_t graph[2][4] = {};           // Krylov chunks [method-1][log2(chunk/8)]
    int64_t graph_kernels[2][4] = {};
};

namespace tf {

void set_error(const std::string& msg);
tf_status cuda_fail(cudaError_t e, const char* what);

#define TF_CUDA(call)                                              \
    do {                                                           \
        cudaError_t _e = (call);                                   \
        if (_e != cudaSuccess) return ::tf::cuda_fail(_e, #call);  \
    } while (0)

#define TF_LAUNCH_CHECK(h)                                                   \
    do {                                                                     \
        (h)->launches++;                                                     \
        cudaError_t _e = cudaGetLastError();                                 \
        if (_e != cudaSuccess) return ::tf::cuda_fail(_e, "kernel launch");  \
    } while (0)

// Launchers implemented in the .cu files (all asynchronous on h->stream).
tf_status launch_prepare(tf_handle* h);
tf_status launch_element(tf_handle* h);
tf_status launch_element_eval(tf_handle* h, int e0, int count, double* Ke, double* Kv, double* fe, double* fv);
tf_status launch_deterministic_gather(tf_handle* h);
tf_status launch_growth(tf_handle* h);
tf_status launch_viscosity_surfaces(tf_handle* h);
tf_status launch_block_inverse(tf_handle* h);
tf_status krylov_solve(tf_handle* h, int* iters, double* relres);
tf_status launch_update(tf_handle* h);
tf_status autotune_element(tf_handle* h);
tf_status launch_adjoint_element(tf_handle* h, const double* lamv, double* carry, double* gr, double* ge, double ndt);
void destroy_graphs(tf_handle* h);

inline int cdiv(int64_t a, int64_t b) { return static_cast<int>((a + b - 1) / b); }

}  // namespace tf
