// Internal declarations shared by the CUDA translation units of libtfgpu.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tf_gpu.h"

namespace tf {

// NVTX range for the phases of a step (begin_step, assembly, solve, Newton
// iteration, multigrid set-up, packing detection, adjoint passes): visible
// to profilers, a no-op without one.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// Checked build (-DTF_CHECKED, libtfgpu_checked.so): the indexed accesses of
// the main kernels test their index first; an index outside its array
// records the site's code in the handle's device word `check` (the first
// failing site wins) and the access is skipped, so nothing reads or writes
// out of bounds.  The host turns a recorded code into TF_CUDA_ERROR after
// the call.  In the normal build the tests compile away.
enum CheckSite {
    CK_ELEM_NODE = 1,    // prism node id < n_nodes (element kernels)
    CK_ELEM_SLOT,        // scatter offset inside the block values
    CK_SPMV_COL,         // column of the Krylov product < n_nodes
    CK_EXTRA_COL,        // column of an extra block < n_nodes
    CK_V0_COL,           // column of the level-0 smoother product < n_nodes
    CK_RESTRICT_ROW,     // fine node of a restriction block < fine level size
    CK_PROLONG_COL,      // coarse node of a prolongation block < coarse level size
    CK_PACK_NODE,        // node of a packing couple < n_nodes
    CK_PACK_BLOCK,       // extra block of a packing couple < extra blocks
    CK_GROW_NODE,        // node of a prism in the growth update < n_nodes
    CK_GROW_PRISM,       // prism whose position a prism takes < n_elems
};
#ifdef TF_CHECKED
__device__ __forceinline__ bool check_in(int* flag, long long i, long long n, int code) {
    if (i >= 0 && i < n) return true;
    if (flag) atomicCAS(flag, 0, code);
    return false;
}
#define TF_IN(flag, i, n, code) ::tf::check_in((flag), (long long)(i), (long long)(n), (code))
#else
#define TF_IN(flag, i, n, code) true
#endif

// Sliced block storage: a slot holds one 3x3 block for each of 32 rows.
constexpr int kSlice = 32;
constexpr int kSlotDoubles = 9 * kSlice;

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
    // block sparse A = K^T, 3x3 blocks.  Logical pattern: CSR over block rows
    // (rowptr, colidx; block index b).  Values are stored sliced: the 32 rows
    // of one warp of the node-parallel kernels share slots, slot s holding the
    // k-th block of each of the 32 rows; entry (r, c) of the block of lane l
    // is val[s * 288 + 32 * (3 r + c) + l].  A block's base offset is
    // s * 288 + l; padding slots hold zeros and a valid column.
    int* rowptr = nullptr;      // [nn+1]
    int* colidx = nullptr;      // [nnzb]
    int* diag = nullptr;        // [nn] base offset of block (i,i)
    int* rowof = nullptr;       // [nnzb] block row of each block
    int* bofs = nullptr;        // [nnzb] base offset of block b
    int* slot = nullptr;        // [36][ne] base offset of the block of pair (a,b)
    int* wslot0 = nullptr;      // [ncta * kWarps + 1] first slot of each warp's rows
    int* scol = nullptr;        // [nslots * 32] column of each slot and lane
    int64_t nval = 0;           // doubles in val (nslots * 288)
    double* val = nullptr;      // [nval]
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
    // blocks of K entries added through tf_add_K_triplets at node pairs outside
    // the element pattern (contact-type couplings): CSR over block rows of A,
    // row-major 3x3 values, cleared at every assembly
    int* xrow = nullptr;        // [nn+1] (null: none)
    int* xcol = nullptr;        // [nxb]
    double* xval = nullptr;     // [9 nxb]
    int64_t nxb = 0;
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
    int* check = nullptr;       // checked build: code of the first failed index check (0: none)
};

// Indices into Device::scal (device-resident Krylov scalars).
enum Scal {
    S_RZ = 0, S_RZ_OLD, S_PQ, S_ALPHA, S_BETA, S_OMEGA, S_RHO, S_RHO_OLD,
    S_TS, S_TT, S_RR, S_BB, S_RR0, S_DU2, S_FLAG, S_ITER, S_TOL2, S_WHY,
    S_SINV,  // largest |du| / |g| of the instance's solves so far (kept across solves)
    S_COUNT = 32
};

constexpr int kNodeThreads = 256;    // nodes per CTA of the node-parallel kernels
constexpr int kWarps = kNodeThreads / 32;
constexpr int kAmgMaxLevels = 10;

struct Amg;      // multigrid hierarchy (tf_amg.cu)
struct Packing;  // packing between tissue surfaces (tf_packing.cu)
struct Growth;   // growth functions (tf_growth.cu)
struct BindPlan; // device program of the bound-DOF merges (tf_api.cu)

// State of the device-side Newton loop (tf_krylov.cu), in device memory with a
// pinned host mirror.
struct NewtonDev {
    int k;                     // Newton iterations of the step so far
    int exc;                   // 1: the loop stopped for the host (solve failed, non-finite or near-threshold update)
    int krylov_total, krylov_max;
    unsigned long long t0, t_asm;  // assembly timing (%globaltimer, ns)
    double dunorm[32];         // largest |du| over the instances, per Newton iteration
};

// A Newton update from a solve stopped at the update accuracy atol (looser
// than krylov_rtol) whose norm dn lies this close to newton_tol is solved
// again to krylov_rtol before the Newton test: the band is a thousand times
// the accuracy asked of the update (at least 1e-3 of the tolerance), so the
// loosening cannot move |du| across the tolerance unnoticed.
__host__ __device__ __forceinline__ bool near_newton_tol(double dn, double tol, double atol) {
    const double band = fmax(1e3 * atol, 1e-3 * tol);
    return fabs(dn - tol) <= band;
}

// Inverse of a 3x3 matrix (row-major) by cofactors.
__device__ __forceinline__ void inv3_cof(const double* M, double* inv) {
    const double c0 = M[4] * M[8] - M[5] * M[7];
    const double c1 = M[5] * M[6] - M[3] * M[8];
    const double c2 = M[3] * M[7] - M[4] * M[6];
    const double det = M[0] * c0 + M[1] * c1 + M[2] * c2;
    const double r = 1.0 / det;
    inv[0] = c0 * r;
    inv[1] = (M[2] * M[7] - M[1] * M[8]) * r;
    inv[2] = (M[1] * M[5] - M[2] * M[4]) * r;
    inv[3] = c1 * r;
    inv[4] = (M[0] * M[8] - M[2] * M[6]) * r;
    inv[5] = (M[2] * M[3] - M[0] * M[5]) * r;
    inv[6] = c2 * r;
    inv[7] = (M[1] * M[6] - M[0] * M[7]) * r;
    inv[8] = (M[0] * M[4] - M[1] * M[3]) * r;
}

// Values combined over a CTA of NT threads: kind[q] 0 sum, 1 min, 2 max; warp
// shuffles, then warp 0 over the warps' values (fixed order: deterministic);
// every thread gets the results in v.  A dependent chain of FP64 operations
// costs on the order of 100 cycles per step on this part, so no fold here
// runs on one thread alone.  sm: shared scratch of N x (NT/32 + 1) doubles.
__device__ __forceinline__ double combine_as(int kind, double a, double b) {
    return kind == 0 ? a + b : (kind == 1 ? fmin(a, b) : fmax(a, b));
}
__device__ __forceinline__ double identity_of(int kind) {
    return kind == 0 ? 0.0 : (kind == 1 ? INFINITY : -INFINITY);
}
template <int NT, int N>
__device__ __forceinline__ void cta_combine(double (&v)[N], const int (&kind)[N], double (*sm)[NT / 32 + 1]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < N; ++q) {
        double x = v[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x = combine_as(kind[q], x, __shfl_down_sync(0xffffffffu, x, o));
        if (lane == 0) sm[q][warp] = x;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int q = 0; q < N; ++q) {
            double x = lane < NT / 32 ? sm[q][lane] : identity_of(kind[q]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x = combine_as(kind[q], x, __shfl_down_sync(0xffffffffu, x, o));
            if (lane == 0) sm[q][NT / 32] = x;
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < N; ++q) v[q] = sm[q][NT / 32];
    __syncthreads();
}

// Sums over the CTA (cta_combine with every kind a sum).
template <int NT, int N>
__device__ __forceinline__ void cta_sum(double (&v)[N], double (*sm)[NT / 32 + 1]) {
    int kind[N];
#pragma unroll
    for (int q = 0; q < N; ++q) kind[q] = 0;
    cta_combine<NT, N>(v, kind, sm);
}

// Simulation::calculateBoundingBox (Simulation.cpp:9148-9185) starts its
// corners at +-1e5 and tests a node for the maximum only when the node did
// not lower the running minimum (a running "else if").  A node other than 0
// that holds the largest coordinate never lowers it, so given hi1, the
// maximum over nodes 1.., the reference's maximum on axis k is hi1 -- unless
// node 0 alone holds the largest coordinate; then the CTA replays the running
// minimum: per-thread chunks in node order, an exclusive min-scan over the
// chunks, the chunks walked in order.  Every thread of the CTA (NT threads)
// calls it with the same hi1; scan is NT doubles of shared memory.
constexpr double kBoxCorner = 100000.0;

template <int NT>
__device__ double reference_box_max(int nn, const double* __restrict__ pos, int k, double hi1, double* scan) {
    if (nn <= 0 || !(pos[k] > hi1)) return fmax(hi1, -kBoxCorner);
    const int t = threadIdx.x;
    const int chunk = (nn + NT - 1) / NT;
    const int i0 = min(nn, t * chunk), i1 = min(nn, i0 + chunk);
    double cm = INFINITY;
    for (int i = i0; i < i1; ++i) cm = fmin(cm, pos[3 * (size_t)i + k]);
    __syncthreads();
    scan[t] = cm;
    __syncthreads();
    for (int o = 1; o < NT; o <<= 1) {
        const double v = t >= o ? scan[t - o] : INFINITY;
        __syncthreads();
        scan[t] = fmin(scan[t], v);
        __syncthreads();
    }
    double run = t > 0 ? fmin(kBoxCorner, scan[t - 1]) : kBoxCorner;
    double up = -kBoxCorner;
    for (int i = i0; i < i1; ++i) {
        const double p = pos[3 * (size_t)i + k];
        if (p < run) run = p;
        else if (p > up) up = p;
    }
    __syncthreads();
    scan[t] = up;
    __syncthreads();
    for (int o = NT / 2; o > 0; o >>= 1) {
        if (t < o) scan[t] = fmax(scan[t], scan[t + o]);
        __syncthreads();
    }
    const double r = scan[0];
    __syncthreads();
    return r;
}

// Programmatic dependent launch for the chains of short kernels of the
// linear solve: a kernel launched with launch_pdl may be scheduled as its
// predecessor's blocks exit, hiding the launch gap; pdl_enter makes it wait
// for the predecessor's completion (and memory) before anything else.  (An
// explicit early trigger, letting the next kernel's blocks sit resident
// while the current one runs, measured 10 % slower on the 320,000-prism
// step; this form measured ~3 % faster than plain launches.)  A no-op for
// ordinary launches.
__device__ __forceinline__ void pdl_enter() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline void launch_pdl_smem(void (*kernel)(KArgs...), int grid, int block, size_t smem, cudaStream_t st,
                            Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

template <class... KArgs, class... Args>
inline void launch_pdl(void (*kernel)(KArgs...), int grid, int block, cudaStream_t st, Args... args) {
    launch_pdl_smem(kernel, grid, block, 0, st, args...);
}

// y = this thread's row of the sliced block matrix times x.  T is the
// storage type of the values (double for the Krylov operator, float for the
// copy the multigrid smoother reads); products and sums are FP64.  The thread is
// node cta_node0[blockIdx.x] + threadIdx.x of a node-parallel kernel (CTAs
// of kNodeThreads); the warp walks its slots together, each lane reading
// its own row's block, so every load of a block entry or column is one
// coalesced access.
template <class T, int U = 2>
__device__ __forceinline__ void sliced_row(const int* __restrict__ wslot0, const int* __restrict__ scol,
                                           const T* __restrict__ val, const double* __restrict__ x, double y[3],
                                           int nn = 0, int* check = nullptr) {
    const int lane = threadIdx.x & 31;
    const int wg = blockIdx.x * kWarps + (threadIdx.x >> 5);
    const int s0 = __ldg(&wslot0[wg]), s1 = __ldg(&wslot0[wg + 1]);
    double y0 = 0.0, y1 = 0.0, y2 = 0.0;
    const int* __restrict__ col = scol + lane;
    const T* __restrict__ a = val + lane;
#pragma unroll U
    for (int s = s0; s < s1; ++s) {
        const int j = __ldg(&col[(size_t)s * kSlice]);
        if (!TF_IN(check, j, nn, CK_SPMV_COL)) continue;
        const T* __restrict__ v = a + (size_t)s * kSlotDoubles;
        const double x0 = x[3 * j], x1 = x[3 * j + 1], x2 = x[3 * j + 2];
        y0 = fma((double)__ldg(&v[0]), x0, fma((double)__ldg(&v[32]), x1, fma((double)__ldg(&v[64]), x2, y0)));
        y1 = fma((double)__ldg(&v[96]), x0, fma((double)__ldg(&v[128]), x1, fma((double)__ldg(&v[160]), x2, y1)));
        y2 = fma((double)__ldg(&v[192]), x0, fma((double)__ldg(&v[224]), x1, fma((double)__ldg(&v[256]), x2, y2)));
    }
    y[0] = y0;
    y[1] = y1;
    y[2] = y2;
}

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
    std::vector<int> h_rowptr, h_colidx, h_bofs;
    std::vector<std::vector<int>> h_xcols;      // extra block columns per block row (sorted)
    std::vector<int> h_xrow;                    // CSR offsets of the extra blocks on the device
    std::vector<int> h_xcol_prev;               // their columns in that layout
    std::vector<int> bind_slave, bind_master;   // bound DOF couples (NRSolver::slaveMasterList)
    bool bound_applied = false;                 // the couples are applied to the current assembly
    double solve_atol = 0.0;                    // absolute update accuracy of the current solve (0: off)
    int mg_kept = 0;                            // time steps since the multigrid's last full rebuild
    int mg_ref_iters = -1;                      // Krylov iterations of the first solve after that rebuild
    bool mg_force = false;                      // rebuild the coarse levels at the next time step
    tf::BindPlan* bind = nullptr;               // device program of the couples' row/column merges
    std::vector<double> h_xval;                 // their values of the current assembly
    int64_t extra_version = 0;                  // changes with every new extra-block layout
    std::vector<uint8_t> h_fixed;
    std::vector<double> h_nu;                   // Poisson ratios, clamped as the material setup does
    std::vector<int> h_apical;                  // 1 for apical nodes (tissue placement 1)
    std::vector<int> h_place;                   // node placement (0 basal, 1 apical, 2 mid, 3 lateral)
    std::vector<double> h_vref;                 // reference volume of each prism
    std::vector<std::vector<int>> h_xuser;      // extra blocks of tf_add_K_triplets and DOF bindings
    std::vector<int> h_seg_node0, h_seg_elem0;  // host copies of the instance offsets
    std::vector<int> h_active;                  // host mirror of seg_active
    int elem_cta = 16;                          // prisms per CTA of the element kernel (autotuned)
    bool tuned = false;
    cudaGraphExec_t graph[2][5] = {};           // Krylov chunks [method-1][log2(chunk/4)]
    int64_t graph_kernels[2][5] = {};
    cudaGraphExec_t kloop[2] = {};              // a whole solve as one graph (device-side while loop) [method-1]
    cudaGraphExec_t nloop = nullptr;            // the Newton iterations after a step's first as one graph
    double nloop_dt = 0.0;                      // the step length that graph was captured with
    bool nloop_off = false;                     // that graph could not be built here: host-driven iterations
    int64_t nloop_kernels = 0;                  // kernels of one of its Newton iterations outside the Krylov loop
    cudaStream_t cap_stream = nullptr;          // second stream for capturing nested loop bodies
    tf::NewtonDev* nd = nullptr;                // device Newton-loop state and its pinned mirror
    tf::NewtonDev* nd_host = nullptr;
    int* nd_seg = nullptr;                      // device [3][nseg]: Newton iterations, converged, capped
    int* nd_seg_host = nullptr;                 // pinned mirror
    bool kloop_off = false;                     // that graph could not be built here: host-checked chunks
    int* kloop_ctl = nullptr;                   // device: [iterations run, iteration cap]
    int* kloop_host = nullptr;                  // pinned copy of the iterations run
    int last_iters[2] = {0, 0};                 // iterations of the last solve per method (chunk planning)
    bool solve_tuned = false;                   // the solve's kernel variants below were chosen by timing
    int spmv_unroll = 2;                        // slots in flight per lane in the FP64 block SpMV (1, 2, 4)
    int plan_iters[2][8] = {};                  // the same per Newton iteration of a step (0-6, 7: later ones)
    int newton_index = -1;                      // Newton iteration of the current solve (-1: outside a step)
    double* du0 = nullptr;                      // the first Newton update of the last step (start of the next)
    bool have_du0 = false;
    tf::Amg* amg = nullptr;                     // multigrid preconditioner (null: block-Jacobi)
    tf::Packing* pk = nullptr;                  // packing between tissue surfaces (null: off)
    tf::Growth* growth = nullptr;               // growth functions (null: none added yet)
    double time = 0.0;                          // simulation time (currSimTimeSec), advanced by tf_end_step
    bool in_step = false;                       // between tf_begin_step and tf_end_step
    std::vector<double> h_pos0;                 // node positions of the mesh at creation
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
tf_status launch_update_norm(tf_handle* h);   // |du|^2 into S_DU2 without applying du
// The Newton iterations after the first of a step on the device (one graph
// launch); io arrays per instance are the host's bookkeeping, updated.
// *ran = false when the loop is not available here (nothing was done).
tf_status newton_device_loop(tf_handle* h, int* it, int* cv, int* capped, int* k, tf_step_stats* st, float* ms_asm,
                             bool* ran, bool* exc);
tf_status autotune_element(tf_handle* h);
tf_status amg_build(tf_handle* h, const double* ref_pos);
tf_status amg_numeric(tf_handle* h);
void amg_refresh(tf_handle* h);     // launches the level-0 smoother copies of the current assembly
tf_status amg_autotune(tf_handle* h);  // picks the level-0 smoother's row-product variant by timing
int amg_smoother_unroll(const tf_handle* h);
void amg_refreshed(tf_handle* h);   // records that amg_refresh ran for the current assembly
void amg_vcycle(tf_handle* h, const double* r, double* out);
int amg_vcycle_kernels(const tf_handle* h);
void amg_free(Amg* a);
void amg_mark_stale(tf_handle* h, int level);  // 1: new assembly, 2: rebuild the hierarchy
tf_status packing_setup(tf_handle* h, int flags); // switch packing on (device tables)
tf_status packing_detect(tf_handle* h);          // couples at the current positions (step start)
tf_status packing_get(tf_handle* h, int64_t* n, int32_t* nodes, double* w, double* mbar, double* threshold,
                      double* detect);
tf_status packing_masses(tf_handle* h, double* mass);
tf_status packing_assemble(tf_handle* h);        // forces and Jacobian into g and K
tf_status packing_relink(tf_handle* h);          // couple blocks in the current extra-block layout
// The multigrid preconditioner is used whenever the handle has a hierarchy
// (the extra blocks -- packing couples among them -- reach its coarse levels
// as X_{l+1} = P^T X_l P).
bool use_multigrid(const tf_handle* h);
void packing_free(Packing* p);
tf_status growth_setup(tf_handle* h);           // growth-function tables from the mesh at creation
constexpr int kMaxGrowthFunctions = 16;         // growth functions per handle
tf_status growth_add_uniform(tf_handle* h, const double* rates, double angle, double t0, double t1, double zmin,
                             double zmax);
tf_status growth_add_ring(tf_handle* h, double cx, double cy, double r_in, double r_out, const double* rates,
                          double angle, double t0, double t1, double zmin, double zmax);
tf_status growth_add_grid(tf_handle* h, int nx, int ny, const double* rates, const double* angles_deg, double t0,
                          double t1, double zmin, double zmax);
void growth_clear(tf_handle* h);
void growth_set_mode(tf_handle* h, int interp, int pinned);
tf_status growth_repin(tf_handle* h);
int growth_count(const tf_handle* h);
tf_status launch_growth_functions(tf_handle* h, bool* done);  // rates + the functions active at h->time
tf_status growth_positions(tf_handle* h, double* relz, double* rel0, double* rel);
void growth_free(Growth* g);
tf_status upload_extra(tf_handle* h, bool pattern_changed);
tf_status sync_extra_to_host(tf_handle* h);      // device extra-block values -> h_xval
void bind_free(tf_handle* h);                     // releases the bound-DOF plan
tf_status take_check(tf_handle* h);              // checked build: report and clear a failed index check
bool amg_reused(const tf_handle* h);
long amg_rebuilds(const tf_handle* h);  // full numeric rebuilds so far
tf_status launch_adjoint_element(tf_handle* h, const double* lamv, double* carry, double* gr, double* ge, double ndt);
void destroy_graphs(tf_handle* h);

inline int cdiv(int64_t a, int64_t b) { return static_cast<int>((a + b - 1) / b); }

}  // namespace tf
