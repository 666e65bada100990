// A linear solve for callers that cannot allocate device memory.
//
// tf_solve_bsr_static solves A x = b for a caller-owned 3x3 block-sparse
// matrix with block-Jacobi preconditioned BiCGStab in FP64, like the solve
// behind tf_solve, but it calls no cudaMalloc, cudaFree or other allocating
// routine.  Its work vectors, reduction partials and scalars live in one
// file-scope device array, g_static_scratch, sized for at most
// kStaticMaxNodes block rows.  Every GPU that loads this library holds that
// array (about 4.3 MB) until the process exits.
//
// Host code cannot use the array's name as a device address, so the first
// call on each device looks the address up with cudaGetSymbolAddress while
// that device is current, and caches it together with the CUDA context it
// came from; a call in another context (after cudaDeviceReset, say) looks it
// up again.  Every call synchronises its stream and reads scalars back to the
// host between chunks of iterations, so no call may be made on a stream that
// is being captured: such a call returns TF_BAD_INPUT and leaves the capture
// untouched.  All calls on a device share the one array: calls that
// overlap on the GPU (two streams, two host threads) race on it and give
// wrong results, so serialise them.  Each call clears the reduction ticket
// and the scalars it reads before its first kernel, and writes every work
// vector before reading it, so nothing carries over from the previous call.
#include <cuda.h>

#include <mutex>

#include "tf_internal.cuh"

namespace tf {
namespace {

constexpr int kStaticMaxNodes = 16384;
constexpr int kStaticThreads = 256;
constexpr int kStaticMaxGrid = (kStaticMaxNodes + kStaticThreads - 1) / kStaticThreads;
constexpr int kNumVec = 8;                    // r, rhat, p, phat, v, s, shat, t
constexpr size_t kVecLen = 3 * (size_t)kStaticMaxNodes;
constexpr size_t kOffDinv = kNumVec * kVecLen;            // 9 doubles per node
constexpr size_t kOffPart = kOffDinv + 9 * (size_t)kStaticMaxNodes;
constexpr size_t kOffScal = kOffPart + 2 * (size_t)kStaticMaxGrid;
constexpr size_t kNumScal = 16;
constexpr size_t kOffTicket = kOffScal + kNumScal;
constexpr size_t kScratchDoubles = kOffTicket + 2;

__device__ __align__(256) double g_static_scratch[kScratchDoubles];

enum { Q_RHO = 0, Q_ALPHA, Q_OMEGA, Q_BETA, Q_BB, Q_RR, Q_ITER, Q_FLAG, Q_TOL2 };
enum { QF_RUNNING = 0, QF_CONVERGED = 1, QF_BREAKDOWN = 2, QF_NAN = 3 };

struct SCtx {
    int n;
    const int* __restrict__ rowptr;
    const int* __restrict__ colidx;
    const double* __restrict__ val;
    double* base;  // device address of g_static_scratch
    __device__ double* vec(int k) const { return base + k * kVecLen; }
    __device__ double* dinv() const { return base + kOffDinv; }
    __device__ double* part() const { return base + kOffPart; }
    __device__ double* q() const { return base + kOffScal; }
    __device__ unsigned* ticket() const { return reinterpret_cast<unsigned*>(base + kOffTicket); }
};

template <int NV>
__device__ bool s_reduce(const SCtx& c, double (&v)[NV], double (&tot)[NV]) {
    __shared__ double sm[NV][kStaticThreads / 32 + 1];
    __shared__ bool last;
    double x[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) x[k] = v[k];
    cta_sum<kStaticThreads, NV>(x, sm);
    if (threadIdx.x == 0) {
        for (int k = 0; k < NV; ++k) c.part()[k * gridDim.x + blockIdx.x] = x[k];
        __threadfence();
        last = atomicAdd(c.ticket(), 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    // all threads of the last CTA fold the partials (fixed order)
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        x[k] = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) x[k] += __ldcg(&c.part()[k * gridDim.x + b]);
    }
    cta_sum<kStaticThreads, NV>(x, sm);
    if (threadIdx.x == 0) {
        for (int k = 0; k < NV; ++k) tot[k] = x[k];
        *c.ticket() = 0u;
    }
    return true;
}

__device__ __forceinline__ bool s_stopped(const SCtx& c) { return __ldcg(&c.q()[Q_FLAG]) != 0.0; }

__device__ __forceinline__ void s_row(const SCtx& c, int i, const double* __restrict__ x, double y[3]) {
    double y0 = 0.0, y1 = 0.0, y2 = 0.0;
    for (int b = c.rowptr[i]; b < c.rowptr[i + 1]; ++b) {
        const int j = c.colidx[b];
        const double* a = c.val + 9 * (size_t)b;
        const double x0 = x[3 * j], x1 = x[3 * j + 1], x2 = x[3 * j + 2];
        y0 = fma(a[0], x0, fma(a[1], x1, fma(a[2], x2, y0)));
        y1 = fma(a[3], x0, fma(a[4], x1, fma(a[5], x2, y1)));
        y2 = fma(a[6], x0, fma(a[7], x1, fma(a[8], x2, y2)));
    }
    y[0] = y0;
    y[1] = y1;
    y[2] = y2;
}

__device__ __forceinline__ void s_prec(const double* D, const double r[3], double z[3]) {
    z[0] = fma(D[0], r[0], fma(D[1], r[1], D[2] * r[2]));
    z[1] = fma(D[3], r[0], fma(D[4], r[1], D[5] * r[2]));
    z[2] = fma(D[6], r[0], fma(D[7], r[1], D[8] * r[2]));
}

// inverse diagonal blocks; r = rhat = b; p = v = 0; x = 0; rho = (b, b)
__global__ void ks_init(SCtx c, const double* __restrict__ b, double* __restrict__ x) {
    const int i = blockIdx.x * kStaticThreads + threadIdx.x;
    double acc[1] = {0.0};
    if (i < c.n) {
        const double* M = nullptr;
        for (int p = c.rowptr[i]; p < c.rowptr[i + 1]; ++p)
            if (c.colidx[p] == i) M = c.val + 9 * (size_t)p;
        double inv[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        if (M) {
            const double c0 = M[4] * M[8] - M[5] * M[7], c1 = M[5] * M[6] - M[3] * M[8], c2 = M[3] * M[7] - M[4] * M[6];
            const double det = M[0] * c0 + M[1] * c1 + M[2] * c2;
            if (det != 0.0) {
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
        }
        for (int k = 0; k < 9; ++k) c.dinv()[9 * (size_t)i + k] = inv[k];
        for (int d = 0; d < 3; ++d) {
            const int k = 3 * i + d;
            const double bk = b[k];
            c.vec(0)[k] = bk;     // r
            c.vec(1)[k] = bk;     // rhat
            c.vec(2)[k] = 0.0;    // p
            c.vec(4)[k] = 0.0;    // v
            x[k] = 0.0;
            acc[0] = fma(bk, bk, acc[0]);
        }
    }
    double tot[1];
    if (s_reduce<1>(c, acc, tot) && threadIdx.x == 0) {
        double* q = c.q();
        q[Q_RHO] = tot[0];
        q[Q_BB] = tot[0];
        q[Q_RR] = tot[0];
        q[Q_ALPHA] = 1.0;
        q[Q_OMEGA] = 1.0;
        q[Q_BETA] = 0.0;
        q[Q_ITER] = 0.0;
        q[Q_FLAG] = tot[0] == 0.0 ? QF_CONVERGED : (isfinite(tot[0]) ? QF_RUNNING : QF_NAN);
    }
}

// p = r + beta (p - omega v); phat = M^-1 p
__global__ void ks_dir(SCtx c) {
    if (s_stopped(c)) return;
    const int i = blockIdx.x * kStaticThreads + threadIdx.x;
    if (i >= c.n) return;
    const double beta = __ldcg(&c.q()[Q_BETA]), omega = __ldcg(&c.q()[Q_OMEGA]);
    double pp[3], z[3];
    for (int d = 0; d < 3; ++d) {
        const int k = 3 * i + d;
        pp[d] = fma(beta, fma(-omega, c.vec(4)[k], c.vec(2)[k]), c.vec(0)[k]);
        c.vec(2)[k] = pp[d];
    }
    s_prec(c.dinv() + 9 * (size_t)i, pp, z);
    for (int d = 0; d < 3; ++d) c.vec(3)[3 * i + d] = z[d];
}

// v = A phat; alpha = rho / (rhat, v)
__global__ void ks_spmv1(SCtx c) {
    if (s_stopped(c)) return;
    const int i = blockIdx.x * kStaticThreads + threadIdx.x;
    double acc[1] = {0.0};
    if (i < c.n) {
        double y[3];
        s_row(c, i, c.vec(3), y);
        for (int d = 0; d < 3; ++d) {
            c.vec(4)[3 * i + d] = y[d];
            acc[0] = fma(c.vec(1)[3 * i + d], y[d], acc[0]);
        }
    }
    double tot[1];
    if (s_reduce<1>(c, acc, tot) && threadIdx.x == 0) {
        double* q = c.q();
        if (tot[0] == 0.0 || !isfinite(tot[0])) q[Q_FLAG] = isfinite(tot[0]) ? QF_BREAKDOWN : QF_NAN;
        else q[Q_ALPHA] = q[Q_RHO] / tot[0];
    }
}

// s = r - alpha v; shat = M^-1 s
__global__ void ks_s(SCtx c) {
    if (s_stopped(c)) return;
    const int i = blockIdx.x * kStaticThreads + threadIdx.x;
    if (i >= c.n) return;
    const double alpha = __ldcg(&c.q()[Q_ALPHA]);
    double ss[3], z[3];
    for (int d = 0; d < 3; ++d) {
        const int k = 3 * i + d;
        ss[d] = fma(-alpha, c.vec(4)[k], c.vec(0)[k]);
        c.vec(5)[k] = ss[d];
    }
    s_prec(c.dinv() + 9 * (size_t)i, ss, z);
    for (int d = 0; d < 3; ++d) c.vec(6)[3 * i + d] = z[d];
}

// t = A shat; omega = (t, s) / (t, t)
__global__ void ks_spmv2(SCtx c) {
    if (s_stopped(c)) return;
    const int i = blockIdx.x * kStaticThreads + threadIdx.x;
    double acc[2] = {0.0, 0.0};
    if (i < c.n) {
        double y[3];
        s_row(c, i, c.vec(6), y);
        for (int d = 0; d < 3; ++d) {
            c.vec(7)[3 * i + d] = y[d];
            acc[0] = fma(y[d], c.vec(5)[3 * i + d], acc[0]);
            acc[1] = fma(y[d], y[d], acc[1]);
        }
    }
    double tot[2];
    if (s_reduce<2>(c, acc, tot) && threadIdx.x == 0) {
        double* q = c.q();
        if (!isfinite(tot[0]) || !isfinite(tot[1])) q[Q_FLAG] = QF_NAN;
        else q[Q_OMEGA] = tot[1] > 0.0 ? tot[0] / tot[1] : 0.0;
    }
}

// x += alpha phat + omega shat; r = s - omega t; rho' = (rhat, r)
__global__ void ks_x(SCtx c, double* __restrict__ x) {
    if (s_stopped(c)) return;
    const int i = blockIdx.x * kStaticThreads + threadIdx.x;
    const double alpha = __ldcg(&c.q()[Q_ALPHA]), omega = __ldcg(&c.q()[Q_OMEGA]);
    double acc[2] = {0.0, 0.0};
    if (i < c.n) {
        for (int d = 0; d < 3; ++d) {
            const int k = 3 * i + d;
            x[k] = fma(omega, c.vec(6)[k], fma(alpha, c.vec(3)[k], x[k]));
            const double rk = fma(-omega, c.vec(7)[k], c.vec(5)[k]);
            c.vec(0)[k] = rk;
            acc[0] = fma(c.vec(1)[k], rk, acc[0]);
            acc[1] = fma(rk, rk, acc[1]);
        }
    }
    double tot[2];
    if (s_reduce<2>(c, acc, tot) && threadIdx.x == 0) {
        double* q = c.q();
        const double om = q[Q_OMEGA];
        q[Q_BETA] = (tot[0] / q[Q_RHO]) * (q[Q_ALPHA] / om);
        q[Q_RHO] = tot[0];
        q[Q_RR] = tot[1];
        q[Q_ITER] += 1.0;
        if (!isfinite(tot[1])) q[Q_FLAG] = QF_NAN;
        else if (tot[1] <= q[Q_TOL2] * q[Q_BB]) q[Q_FLAG] = QF_CONVERGED;
        else if (om == 0.0 || tot[0] == 0.0) q[Q_FLAG] = QF_BREAKDOWN;
    }
}

std::mutex g_addr_mutex;
struct ScratchAddr {
    CUcontext ctx;
    double* ptr;
};
ScratchAddr g_addr[64] = {};
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
CtxGetCurrentFn g_ctx_get = nullptr;

// The current CUDA context, through the driver entry point the runtime hands
// out (the library does not link the driver library itself).
tf_status current_context(CUcontext* ctx) {
    if (!g_ctx_get) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetDriverEntryPointByVersion(cuCtxGetCurrent)");
        if (q != cudaDriverEntryPointSuccess || !fn) {
            set_error("tf_solve_bsr_static: the driver offers no cuCtxGetCurrent");
            return TF_CUDA_ERROR;
        }
        g_ctx_get = reinterpret_cast<CtxGetCurrentFn>(fn);
    }
    *ctx = nullptr;
    if (g_ctx_get(ctx) != CUDA_SUCCESS || !*ctx) {
        set_error("tf_solve_bsr_static: no current CUDA context");
        return TF_CUDA_ERROR;
    }
    return TF_OK;
}

// Device address of g_static_scratch for `device`, looked up once per device
// and context with that device current.
tf_status scratch_address(int device, double** out) {
    if (device < 0 || device >= 64) {
        set_error("device ordinal out of range for the static solve");
        return TF_BAD_INPUT;
    }
    std::lock_guard<std::mutex> lock(g_addr_mutex);
    CUcontext ctx = nullptr;
    tf_status s = current_context(&ctx);
    if (s != TF_OK) return s;
    if (!g_addr[device].ptr || g_addr[device].ctx != ctx) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_static_scratch)");
        g_addr[device].ptr = static_cast<double*>(p);
        g_addr[device].ctx = ctx;
    }
    *out = g_addr[device].ptr;
    return TF_OK;
}

}  // namespace
}  // namespace tf

using namespace tf;

extern "C" TF_API tf_status tf_solve_bsr_static(int32_t n_block_rows, const int32_t* rowptr, const int32_t* colidx,
                                                const double* val, const double* b, double* x, double rtol,
                                                int32_t max_iter, void* stream, int32_t* iters, double* relres) {
    if (n_block_rows <= 0 || !rowptr || !colidx || !val || !b || !x || !(rtol > 0.0) || max_iter <= 0) {
        set_error("tf_solve_bsr_static: bad arguments");
        return TF_BAD_INPUT;
    }
    if (n_block_rows > kStaticMaxNodes) {
        set_error("tf_solve_bsr_static: " + std::to_string(n_block_rows) + " block rows exceed the static limit of " +
                  std::to_string(kStaticMaxNodes));
        return TF_BAD_INPUT;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    TF_CUDA(cudaStreamIsCapturing(st, &cap));
    if (cap != cudaStreamCaptureStatusNone) {
        set_error("tf_solve_bsr_static: the stream is being captured; this call synchronises and reads back, "
                  "so it cannot run inside a capture");
        return TF_BAD_INPUT;
    }
    int device = 0;
    TF_CUDA(cudaGetDevice(&device));
    double* base = nullptr;
    tf_status s = scratch_address(device, &base);
    if (s != TF_OK) return s;
    SCtx c{n_block_rows, rowptr, colidx, val, base};
    const int grid = cdiv(n_block_rows, kStaticThreads);
    // clear the ticket and scalars, then the tolerance
    TF_CUDA(cudaMemsetAsync(base + kOffScal, 0, sizeof(double) * (kNumScal + 2), st));
    const double tol2 = rtol * rtol;
    TF_CUDA(cudaMemcpyAsync(base + kOffScal + Q_TOL2, &tol2, sizeof(double), cudaMemcpyHostToDevice, st));
    ks_init<<<grid, kStaticThreads, 0, st>>>(c, b, x);
    TF_CUDA(cudaGetLastError());
    double q[kNumScal];
    int launched = 0, chunk = 8;
    while (launched < max_iter) {
        const int n = chunk < max_iter - launched ? chunk : max_iter - launched;
        for (int it = 0; it < n; ++it) {
            ks_dir<<<grid, kStaticThreads, 0, st>>>(c);
            ks_spmv1<<<grid, kStaticThreads, 0, st>>>(c);
            ks_s<<<grid, kStaticThreads, 0, st>>>(c);
            ks_spmv2<<<grid, kStaticThreads, 0, st>>>(c);
            ks_x<<<grid, kStaticThreads, 0, st>>>(c, x);
        }
        TF_CUDA(cudaGetLastError());
        launched += n;
        TF_CUDA(cudaMemcpyAsync(q, base + kOffScal, sizeof(q), cudaMemcpyDeviceToHost, st));
        TF_CUDA(cudaStreamSynchronize(st));
        if (q[Q_FLAG] != QF_RUNNING) break;
        if (chunk < 64) chunk *= 2;
    }
    if (iters) *iters = static_cast<int32_t>(q[Q_ITER]);
    if (relres) *relres = q[Q_BB] > 0.0 ? sqrt(q[Q_RR] / q[Q_BB]) : 0.0;
    if (q[Q_FLAG] == QF_CONVERGED) return TF_OK;
    if (q[Q_FLAG] == QF_NAN) {
        set_error("tf_solve_bsr_static: non-finite value");
        return TF_NAN_DETECTED;
    }
    if (q[Q_FLAG] == QF_BREAKDOWN) {
        set_error("tf_solve_bsr_static: BiCGStab breakdown");
        return TF_KRYLOV_BREAKDOWN;
    }
    set_error("tf_solve_bsr_static: iteration cap reached");
    return TF_KRYLOV_NOT_CONVERGED;
}
