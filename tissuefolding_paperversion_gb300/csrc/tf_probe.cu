// Memory-roofline probe: the HBM bandwidth this device gives three access
// patterns, measured with kernels of this library.  No counterpart in the
// reference; it supplies the denominators the read-dominated kernels of the
// solve (the block SpMVs, the multigrid smoothers and transfers) are judged
// against, next to the copy bandwidth the benchmark's roofline uses.
//
//   read  : every thread keeps eight independent 16-byte loads in flight
//           (grid-stride over the buffer, a sum kept so the loads stay);
//   bulk  : one-dimensional bulk copies (cp.async.bulk, the TMA engine) of
//           32 KB chunks into a four-stage shared-memory ring per CTA, one
//           CTA per SM, the threads summing each chunk as it lands;
//   copy  : 16-byte loads and stores, read + write bytes counted.
//
// Every mbarrier wait of the bulk kernel gives up after a bounded number of
// polls and raises an error flag the host reads (no endless spin).
#include <algorithm>

#include "tf_internal.cuh"

namespace tf {
namespace {

constexpr int kProbeThreads = 256;
constexpr int kBulkStages = 4;
constexpr int kBulkChunk = 32768;

// Buffer contents: a hash of the index (not zeros, so nothing downstream can
// treat the data as trivially compressible).
__global__ void k_probe_fill(uint32_t* __restrict__ a, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        uint32_t x = (uint32_t)i * 2654435761u;
        x ^= x >> 15;
        a[i] = (x & 0x007fffffu) | 0x3f800000u;  // a float in [1, 2)
    }
}

__global__ void __launch_bounds__(kProbeThreads) k_probe_read(const float4* __restrict__ a, size_t n4,
                                                               float* __restrict__ sink) {
    float s = 0.f;
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (; i + 7 * stride < n4; i += 8 * stride) {
        float4 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = __ldg(&a[i + u * stride]);
#pragma unroll
        for (int u = 0; u < 8; ++u) s += (v[u].x + v[u].y) + (v[u].z + v[u].w);
    }
    for (; i < n4; i += stride) {
        const float4 v = __ldg(&a[i]);
        s += (v.x + v.y) + (v.z + v.w);
    }
    if (s == -1.f) sink[0] = s;  // never true for data in [1, 2): keeps the loads
}

__global__ void __launch_bounds__(kProbeThreads) k_probe_copy(const float4* __restrict__ a, float4* __restrict__ b,
                                                               size_t n4) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x)
        b[i] = a[i];
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__global__ void __launch_bounds__(kProbeThreads) k_probe_bulk(const char* __restrict__ a, size_t nchunks,
                                                               float* __restrict__ sink, int* __restrict__ err) {
    extern __shared__ __align__(128) char ring[];
    __shared__ __align__(8) uint64_t bar[kBulkStages];
    const int tid = threadIdx.x;
    if (tid == 0) {
        for (int s = 0; s < kBulkStages; ++s)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bar[s])));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    auto issue = [&](int s, size_t c) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(&bar[s])),
                     "r"(kBulkChunk)
                     : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_addr(ring + (size_t)s * kBulkChunk)),
            "l"(a + c * kBulkChunk), "r"(kBulkChunk), "r"(smem_addr(&bar[s]))
            : "memory");
    };
    const size_t c0 = blockIdx.x, step = gridDim.x;
    if (tid == 0)
        for (int s = 0; s < kBulkStages; ++s)
            if (c0 + s * step < nchunks) issue(s, c0 + s * step);
    float acc = 0.f;
    int k = 0;
    for (size_t c = c0; c < nchunks; c += step, ++k) {
        const int s = k % kBulkStages;
        const uint32_t parity = (k / kBulkStages) & 1;
        uint32_t ready = 0;
        for (int it = 0; it < (1 << 22) && !ready; ++it)
            asm volatile(
                "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                : "=r"(ready)
                : "r"(smem_addr(&bar[s])), "r"(parity)
                : "memory");
        if (!ready) atomicExch(err, 1);  // every thread still takes the barrier below
        const float4* v = reinterpret_cast<const float4*>(ring + (size_t)s * kBulkChunk);
#pragma unroll 4
        for (int q = tid; q < kBulkChunk / 16; q += kProbeThreads) {
            const float4 x = v[q];
            acc += (x.x + x.y) + (x.z + x.w);
        }
        __syncthreads();
        const size_t cn = c + (size_t)kBulkStages * step;
        if (tid == 0 && cn < nchunks) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(s, cn);
        }
    }
    if (acc == -1.f) sink[0] = acc;
}

struct ProbeBuffers {
    char* a = nullptr;
    char* b = nullptr;
    float* sink = nullptr;
    int* err = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ~ProbeBuffers() {
        cudaFree(a);
        cudaFree(b);
        cudaFree(sink);
        cudaFree(err);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    }
};

template <class F>
tf_status best_ms(ProbeBuffers& B, int reps, F launch, float* best) {
    for (int w = 0; w < 2; ++w) launch();
    TF_CUDA(cudaGetLastError());
    *best = 1e30f;
    for (int r = 0; r < reps; ++r) {
        TF_CUDA(cudaEventRecord(B.e0));
        launch();
        TF_CUDA(cudaEventRecord(B.e1));
        TF_CUDA(cudaEventSynchronize(B.e1));
        float ms = 0.f;
        TF_CUDA(cudaEventElapsedTime(&ms, B.e0, B.e1));
        *best = std::min(*best, ms);
    }
    return TF_OK;
}

}  // namespace
}  // namespace tf

extern "C" TF_API tf_status tf_measure_bandwidth(int32_t device, int64_t bytes, int32_t reps, double* read_gbs,
                                                 double* bulk_gbs, double* copy_gbs) {
    using namespace tf;
    if (bytes < (int64_t)kBulkChunk * 152 || bytes % kBulkChunk != 0 || reps < 1 || !read_gbs || !bulk_gbs ||
        !copy_gbs) {
        set_error("tf_measure_bandwidth: bytes must be a multiple of 32 KB and at least 152 chunks; reps >= 1");
        return TF_BAD_INPUT;
    }
    TF_CUDA(cudaSetDevice(device));
    int sms = 0;
    TF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    ProbeBuffers B;
    TF_CUDA(cudaMalloc(&B.a, (size_t)bytes));
    TF_CUDA(cudaMalloc(&B.b, (size_t)bytes));
    TF_CUDA(cudaMalloc(&B.sink, sizeof(float)));
    TF_CUDA(cudaMalloc(&B.err, sizeof(int)));
    TF_CUDA(cudaMemset(B.err, 0, sizeof(int)));
    TF_CUDA(cudaEventCreate(&B.e0));
    TF_CUDA(cudaEventCreate(&B.e1));
    k_probe_fill<<<4 * sms, kProbeThreads>>>(reinterpret_cast<uint32_t*>(B.a), (size_t)bytes / 4);
    TF_CUDA(cudaGetLastError());
    const size_t n4 = (size_t)bytes / 16;
    const size_t smem = (size_t)kBulkStages * kBulkChunk;
    TF_CUDA(cudaFuncSetAttribute(k_probe_bulk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    float ms_read = 0.f, ms_bulk = 0.f, ms_copy = 0.f;
    tf_status s = best_ms(
        B, reps, [&] { k_probe_read<<<4 * sms, kProbeThreads>>>((const float4*)B.a, n4, B.sink); }, &ms_read);
    if (s == TF_OK)
        s = best_ms(
            B, reps,
            [&] { k_probe_bulk<<<sms, kProbeThreads, smem>>>(B.a, (size_t)bytes / kBulkChunk, B.sink, B.err); },
            &ms_bulk);
    if (s == TF_OK)
        s = best_ms(
            B, reps, [&] { k_probe_copy<<<8 * sms, kProbeThreads>>>((const float4*)B.a, (float4*)B.b, n4); },
            &ms_copy);
    if (s != TF_OK) return s;
    int err = 0;
    TF_CUDA(cudaMemcpy(&err, B.err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
        set_error("tf_measure_bandwidth: a bulk-copy wait gave up");
        return TF_CUDA_ERROR;
    }
    *read_gbs = (double)bytes / (ms_read * 1e-3) / 1e9;
    *bulk_gbs = (double)bytes / (ms_bulk * 1e-3) / 1e9;
    *copy_gbs = 2.0 * (double)bytes / (ms_copy * 1e-3) / 1e9;
    return TF_OK;
}
