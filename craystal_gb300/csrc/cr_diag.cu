// cr_diag.cu -- device read bandwidth of the memory level a buffer of a
// given size lives in, for the roofline of the ray queries.
//
// The closest-hit ray cast of a 1M-triangle scene reads 72 MiB of nodes and
// triangle blocks, which stay in the 129 MB L2: its bound is L2 bandwidth,
// not HBM.  cr_device_read_bandwidth measures it: a buffer of `bytes` is
// read `passes` times by a grid of persistent blocks (16-byte loads cached
// in L2 only, ld.global.cg, so that L1 does not serve repeats), after one
// untimed pass that makes it resident; CUDA events time the passes.  A
// buffer well below the L2 size gives the L2 read bandwidth, one well above
// it the HBM read bandwidth.

#include "cr_internal.cuh"

namespace cr {
namespace {

constexpr int kDiagThreads = 512;
constexpr int kDiagUnroll = 4;

__global__ void __launch_bounds__(kDiagThreads) kReadPasses(const float4* __restrict__ p, uint64_t n4,
                                                            uint32_t passes, float* __restrict__ sink) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t t0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float acc = 0.0f;
    for (uint32_t pass = 0; pass < passes; pass++) {
        uint64_t i = t0;
        for (; i + (kDiagUnroll - 1) * stride < n4; i += kDiagUnroll * stride) {
            float4 v[kDiagUnroll];
#pragma unroll
            for (int k = 0; k < kDiagUnroll; k++) v[k] = __ldcg(p + i + k * stride);
#pragma unroll
            for (int k = 0; k < kDiagUnroll; k++) acc += (v[k].x + v[k].y) + (v[k].z + v[k].w);
        }
        for (; i < n4; i += stride) {
            const float4 v = __ldcg(p + i);
            acc += (v.x + v.y) + (v.z + v.w);
        }
    }
    if (acc == 1234.5f) *sink = acc;  // keeps the loads; the buffer holds zeros
}

}  // namespace
}  // namespace cr

using namespace cr;

extern "C" int cr_device_read_bandwidth(uint64_t bytes, uint32_t passes, double* gbs) {
    clearError();
    if (!gbs || passes == 0 || bytes < 16 * 1024) return fail(CR_ERR_INVALID_ARGUMENT, "bytes / passes / gbs");
    *gbs = 0.0;
    int dev = 0, sms = 0, perSm = 0;
    CR_CUDA(cudaGetDevice(&dev));
    CR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kReadPasses, kDiagThreads, 0));
    const uint64_t n4 = bytes / 16;
    float4* buf = nullptr;
    float* sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = CR_OK;
    auto run = [&]() -> int {
        CR_CUDA(cudaMalloc(&buf, n4 * 16));
        CR_CUDA(cudaMalloc(&sink, sizeof(float)));
        CR_CUDA(cudaMemset(buf, 0, n4 * 16));
        CR_CUDA(cudaEventCreate(&e0));
        CR_CUDA(cudaEventCreate(&e1));
        const unsigned blocks = (unsigned)(sms * std::max(perSm, 1));
        kReadPasses<<<blocks, kDiagThreads>>>(buf, n4, 1, sink);  // makes the buffer resident
        CR_LAUNCH_CHECK();
        CR_CUDA(cudaEventRecord(e0, 0));
        kReadPasses<<<blocks, kDiagThreads>>>(buf, n4, passes, sink);
        CR_LAUNCH_CHECK();
        CR_CUDA(cudaEventRecord(e1, 0));
        CR_CUDA(cudaEventSynchronize(e1));
        float ms = 0.0f;
        CR_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        *gbs = (double)n4 * 16.0 * passes / (ms * 1e-3) / 1e9;
        return CR_OK;
    };
    rc = run();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (buf) cudaFree(buf);
    if (sink) cudaFree(sink);
    return rc;
}
