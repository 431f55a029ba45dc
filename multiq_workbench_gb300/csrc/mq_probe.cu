// L2 read bandwidth, the denominator of the gather kernels' L2 roofline: sweeps over a buffer
// small enough to stay resident in L2, loaded with ld.global.cg (cached in L2, not in L1).
#include <cuda_runtime.h>

#include "mq_engine.h"
#include "mq_check.h"

namespace {

__global__ void __launch_bounds__(512) k_l2_read(const float4* __restrict__ buf, size_t n4, int passes,
                                                 unsigned* __restrict__ sink) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    float acc = 0.0f;
    for (int p = 0; p < passes; ++p) {
        // a different starting block each sweep, so no thread re-reads its own previous line
        const size_t shift = ((size_t)p * 7919u * blockDim.x) % n4;
        size_t i = tid;
#pragma unroll 4
        for (; i < n4; i += stride) {
            size_t j = i + shift;
            if (j >= n4) j -= n4;
            const float4 v = __ldcg(buf + j);
            acc += (v.x + v.y) + (v.z + v.w);
        }
    }
    if (acc == -1.0f) atomicAdd(sink, 1u);   // the buffer holds zeros: never taken, keeps the loads
}

// one index equal to its limit, through the check (no memory is accessed): a check build records it
__global__ void k_check_selftest(unsigned long long* out) {
    out[0] = (unsigned long long)MQ_CHK(7u, 7u, MQ_SITE_SELFTEST);
}

}  // namespace

MQ_CHECK_READER(mq_check_read_probe)

extern "C" int mq_check_selftest_launch(void) {
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, sizeof(unsigned long long)) != cudaSuccess) { cudaGetLastError(); return -3; }
    k_check_selftest<<<1, 1>>>(d);
    unsigned long long h = 1;
    const cudaError_t e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) { cudaGetLastError(); return -2; }
    return 0;
}

extern "C" mq_status mq_measure_l2_read_gbs(int32_t device, size_t bytes, int32_t passes, double* gbs) {
    if (!gbs || passes < 1 || passes > 10000 || bytes < ((size_t)16 << 20) || bytes > ((size_t)96 << 20))
        return MQ_ERR_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return MQ_ERR_NO_DEVICE;
    int prev = 0;
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) return MQ_ERR_CUDA;
    const size_t n4 = bytes / sizeof(float4);
    float4* buf = nullptr;
    unsigned* sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    mq_status rc = MQ_ERR_CUDA;
    int sms = 0, per_sm = 0;
    if (cudaMalloc(&buf, n4 * sizeof(float4)) != cudaSuccess || cudaMalloc(&sink, sizeof(unsigned)) != cudaSuccess) {
        rc = MQ_ERR_NOMEM;
        goto done;
    }
    if (cudaMemset(buf, 0, n4 * sizeof(float4)) != cudaSuccess || cudaMemset(sink, 0, sizeof(unsigned)) != cudaSuccess)
        goto done;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) goto done;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_l2_read, 512, 0) != cudaSuccess || per_sm < 1)
        goto done;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) goto done;
    {
        const unsigned grid = (unsigned)(sms * per_sm);
        k_l2_read<<<grid, 512>>>(buf, n4, 1, sink);   // brings the buffer into L2
        cudaEventRecord(e0);
        k_l2_read<<<grid, 512>>>(buf, n4, passes, sink);
        cudaEventRecord(e1);
        if (cudaEventSynchronize(e1) != cudaSuccess || cudaGetLastError() != cudaSuccess) goto done;
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        *gbs = (double)n4 * sizeof(float4) * passes / (ms * 1e-3) / 1e9;
        rc = MQ_OK;
    }
done:
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(buf);
    cudaFree(sink);
    cudaSetDevice(prev);
    return rc;
}
