// swm_probe.cu -- measured ceiling for the roofline of the gather kernels.
//
// The seed lookups and the candidate gathers read scattered 32-byte sectors
// (a 2-byte flank code, a 4-byte position, an 8-byte bucket-offset pair), so
// their bound is the rate at which the memory system serves independent
// random sectors, not the streaming copy bandwidth. This probe measures that
// rate on the device it runs on: every thread keeps 8 loads of 4 bytes from
// random sectors of a buffer in flight.
#include <stdio.h>

#include "swm_common.cuh"

#define PROBE_INFLIGHT 8

__global__ void __launch_bounds__(256) k_probe_gather(const uint32_t *__restrict__ buf, uint64_t nsec,
                                                      uint32_t iters, uint32_t seed, uint32_t *out) {
    const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    uint32_t x = seed ^ (uint32_t)(tid * 0x9E3779B9u) ^ 0x6A09E667u;
    if (x == 0) x = 1;
    uint32_t acc = 0;
    for (uint32_t it = 0; it < iters; it++) {
        uint32_t v[PROBE_INFLIGHT];
#pragma unroll
        for (int k = 0; k < PROBE_INFLIGHT; k++) {
            x ^= x << 13; // xorshift32
            x ^= x >> 17;
            x ^= x << 5;
            const uint64_t s = ((uint64_t)x * nsec) >> 32; // sector in [0, nsec)
            v[k] = __ldcg(buf + s * 8 + (x & 7u));
        }
#pragma unroll
        for (int k = 0; k < PROBE_INFLIGHT; k++) acc ^= v[k];
    }
    if (acc == 0x9E3779B9u) out[0] = acc; // keeps the loads
}

extern "C" int swm_probe_random_reads(int device, uint64_t bytes, double *sectors_per_s) {
    if (!sectors_per_s || bytes < (1u << 20) || bytes > (64ull << 30)) return SWM_ERR_ARG;
    *sectors_per_s = 0.0;
    SWM_CUDA(cudaSetDevice(device));
    int sms = 0;
    SWM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    uint32_t *buf = nullptr, *out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = SWM_OK;
    const uint64_t nsec = bytes / 32;
    const unsigned threads = 256, blocks = (unsigned)sms * 8;
    const uint32_t iters = 64;
    float best = 0.0f;
    if (cudaMalloc((void **)&buf, nsec * 32) != cudaSuccess || cudaMalloc((void **)&out, 4) != cudaSuccess) {
        swm_set_error("probe: cudaMalloc of %llu bytes failed", (unsigned long long)(nsec * 32));
        rc = SWM_ERR_OOM;
        goto done;
    }
    if (cudaMemset(buf, 0x5a, nsec * 32) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess) {
        rc = SWM_ERR_CUDA;
        goto done;
    }
    for (int rep = 0; rep < 6; rep++) { // the first launch is a warm-up
        cudaEventRecord(e0);
        k_probe_gather<<<blocks, threads>>>(buf, nsec, iters, 0x1234567u + rep, out);
        cudaEventRecord(e1);
        if (cudaEventSynchronize(e1) != cudaSuccess) {
            rc = SWM_ERR_CUDA;
            goto done;
        }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms > 0.0f) {
            const float rate = (float)((double)blocks * threads * iters * PROBE_INFLIGHT / (ms * 1e-3));
            if (rate > best) best = rate;
        }
    }
    *sectors_per_s = best;
done:
    if (rc == SWM_ERR_CUDA) swm_set_error("probe: %s", cudaGetErrorString(cudaGetLastError()));
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(buf);
    cudaFree(out);
    return rc;
}
