/*
 * The L2 ceiling that bounds the DROP block update, measured on the device at
 * hand: float reductions (red.global.add.f32) at pseudo-random 32-byte sectors
 * of an array that stays resident in L2 (the size of a 256x256x32 update
 * image), one element per sector and warp instruction.  Mode 1 first reads the
 * same sector of a second array of that size, as the DROP row pass gathers
 * x[v] and then adds into x_update[v].  Not part of the reference interface: a measurement aid
 * for the benchmark's roofline.
 */
#include "pct_device.cuh"
#include "pct_probe.h"

namespace {

constexpr int PROBE_THREADS = 256;
constexpr int PROBE_SECTORS_LOG2 = 18; /* 2^18 sectors x 32 B = 8 MB */

__device__ __forceinline__ uint32_t probe_hash(uint32_t a) {
    /* a 32-bit integer mix (xorshift-multiply), one index per call */
    a ^= a >> 16;
    a *= 0x7feb352du;
    a ^= a >> 15;
    a *= 0x846ca68bu;
    a ^= a >> 16;
    return a;
}

__global__ void __launch_bounds__(PROBE_THREADS) k_probe_l2(int mode, int per_thread, float* __restrict__ sectors,
                                                            const float* __restrict__ gather) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t mask = (1u << PROBE_SECTORS_LOG2) - 1u;
    for (int k = 0; k < per_thread; ++k) {
        const uint32_t s = probe_hash(tid * 0x9e3779b9u + (uint32_t)k) & mask;
        float v = 1.0f;
        if (mode == 1) v += gather[(size_t)s * 8];
        atomicAdd(sectors + (size_t)s * 8, v);
    }
}

}  // namespace

extern "C" pct_status pct_probe_l2(int device, int mode, double* sectors_per_second) {
    if (!sectors_per_second || (mode != 0 && mode != 1)) return PCT_ERR_ARGUMENT;
    *sectors_per_second = 0.0;
    int prev = 0;
    if (cudaGetDevice(&prev) != cudaSuccess || cudaSetDevice(device) != cudaSuccess) return PCT_ERR_CUDA;
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_probe_l2, PROBE_THREADS, 0);
    if (sms < 1) sms = 1;
    if (per_sm < 1) per_sm = 1;
    const size_t floats = (size_t)8 << PROBE_SECTORS_LOG2;
    const unsigned grid = (unsigned)(sms * per_sm);
    const int per_thread = 1024;
    float* buf = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    pct_status rc = PCT_OK;
    float ms = 0.0f;
    if (cudaMalloc(&buf, 2 * floats * sizeof(float)) != cudaSuccess || cudaStreamCreate(&st) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        rc = PCT_ERR_CUDA;
    } else {
        cudaMemsetAsync(buf, 0, 2 * floats * sizeof(float), st);
        for (int rep = 0; rep < 3; ++rep) /* warm-up: the array into L2, clocks up */
            k_probe_l2<<<grid, PROBE_THREADS, 0, st>>>(mode, per_thread, buf, buf + floats);
        cudaEventRecord(e0, st);
        const int reps = 5;
        for (int rep = 0; rep < reps; ++rep)
            k_probe_l2<<<grid, PROBE_THREADS, 0, st>>>(mode, per_thread, buf, buf + floats);
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess || ms <= 0.0f)
            rc = PCT_ERR_CUDA;
        else
            *sectors_per_second = (double)grid * PROBE_THREADS * per_thread * reps / (ms * 1e-3);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    if (buf) cudaFree(buf);
    cudaGetLastError();
    cudaSetDevice(prev);
    return rc;
}
