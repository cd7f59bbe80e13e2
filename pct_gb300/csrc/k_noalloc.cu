/*
 * pct_drop_noalloc: DROP iterations over caller-owned device arrays, with no
 * device or host allocation inside the call.
 *
 * Who needs it: a caller whose process may not allocate at this point, for
 * example one that runs on a pre-sized memory pool with the CUDA allocator
 * locked, or one that must not let cudaMalloc/cudaFree (which synchronise the
 * device) run in the middle of its own sequence of work on a stream.
 * pct_drop() keeps its scratch in the context and may (re)allocate it; this
 * entry point needs no context at all.
 *
 * Scratch: the per-voxel update sums and the per-voxel row counts s_j of the
 * current block live in one file-scope __device__ array sized for
 * PCT_NOALLOC_MAX_VOXELS voxels (2 x 4 bytes per voxel, 16 MiB in all).  Its
 * address is looked up once per device with cudaGetSymbolAddress (that lookup
 * can load the module; pct_noalloc_setup() does it ahead of the first call).
 * There is one
 * scratch per device: two calls that overlap on one device (different
 * streams or host threads) race on it and give wrong images.
 *
 * Arithmetic: the same block update as pct_drop() (block_update_GPU and
 * image_update_GPU, src/pCT_Reconstruction_Data_Segments.cu:5774-5841 and
 * :5900-5938) but the diagonal weights s_j are counted again in every block
 * of every iteration (as the reference does) and 1/||a_i||^2 = 1/(c^2 n) is
 * formed from the binary32 chord length; binary32 scatter-adds make the sum
 * order run-dependent, so results agree with pct_drop() to rounding.
 */
#include <cuda_runtime.h>
#include <mutex>
#include "pct_internal.h"

namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_WARPS = NA_THREADS / 32;
constexpr int NA_MAX_DEVICES = 64;

/* [0, MAX): binary32 update sums; [MAX, 2 MAX): uint32 row counts. */
__device__ __align__(256) unsigned char g_drop_scratch[(size_t)PCT_NOALLOC_MAX_VOXELS * 8];

std::mutex g_setup_mutex;
void* g_scratch_ptr[NA_MAX_DEVICES];

__global__ void k_na_counts(int64_t start, int64_t end, const int64_t* __restrict__ off,
                            const uint32_t* __restrict__ rows, uint32_t nv, uint32_t* __restrict__ cnt) {
    int lane = threadIdx.x & 31;
    int64_t i = start + ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    if (i >= end) return;
    for (int64_t p = off[i] + lane; p < off[i + 1]; p += 32) {
        uint32_t v = rows[p];
        if (v < nv) atomicAdd(cnt + v, 1u);
    }
}

__global__ void __launch_bounds__(NA_THREADS) k_na_rows(int64_t start, int64_t end, const int64_t* __restrict__ off,
                                                        const uint32_t* __restrict__ rows,
                                                        const float* __restrict__ chord,
                                                        const float* __restrict__ wepl, float lambda,
                                                        const float* __restrict__ x, float* __restrict__ upd,
                                                        uint32_t nv, double* __restrict__ resid) {
    __shared__ double sres[NA_WARPS];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int64_t i = start + (int64_t)blockIdx.x * NA_WARPS + w;
    double r2 = 0.0; /* the squared residual and its sums in binary64 */
    if (i < end) {
        int64_t a = off[i], b = off[i + 1];
        float dot = 0.0f;
        for (int64_t p = a + lane; p < b; p += 32) {
            uint32_t v = rows[p];
            if (v < nv) dot += x[v];
        }
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
        const float c = chord[i];
        const float res = fmaf(-c, dot, wepl[i]);
        const float value = (res / (c * (float)(b - a))) * lambda; /* lambda res c / (c^2 len) */
        for (int64_t p = a + lane; p < b; p += 32) {
            uint32_t v = rows[p];
            if (v < nv) atomicAdd(upd + v, value);
        }
        r2 = (double)res * (double)res; /* exact */
    }
    if (lane == 0) sres[w] = r2;
    __syncthreads();
    if (threadIdx.x == 0 && resid) {
        double s = 0.0;
        for (int k = 0; k < NA_WARPS; ++k) s += sres[k];
        if (s != 0.0) atomicAdd(resid, s);
    }
}

/* x += upd / s_j, then clears both scratch entries for the next block. */
__global__ void k_na_relax(int nv, uint32_t* __restrict__ cnt, float* __restrict__ x, float* __restrict__ upd) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    uint32_t s = cnt[v];
    if (s > 0) {
        x[v] += upd[v] / (float)s;
        upd[v] = 0.0f;
        cnt[v] = 0u;
    }
}

unsigned grid_for(int64_t threads, int block) { return (unsigned)((threads + block - 1) / block); }

}  // namespace

extern "C" pct_status pct_noalloc_setup(void) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return pct_fail(PCT_ERR_CUDA, "pct_noalloc_setup: cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= NA_MAX_DEVICES)
        return pct_fail(PCT_ERR_ARGUMENT, "pct_noalloc_setup: device %d beyond the %d supported", dev, NA_MAX_DEVICES);
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (g_scratch_ptr[dev]) return PCT_OK;
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_drop_scratch);
    if (e != cudaSuccess || !p)
        return pct_fail(PCT_ERR_CUDA, "pct_noalloc_setup: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    g_scratch_ptr[dev] = p;
    return PCT_OK;
}

extern "C" pct_status pct_drop_noalloc(int64_t n, const int64_t* row_offsets, const uint32_t* rows, const float* chord,
                                       const float* wepl, int num_voxels, int block_size, float lambda,
                                       int iterations, float* x, double* residual_sq, void* stream) {
    if (num_voxels <= 0) return pct_fail(PCT_ERR_ARGUMENT, "pct_drop_noalloc: num_voxels %d", num_voxels);
    if (num_voxels > PCT_NOALLOC_MAX_VOXELS)
        return pct_fail(PCT_ERR_ARGUMENT,
                        "pct_drop_noalloc: %d voxels exceed the static scratch of %d voxels (use pct_drop)",
                        num_voxels, PCT_NOALLOC_MAX_VOXELS);
    if (n < 0 || block_size <= 0 || iterations < 0)
        return pct_fail(PCT_ERR_ARGUMENT, "pct_drop_noalloc: n %lld, block_size %d, iterations %d", (long long)n,
                        block_size, iterations);
    if (!x || (n > 0 && (!row_offsets || !rows || !chord || !wepl)))
        return pct_fail(PCT_ERR_ARGUMENT, "pct_drop_noalloc: null array");
    pct_status s = pct_noalloc_setup();
    if (s != PCT_OK) return s;
    int dev = 0;
    cudaGetDevice(&dev);
    unsigned char* base = (unsigned char*)g_scratch_ptr[dev];
    float* upd = (float*)base;
    uint32_t* cnt = (uint32_t*)(base + (size_t)PCT_NOALLOC_MAX_VOXELS * 4);
    cudaStream_t st = (cudaStream_t)stream;
    /* a call that failed half-way may have left partial sums behind */
    cudaError_t e = cudaMemsetAsync(upd, 0, sizeof(float) * (size_t)num_voxels, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * (size_t)num_voxels, st);
    if (e == cudaSuccess && residual_sq && iterations > 0)
        e = cudaMemsetAsync(residual_sq, 0, sizeof(double) * (size_t)iterations, st);
    if (e != cudaSuccess) return pct_fail(PCT_ERR_CUDA, "pct_drop_noalloc: clear: %s", cudaGetErrorString(e));
    const int64_t B = block_size;
    for (int it = 0; it < iterations; ++it) {
        double* r = residual_sq ? residual_sq + it : nullptr;
        for (int64_t a = 0; a < n; a += B) {
            int64_t b = a + B < n ? a + B : n;
            k_na_counts<<<grid_for((b - a) * 32, NA_THREADS), NA_THREADS, 0, st>>>(a, b, row_offsets, rows,
                                                                                 (uint32_t)num_voxels, cnt);
            k_na_rows<<<grid_for(b - a, NA_WARPS), NA_THREADS, 0, st>>>(a, b, row_offsets, rows, chord, wepl, lambda,
                                                                       x, upd, (uint32_t)num_voxels, r);
            k_na_relax<<<grid_for(num_voxels, NA_THREADS), NA_THREADS, 0, st>>>(num_voxels, cnt, x, upd);
        }
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return pct_fail(PCT_ERR_CUDA, "pct_drop_noalloc: launch: %s", cudaGetErrorString(e));
    return PCT_OK;
}
