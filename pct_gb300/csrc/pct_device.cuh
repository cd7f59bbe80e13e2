/*
 * Device helpers shared by the kernels: voxel arithmetic of the reference
 * walks, the brick voxel order, certified binary32 walk arithmetic and block
 * scans.
 *
 * The voxel helpers evaluate the reference's expressions
 * (src/pCT_Reconstruction_Data_Segments.cu:8508-8752) in binary64 in source
 * order; the library is compiled with -fmad=false, so no multiply-add pair
 * is fused behind the source's back and the results equal the CPU oracle's.
 */
#ifndef PCT_DEVICE_CUH
#define PCT_DEVICE_CUH

#include <cstdint>
#include "pct_ctx.h"

#define PCT_X_INC 1    /* X_INCREASING_DIRECTION = RIGHT (pCT_data.h:275) */
#define PCT_Y_INC (-1) /* DOWN */
#define PCT_Z_INC (-1) /* DOWN */

/* calculate_voxel_GPU (.cu:8508) */
__device__ __forceinline__ int dev_calculate_voxel(double zero, double pos, double size) {
    return pct_d2i(fabs(pos - zero) / size);
}
/* edge_coordinate_GPU (.cu:8735) */
__device__ __forceinline__ double dev_edge_coordinate(double zero, int voxel_entered, double size, int inc, int step) {
    int on_edge = (step == inc) ? voxel_entered : voxel_entered + 1;
    return zero + (inc * on_edge * size);
}
/* distance_remaining_GPU (.cu:8721) */
__device__ __forceinline__ double dev_distance_remaining(double zero, double pos, int inc, int step, double size,
                                                         int voxel) {
    return fabs(dev_edge_coordinate(zero, voxel + inc * step, size, inc, step) - pos);
}
/* corresponding_coordinate_GPU (.cu:8748) */
__device__ __forceinline__ double dev_corresponding(double m, double x, double x0, double y0) {
    return m * (x - x0) + y0;
}

/* relative angle with the +-2 pi wrap (.cu:2557-2566) */
__device__ __forceinline__ double dev_rel_angle(float exit_angle, float entry_angle) {
    double r = exit_angle - entry_angle;
    if (r > PCT_PI) r -= 2 * PCT_PI;
    if (r < -PCT_PI) r += 2 * PCT_PI;
    return r;
}

__device__ __forceinline__ void dev_flag(unsigned long long* flags, int which) {
    atomicAdd(flags + which, 1ull);
}

/* Brick voxel order of the MLP rows and the DROP iterate: 4x2x1 voxel bricks
 * (one 32-byte sector of floats), bricks in x, y, z order.  A path step in x
 * or y then stays in the same sector more often than in the linear order, so
 * the DROP gathers and reductions touch fewer L2 sectors.  Indices >= the
 * voxel count (row entries outside the image) are kept as they are. */
__host__ __device__ __forceinline__ uint32_t dev_brick_xyz(uint32_t C, uint32_t R, uint32_t x, uint32_t y, uint32_t z) {
    return (((x >> 2) + (C >> 2) * ((y >> 1) + (R >> 1) * z)) << 3) | (x & 3u) | ((y & 1u) << 2);
}
__host__ __device__ __forceinline__ uint32_t dev_div(uint32_t n, uint32_t d, unsigned long long m) {
#if defined(__CUDA_ARCH__)
    return d > 1 ? (uint32_t)__umul64hi((unsigned long long)n, m) : n;
#else
    (void)m;
    return n / d;
#endif
}
__host__ __device__ __forceinline__ uint32_t dev_to_brick(const DevGeom& g, uint32_t v) {
    if (!g.brick || v >= (uint32_t)g.num_voxels) return v;
    const uint32_t C = (uint32_t)g.columns, R = (uint32_t)g.rows;
    const uint32_t r = dev_div(v, C, g.div_c), x = v - r * C, z = dev_div(r, R, g.div_r), y = r - z * R;
    return dev_brick_xyz(C, R, x, y, z);
}
__host__ __device__ __forceinline__ uint32_t dev_from_brick(const DevGeom& g, uint32_t b) {
    if (!g.brick || b >= (uint32_t)g.num_voxels) return b;
    const uint32_t C4 = (uint32_t)g.columns >> 2, R2 = (uint32_t)g.rows >> 1;
    const uint32_t w = b & 7u, q = b >> 3;
    const uint32_t t = q / C4, bx = q - t * C4, z = t / R2, by = t - z * R2;
    const uint32_t x = bx * 4u + (w & 3u), y = by * 2u + (w >> 2);
    return x + (uint32_t)g.columns * (y + (uint32_t)g.rows * z);
}

/* ---- binary32 walk arithmetic with error bounds (certified walks) ---- */
constexpr float WU = 1.2e-7f; /* twice the binary32 unit roundoff */

/* edge_coordinate_GPU in binary32 and a bound on its error */
__device__ __forceinline__ float edge32(float zero, int voxel_entered, float size, int inc, int step, float* err) {
    int on_edge = (step == inc) ? voxel_entered : voxel_entered + 1;
    float k = (float)(inc * on_edge);
    float prod = k * size;
    float e = zero + prod;
    *err = WU * (fabsf(zero) + 2.0f * fabsf(prod) + fabsf(e));
    return e;
}

/* corresponding_coordinate in binary32: m (p - p0) + q0 with |error of p| <= ep */
__device__ __forceinline__ float corr32(float m, float p, float p0, float q0, float ep, float* err) {
    float d = p - p0;
    float md = m * d;
    float r = md + q0;
    *err = fabsf(m) * (ep + WU * fabsf(d)) + WU * (fabsf(md) + fabsf(r));
    return r;
}

/* a <= b decided with certainty: 1 / 0, or -1 when the bounds overlap */
__device__ __forceinline__ int cmp_le(float a, float ea, float b, float eb) {
    float d = b - a;
    float tol = ea + eb + WU * (fabsf(a) + fabsf(b));
    if (d > tol) return 1;
    if (-d > tol) return 0;
    return -1;
}

/* Launch order for per-history kernels whose work per thread varies: each chunk
 * of ORDER_CHUNK histories counting-sorted by an integer work estimate (clamped
 * to ORDER_KEYS - 1), so that the 32 histories of a warp do about the same
 * amount of work.  order[] is a permutation of [0, n) within each chunk; the
 * results of the ordered kernels do not depend on it.  1024 threads per CTA. */
constexpr int ORDER_CHUNK = 4096;
constexpr int ORDER_KEYS = 1024;
template <typename K>
__global__ void __launch_bounds__(1024) k_chunk_order(int64_t n, const K* __restrict__ key,
                                                      uint32_t* __restrict__ order) {
    __shared__ int cnt[ORDER_KEYS];
    __shared__ int wsum[32];
    const int64_t base = (int64_t)blockIdx.x * ORDER_CHUNK;
    const int m = (int)(n - base < ORDER_CHUNK ? n - base : ORDER_CHUNK);
    for (int k = threadIdx.x; k < ORDER_KEYS; k += blockDim.x) cnt[k] = 0;
    __syncthreads();
    constexpr int PER = ORDER_CHUNK / 1024;
    int kk[PER], rank[PER];
#pragma unroll
    for (int r = 0; r < PER; ++r) {
        const int t = threadIdx.x + r * 1024;
        kk[r] = -1;
        if (t < m) {
            const K b = key[base + t];
            kk[r] = b <= (K)0 ? 0 : (b < (K)(ORDER_KEYS - 1) ? (int)b : ORDER_KEYS - 1);
            rank[r] = atomicAdd(&cnt[kk[r]], 1);
        }
    }
    __syncthreads();
    /* exclusive scan of the 1024 bucket counts, one per thread */
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int v = cnt[threadIdx.x];
    int incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    if (w == 0) {
        const int s = wsum[lane];
        int si = s;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, si, o);
            if (lane >= o) si += y;
        }
        wsum[lane] = si - s;
    }
    __syncthreads();
    const int excl = incl - v + wsum[w];
    __syncthreads();
    cnt[threadIdx.x] = excl;
    __syncthreads();
#pragma unroll
    for (int r = 0; r < PER; ++r)
        if (kk[r] >= 0) order[base + cnt[kk[r]] + rank[r]] = (uint32_t)(base + threadIdx.x + r * 1024);
}

/* Exclusive scan of one value per thread over the CTA (blockDim.x a multiple
 * of 32, at most 1024); ws holds 32 words of shared memory; *total receives the
 * CTA's sum.  Every thread of the CTA must call it. */
__device__ __forceinline__ uint32_t dev_block_exclusive_scan_u32(uint32_t v, uint32_t* ws, uint32_t* total) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t s = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        ws[lane] = s;
    }
    __syncthreads();
    uint32_t r = x - v + (w > 0 ? ws[w - 1] : 0u);
    *total = ws[(blockDim.x >> 5) - 1];
    __syncthreads();
    return r;
}

static inline unsigned pct_grid_for(int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    return (unsigned)(b > 0 ? b : 1);
}

#endif
