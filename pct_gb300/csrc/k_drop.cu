/*
 * Stages a16-a18: the DROP block-iterative solver on resident MLP rows.
 *
 * Per block of B consecutive recon histories (BLOCK_SIZE_RECON, the
 * reference's block loop .cu:6803-6844) one launch does block_update_GPU
 * (.cu:5774-5841) without the MLP: the dot of every row with the iterate at
 * the start of the block, the update value c * lambda * (b - c sum x) / ||a||^2
 * with ||a||^2 in binary64, its addition to every voxel of the row, and the
 * binary64 squared residual; a second launch is image_update_GPU
 * (.cu:5900-5938): x += x_update / s_j with s_j the number of block row
 * entries in voxel j (the DROP diagonal weight).  s_j depends only on the
 * rows and the block split, so it is counted once per set of rows instead of
 * in every iteration.  One CUDA graph holds the 2 * blocks launches of an
 * iteration.
 *
 * Aggregated form (default): the rows of each block are visited in sinogram
 * bin order (a per-block counting sort by bin, once per set of rows), and one
 * warp walks 32 consecutive rows in step, one per lane (k_drop_lanes).  Rows
 * of one bin follow nearly the same path, so the iterate gathers of a step
 * coalesce and the lanes on one voxel add their summed update with a single
 * L2 reduction.  The diagonal weights come from the same kernel adding 1 per
 * entry.
 * Scatter form: one warp per row in history order and one L2 reduction per
 * row entry (k_drop_rows), the direct transcription of the block update.
 */
#include <cstring>
#include "pct_device.cuh"

namespace {

constexpr int DROP_THREADS = 256;
constexpr int DROP_WARPS = DROP_THREADS / 32;

/* ---- scatter form ------------------------------------------------------------ */

/* s_j of one block: one warp per row */
__global__ void k_block_counts(int64_t start, int64_t end, const int64_t* __restrict__ row_start,
                               const int* __restrict__ row_len, const uint32_t* __restrict__ rows, uint32_t nv,
                               uint32_t* __restrict__ cnt) {
    int lane = threadIdx.x & 31;
    int64_t i = start + ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    if (i >= end) return;
    int64_t a = row_start[i], b = a + row_len[i];
    for (int64_t p = a + lane; p < b; p += 32) {
        uint32_t v = rows[p];
        if (v < nv) atomicAdd(cnt + v, 1u);
    }
}

__global__ void __launch_bounds__(DROP_THREADS) k_drop_rows(int64_t start, int64_t end,
                                                            const uint32_t* __restrict__ perm,
                                                            const int64_t* __restrict__ row_start,
                                                            const int* __restrict__ row_len,
                                                            const uint32_t* __restrict__ rows,
                                                            const float* __restrict__ chord,
                                                            const double* __restrict__ inv_norm,
                                                            const float* __restrict__ wepl, float lambda,
                                                            const float* __restrict__ x, float* __restrict__ upd,
                                                            uint32_t nv, double* __restrict__ resid) {
    __shared__ double sres[DROP_WARPS];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int64_t i = start + (int64_t)blockIdx.x * DROP_WARPS + w;
    double r2 = 0.0;
    if (i < end) {
        if (perm) i = start + perm[i];
        int64_t a = row_start[i], b = a + row_len[i];
        float dot = 0.0f;
        for (int64_t p = a + lane; p < b; p += 32) {
            uint32_t v = rows[p];
            if (v < nv) dot += x[v];
        }
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
        double c = chord[i];
        double res = (double)wepl[i] - c * (double)dot;
        float value = (float)(c * res * inv_norm[i] * (double)lambda);
        for (int64_t p = a + lane; p < b; p += 32) {
            uint32_t v = rows[p];
            if (v < nv) atomicAdd(upd + v, value);
        }
        r2 = res * res;
    }
    if (lane == 0) sres[w] = r2;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < DROP_WARPS; ++k) s += sres[k];
        if (s != 0.0) atomicAdd(resid, s);
    }
}

__global__ void k_drop_relax(int nv, const uint32_t* __restrict__ cnt, float* __restrict__ x, float* __restrict__ upd) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    uint32_t s = cnt[v];
    if (s > 0) {
        x[v] += upd[v] / (float)s;
        upd[v] = 0.0f;
    }
}

/* ---- aggregated form ----------------------------------------------------------- */
constexpr int SCAN_TILE = 4096;       /* keys per scan tile: 1024 threads x 4 */

/* Counting sort of one block's rows by sinogram bin: counts, scan, placement. */
__global__ void k_sort_count(int64_t start, int64_t end, const int32_t* __restrict__ bin_num, uint32_t nkeys,
                             uint32_t* __restrict__ cnt) {
    int64_t i = start + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= end) return;
    uint32_t key = (uint32_t)bin_num[i];
    atomicAdd(cnt + (key < nkeys ? key : 0u), 1u);
}

__device__ __forceinline__ uint32_t block_exclusive_scan_u32(uint32_t v, uint32_t* ws, uint32_t* total) {
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

/* tile sums of the counts (one CTA per 4096 keys) */
__global__ void __launch_bounds__(1024) k_scan_tile_sum_u32(const uint32_t* __restrict__ cnt, uint32_t nkeys,
                                                            uint32_t* __restrict__ tsum) {
    __shared__ uint32_t ws[32];
    uint32_t k0 = blockIdx.x * SCAN_TILE + threadIdx.x * 4, s = 0;
    for (int k = 0; k < 4; ++k) s += k0 + k < nkeys ? cnt[k0 + k] : 0u;
    uint32_t total;
    block_exclusive_scan_u32(s, ws, &total);
    if (threadIdx.x == 0) tsum[blockIdx.x] = total;
}

/* exclusive scan of the tile sums (one CTA) */
__global__ void __launch_bounds__(1024) k_scan_tiles_u32(uint32_t* __restrict__ tsum, int tiles) {
    __shared__ uint32_t ws[32];
    uint32_t carry = 0;
    for (int base = 0; base < tiles; base += 1024) {
        int k = base + threadIdx.x;
        uint32_t v = k < tiles ? tsum[k] : 0u, total;
        uint32_t ex = block_exclusive_scan_u32(v, ws, &total);
        if (k < tiles) tsum[k] = carry + ex;
        carry += total;
    }
}

/* off[k] = exclusive prefix of the counts */
__global__ void __launch_bounds__(1024) k_scan_apply_u32(const uint32_t* __restrict__ cnt, uint32_t nkeys,
                                                         const uint32_t* __restrict__ tsum,
                                                         uint32_t* __restrict__ off) {
    __shared__ uint32_t ws[32];
    uint32_t k0 = blockIdx.x * SCAN_TILE + threadIdx.x * 4;
    uint32_t e[4], s = 0;
    for (int k = 0; k < 4; ++k) {
        e[k] = k0 + k < nkeys ? cnt[k0 + k] : 0u;
        s += e[k];
    }
    uint32_t total;
    uint32_t run = block_exclusive_scan_u32(s, ws, &total) + tsum[blockIdx.x];
    for (int k = 0; k < 4; ++k) {
        if (k0 + k < nkeys) off[k0 + k] = run;
        run += e[k];
    }
}

/* perm[start + off[key] + slot] = block-local row index (counts consumed as cursors) */
__global__ void k_sort_fill(int64_t start, int64_t end, const int32_t* __restrict__ bin_num, uint32_t nkeys,
                            uint32_t* __restrict__ cnt, const uint32_t* __restrict__ off,
                            uint32_t* __restrict__ perm) {
    int64_t i = start + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= end) return;
    uint32_t key = (uint32_t)bin_num[i];
    key = key < nkeys ? key : 0u;
    uint32_t slot = atomicSub(cnt + key, 1u) - 1u;
    perm[start + off[key] + slot] = (uint32_t)(i - start);
}

/* Sum of val over this lane's run of equal v up to the run's end (runs are
 * maximal sequences of consecutive lanes with equal v), by a segmented suffix
 * scan; the run's first lane gets the whole run's sum. */
__device__ __forceinline__ float run_sum(uint32_t v, float val, int lane, int* is_head) {
    uint32_t nxt = __shfl_down_sync(0xffffffffu, v, 1);
    uint32_t prv = __shfl_up_sync(0xffffffffu, v, 1);
    int f = lane == 31 || nxt != v; /* a run ends inside this lane's window */
    float sum = val;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        float ts = __shfl_down_sync(0xffffffffu, sum, o);
        int tf = __shfl_down_sync(0xffffffffu, f, o);
        if (!f) {
            sum += ts;
            f = tf;
        }
    }
    *is_head = lane == 0 || prv != v;
    return sum;
}

/* One warp: 32 consecutive rows of the block's bin order, one per lane, walked
 * entry by entry in step.  The rows are read in coalesced 32-entry chunks
 * (row by row) and transposed through shared memory.  Rows of one bin follow
 * nearly the same path, so at each step the lanes hold a few distinct voxels:
 * the iterate gathers coalesce, and each run of lanes on one voxel adds its
 * summed update with a single reduction.  COUNT: adds 1 per row entry (the
 * diagonal weights, exact in binary32 below 2^24); otherwise the block update
 * into out (x_update). */
constexpr int LANE_WARPS = 4;
constexpr uint32_t NO_VOXEL = 0xffffffffu;

struct LaneRows {
    int64_t a[32];
    int len[32];
    uint32_t buf[32][33];
};

/* Stages entries [k0, k0 + 32) of the warp's 32 rows: buf[r][e] = entry k0 + e of row r. */
__device__ __forceinline__ void stage_chunk(LaneRows& L, const uint32_t* __restrict__ rows, int k0, int lane) {
    __syncwarp();
    for (int r = 0; r < 32; ++r) {
        int k = k0 + lane;
        L.buf[r][lane] = k < L.len[r] ? rows[L.a[r] + k] : NO_VOXEL;
    }
    __syncwarp();
}

template <bool COUNT>
__global__ void __launch_bounds__(LANE_WARPS * 32) k_drop_lanes(int64_t start, int64_t end,
                                                                const uint32_t* __restrict__ perm,
                                                                const int64_t* __restrict__ row_start,
                                                                const int* __restrict__ row_len,
                                                                const uint32_t* __restrict__ rows,
                                                                const float* __restrict__ chord,
                                                                const double* __restrict__ inv_norm,
                                                                const float* __restrict__ wepl, float lambda,
                                                                const float* __restrict__ x, uint32_t nv,
                                                                float* __restrict__ out, double* __restrict__ resid) {
    __shared__ LaneRows lr[LANE_WARPS];
    __shared__ double sres[LANE_WARPS];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    LaneRows& L = lr[w];
    const int64_t j = start + ((int64_t)blockIdx.x * LANE_WARPS + w) * 32 + lane;
    const bool have = j < end;
    int64_t i = 0;
    int len = 0;
    if (have) {
        i = start + perm[j];
        L.a[lane] = row_start[i];
        len = row_len[i];
    } else {
        L.a[lane] = 0;
    }
    L.len[lane] = len;
    int maxlen = len;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        int t = __shfl_xor_sync(0xffffffffu, maxlen, o);
        maxlen = t > maxlen ? t : maxlen;
    }
    float val = 1.0f;
    double r2 = 0.0;
    if (!COUNT) {
        float dot = 0.0f;
        for (int k0 = 0; k0 < maxlen; k0 += 32) {
            stage_chunk(L, rows, k0, lane);
#pragma unroll 4
            for (int e = 0; e < 32; ++e) {
                uint32_t v = L.buf[lane][e];
                if (v < nv) dot += x[v];
            }
        }
        if (have) {
            double c = chord[i];
            double res = (double)wepl[i] - c * (double)dot;
            val = (float)(c * res * inv_norm[i] * (double)lambda);
            r2 = res * res;
        }
    }
    for (int k0 = 0; k0 < maxlen; k0 += 32) {
        stage_chunk(L, rows, k0, lane);
        int kend = maxlen - k0 < 32 ? maxlen - k0 : 32;
        for (int e = 0; e < kend; ++e) {
            uint32_t v = L.buf[lane][e];
            float contrib = v < nv ? val : 0.0f;
            int head;
            float sum = run_sum(v, contrib, lane, &head);
            if (head && v < nv) atomicAdd(out + v, sum);
        }
    }
    if (!COUNT) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r2 += __shfl_xor_sync(0xffffffffu, r2, o);
        if (lane == 0) sres[w] = r2;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int k = 0; k < LANE_WARPS; ++k) t += sres[k];
            if (t != 0.0) atomicAdd(resid, t);
        }
    }
}

/* x += x_update / s_j and x_update = 0 where s_j > 0; four voxels per thread
 * (float4 accesses when nv is a multiple of 4, else scalar). */
__global__ void k_drop_relax4(int nv, const float* __restrict__ cnt, float* __restrict__ x, float* __restrict__ upd) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    int v0 = 4 * q;
    if (v0 >= nv) return;
    /* the block's weights start at k * nv floats: 16-byte aligned only when nv % 4 == 0 */
    if ((nv & 3) == 0 && v0 + 3 < nv) {
        float4 s = *reinterpret_cast<const float4*>(cnt + v0);
        if (s.x == 0.0f && s.y == 0.0f && s.z == 0.0f && s.w == 0.0f) return;
        float4 u = *reinterpret_cast<const float4*>(upd + v0);
        float4 xv = *reinterpret_cast<float4*>(x + v0);
        if (s.x > 0.0f) xv.x += u.x / s.x;
        if (s.y > 0.0f) xv.y += u.y / s.y;
        if (s.z > 0.0f) xv.z += u.z / s.z;
        if (s.w > 0.0f) xv.w += u.w / s.w;
        *reinterpret_cast<float4*>(x + v0) = xv;
        *reinterpret_cast<float4*>(upd + v0) = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    } else {
        for (int v = v0; v < nv; ++v) {
            float s = cnt[v];
            if (s > 0.0f) {
                x[v] += upd[v] / s;
                upd[v] = 0.0f;
            }
        }
    }
}

/* Moves the iteration's residual accumulator into its history slot. */
__global__ void k_store_resid(double* __restrict__ acc, double* __restrict__ slot) {
    *slot = *acc;
    *acc = 0.0;
}

__global__ void k_wepl_norm(int64_t n, const float* __restrict__ wepl, double* __restrict__ out) {
    __shared__ double red[32];
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double w = wepl[i];
        s += w * w;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
        atomicAdd(out, t);
    }
}

}  // namespace

/* Per-block voxel counts for the scatter form. */
static pct_status build_scatter(pct_ctx* c) {
    const int64_t n = c->h.n;
    const int64_t B = c->cfg.block_size;
    const int nv = c->geo.num_voxels;
    int nb = (int)((n + B - 1) / B);
    PCT_TRY(c->block_diag.alloc(sizeof(uint32_t) * (size_t)nv * (nb > 0 ? nb : 1)));
    PCT_CUDA(cudaMemsetAsync(c->block_diag.p, 0, sizeof(uint32_t) * (size_t)nv * (nb > 0 ? nb : 1), c->stream));
    for (int k = 0; k < nb; ++k) {
        int64_t s = k * B, e = s + B < n ? s + B : n;
        ++c->launches;
        k_block_counts<<<pct_grid_for((e - s) * 32, 256), 256, 0, c->stream>>>(
            s, e, c->row_offsets.as<int64_t>(), c->row_len.as<int>(), c->rows.as<uint32_t>(), (uint32_t)nv,
            c->block_diag.as<uint32_t>() + (size_t)k * nv);
    }
    PCT_CUDA(cudaGetLastError());
    c->num_blocks = nb;
    c->drop_aggregated = 0;
    c->diag_ready = 1;
    return PCT_OK;
}

/* Bin order of every block and the per-block diagonal weights (binary32) for
 * the aggregated form. */
static pct_status build_aggregated(pct_ctx* c) {
    const int64_t n = c->h.n;
    const int64_t B = c->cfg.block_size;
    const int nv = c->geo.num_voxels;
    const uint32_t nkeys = (uint32_t)c->geo.num_bins;
    const int tiles = (int)((nkeys + SCAN_TILE - 1) / SCAN_TILE);
    int nb = (int)((n + B - 1) / B);
    PCT_TRY(c->drop_perm.alloc(sizeof(uint32_t) * (n > 0 ? n : 1)));
    PCT_TRY(c->drop_sort.alloc(sizeof(uint32_t) * ((size_t)2 * nkeys + tiles)));
    uint32_t* cnt = c->drop_sort.as<uint32_t>();
    uint32_t* off = cnt + nkeys;
    uint32_t* tsum = off + nkeys;
    const int32_t* bin = c->h.bin_num.as<int32_t>();
    uint32_t* perm = c->drop_perm.as<uint32_t>();
    for (int k = 0; k < nb; ++k) {
        int64_t s = k * B, e = s + B < n ? s + B : n;
        PCT_CUDA(cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * nkeys, c->stream));
        c->launches += 5;
        k_sort_count<<<pct_grid_for(e - s, 256), 256, 0, c->stream>>>(s, e, bin, nkeys, cnt);
        k_scan_tile_sum_u32<<<tiles, 1024, 0, c->stream>>>(cnt, nkeys, tsum);
        k_scan_tiles_u32<<<1, 1024, 0, c->stream>>>(tsum, tiles);
        k_scan_apply_u32<<<tiles, 1024, 0, c->stream>>>(cnt, nkeys, tsum, off);
        k_sort_fill<<<pct_grid_for(e - s, 256), 256, 0, c->stream>>>(s, e, bin, nkeys, cnt, off, perm);
    }
    PCT_TRY(c->block_diag.alloc(sizeof(float) * (size_t)nv * (nb > 0 ? nb : 1)));
    PCT_CUDA(cudaMemsetAsync(c->block_diag.p, 0, sizeof(float) * (size_t)nv * (nb > 0 ? nb : 1), c->stream));
    for (int k = 0; k < nb; ++k) {
        int64_t s = k * B, e = s + B < n ? s + B : n;
        ++c->launches;
        k_drop_lanes<true><<<(unsigned)((e - s + LANE_WARPS * 32 - 1) / (LANE_WARPS * 32)), LANE_WARPS * 32, 0, c->stream>>>(
            s, e, perm, c->row_offsets.as<int64_t>(), c->row_len.as<int>(), c->rows.as<uint32_t>(), nullptr,
            nullptr, nullptr, 0.0f, nullptr, (uint32_t)nv, c->block_diag.as<float>() + (size_t)k * nv, nullptr);
    }
    PCT_CUDA(cudaGetLastError());
    c->num_blocks = nb;
    c->drop_aggregated = c->cfg.drop_form == 1 ? 2 : 1;
    c->diag_ready = 1;
    return PCT_OK;
}

/* Enqueues one DROP iteration (all blocks) on the context stream. */
static void enqueue_iteration(pct_ctx* c, double* resid) {
    const int64_t n = c->h.n;
    const int64_t B = c->cfg.block_size;
    const int nv = c->geo.num_voxels;
    for (int k = 0; k < c->num_blocks; ++k) {
        int64_t s = k * B, e = s + B < n ? s + B : n;
        if (c->drop_aggregated == 2) {
            unsigned grid = (unsigned)((e - s + DROP_WARPS - 1) / DROP_WARPS);
            k_drop_rows<<<grid, DROP_THREADS, 0, c->stream>>>(s, e, c->drop_perm.as<uint32_t>(),
                                                              c->row_offsets.as<int64_t>(), c->row_len.as<int>(),
                                                              c->rows.as<uint32_t>(), c->chord.as<float>(),
                                                              c->inv_norm.as<double>(), c->h.wepl.as<float>(),
                                                              c->cfg.lambda, c->x.as<float>(), c->x_update.as<float>(),
                                                              (uint32_t)nv, resid);
            k_drop_relax4<<<pct_grid_for((nv + 3) / 4, 256), 256, 0, c->stream>>>(
                nv, c->block_diag.as<float>() + (size_t)k * nv, c->x.as<float>(), c->x_update.as<float>());
        } else if (c->drop_aggregated) {
            k_drop_lanes<false><<<(unsigned)((e - s + LANE_WARPS * 32 - 1) / (LANE_WARPS * 32)), LANE_WARPS * 32, 0,
                                  c->stream>>>(
                s, e, c->drop_perm.as<uint32_t>(), c->row_offsets.as<int64_t>(), c->row_len.as<int>(),
                c->rows.as<uint32_t>(), c->chord.as<float>(), c->inv_norm.as<double>(), c->h.wepl.as<float>(),
                c->cfg.lambda, c->x.as<float>(), (uint32_t)nv, c->x_update.as<float>(), resid);
            k_drop_relax4<<<pct_grid_for((nv + 3) / 4, 256), 256, 0, c->stream>>>(
                nv, c->block_diag.as<float>() + (size_t)k * nv, c->x.as<float>(), c->x_update.as<float>());
        } else {
            unsigned grid = (unsigned)((e - s + DROP_WARPS - 1) / DROP_WARPS);
            k_drop_rows<<<grid, DROP_THREADS, 0, c->stream>>>(s, e, nullptr, c->row_offsets.as<int64_t>(),
                                                              c->row_len.as<int>(),
                                                              c->rows.as<uint32_t>(), c->chord.as<float>(),
                                                              c->inv_norm.as<double>(), c->h.wepl.as<float>(),
                                                              c->cfg.lambda, c->x.as<float>(), c->x_update.as<float>(),
                                                              (uint32_t)nv, resid);
            k_drop_relax<<<pct_grid_for(nv, 256), 256, 0, c->stream>>>(nv, c->block_diag.as<uint32_t>() + (size_t)k * nv,
                                                                       c->x.as<float>(), c->x_update.as<float>());
        }
    }
}

static pct_status capture_iteration(pct_ctx* c, double* acc) {
    if (c->drop_graph_exec) return PCT_OK;
    cudaGraph_t graph = nullptr;
    PCT_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    enqueue_iteration(c, acc);
    cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
    if (e != cudaSuccess) return pct_fail(PCT_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return pct_fail(PCT_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    c->drop_graph_exec = exec;
    return PCT_OK;
}

pct_status pct_stage_drop(pct_ctx* c, int iterations, pct_drop_stats* stats) {
    if (c->stage != ST_ROWS) return pct_fail(PCT_ERR_STATE, "drop needs MLP rows");
    if (iterations < 0) return pct_fail(PCT_ERR_ARGUMENT, "drop: negative iteration count");
    const int nv = c->geo.num_voxels;
    if (!c->diag_ready) {
        if (c->cfg.drop_form == PCT_DROP_SCATTER) PCT_TRY(build_scatter(c));
        else PCT_TRY(build_aggregated(c));
        pct_drop_release_graph(c);
    }
    PCT_TRY(c->x_update.alloc(sizeof(float) * nv));
    PCT_CUDA(cudaMemsetAsync(c->x_update.p, 0, sizeof(float) * nv, c->stream));
    const int maxit = 64;
    /* [0, maxit): per-iteration squared residual, maxit: accumulator, maxit+1: ||b||^2 */
    PCT_TRY(c->drop_resid.alloc(sizeof(double) * (maxit + 2)));
    double* d_res = c->drop_resid.as<double>();
    PCT_CUDA(cudaMemsetAsync(d_res, 0, sizeof(double) * (maxit + 2), c->stream));
    if (c->h.n > 0) k_wepl_norm<<<304, 256, 0, c->stream>>>(c->h.n, c->h.wepl.as<float>(), d_res + maxit + 1);
    PCT_TRY(capture_iteration(c, d_res + maxit));
    cudaEvent_t e0, e1;
    PCT_CUDA(cudaEventCreate(&e0));
    PCT_CUDA(cudaEventCreate(&e1));
    PCT_CUDA(cudaEventRecord(e0, c->stream));
    int done = 0;
    double res_host[maxit + 2];
    for (int it = 0; it < iterations; ++it) {
        PCT_CUDA(cudaGraphLaunch(c->drop_graph_exec, c->stream));
        c->launches += 2 * (int64_t)c->num_blocks;
        ++c->launches;
        k_store_resid<<<1, 1, 0, c->stream>>>(d_res + maxit, d_res + (it < maxit ? it : maxit - 1));
        ++done;
        if (c->cfg.residual_tol > 0.0) {
            PCT_CUDA(cudaMemcpyAsync(res_host, d_res, sizeof(double) * (maxit + 2), cudaMemcpyDeviceToHost, c->stream));
            PCT_CUDA(cudaStreamSynchronize(c->stream));
            double b2 = res_host[maxit + 1];
            double rel = b2 > 0 ? sqrt(res_host[it < maxit ? it : maxit - 1] / b2) : 0.0;
            if (rel < c->cfg.residual_tol) break;
        }
    }
    PCT_CUDA(cudaEventRecord(e1, c->stream));
    PCT_CUDA(cudaGetLastError());
    PCT_CUDA(cudaMemcpyAsync(res_host, d_res, sizeof(double) * (maxit + 2), cudaMemcpyDeviceToHost, c->stream));
    PCT_CUDA(cudaStreamSynchronize(c->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->iterations_run = done;
        double b2 = res_host[maxit + 1];
        for (int k = 0; k < done && k < maxit; ++k) stats->residual[k] = b2 > 0 ? sqrt(res_host[k] / b2) : 0.0;
        stats->seconds = ms * 1e-3;
    }
    return PCT_OK;
}

void pct_drop_release_graph(pct_ctx* c) {
    if (c->drop_graph_exec) cudaGraphExecDestroy(c->drop_graph_exec);
    c->drop_graph_exec = nullptr;
}
