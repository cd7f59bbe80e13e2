/*
 * Stages a16-a18: the DROP block-iterative solver on resident MLP rows.
 *
 * Per block of B consecutive recon histories (BLOCK_SIZE_RECON, the
 * reference's block loop .cu:6803-6844) one launch does block_update_GPU
 * (.cu:5774-5841) without the MLP: the dot of every row with the iterate at
 * the start of the block, the update value c * lambda * (b - c sum x) / ||a||^2
 * (binary32, with 1 / (c |a|) rounded once from binary64), its addition to every
 * voxel of the row, and the squared residual (each row's square and every sum
 * of them in binary64); a second launch is image_update_GPU
 * (.cu:5900-5938): x += x_update / s_j with s_j the number of block row
 * entries in voxel j (the DROP diagonal weight).  s_j depends only on the
 * rows and the block split, so it is counted once per set of rows instead of
 * in every iteration.  One CUDA graph holds the 2 * blocks launches of an
 * iteration.
 *
 * Forms: the scatter form (the default) runs one warp per row in history
 * order with one L2 reduction per row entry (k_drop_rows + k_drop_relax), the
 * direct transcription of the block update; the sorted form is the scatter
 * form visiting each block's rows in sinogram bin order (a per-block
 * counting sort, once per set of rows); the tiled form (k_drop_tiled.cu)
 * regroups the rows by image tile and sums in fixed point (reproducible).
 */
#include <cstring>
#include "pct_device.cuh"

namespace {

constexpr int DROP_THREADS = 256;
constexpr int DROP_WARPS = DROP_THREADS / 32;
constexpr int DROP_REG = 8; /* row entries per lane held in registers (256 per row) */

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
        uint32_t v = __ldcs(rows + p); /* streamed once: evict first */
        if (v < nv) atomicAdd(cnt + v, 1u);
    }
}

/* VARIANT 0: block_update_GPU; 1: DROP_blocks_red (.cu:7998-8021), the entry's
 * update c lambda r / (||a||^2 + psi_j) with psi_j = ((1 - x_j) eta) psi_sign,
 * in binary32; 2: DROP_blocks_robust2 (.cu:7871-7885), the standard update (its
 * per-voxel sums of c^2 per block are fixed by the rows and counted once,
 * k_block_norms; DROP_update_robust2 adds them up as the blocks go by). */
template <int VARIANT>
__global__ void __launch_bounds__(DROP_THREADS) k_drop_rows(int64_t start, int64_t end,
                                                            const uint32_t* __restrict__ perm,
                                                            const int64_t* __restrict__ row_start,
                                                            const int* __restrict__ row_len,
                                                            const uint32_t* __restrict__ rows,
                                                            const float* __restrict__ chord,
                                                            const float* __restrict__ row_scale,
                                                            const float* __restrict__ wepl, float lambda,
                                                            const float* __restrict__ x, float* __restrict__ upd,
                                                            uint32_t nv, double* __restrict__ resid, float eta,
                                                            float psi_sign) {
    __shared__ double sres[DROP_WARPS];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t stride = (int64_t)gridDim.x * DROP_WARPS;
    /* The squared residuals in binary64: lane (k mod 32) keeps the residual of
     * the warp's k-th row until 32 rows are pending, then every lane adds its
     * exact square with one FMA (one binary64 warp instruction per 32 rows). */
    double r2 = 0.0;
    float pend = 0.0f;
    int nrow = 0;
    /* persistent warps: one row at a time, its first 32 * DROP_REG entries held in
     * registers between the dot and the update (independent loads, one read of the row) */
    for (int64_t j = start + (int64_t)blockIdx.x * DROP_WARPS + w; j < end; j += stride) {
        const int64_t i = perm ? start + perm[j] : j;
        const int64_t a = row_start[i];
        const int len = row_len[i];
        uint32_t e[DROP_REG];
        float xv[DROP_REG];
#pragma unroll
        for (int k = 0; k < DROP_REG; ++k) {
            const int q = lane + 32 * k;
            e[k] = q < len ? __ldcs(rows + a + q) : 0xffffffffu; /* streamed once: evict first */
        }
#pragma unroll
        for (int k = 0; k < DROP_REG; ++k) xv[k] = e[k] < nv ? x[e[k]] : 0.0f;
        float dot = 0.0f;
#pragma unroll
        for (int k = 0; k < DROP_REG; ++k) dot += xv[k];
        for (int q = 32 * DROP_REG + lane; q < len; q += 32) {
            const uint32_t v = __ldcs(rows + a + q);
            if (v < nv) dot += x[v];
        }
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
        /* binary32 throughout: an FP64 warp instruction costs 16 SM cycles on this part */
        const float c = chord[i];
        const float res = fmaf(-c, dot, wepl[i]); /* one rounding */
        if (VARIANT == 1) {
            const float cl_res = (c * lambda) * res;
            const float aa = (c * c) * (float)len;
#pragma unroll
            for (int k = 0; k < DROP_REG; ++k)
                if (e[k] < nv) atomicAdd(upd + e[k], cl_res / (aa + ((1.0f - xv[k]) * eta) * psi_sign));
            for (int q = 32 * DROP_REG + lane; q < len; q += 32) {
                const uint32_t v = __ldcs(rows + a + q);
                if (v < nv) atomicAdd(upd + v, cl_res / (aa + ((1.0f - x[v]) * eta) * psi_sign));
            }
        } else {
            const float value = (res * row_scale[i]) * lambda;
#pragma unroll
            for (int k = 0; k < DROP_REG; ++k)
                if (e[k] < nv) atomicAdd(upd + e[k], value);
            for (int q = 32 * DROP_REG + lane; q < len; q += 32) {
                const uint32_t v = __ldcs(rows + a + q);
                if (v < nv) atomicAdd(upd + v, value);
            }
        }
        if (lane == (nrow & 31)) pend = res;
        if ((++nrow & 31) == 0) {
            r2 = fma((double)pend, (double)pend, r2);
            pend = 0.0f;
        }
    }
    r2 = fma((double)pend, (double)pend, r2);
    for (int o = 16; o > 0; o >>= 1) r2 += __shfl_xor_sync(0xffffffffu, r2, o);
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

/* k_drop_relax on four voxels per thread (16-byte loads); used when nv % 4 == 0
 * so that every block's slice of the counts is 16-byte aligned. */
__global__ void k_drop_relax4(int nv4, const uint4* __restrict__ cnt, float4* __restrict__ x, float4* __restrict__ upd) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nv4) return;
    const uint4 s = cnt[q];
    if ((s.x | s.y | s.z | s.w) == 0u) return;
    float4 u = upd[q], xv = x[q];
    if (s.x > 0) xv.x += u.x / (float)s.x;
    if (s.y > 0) xv.y += u.y / (float)s.y;
    if (s.z > 0) xv.z += u.z / (float)s.z;
    if (s.w > 0) xv.w += u.w / (float)s.w;
    x[q] = xv;
    upd[q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f); /* entries with s = 0 are already 0 */
}

/* ||A||_j of one block: the sum of c^2 over the block's entries in voxel j
 * (DROP_blocks_robust2, .cu:7884), one warp per row. */
__global__ void k_block_norms(int64_t start, int64_t end, const int64_t* __restrict__ row_start,
                              const int* __restrict__ row_len, const uint32_t* __restrict__ rows,
                              const float* __restrict__ chord, uint32_t nv, float* __restrict__ norm) {
    int lane = threadIdx.x & 31;
    int64_t i = start + ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    if (i >= end) return;
    const float c2 = (float)((double)chord[i] * (double)chord[i]);
    int64_t a = row_start[i], b = a + row_len[i];
    for (int64_t p = a + lane; p < b; p += 32) {
        uint32_t v = rows[p];
        if (v < nv) atomicAdd(norm + v, c2);
    }
}

/* DROP_update_robust2 (.cu:7887-7901): x += ||A|| / (||A|| + psi) * x_update / s,
 * psi = psi_sign (1 - x) eta, in binary64 as the reference.  ||A||_j is the sum
 * of c^2 over every entry in voxel j of all blocks processed since the
 * reconstruction started: the reference allocates norm_Ai once (.cu:7448) and
 * never clears it, so `acc` gains this block's sums before they are used. */
__global__ void k_drop_relax_robust2(int nv, const uint32_t* __restrict__ cnt, const float* __restrict__ norm,
                                     double* __restrict__ acc, float* __restrict__ x, float* __restrict__ upd,
                                     double eta, double psi_sign) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    uint32_t s = cnt[v];
    if (s > 0) {
        const double na = acc[v] + (double)norm[v];
        acc[v] = na;
        const float xv = x[v];
        const double psi = psi_sign * (1.0 - (double)xv) * eta;
        x[v] = (float)((double)xv + (na / (na + psi)) * (double)upd[v] / (double)s);
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

/* tile sums of the counts (one CTA per 4096 keys) */
__global__ void __launch_bounds__(1024) k_scan_tile_sum_u32(const uint32_t* __restrict__ cnt, uint32_t nkeys,
                                                            uint32_t* __restrict__ tsum) {
    __shared__ uint32_t ws[32];
    uint32_t k0 = blockIdx.x * SCAN_TILE + threadIdx.x * 4, s = 0;
    for (int k = 0; k < 4; ++k) s += k0 + k < nkeys ? cnt[k0 + k] : 0u;
    uint32_t total;
    dev_block_exclusive_scan_u32(s, ws, &total);
    if (threadIdx.x == 0) tsum[blockIdx.x] = total;
}

/* exclusive scan of the tile sums (one CTA) */
__global__ void __launch_bounds__(1024) k_scan_tiles_u32(uint32_t* __restrict__ tsum, int tiles) {
    __shared__ uint32_t ws[32];
    uint32_t carry = 0;
    for (int base = 0; base < tiles; base += 1024) {
        int k = base + threadIdx.x;
        uint32_t v = k < tiles ? tsum[k] : 0u, total;
        uint32_t ex = dev_block_exclusive_scan_u32(v, ws, &total);
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
    uint32_t run = dev_block_exclusive_scan_u32(s, ws, &total) + tsum[blockIdx.x];
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

/* The iterate between the linear and the brick voxel order. */
__global__ void k_image_to_brick(DevGeom g, const float* __restrict__ lin, float* __restrict__ brk) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < g.num_voxels) brk[dev_to_brick(g, (uint32_t)v)] = lin[v];
}
__global__ void k_image_from_brick(DevGeom g, const float* __restrict__ brk, float* __restrict__ lin) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < g.num_voxels) lin[v] = brk[dev_to_brick(g, (uint32_t)v)];
}

}  // namespace

/* Per-block voxel counts for the scatter form. */
/* Number of DROP blocks: of this context's rows, or of the global rows when the
 * rows are one shard of a sharded DROP (every rank runs every block). */
int pct_drop_num_blocks(const pct_ctx* c) {
    const int64_t B = c->cfg.block_size;
    if (c->num_shards > 1) {
        const int64_t Bg = B * c->num_shards;
        return (int)((c->shard_total + Bg - 1) / Bg);
    }
    return (int)((c->h.n + B - 1) / B);
}

/* Rows [s, e) of block k (empty past the end of a shard). */
void pct_drop_block_range(const pct_ctx* c, int k, int64_t* s, int64_t* e) {
    const int64_t n = c->h.n, B = c->cfg.block_size;
    const int64_t a = (int64_t)k * B;
    *s = a < n ? a : n;
    *e = a + B < n ? a + B : n;
    if (*e < *s) *e = *s;
}

/* Sum over the ranks of a sharded DROP (no-op without a callback). */
static pct_status drop_allreduce(pct_ctx* c, void* data, int64_t count, int dtype) {
    if (!c->allreduce) return PCT_OK;
    PCT_CUDA(cudaStreamSynchronize(c->stream));
    const int rc = c->allreduce(c->allreduce_user, data, count, dtype, 1);
    if (rc != 0) return pct_fail(PCT_ERR_ARGUMENT, "sharded DROP: the all-reduce callback returned %d", rc);
    return PCT_OK;
}

static pct_status build_scatter(pct_ctx* c) {
    const int nv = c->geo.num_voxels;
    int nb = pct_drop_num_blocks(c);
    PCT_TRY(c->block_diag.alloc(sizeof(uint32_t) * (size_t)nv * (nb > 0 ? nb : 1)));
    PCT_CUDA(cudaMemsetAsync(c->block_diag.p, 0, sizeof(uint32_t) * (size_t)nv * (nb > 0 ? nb : 1), c->stream));
    for (int k = 0; k < nb; ++k) {
        int64_t s, e;
        pct_drop_block_range(c, k, &s, &e);
        if (e == s) continue;
        ++c->launches;
        k_block_counts<<<pct_grid_for((e - s) * 32, 256), 256, 0, c->stream>>>(
            s, e, c->row_offsets.as<int64_t>(), c->row_len.as<int>(), c->rows.as<uint32_t>(), (uint32_t)nv,
            c->block_diag.as<uint32_t>() + (size_t)k * nv);
    }
    if (c->cfg.drop_variant == PCT_DROP_ROBUST2) {
        PCT_TRY(c->block_norm.alloc(sizeof(float) * (size_t)nv * (nb > 0 ? nb : 1)));
        PCT_CUDA(cudaMemsetAsync(c->block_norm.p, 0, sizeof(float) * (size_t)nv * (nb > 0 ? nb : 1), c->stream));
        PCT_TRY(c->robust_norm.alloc(sizeof(double) * (size_t)nv));
        PCT_CUDA(cudaMemsetAsync(c->robust_norm.p, 0, sizeof(double) * (size_t)nv, c->stream));
        for (int k = 0; k < nb; ++k) {
            int64_t s, e;
            pct_drop_block_range(c, k, &s, &e);
            if (e == s) continue;
            ++c->launches;
            k_block_norms<<<pct_grid_for((e - s) * 32, 256), 256, 0, c->stream>>>(
                s, e, c->row_offsets.as<int64_t>(), c->row_len.as<int>(), c->rows.as<uint32_t>(), c->chord.as<float>(),
                (uint32_t)nv, c->block_norm.as<float>() + (size_t)k * nv);
        }
    }
    PCT_CUDA(cudaGetLastError());
    if (nb > 0) {
        PCT_TRY(drop_allreduce(c, c->block_diag.p, (int64_t)nv * nb, PCT_DT_U32));
        if (c->cfg.drop_variant == PCT_DROP_ROBUST2)
            PCT_TRY(drop_allreduce(c, c->block_norm.p, (int64_t)nv * nb, PCT_DT_F32));
    }
    c->num_blocks = nb;
    c->drop_mode = PCT_DROP_SCATTER;
    c->drop_launches_per_iter = 2 * nb;
    c->diag_ready = 1;
    return PCT_OK;
}

/* Bin order of every block's rows: drop_perm[start + j] is the block-local
 * index of the block's j-th row in sinogram bin order (a counting sort per
 * block, once per set of rows). */
pct_status pct_drop_bin_order(pct_ctx* c) {
    const int64_t n = c->h.n;
    const uint32_t nkeys = (uint32_t)c->geo.num_bins;
    const int tiles = (int)((nkeys + SCAN_TILE - 1) / SCAN_TILE);
    int nb = pct_drop_num_blocks(c);
    PCT_TRY(c->drop_perm.alloc(sizeof(uint32_t) * (n > 0 ? n : 1)));
    PCT_TRY(c->drop_sort.alloc(sizeof(uint32_t) * ((size_t)2 * nkeys + tiles)));
    uint32_t* cnt = c->drop_sort.as<uint32_t>();
    uint32_t* off = cnt + nkeys;
    uint32_t* tsum = off + nkeys;
    const int32_t* bin = c->h.bin_num.as<int32_t>();
    uint32_t* perm = c->drop_perm.as<uint32_t>();
    for (int k = 0; k < nb; ++k) {
        int64_t s, e;
        pct_drop_block_range(c, k, &s, &e);
        if (e == s) continue;
        PCT_CUDA(cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * nkeys, c->stream));
        c->launches += 5;
        k_sort_count<<<pct_grid_for(e - s, 256), 256, 0, c->stream>>>(s, e, bin, nkeys, cnt);
        k_scan_tile_sum_u32<<<tiles, 1024, 0, c->stream>>>(cnt, nkeys, tsum);
        k_scan_tiles_u32<<<1, 1024, 0, c->stream>>>(tsum, tiles);
        k_scan_apply_u32<<<tiles, 1024, 0, c->stream>>>(cnt, nkeys, tsum, off);
        k_sort_fill<<<pct_grid_for(e - s, 256), 256, 0, c->stream>>>(s, e, bin, nkeys, cnt, off, perm);
    }
    PCT_CUDA(cudaGetLastError());
    return PCT_OK;
}

/* The sorted form: the scatter form visiting each block's rows in bin order. */
static pct_status build_sorted(pct_ctx* c) {
    PCT_TRY(pct_drop_bin_order(c));
    PCT_TRY(build_scatter(c));
    c->drop_mode = PCT_DROP_SORTED;
    return PCT_OK;
}

/* CTAs of a persistent k_drop_rows launch: every resident slot of the device,
 * or fewer when the block has fewer rows than warps. */
static unsigned drop_rows_grid(pct_ctx* c, int64_t rows, const void* fn) {
    int sms = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess || sms < 1) sms = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, DROP_THREADS, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    const int64_t need = (rows + DROP_WARPS - 1) / DROP_WARPS;
    const int64_t cap = (int64_t)sms * per_sm;
    return (unsigned)(need < cap ? (need > 0 ? need : 1) : cap);
}

/* The row pass of block k (scatter and sorted forms): x_update and the
 * residual accumulator; returns the number of launches. */
static int enqueue_block_rows(pct_ctx* c, int k, double* resid) {
    int64_t s, e;
    pct_drop_block_range(c, k, &s, &e);
    if (e == s) return 0;
    const int nv = c->geo.num_voxels;
    const uint32_t* perm = c->drop_mode == PCT_DROP_SORTED ? c->drop_perm.as<uint32_t>() : nullptr;
    float* xi = c->dg.brick ? c->x_brick.as<float>() : c->x.as<float>(); /* the rows' voxel order */
    const int var = c->cfg.drop_variant;
    const float eta = (float)c->cfg.eta, sgn = (float)c->cfg.psi_sign;
    auto rows_kernel = var == PCT_DROP_RED ? k_drop_rows<1> : (var == PCT_DROP_ROBUST2 ? k_drop_rows<2> : k_drop_rows<0>);
    const unsigned grid = drop_rows_grid(c, e - s, (const void*)rows_kernel);
    rows_kernel<<<grid, DROP_THREADS, 0, c->stream>>>(s, e, perm, c->row_offsets.as<int64_t>(), c->row_len.as<int>(),
                                                      c->rows.as<uint32_t>(), c->chord.as<float>(),
                                                      c->row_scale.as<float>(), c->h.wepl.as<float>(), c->cfg.lambda,
                                                      xi, c->x_update.as<float>(), (uint32_t)nv, resid, eta, sgn);
    return 1;
}

/* x += x_update / s_j for block k (and x_update cleared); one launch. */
static void enqueue_block_relax(pct_ctx* c, int k) {
    const int nv = c->geo.num_voxels;
    float* xi = c->dg.brick ? c->x_brick.as<float>() : c->x.as<float>();
    const float eta = (float)c->cfg.eta, sgn = (float)c->cfg.psi_sign;
    if (c->cfg.drop_variant == PCT_DROP_ROBUST2)
        k_drop_relax_robust2<<<pct_grid_for(nv, 256), 256, 0, c->stream>>>(
            nv, c->block_diag.as<uint32_t>() + (size_t)k * nv, c->block_norm.as<float>() + (size_t)k * nv,
            c->robust_norm.as<double>(), xi, c->x_update.as<float>(), c->cfg.eta, (double)c->cfg.psi_sign);
    else if (nv % 4 == 0)
        k_drop_relax4<<<pct_grid_for(nv / 4, 256), 256, 0, c->stream>>>(
            nv / 4, reinterpret_cast<const uint4*>(c->block_diag.as<uint32_t>() + (size_t)k * nv),
            reinterpret_cast<float4*>(xi), reinterpret_cast<float4*>(c->x_update.as<float>()));
    else
        k_drop_relax<<<pct_grid_for(nv, 256), 256, 0, c->stream>>>(nv, c->block_diag.as<uint32_t>() + (size_t)k * nv,
                                                                   xi, c->x_update.as<float>());
}

/* One iteration of a sharded DROP: every block's update summed over the ranks
 * before it is applied, then the iteration's squared residual; not captured
 * (the callback runs on the host between the launches). */
static pct_status run_iteration_sharded(pct_ctx* c, double* resid) {
    for (int k = 0; k < c->num_blocks; ++k) {
        c->launches += enqueue_block_rows(c, k, resid);
        PCT_TRY(drop_allreduce(c, c->x_update.p, c->geo.num_voxels, PCT_DT_F32));
        enqueue_block_relax(c, k);
        ++c->launches;
    }
    PCT_CUDA(cudaGetLastError());
    return drop_allreduce(c, resid, 1, PCT_DT_F64);
}

/* Enqueues one DROP iteration (all blocks) on the context stream. */
static void enqueue_iteration(pct_ctx* c, double* resid) {
    for (int k = 0; k < c->num_blocks; ++k) {
        if (c->drop_mode == PCT_DROP_TILED) {
            pct_drop_tiled_enqueue(c, k, resid);
            continue;
        }
        if (c->drop_mode == PCT_DROP_GATHER) {
            pct_drop_gather_enqueue(c, k, resid);
            continue;
        }
        enqueue_block_rows(c, k, resid);
        enqueue_block_relax(c, k);
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

/* Builds the per-block structures of the configured DROP form once per set of
 * rows and block size (diagonal counts; sort order; tiled segments). */
pct_status pct_drop_prepare(pct_ctx* c) {
    if (!c->diag_ready) {
        pct_drop_release_graph(c);
        c->td.release();
        const int form = c->cfg.drop_form;
        /* the gather form's buffers are kept for its next build (they only grow) */
        if (form != PCT_DROP_GATHER) pct_drop_gather_release(c);
        c->gather_entries = 0;
        if (form == PCT_DROP_TILED && !c->allreduce && c->num_shards == 1 && pct_drop_tiled_fits(c)) {
            PCT_TRY(pct_drop_tiled_build(c));
            const int64_t B = c->cfg.block_size;
            c->num_blocks = c->td.num_blocks;
            c->drop_mode = PCT_DROP_TILED;
            c->drop_launches_per_iter = 0;
            for (int b = 0; b < c->num_blocks; ++b)
                c->drop_launches_per_iter += 2 + (c->td.fw_base[b + 1] > c->td.fw_base[b] ? 1 : 0);
            (void)B;
            c->diag_ready = 1;
        } else if (form == PCT_DROP_SORTED) {
            PCT_TRY(build_sorted(c));
        } else if (form == PCT_DROP_GATHER && c->cfg.drop_variant == PCT_DROP_STANDARD && !c->allreduce &&
                   c->num_shards == 1) {
            /* the scatter form's per-block counts size the gather lists; without the
             * memory for the lists the scatter form runs */
            PCT_TRY(build_scatter(c));
            const pct_status st = pct_drop_gather_build(c);
            if (st == PCT_OK) c->drop_mode = PCT_DROP_GATHER;
            else if (st != PCT_ERR_ALLOC) return st;
        } else {
            PCT_TRY(build_scatter(c));
        }
    }
    return PCT_OK;
}

/* Everything a run of DROP iterations needs before the first one: the
 * per-block structures, a zero x_update, the iterate in the rows' voxel order
 * and the residual slots ([0, maxit): per-iteration squared residual, maxit:
 * accumulator, maxit+1: ||b||^2). */
pct_status pct_drop_begin(pct_ctx* c) {
    if (c->stage != ST_ROWS) return pct_fail(PCT_ERR_STATE, "drop needs MLP rows");
    const int nv = c->geo.num_voxels;
    PCT_TRY(pct_drop_prepare(c));
    PCT_TRY(c->x_update.alloc(sizeof(float) * nv));
    PCT_CUDA(cudaMemsetAsync(c->x_update.p, 0, sizeof(float) * nv, c->stream));
    if (c->dg.brick && c->drop_mode != PCT_DROP_TILED) {
        PCT_TRY(c->x_brick.alloc(sizeof(float) * nv));
        ++c->launches;
        k_image_to_brick<<<pct_grid_for(nv, 256), 256, 0, c->stream>>>(c->dg, c->x.as<float>(), c->x_brick.as<float>());
    }
    PCT_TRY(c->drop_resid.alloc(sizeof(double) * (PCT_DROP_MAXIT + 2)));
    double* d_res = c->drop_resid.as<double>();
    PCT_CUDA(cudaMemsetAsync(d_res, 0, sizeof(double) * (PCT_DROP_MAXIT + 2), c->stream));
    if (c->h.n > 0)
        k_wepl_norm<<<304, 256, 0, c->stream>>>(c->h.n, c->h.wepl.as<float>(), d_res + PCT_DROP_MAXIT + 1);
    PCT_CUDA(cudaGetLastError());
    return PCT_OK;
}

/* After the iterations: the iterate back in linear order, and the stats of
 * `done` iterations that took `ms` milliseconds. */
pct_status pct_drop_end(pct_ctx* c, int done, float ms, pct_drop_stats* stats) {
    const int nv = c->geo.num_voxels, maxit = PCT_DROP_MAXIT;
    if (c->dg.brick && c->drop_mode != PCT_DROP_TILED) {
        ++c->launches;
        k_image_from_brick<<<pct_grid_for(nv, 256), 256, 0, c->stream>>>(c->dg, c->x_brick.as<float>(), c->x.as<float>());
    }
    PCT_CUDA(cudaGetLastError());
    double res_host[PCT_DROP_MAXIT + 2];
    PCT_CUDA(cudaMemcpyAsync(res_host, c->drop_resid.p, sizeof(double) * (maxit + 2), cudaMemcpyDeviceToHost,
                             c->stream));
    PCT_CUDA(cudaStreamSynchronize(c->stream));
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->iterations_run = done;
        double b2 = res_host[maxit + 1];
        for (int k = 0; k < done && k < maxit; ++k) stats->residual[k] = b2 > 0 ? sqrt(res_host[k] / b2) : 0.0;
        stats->seconds = ms * 1e-3;
        stats->drop_form = c->drop_mode;
    }
    return PCT_OK;
}

/* Copies the iteration's squared residual into slot `it` and clears the accumulator. */
void pct_drop_store_resid(pct_ctx* c, int it) {
    double* d_res = c->drop_resid.as<double>();
    ++c->launches;
    k_store_resid<<<1, 1, 0, c->stream>>>(d_res + PCT_DROP_MAXIT, d_res + (it < PCT_DROP_MAXIT ? it : PCT_DROP_MAXIT - 1));
}

pct_status pct_stage_drop(pct_ctx* c, int iterations, pct_drop_stats* stats) {
    if (c->stage != ST_ROWS) return pct_fail(PCT_ERR_STATE, "drop needs MLP rows");
    if (iterations < 0) return pct_fail(PCT_ERR_ARGUMENT, "drop: negative iteration count");
    PCT_TRY(pct_drop_begin(c));
    const int maxit = PCT_DROP_MAXIT;
    double* d_res = c->drop_resid.as<double>();
    PCT_TRY(drop_allreduce(c, d_res + maxit + 1, 1, PCT_DT_F64));
    if (!c->allreduce) PCT_TRY(capture_iteration(c, d_res + maxit));
    cudaEvent_t e0, e1;
    PCT_CUDA(cudaEventCreate(&e0));
    PCT_CUDA(cudaEventCreate(&e1));
    PCT_CUDA(cudaEventRecord(e0, c->stream));
    int done = 0;
    double res_host[maxit + 2];
    for (int it = 0; it < iterations; ++it) {
        if (c->allreduce) {
            PCT_TRY(run_iteration_sharded(c, d_res + maxit));
        } else {
            PCT_CUDA(cudaGraphLaunch(c->drop_graph_exec, c->stream));
            c->launches += c->drop_launches_per_iter;
        }
        pct_drop_store_resid(c, it);
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
    PCT_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return pct_drop_end(c, done, ms, stats);
}

void pct_drop_release_graph(pct_ctx* c) {
    if (c->drop_graph_exec) cudaGraphExecDestroy(c->drop_graph_exec);
    c->drop_graph_exec = nullptr;
}
