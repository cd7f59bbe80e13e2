/*
 * Gather form of the DROP block step (drop_form = PCT_DROP_GATHER).
 *
 * The reference's block step (block_update_GPU .cu:5774-5841, then
 * image_update_GPU .cu:5900-5938) adds every row's update value to each of
 * its voxels with a float atomicAdd and then divides by the voxel's entry
 * count s_j.  Transcribed directly (the scatter form, k_drop.cu) that is one
 * L2 float reduction per row entry, and those reductions bound the step.  The
 * gather form computes the same block update without them:
 *
 *   row pass     k_gather_rows: per row (in sinogram bin order) the dot with
 *                the iterate at the start of the block, the residual and the
 *                row's update value c lambda (b - c sum x) / ||a||^2, stored
 *                once per row (val[rank]); no atomics.
 *   column pass  k_gather_cols: per voxel the sum of val over the block's row
 *                entries in that voxel and their count s_j, then
 *                x_j += sum / s_j (the relaxation, fused).
 *
 * The column pass reads, per block, the transposed incidence: for each voxel
 * the bin-order ranks of the rows that touch it (with multiplicity: a row that
 * revisits a voxel appears twice, as the reference adds twice).  It is stored
 * per slice of 32 consecutive voxels (of the rows' voxel order) as jagged
 * diagonals: the slice's voxels ordered by decreasing entry count c_(0) >=
 * c_(1) >= ...; step k holds entry k of the n_k voxels with c > k, at
 * positions P(k) .. P(k) + n_k - 1 with P(k) = sum_q min(c_(q), k).  A warp
 * (lane p = the voxel at position p) reads step k as one contiguous run of
 * n_k entries: coalesced, unpadded, every active lane adds.  The lists are
 * built once per set of rows and block size (k_gather_fill), like the scatter
 * form's s_j.  Visiting the rows in bin order makes neighbouring rows (nearly
 * the same path) neighbours in rank, so the iterate gathers of the row pass
 * and the value gathers of the column pass hit the SM's L1.
 *
 * Within a block the update is a sum over the block's rows, so the order in
 * which rows are visited and entries added changes only the binary32 rounding
 * (the reference adds in atomic order).  The list order follows the fill's
 * atomics, so results may differ between runs in the last bits, as the
 * reference's own.
 *
 * Bytes per iteration (HBM): the row pass streams 4 B per row entry plus 24 B
 * per row (start, length, chord, row scale, WEPL), the column pass 4 B per
 * list entry (one per row entry inside the image), 4 B per voxel (its slot:
 * voxel and count) and 8 B per slice; the iterate (8 MB at 256x256x32) and
 * the value array (4 B per row of a block) stay in L2.
 */
#include "pct_device.cuh"

int pct_drop_num_blocks(const pct_ctx* c);                                  /* k_drop.cu */
void pct_drop_block_range(const pct_ctx* c, int k, int64_t* s, int64_t* e); /* k_drop.cu */
pct_status pct_drop_bin_order(pct_ctx* c);                                  /* k_drop.cu */

namespace {

constexpr int GR_THREADS = 256;
constexpr int GR_WARPS = GR_THREADS / 32;
constexpr int GR_REG = 8; /* row entries per lane held in registers (256 per row) */
constexpr int GC_UNROLL = 8;  /* jagged-diagonal steps whose loads a warp issues together */
constexpr uint32_t ROW_END = 0xffffffffu; /* register slots past a row's end */

/* Per-row data in bin-rank order (all blocks), so that the row pass reads it
 * contiguously. */
struct RankRows {
    int64_t* start;
    int* len;
    float* chord;
    float* scale;
    float* wepl;
};

__global__ void k_gather_meta(int64_t n, int64_t B, const uint32_t* __restrict__ perm,
                              const int64_t* __restrict__ row_start, const int* __restrict__ row_len,
                              const float* __restrict__ chord, const float* __restrict__ row_scale,
                              const float* __restrict__ wepl, RankRows m) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int64_t i = (p / B) * B + perm[p];
    m.start[p] = row_start[i];
    m.len[p] = row_len[i];
    m.chord[p] = chord[i];
    m.scale[p] = row_scale[i];
    m.wepl[p] = wepl[i];
}

/* Slots of one block's slices (one warp per slice): the slice's voxels in
 * decreasing order of their entry count (ties by voxel), slot[32 s + p] =
 * voxel lane | count << 5 for the voxel at position p; size[s] = the slice's
 * entries; *kmax = the largest count. */
__global__ void k_jds_slots(int nv, int S, const uint32_t* __restrict__ cnt, uint32_t* __restrict__ slot,
                            int64_t* __restrict__ size, unsigned* __restrict__ kmax) {
    const int s = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (s >= S) return;
    const int v = s * 32 + lane;
    const uint32_t c = v < nv ? cnt[v] : 0u;
    int p = 0;
    for (int m = 0; m < 32; ++m) {
        const uint32_t cm = __shfl_sync(0xffffffffu, c, m);
        p += (cm > c) || (cm == c && m < lane);
    }
    slot[(size_t)s * 32 + p] = (uint32_t)lane | (c << 5);
    const uint32_t total = __reduce_add_sync(0xffffffffu, c);
    const uint32_t mx = __reduce_max_sync(0xffffffffu, c);
    if (lane == 0) {
        size[s] = (int64_t)total;
        if (mx) atomicMax(kmax, mx);
    }
}

/* For the fill of one block (one warp per slice): each voxel's position p in
 * its slice (pos[v]) and the step starts P(k) = sum_q min(c_(q), k) of the
 * slice (ptab[s * kcap + k], k < c_(0)). */
__global__ void k_jds_steps(int nv, int S, int kcap, const uint32_t* __restrict__ slot, uint8_t* __restrict__ pos,
                            uint32_t* __restrict__ ptab) {
    const int s = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (s >= S) return;
    const uint32_t sl = slot[(size_t)s * 32 + lane];
    const uint32_t c = sl >> 5;
    const int v = s * 32 + (int)(sl & 31u);
    if (v < nv) pos[v] = (uint8_t)lane;
    const int K = (int)__shfl_sync(0xffffffffu, c, 0);
    for (int kk = 0; kk < K; kk += 32) {
        const uint32_t k = (uint32_t)(kk + lane);
        uint32_t P = 0;
        for (int q = 0; q < 32; ++q) {
            const uint32_t cq = __shfl_sync(0xffffffffu, c, q);
            P += cq < k ? cq : k;
        }
        if ((int)k < K) ptab[(size_t)s * kcap + k] = P;
    }
}

/* The transposed incidence of one block: every row entry's rank at its
 * voxel's next free step.  A warp takes FILL_ROWS consecutive ranks (rows of
 * neighbouring sinogram bins, most of them in one bin, whose paths cross
 * nearly the same voxels) and walks them in windows of FILL_WIN entries per
 * row; lanes that hold the same voxel claim their steps with one atomic
 * (match_any), so that a voxel the rows share costs one L2 atomic, not one per
 * row.  (A row that revisits a voxel inside a window claims two steps, as the
 * reference adds twice.) */
constexpr int FILL_ROWS = 4;
constexpr int FILL_WIN = 32 / FILL_ROWS;
__global__ void k_gather_fill(int nrows, const int64_t* __restrict__ mstart, const int* __restrict__ mlen,
                              const uint32_t* __restrict__ rows, uint32_t nv, const int64_t* __restrict__ slice_off,
                              int kcap, const uint32_t* __restrict__ ptab, const uint8_t* __restrict__ pos,
                              uint32_t* __restrict__ cursor, uint32_t* __restrict__ lists) {
    const int g = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    const int j0 = g * FILL_ROWS;
    if (j0 >= nrows) return; /* the whole warp */
    const int j = j0 + lane / FILL_WIN, o = lane % FILL_WIN;
    int64_t a = 0;
    int len = 0;
    if (j < nrows) {
        a = mstart[j];
        len = mlen[j];
    }
    int maxlen = len;
    for (int d = 16; d > 0; d >>= 1) maxlen = max(maxlen, __shfl_xor_sync(0xffffffffu, maxlen, d));
    for (int e0 = 0; e0 < maxlen; e0 += FILL_WIN) {
        const int q = e0 + o;
        const uint32_t v = q < len ? rows[a + q] : 0xffffffffu;
        const bool act = v < nv;
        const uint32_t key = act ? v : nv + (uint32_t)lane; /* inactive lanes stay alone */
        const unsigned grp = __match_any_sync(0xffffffffu, key);
        const int leader = __ffs(grp) - 1;
        uint32_t base = 0;
        if (act && lane == leader) base = atomicAdd(cursor + v, (uint32_t)__popc(grp));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (act) {
            const uint32_t k = base + (uint32_t)__popc(grp & ((1u << lane) - 1u));
            const uint32_t s = v >> 5;
            lists[slice_off[s] + ptab[(size_t)s * kcap + k] + pos[v]] = (uint32_t)j;
        }
    }
}

/* Row pass of one block: each CTA takes one contiguous run of ranks (bin
 * neighbours share voxels, so some iterate gathers hit L1), a warp per row;
 * the next row's first 32 * GR_REG entries are loaded into registers while
 * the current row's iterate gathers are in flight.  Bound by L2 read sectors
 * of the iterate gathers (about 0.6 per row entry). */
__global__ void __launch_bounds__(GR_THREADS) k_gather_rows(int nrows, const int64_t* __restrict__ mstart,
                                                            const int* __restrict__ mlen,
                                                            const float* __restrict__ mchord,
                                                            const float* __restrict__ mscale,
                                                            const float* __restrict__ mwepl,
                                                            const uint32_t* __restrict__ rows, float lambda,
                                                            const float* __restrict__ x, uint32_t nv,
                                                            float* __restrict__ val, double* __restrict__ resid) {
    __shared__ double sres[GR_WARPS];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int chunk = (nrows + gridDim.x - 1) / gridDim.x;
    const int j0 = blockIdx.x * chunk;
    const int j1 = j0 + chunk < nrows ? j0 + chunk : nrows;
    /* squared residuals in binary64: lane (k mod 32) keeps the warp's k-th
     * residual until 32 are pending, then each lane adds its exact square */
    double r2 = 0.0;
    float pend = 0.0f;
    int nrow = 0;
    int j = j0 + w;
    uint32_t e[GR_REG];
    int64_t a = 0;
    int len = 0;
    if (j < j1) {
        a = mstart[j];
        len = mlen[j];
    }
#pragma unroll
    for (int k = 0; k < GR_REG; ++k) {
        const int q = lane + 32 * k;
        e[k] = q < len ? __ldcs(rows + a + q) : ROW_END; /* streamed once per iteration */
    }
    for (; j < j1; j += GR_WARPS) {
        const int jn = j + GR_WARPS;
        int64_t an = 0;
        int lenn = 0;
        if (jn < j1) {
            an = mstart[jn];
            lenn = mlen[jn];
        }
        uint32_t en[GR_REG];
#pragma unroll
        for (int k = 0; k < GR_REG; ++k) {
            const int q = lane + 32 * k;
            en[k] = q < lenn ? __ldcs(rows + an + q) : ROW_END;
        }
        float dot = 0.0f;
#pragma unroll
        for (int k = 0; k < GR_REG; ++k) dot += e[k] < nv ? x[e[k]] : 0.0f;
        for (int q = 32 * GR_REG + lane; q < len; q += 32) {
            const uint32_t v = __ldcs(rows + a + q);
            if (v < nv) dot += x[v];
        }
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
        const float c = mchord[j];
        const float res = fmaf(-c, dot, mwepl[j]); /* one rounding */
        if (lane == 0) val[j] = (res * mscale[j]) * lambda;
        if (lane == (nrow & 31)) pend = res;
        if ((++nrow & 31) == 0) {
            r2 = fma((double)pend, (double)pend, r2);
            pend = 0.0f;
        }
#pragma unroll
        for (int k = 0; k < GR_REG; ++k) e[k] = en[k];
        a = an;
        len = lenn;
    }
    r2 = fma((double)pend, (double)pend, r2);
    for (int o = 16; o > 0; o >>= 1) r2 += __shfl_xor_sync(0xffffffffu, r2, o);
    if (lane == 0) sres[w] = r2;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < GR_WARPS; ++k) s += sres[k];
        if (s != 0.0) atomicAdd(resid, s);
    }
}

/* Column pass of one block: one warp per slice of 32 voxels, lane p = the
 * voxel at position p; step k is the contiguous run of the n_k = |{c > k}|
 * entries starting at P(k).  Steps go in groups of GC_UNROLL: the loads of
 * the next group are issued before the current group's values are gathered,
 * so two groups of loads are in flight.  Then x_j += sum / s_j with s_j the
 * voxel's entry count. */
__global__ void __launch_bounds__(GR_THREADS) k_gather_cols(int S, int nv, const int64_t* __restrict__ slice_off,
                                                            const uint32_t* __restrict__ slot,
                                                            const uint32_t* __restrict__ lists,
                                                            const float* __restrict__ val, float* __restrict__ x) {
    const int s = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (s >= S) return;
    const int64_t p0 = slice_off[s];
    if (slice_off[s + 1] == p0) return;
    const uint32_t sl = slot[(size_t)s * 32 + lane];
    const int c = (int)(sl >> 5);
    const int K = __shfl_sync(0xffffffffu, c, 0);
    const uint32_t* e = lists + p0 + lane;
    uint32_t r[GC_UNROLL];
#pragma unroll
    for (int u = 0; u < GC_UNROLL; ++u) {
        r[u] = c > u ? __ldcs(e) : 0u;
        e += __popc(__ballot_sync(0xffffffffu, c > u));
    }
    float acc = 0.0f;
    for (int k = 0; k < K; k += GC_UNROLL) {
        uint32_t rn[GC_UNROLL];
#pragma unroll
        for (int u = 0; u < GC_UNROLL; ++u) {
            const int kn = k + GC_UNROLL + u;
            rn[u] = c > kn ? __ldcs(e) : 0u;
            e += __popc(__ballot_sync(0xffffffffu, c > kn));
        }
#pragma unroll
        for (int u = 0; u < GC_UNROLL; ++u)
            if (c > k + u) acc += val[r[u]];
#pragma unroll
        for (int u = 0; u < GC_UNROLL; ++u) r[u] = rn[u];
    }
    const int v = s * 32 + (int)(sl & 31u);
    if (c > 0 && v < nv) x[v] += acc / (float)c;
}

}  // namespace

static RankRows rank_rows(pct_ctx* c) {
    const size_t n = (size_t)(c->h.n > 0 ? c->h.n : 1);
    char* p = c->gather_meta.as<char>();
    RankRows m;
    m.start = reinterpret_cast<int64_t*>(p);
    m.len = reinterpret_cast<int*>(p + 8 * n);
    m.chord = reinterpret_cast<float*>(p + 12 * n);
    m.scale = reinterpret_cast<float*>(p + 16 * n);
    m.wepl = reinterpret_cast<float*>(p + 20 * n);
    return m;
}

void pct_drop_gather_release(pct_ctx* c) {
    c->gather_meta.release();
    c->gather_off.release();
    c->gather_lists.release();
    c->gather_val.release();
    c->gather_tmp.release();
    c->gather_slot.release();
    c->gather_steps.release();
    c->gather_entries = 0;
}

/* Builds the gather form's structures on top of the scatter form's per-block
 * counts (block_diag): bin order, rank-ordered row data, slice slots and
 * offsets, jagged-diagonal lists.
 * On an allocation failure the structures are released and PCT_ERR_ALLOC is
 * returned (the caller falls back to the scatter form). */
pct_status pct_drop_gather_build(pct_ctx* c) {
    const int64_t n = c->h.n;
    const int nv = c->geo.num_voxels;
    const int S = (nv + 31) / 32;
    const int nb = c->num_blocks;
    const int64_t B = c->cfg.block_size;
    if (nb == 0) return PCT_OK; /* no rows: nothing to iterate */
    /* neither pass uses shared memory: all of it as L1 for the gathers */
    PCT_CUDA(cudaFuncSetAttribute(k_gather_rows, cudaFuncAttributePreferredSharedMemoryCarveout, 0));
    PCT_CUDA(cudaFuncSetAttribute(k_gather_cols, cudaFuncAttributePreferredSharedMemoryCarveout, 0));
    PCT_TRY(pct_drop_bin_order(c));
    const size_t nn = (size_t)(n > 0 ? n : 1);
    pct_status st = c->gather_meta.alloc(24 * nn);
    if (st == PCT_OK) st = c->gather_off.alloc(sizeof(int64_t) * ((size_t)nb * S + 1));
    /* slice sizes for the scan and the largest count, then the fill's per-voxel cursors */
    const size_t tmp_bytes = sizeof(int64_t) * ((size_t)nb * S + 2);
    if (st == PCT_OK) st = c->gather_tmp.alloc(tmp_bytes > sizeof(uint32_t) * (size_t)nv
                                                   ? tmp_bytes : sizeof(uint32_t) * (size_t)nv);
    if (st == PCT_OK) st = c->gather_slot.alloc(sizeof(uint32_t) * (size_t)nb * S * 32);
    if (st == PCT_OK) st = c->gather_val.alloc(sizeof(float) * (size_t)(B < n ? B : nn));
    if (st != PCT_OK) {
        pct_drop_gather_release(c);
        return PCT_ERR_ALLOC;
    }
    RankRows m = rank_rows(c);
    if (n > 0) {
        ++c->launches;
        k_gather_meta<<<pct_grid_for(n, 256), 256, 0, c->stream>>>(
            n, B, c->drop_perm.as<uint32_t>(), c->row_offsets.as<int64_t>(), c->row_len.as<int>(),
            c->chord.as<float>(), c->row_scale.as<float>(), c->h.wepl.as<float>(), m);
    }
    int64_t* size = c->gather_tmp.as<int64_t>();
    unsigned* d_kmax = reinterpret_cast<unsigned*>(size + (size_t)nb * S + 1);
    PCT_CUDA(cudaMemsetAsync(d_kmax, 0, sizeof(unsigned), c->stream));
    for (int k = 0; k < nb; ++k) {
        ++c->launches;
        k_jds_slots<<<pct_grid_for((int64_t)S * 32, 256), 256, 0, c->stream>>>(
            nv, S, c->block_diag.as<uint32_t>() + (size_t)k * nv, c->gather_slot.as<uint32_t>() + (size_t)k * S * 32,
            size + (size_t)k * S, d_kmax);
    }
    PCT_CUDA(cudaGetLastError());
    unsigned kmax = 0;
    PCT_CUDA(cudaMemcpyAsync(&kmax, d_kmax, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    int64_t total = 0;
    PCT_TRY(pct_scan_lengths(c, size, (int64_t)nb * S, c->gather_off.as<int64_t>(), &total));
    const int kcap = kmax > 0 ? (int)kmax : 1;
    st = c->gather_lists.alloc(sizeof(uint32_t) * (size_t)(total > 0 ? total : 1));
    if (st == PCT_OK) st = c->gather_steps.alloc(sizeof(uint32_t) * (size_t)S * kcap + (size_t)nv);
    if (st != PCT_OK) {
        pct_drop_gather_release(c);
        return PCT_ERR_ALLOC;
    }
    c->gather_entries = total;
    uint32_t* ptab = c->gather_steps.as<uint32_t>();
    uint8_t* pos = reinterpret_cast<uint8_t*>(ptab + (size_t)S * kcap);
    uint32_t* cursor = reinterpret_cast<uint32_t*>(size); /* the sizes are no longer needed */
    for (int k = 0; k < nb; ++k) {
        int64_t s, e;
        pct_drop_block_range(c, k, &s, &e);
        if (e == s) continue;
        PCT_CUDA(cudaMemsetAsync(cursor, 0, sizeof(uint32_t) * (size_t)nv, c->stream));
        c->launches += 2;
        k_jds_steps<<<pct_grid_for((int64_t)S * 32, 256), 256, 0, c->stream>>>(
            nv, S, kcap, c->gather_slot.as<uint32_t>() + (size_t)k * S * 32, pos, ptab);
        k_gather_fill<<<pct_grid_for((e - s + FILL_ROWS - 1) / FILL_ROWS * 32, 256), 256, 0, c->stream>>>(
            (int)(e - s), m.start + s, m.len + s, c->rows.as<uint32_t>(), (uint32_t)nv,
            c->gather_off.as<int64_t>() + (size_t)k * S, kcap, ptab, pos, cursor, c->gather_lists.as<uint32_t>());
    }
    PCT_CUDA(cudaGetLastError());
    PCT_CUDA(cudaStreamSynchronize(c->stream));
    return PCT_OK;
}

/* CTAs of a k_gather_rows launch: every resident slot, or fewer for a small block. */
static unsigned gather_rows_grid(pct_ctx* c, int64_t rows) {
    int sms = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess || sms < 1) sms = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gather_rows, GR_THREADS, 0) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    const int64_t need = (rows + GR_WARPS - 1) / GR_WARPS;
    const int64_t cap = (int64_t)sms * per_sm;
    return (unsigned)(need < cap ? (need > 0 ? need : 1) : cap);
}

/* The two launches of block k. */
void pct_drop_gather_enqueue(pct_ctx* c, int k, double* resid) {
    int64_t s, e;
    pct_drop_block_range(c, k, &s, &e);
    if (e == s) return;
    const int nv = c->geo.num_voxels;
    const int S = (nv + 31) / 32;
    RankRows m = rank_rows(c);
    float* xi = c->dg.brick ? c->x_brick.as<float>() : c->x.as<float>();
    float* val = c->gather_val.as<float>();
    k_gather_rows<<<gather_rows_grid(c, e - s), GR_THREADS, 0, c->stream>>>(
        (int)(e - s), m.start + s, m.len + s, m.chord + s, m.scale + s, m.wepl + s, c->rows.as<uint32_t>(),
        c->cfg.lambda, xi, (uint32_t)nv, val, resid);
    k_gather_cols<<<pct_grid_for((int64_t)S * 32, GR_THREADS), GR_THREADS, 0, c->stream>>>(
        S, nv, c->gather_off.as<int64_t>() + (size_t)k * S, c->gather_slot.as<uint32_t>() + (size_t)k * S * 32,
        c->gather_lists.as<uint32_t>(), val, xi);
}
