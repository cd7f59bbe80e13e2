/*
 * Stages a4-a6 of the path: per-bin means and standard deviations, the
 * 3-sigma cuts and the sinogram, with the reference's binary32 sums.
 *
 * The reference adds every per-bin sum with binary32 atomicAdd:
 *   binning_GPU                 .cu:2567-2570  WEPL and the two relative angles
 *   sum_squared_deviations_GPU  .cu:2695-2697  the three squared deviations
 *   statistical_cuts_GPU        .cu:2865-2866  the WEPL of the kept histories
 * Its result is the left-to-right binary32 sum of each bin's summands in the
 * order the additions happen.  Here that order is defined as the history order
 * of the resident store (the reference's *_vector order, chunk after chunk),
 * which is the order of a sequential run of those kernels, so the sums, the
 * means and sigmas (.cu:2618-2627, .cu:2718-2730), the cut decisions
 * (.cu:2844-2868) and the sinogram (.cu:2912-2917) are deterministic and equal
 * the reference's sequential run bit for bit.
 *
 *   k_rs_hist / k_rs_scan_rows / k_rs_scatter
 *                 stable LSD radix sort of the store indices by bin (8-bit
 *                 digits); afterwards each bin's histories are one contiguous
 *                 segment, in store order.
 *   k_seg_bounds  the segment [begin, end) of every bin.
 *   k_bin_stats   one thread per bin: the binary32 sums of its segment in
 *                 order, the means, the squared deviations from its own means
 *                 and the sigmas.
 *   k_cuts        one thread per history: the cut decision.
 *   k_sinogram_seq one thread per bin: kept count and binary32 WEPL sum in order.
 * All are bound by memory latency and bandwidth (a few passes of 4-byte keys
 * and gathers of the history fields); none needs floating-point atomics.
 */
#include "pct_device.cuh"

namespace {

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ROUNDS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS; /* keys per CTA */
constexpr int RS_DIGITS = 256;                  /* == RS_THREADS: one digit per thread */
static_assert(RS_DIGITS == RS_THREADS, "one digit per thread");

/* Digit histogram of one tile: tile_hist[digit * ntiles + tile]. */
__global__ void __launch_bounds__(RS_THREADS) k_rs_hist(int64_t n, const uint32_t* __restrict__ keys, int shift,
                                                       int ntiles, uint32_t* __restrict__ tile_hist) {
    __shared__ uint32_t h[RS_DIGITS];
    h[threadIdx.x] = 0u;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ROUNDS; ++r) {
        const int64_t i = base + r * RS_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & (RS_DIGITS - 1)], 1u);
    }
    __syncthreads();
    tile_hist[(size_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

/* Exclusive scan of one digit's row of tile counts, in place; the row total
 * goes to digit_tot[digit].  One CTA per digit. */
__global__ void __launch_bounds__(1024) k_rs_scan_rows(uint32_t* __restrict__ tile_hist, int ntiles,
                                                       uint32_t* __restrict__ digit_tot) {
    __shared__ uint32_t ws[32];
    uint32_t* row = tile_hist + (size_t)blockIdx.x * ntiles;
    uint32_t carry = 0;
    for (int b = 0; b < ntiles; b += 1024) {
        const int k = b + threadIdx.x;
        uint32_t v = k < ntiles ? row[k] : 0u, tot;
        const uint32_t ex = dev_block_exclusive_scan_u32(v, ws, &tot);
        if (k < ntiles) row[k] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) digit_tot[blockIdx.x] = carry;
}

/* Stable scatter of one tile.  The tile's keys are ranked in rounds of 256
 * consecutive keys; within a round by warp, then by lane, so a key's rank
 * among the tile's keys of the same digit follows its position.  vals_in null:
 * the values are the key positions (first pass). */
__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(int64_t n, const uint32_t* __restrict__ keys_in,
                                                          const uint32_t* __restrict__ vals_in, int shift, int ntiles,
                                                          const uint32_t* __restrict__ tile_off,
                                                          const uint32_t* __restrict__ digit_tot,
                                                          uint32_t* __restrict__ keys_out,
                                                          uint32_t* __restrict__ vals_out) {
    __shared__ uint32_t s_base[RS_DIGITS];
    __shared__ uint32_t s_warp[RS_WARPS][RS_DIGITS];
    __shared__ uint32_t ws[32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    uint32_t tot;
    const uint32_t digit_base = dev_block_exclusive_scan_u32(digit_tot[tid], ws, &tot);
    s_base[tid] = digit_base + tile_off[(size_t)tid * ntiles + blockIdx.x];
    const int64_t base = (int64_t)blockIdx.x * RS_TILE;
    const unsigned lanes_below = (1u << lane) - 1u;
    for (int r = 0; r < RS_ROUNDS; ++r) {
#pragma unroll
        for (int k = 0; k < RS_WARPS; ++k) s_warp[k][tid] = 0u;
        __syncthreads();
        const int64_t i = base + r * RS_THREADS + tid;
        const bool ok = i < n;
        uint32_t key = 0u, val = 0u, d = RS_DIGITS; /* RS_DIGITS: no key (never matches a digit) */
        if (ok) {
            key = keys_in[i];
            val = vals_in ? vals_in[i] : (uint32_t)i;
            d = (key >> shift) & (RS_DIGITS - 1);
        }
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int rank = __popc(peers & lanes_below);
        if (ok && rank == 0) s_warp[w][d] = (uint32_t)__popc(peers);
        __syncthreads();
        if (ok) {
            uint32_t pos = s_base[d] + (uint32_t)rank;
            for (int k = 0; k < w; ++k) pos += s_warp[k][d];
            keys_out[pos] = key;
            vals_out[pos] = val;
        }
        __syncthreads();
        uint32_t add = 0u;
#pragma unroll
        for (int k = 0; k < RS_WARPS; ++k) add += s_warp[k][tid];
        s_base[tid] += add;
    }
}

/* seg_begin[b], seg_end[b] of every bin present in the sorted keys (both
 * zero-filled before: absent bins get an empty segment). */
__global__ void k_seg_bounds(int64_t n, const uint32_t* __restrict__ keys, uint32_t nb,
                             uint32_t* __restrict__ seg_begin, uint32_t* __restrict__ seg_end) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t b = keys[k];
    if (b >= nb) return; /* bins are in [0, nb) by construction (k_preprocess) */
    if (k == 0 || keys[k - 1] != b) seg_begin[b] = (uint32_t)k;
    if (k == n - 1 || keys[k + 1] != b) seg_end[b] = (uint32_t)(k + 1);
}

/* One bin: binning_GPU's sums (.cu:2567-2570; histories with a valid bin),
 * calculate_means_GPU (.cu:2618-2627), sum_squared_deviations_GPU
 * (.cu:2678-2698; every stored history, invalid ones sit in bin 0) and
 * calculate_standard_deviations_GPU (.cu:2718-2730).  Each sum is binary32,
 * left to right over the bin's segment. */
__global__ void k_bin_stats(int nb, const uint32_t* __restrict__ seg_begin, const uint32_t* __restrict__ seg_end,
                            const uint32_t* __restrict__ order, HistView h, const int* __restrict__ counts,
                            int sample, float* __restrict__ mw, float* __restrict__ mut, float* __restrict__ muv,
                            float* __restrict__ sw, float* __restrict__ sut, float* __restrict__ suv) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const uint32_t a = seg_begin[b], e = seg_end[b];
    float s_w = 0.0f, s_u = 0.0f, s_v = 0.0f;
    for (uint32_t k = a; k < e; ++k) {
        const uint32_t i = order[k];
        if (!h.bin_valid[i]) continue;
        s_w = s_w + h.wepl[i];
        s_u = s_u + (float)dev_rel_angle(h.xy_exit_angle[i], h.xy_entry_angle[i]);
        s_v = s_v + (float)dev_rel_angle(h.xz_exit_angle[i], h.xz_entry_angle[i]);
    }
    const int c = counts[b];
    if (c > 0) {
        s_w /= c;
        s_u /= c;
        s_v /= c;
    }
    mw[b] = s_w;
    mut[b] = s_u;
    muv[b] = s_v;
    float q_w = 0.0f, q_u = 0.0f, q_v = 0.0f;
    for (uint32_t k = a; k < e; ++k) {
        const uint32_t i = order[k];
        const double dw = h.wepl[i] - s_w; /* binary32 difference, as the reference's float operands */
        const double du = dev_rel_angle(h.xy_exit_angle[i], h.xy_entry_angle[i]) - s_u;
        const double dv = dev_rel_angle(h.xz_exit_angle[i], h.xz_entry_angle[i]) - s_v;
        q_w = q_w + (float)(dw * dw);
        q_u = q_u + (float)(du * du);
        q_v = q_v + (float)(dv * dv);
    }
    if (c > 1) {
        const int div = c - sample;
        q_w = sqrtf(q_w / div);
        q_u = sqrtf(q_u / div);
        q_v = sqrtf(q_v / div);
    }
    sw[b] = q_w;
    sut[b] = q_u;
    suv[b] = q_v;
}

/* statistical_cuts_GPU (.cu:2844-2862): the decision of each history;
 * keep[i] = passed.  Strict < for the angles, <= for WEPL. */
__global__ void __launch_bounds__(256) k_cuts(int64_t n, HistView h, int K, const float* __restrict__ mw,
                                              const float* __restrict__ mut, const float* __restrict__ muv,
                                              const float* __restrict__ sw, const float* __restrict__ sut,
                                              const float* __restrict__ suv, uint8_t* __restrict__ keep) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int b = h.bin_num[i];
    const double rut = dev_rel_angle(h.xy_exit_angle[i], h.xy_entry_angle[i]);
    const double ruv = dev_rel_angle(h.xz_exit_angle[i], h.xz_entry_angle[i]);
    const float w = h.wepl[i];
    const int p_ut = fabs(rut - mut[b]) < (K * sut[b]);
    const int p_uv = fabs(ruv - muv[b]) < (K * suv[b]);
    const int p_w = fabsf(mw[b] - w) <= (K * sw[b]);
    const int f = !p_ut || !p_uv || !p_w;
    h.failed[i] = (uint8_t)f;
    keep[i] = (uint8_t)!f;
}

/* The post-cut count and the sinogram of one bin: statistical_cuts_GPU's
 * count and binary32 WEPL sum (.cu:2863-2866) over the kept histories of the
 * segment in order, then construct_sinogram_GPU (.cu:2912-2917). */
__global__ void k_sinogram_seq(int nb, const uint32_t* __restrict__ seg_begin, const uint32_t* __restrict__ seg_end,
                               const uint32_t* __restrict__ order, const uint8_t* __restrict__ keep,
                               const float* __restrict__ wepl, int* __restrict__ counts_post,
                               float* __restrict__ sino) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    float s = 0.0f;
    int c = 0;
    for (uint32_t k = seg_begin[b], e = seg_end[b]; k < e; ++k) {
        const uint32_t i = order[k];
        if (keep[i]) {
            s = s + wepl[i];
            ++c;
        }
    }
    if (c > 0) s /= c;
    counts_post[b] = c;
    sino[b] = s;
}

}  // namespace

pct_status pct_ensure_bins(pct_ctx* c); /* k_preprocess.cu */

/* Stable sort of the store indices [0, n) by bin: afterwards order[] lists the
 * store indices bin after bin, each bin's in store order, and [seg_begin[b],
 * seg_end[b]) is bin b's segment.  The buffers live in c->bin_sort/bin_seg. */
static pct_status sort_store_by_bin(pct_ctx* c, int64_t n, const uint32_t** order_out, const uint32_t** begin_out,
                                    const uint32_t** end_out) {
    const int nb = c->geo.num_bins;
    const int ntiles = (int)((n + RS_TILE - 1) / RS_TILE);
    int bits = 0;
    while (bits < 32 && ((uint64_t)(nb - 1) >> bits) != 0) ++bits;
    const int passes = bits > 0 ? (bits + 7) / 8 : 1;
    const size_t nn = (size_t)n;
    PCT_TRY(c->bin_sort.alloc(sizeof(uint32_t) * (4 * nn + (size_t)RS_DIGITS * ntiles + RS_DIGITS)));
    uint32_t* keys_a = c->bin_sort.as<uint32_t>();
    uint32_t* vals_a = keys_a + nn;
    uint32_t* keys_b = vals_a + nn;
    uint32_t* vals_b = keys_b + nn;
    uint32_t* tile_hist = vals_b + nn;
    uint32_t* digit_tot = tile_hist + (size_t)RS_DIGITS * ntiles;
    const uint32_t* kin = reinterpret_cast<const uint32_t*>(c->h.bin_num.as<int32_t>()); /* bins are in [0, nb) */
    const uint32_t* vin = nullptr;
    uint32_t* kout = keys_a;
    uint32_t* vout = vals_a;
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        c->launches += 3;
        k_rs_hist<<<ntiles, RS_THREADS, 0, c->stream>>>(n, kin, shift, ntiles, tile_hist);
        k_rs_scan_rows<<<RS_DIGITS, 1024, 0, c->stream>>>(tile_hist, ntiles, digit_tot);
        k_rs_scatter<<<ntiles, RS_THREADS, 0, c->stream>>>(n, kin, vin, shift, ntiles, tile_hist, digit_tot, kout,
                                                           vout);
        kin = kout;
        vin = vout;
        kout = kout == keys_a ? keys_b : keys_a;
        vout = vout == vals_a ? vals_b : vals_a;
    }
    PCT_TRY(c->bin_seg.alloc(sizeof(uint32_t) * 2 * (size_t)nb));
    uint32_t* seg_begin = c->bin_seg.as<uint32_t>();
    uint32_t* seg_end = seg_begin + nb;
    PCT_CUDA(cudaMemsetAsync(seg_begin, 0, sizeof(uint32_t) * 2 * (size_t)nb, c->stream));
    ++c->launches;
    k_seg_bounds<<<pct_grid_for(n, 256), 256, 0, c->stream>>>(n, kin, (uint32_t)nb, seg_begin, seg_end);
    PCT_CUDA(cudaGetLastError());
    *order_out = vin;
    *begin_out = seg_begin;
    *end_out = seg_end;
    return PCT_OK;
}

pct_status pct_stage_cuts(pct_ctx* c) {
    if (c->stage < ST_BINNED) return pct_fail(PCT_ERR_STATE, "statistical_cuts before any chunk");
    if (c->stage >= ST_CUT) return pct_fail(PCT_ERR_STATE, "statistical_cuts already done");
    PCT_TRY(pct_ensure_bins(c));
    const int nb = c->geo.num_bins;
    const int64_t n = c->h.n;
    if (n >= (int64_t)0xffffffffu) return pct_fail(PCT_ERR_ARGUMENT, "statistical_cuts: more than 2^32 - 2 histories");
    HistView h = c->view(c->h);
    PCT_TRY(c->tmp_missed.alloc(n > 0 ? n : 1));
    uint8_t* keep = c->tmp_missed.as<uint8_t>();
    if (n > 0) {
        const uint32_t *order = nullptr, *seg_begin = nullptr, *seg_end = nullptr;
        PCT_TRY(sort_store_by_bin(c, n, &order, &seg_begin, &seg_end));
        ++c->launches;
        k_bin_stats<<<pct_grid_for(nb, 128), 128, 0, c->stream>>>(
            nb, seg_begin, seg_end, order, h, c->bin_counts.as<int>(), c->cfg.sample_std_dev ? 1 : 0,
            c->mean_wepl.as<float>(), c->mean_ut.as<float>(), c->mean_uv.as<float>(), c->sd_wepl.as<float>(),
            c->sd_ut.as<float>(), c->sd_uv.as<float>());
        ++c->launches;
        k_cuts<<<pct_grid_for(n, 256), 256, 0, c->stream>>>(
            n, h, c->cfg.sigmas_to_keep, c->mean_wepl.as<float>(), c->mean_ut.as<float>(), c->mean_uv.as<float>(),
            c->sd_wepl.as<float>(), c->sd_ut.as<float>(), c->sd_uv.as<float>(), keep);
        ++c->launches;
        k_sinogram_seq<<<pct_grid_for(nb, 128), 128, 0, c->stream>>>(nb, seg_begin, seg_end, order, keep,
                                                                    c->h.wepl.as<float>(),
                                                                    c->bin_counts_post.as<int>(),
                                                                    c->sinogram.as<float>());
        PCT_CUDA(cudaGetLastError());
    } else {
        /* no histories: every bin is empty (means, sigmas, counts and sinogram 0) */
        DevBuf* f[] = {&c->mean_wepl, &c->mean_ut, &c->mean_uv, &c->sd_wepl, &c->sd_ut, &c->sd_uv, &c->sinogram,
                       &c->bin_counts_post};
        for (DevBuf* b : f) PCT_CUDA(cudaMemsetAsync(b->p, 0, (size_t)nb * 4, c->stream));
    }
    int64_t kept = 0;
    PCT_TRY(pct_compact_histories(c, keep, n, &kept));
    c->counts.post_cut_histories = kept;
    /* the sort is not needed after the cuts */
    c->bin_sort.release();
    c->bin_seg.release();
    c->stage = ST_CUT;
    return PCT_OK;
}
