/*
 * DROP block step on image tiles (the tiled form, default where it fits).
 *
 * The block update of block_update_GPU / image_update_GPU
 * (src/pCT_Reconstruction_Data_Segments.cu:5774-5841, :5900-5938) gathers the
 * iterate over every row entry and adds each row's update to every voxel of
 * the row.  Done row by row, every entry costs a random 4-byte gather and a
 * random 4-byte reduction in L2 (the scatter form, bound by L2 reduction
 * throughput).  Here the image is cut into tiles of at most 8192 voxels and
 * the rows of each DROP block are regrouped once per set of rows into
 * segments: maximal runs of consecutive in-image entries of one row that lie
 * in one tile, stored per (block, tile) as 16-bit tile-local voxel indices.
 * Per block and iteration:
 *   k_tile_fwd   one CTA per chunk of a tile's segments stages the tile of x in
 *                shared memory (as x * 2^32 in int64); warps read the entries
 *                32 at a time and a segmented scan over the lanes forms each
 *                segment's partial dot, stored in the row's slot.
 *   k_tile_rows  one thread per row adds its partial dots (exact, integer) and
 *                forms the update value u = c lambda (b - c dot) / ||a||^2
 *                (binary64 scalars), the squared residual, and max |u|.
 *   k_tile_bwd   a cluster of CTAs per tile adds u of every segment to its
 *                voxels in shared-memory int32 accumulators (fixed point with a
 *                per-block power-of-two scale chosen from max |u| and the
 *                block's largest s_j so no sum can overflow), reduces the
 *                cluster's accumulators over distributed shared memory and
 *                applies x += update / s_j to the tile.
 * Integer sums make the dots and the update independent of the order of
 * addition, so the iterate is reproducible bit for bit (and the dots are
 * exact where the reference rounds a binary32 sum at every entry).  The diagonal weights s_j come from
 * k_tile_bwd in count mode at build time.
 */
#include <cooperative_groups.h>
#include <cstring>
#include <vector>
#include "pct_device.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int TILE_MAX = 8192;     /* voxels per tile (x tile 32 KB, accumulators 32 KB) */
constexpr int BWD_CLUSTER = 8;     /* CTAs per tile in k_tile_bwd */
constexpr int BWD_THREADS = 256;
constexpr int FWD_THREADS = 256;
constexpr int FWD_SEGS = 1024;     /* segments per k_tile_fwd CTA */
constexpr int ROWS_THREADS = 256;

constexpr int TX = 32, TY = 32;   /* tile extent in x and y; z extent T.tz <= 8 */
constexpr int SUBS = 32;          /* cursors per (block, tile), by row index mod 32 */
constexpr int CHUNK_ENTRIES = 8192; /* longest row the tiled form accepts */
constexpr uint16_t SEG_HEAD = 0x8000; /* entry flag: first entry of a segment */
constexpr uint16_t SEG_LOCAL = 0x1fff; /* entry bits: tile-local voxel index (< 8192) */
/* The forward dots are exact sums in fixed point: x * 2^32 as int64 (|x| < 2^30). */
constexpr float X_FIXED_SCALE = 4294967296.0f;
constexpr float X_FIXED_LIMIT = 1073741824.0f;

/* Division of n < 2^31 by a fixed d >= 1: q = high 64 bits of n * ceil(2^64 / d)
 * (exact since 64 >= 31 + log2(d) for d < 2^32). */
struct FastDiv {
    unsigned long long m;
    uint32_t d;
};
static FastDiv fast_div(uint32_t d) {
    FastDiv f;
    f.d = d;
    f.m = d == 1 ? 0ull : (unsigned long long)((~0ull) / d) + 1ull;
    return f;
}
__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) {
    return f.d == 1 ? n : (uint32_t)__umul64hi((unsigned long long)n, f.m);
}

struct TileGeom {
    int C, R, S, nv;
    int tz, ntx, nty, ntz, nt, tv;
    FastDiv divC, divCR;
};

__device__ __forceinline__ void tile_of(const TileGeom& T, uint32_t v, int* t, int* l) {
    uint32_t z = fdiv(v, T.divCR);
    uint32_t r = v - z * (uint32_t)(T.C * T.R);
    uint32_t y = fdiv(r, T.divC);
    uint32_t x = r - y * (uint32_t)T.C;
    uint32_t bz = z / (uint32_t)T.tz; /* tz <= 8: a short division */
    uint32_t lz = z - bz * (uint32_t)T.tz;
    *t = (int)((x >> 5) + T.ntx * ((y >> 5) + T.nty * bz));
    *l = (int)((x & 31u) + TX * ((y & 31u) + TY * lz));
}

/* origin of tile t in voxels */
__device__ __forceinline__ void tile_origin(const TileGeom& T, int t, int* ox, int* oy, int* oz) {
    int bx = t % T.ntx, by = (t / T.ntx) % T.nty, bz = t / (T.ntx * T.nty);
    *ox = bx * TX;
    *oy = by * TY;
    *oz = bz * T.tz;
}

/* global voxel of local index l of the tile at (ox, oy, oz), or -1 outside the image */
__device__ __forceinline__ int tile_voxel(const TileGeom& T, int ox, int oy, int oz, int l) {
    int x = ox + (l & 31), y = oy + ((l >> 5) & 31), z = oz + (l >> 10);
    if (x >= T.C || y >= T.R || z >= T.S) return -1;
    return x + T.C * (y + T.R * z);
}

/* Build pass 1: segments per row, and per (block, tile, row mod 32) the segment
 * and entry counts packed as (segments << 32) | entries. */
__global__ void k_tile_count(DevGeom dg, int64_t n, int64_t B, TileGeom T, const int64_t* __restrict__ row_start,
                             const int* __restrict__ row_len, const uint32_t* __restrict__ rows,
                             int64_t* __restrict__ row_nseg, unsigned long long* __restrict__ bt_cnt) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t b = i / B;
    const int64_t a = row_start[i];
    const int len = row_len[i];
    int cur = -1, seg = 0, nseg = 0;
    for (int k = 0; k < len; ++k) {
        uint32_t v = dev_from_brick(dg, rows[a + k]); /* linear order */
        if (v >= (uint32_t)T.nv) continue;
        int t, l;
        tile_of(T, v, &t, &l);
        if (t != cur) {
            if (seg) {
                atomicAdd(bt_cnt + (b * T.nt + cur) * SUBS + (i & (SUBS - 1)), (1ull << 32) | (unsigned long long)seg);
                ++nseg;
            }
            cur = t;
            seg = 0;
        }
        ++seg;
    }
    if (seg) {
        atomicAdd(bt_cnt + (b * T.nt + cur) * SUBS + (i & (SUBS - 1)), (1ull << 32) | (unsigned long long)seg);
        ++nseg;
    }
    row_nseg[i] = nseg;
}

/* Build pass 2: segment records and tile-local entries.  A packed cursor per
 * (block, tile, row mod 32) hands out the segment slot and its entry range
 * together, so the entries of consecutive segments are consecutive; the 32
 * cursors of a (block, tile) own consecutive ranges. */
__global__ void k_tile_fill(DevGeom dg, int64_t n, int64_t B, TileGeom T, const int64_t* __restrict__ row_start,
                            const int* __restrict__ row_len, const uint32_t* __restrict__ rows,
                            const int64_t* __restrict__ row_seg_off, const int64_t* __restrict__ seg_sub,
                            const int64_t* __restrict__ ent_sub, const int64_t* __restrict__ ent_base,
                            unsigned long long* __restrict__ cursor, uint32_t* __restrict__ seg_row,
                            uint32_t* __restrict__ seg_slot, uint32_t* __restrict__ seg_ent,
                            uint16_t* __restrict__ ent) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t b = i / B;
    const int64_t a = row_start[i];
    const int len = row_len[i];
    int cur = -1, seg = 0, q = 0, k0 = 0;
    for (int k = 0; k <= len; ++k) {
        int t = -1, l = 0;
        bool in = false;
        if (k < len) {
            uint32_t v = dev_from_brick(dg, rows[a + k]); /* linear order */
            if (v >= (uint32_t)T.nv) continue;
            tile_of(T, v, &t, &l);
            in = true;
        }
        if (t != cur || !in) {
            if (seg) {
                const int64_t bt = (b * T.nt + cur) * SUBS + (i & (SUBS - 1));
                unsigned long long old = atomicAdd(cursor + bt, (1ull << 32) | (unsigned long long)seg);
                const int64_t g = seg_sub[bt] + (int64_t)(old >> 32);
                const int64_t e0 = ent_sub[bt] + (int64_t)(uint32_t)old;
                seg_row[g] = (uint32_t)(i - b * B);
                seg_slot[g] = (uint32_t)(row_seg_off[i] + q);
                seg_ent[g] = (uint32_t)(e0 - ent_base[b]);
                int m = 0;
                for (int kk = k0; m < seg; ++kk) {
                    uint32_t vv = dev_from_brick(dg, rows[a + kk]);
                    if (vv >= (uint32_t)T.nv) continue;
                    int tt, ll;
                    tile_of(T, vv, &tt, &ll);
                    ent[e0 + m] = (uint16_t)(ll | (m == 0 ? SEG_HEAD : 0));
                    ++m;
                }
                ++q;
            }
            cur = t;
            seg = 0;
            k0 = k;
        }
        if (in) ++seg;
    }
}

__device__ __forceinline__ int seg_len(int64_t g, int64_t g_end, const uint32_t* __restrict__ seg_ent,
                                       uint32_t ent_total) {
    uint32_t e1 = g + 1 < g_end ? seg_ent[g + 1] : ent_total;
    return (int)(e1 - seg_ent[g]);
}

/* Forward: partial dots of the segments [wk.y, wk.y + wk.z) (block-relative)
 * of tile wk.x, one thread per segment; the entries are read eight at a time
 * with aligned 16-byte loads (the entry array starts 256-byte aligned). */
__global__ void __launch_bounds__(FWD_THREADS) k_tile_fwd(TileGeom T, int b, int work0,
                                                          const int4* __restrict__ work,
                                                          const int64_t* __restrict__ seg_base,
                                                          const int64_t* __restrict__ ent_base,
                                                          const uint32_t* __restrict__ seg_slot,
                                                          const uint32_t* __restrict__ seg_ent,
                                                          const uint16_t* __restrict__ ent,
                                                          const float* __restrict__ x, long long* __restrict__ partial,
                                                          unsigned long long* __restrict__ flags) {
    extern __shared__ long long xs[]; /* the tile of x in fixed point, T.tv entries */
    const int4 wk = work[work0 + blockIdx.x];
    int ox, oy, oz;
    tile_origin(T, wk.x, &ox, &oy, &oz);
    for (int l = threadIdx.x; l < T.tv; l += FWD_THREADS) {
        int v = tile_voxel(T, ox, oy, oz, l);
        float xv = v >= 0 ? x[v] : 0.0f;
        if (!(fabsf(xv) < X_FIXED_LIMIT)) {
            atomicAdd(flags + ERR_DROP_NONFINITE, 1ull);
            xv = 0.0f;
        }
        xs[l] = __float2ll_rn(xv * X_FIXED_SCALE); /* exact: a power-of-two scaling */
    }
    __syncthreads();
    const int64_t sb = seg_base[b], se = seg_base[b + 1];
    const int64_t eb0 = ent_base[b];
    const uint32_t ent_total = (uint32_t)(ent_base[b + 1] - ent_base[b]);
    for (int64_t g = sb + wk.y + threadIdx.x; g < sb + wk.y + wk.z; g += FWD_THREADS) {
        const int64_t A0 = eb0 + seg_ent[g];
        const int64_t A1 = eb0 + (g + 1 < se ? seg_ent[g + 1] : ent_total);
        long long sum = 0;
        for (int64_t a8 = A0 & ~(int64_t)7; a8 < A1; a8 += 8) {
            const uint4 w = *reinterpret_cast<const uint4*>(ent + a8);
            const uint32_t wd[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int64_t idx = a8 + k;
                const uint32_t q = (wd[k >> 1] >> ((k & 1) * 16)) & SEG_LOCAL;
                if (idx >= A0 && idx < A1) sum += xs[q];
            }
        }
        partial[seg_slot[g]] = sum;
    }
}

/* Row updates of one block from the partial dots (row order). */
__global__ void __launch_bounds__(ROWS_THREADS) k_tile_rows(int64_t start, int64_t end, const int64_t* __restrict__ row_seg_off,
                                                            const long long* __restrict__ partial,
                                                            const float* __restrict__ chord,
                                                            const float* __restrict__ row_scale,
                                                            const float* __restrict__ wepl, float lambda,
                                                            float* __restrict__ u, unsigned* __restrict__ umax,
                                                            double* __restrict__ resid) {
    __shared__ double sres[ROWS_THREADS / 32];
    __shared__ unsigned smax[ROWS_THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t i = start + (int64_t)blockIdx.x * ROWS_THREADS + threadIdx.x;
    double r2 = 0.0; /* the squared residual and its sums in binary64 */
    unsigned mx = 0;
    if (i < end) {
        long long sum = 0;
        for (int64_t p = row_seg_off[i]; p < row_seg_off[i + 1]; ++p) sum += partial[p];
        const float dot = __ll2float_rn(sum) * (1.0f / 4294967296.0f); /* exact sum, rounded once */
        const float c = chord[i];
        const float res = fmaf(-c, dot, wepl[i]);
        const float val = (res * row_scale[i]) * lambda;
        u[i - start] = val;
        r2 = (double)res * (double)res; /* exact */
        mx = __float_as_uint(fabsf(val)); /* non-negative floats order like their bits; NaN sorts above inf */
    }
    for (int o = 16; o > 0; o >>= 1) {
        r2 += __shfl_xor_sync(0xffffffffu, r2, o);
        unsigned t = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = t > mx ? t : mx;
    }
    if (lane == 0) {
        sres[w] = r2;
        smax[w] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        unsigned m = 0;
        for (int k = 0; k < ROWS_THREADS / 32; ++k) {
            s += sres[k];
            m = smax[k] > m ? smax[k] : m;
        }
        if (s != 0.0) atomicAdd(resid, s);
        if (m) atomicMax(umax, m);
    }
}

/* Backward (COUNT = false) or diagonal weights (COUNT = true) of one block:
 * cluster `blockIdx.x / BWD_CLUSTER` owns tile t; its CTAs split the tile's
 * segments, accumulate in shared memory, then each reduces a quarter of the
 * tile over the cluster and writes it. */
template <bool COUNT>
__global__ void __cluster_dims__(BWD_CLUSTER, 1, 1) __launch_bounds__(BWD_THREADS)
    k_tile_bwd(TileGeom T, int b, const int64_t* __restrict__ seg_bt, const int64_t* __restrict__ seg_base,
               const int64_t* __restrict__ ent_base, const uint32_t* __restrict__ seg_row,
               const uint32_t* __restrict__ seg_ent, const uint16_t* __restrict__ ent, const float* __restrict__ u,
               const unsigned* __restrict__ umax, const unsigned* __restrict__ smax, uint32_t* __restrict__ counts,
               unsigned* __restrict__ smax_out, float* __restrict__ x, unsigned long long* __restrict__ flags) {
    __shared__ int acc[TILE_MAX];
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int t = blockIdx.x / BWD_CLUSTER;
    for (int l = threadIdx.x; l < T.tv; l += BWD_THREADS) acc[l] = 0;
    double scale = 1.0;
    if (!COUNT) {
        const float um = __uint_as_float(umax[b]);
        if (!(um <= 3.0e38f)) {
            scale = 0.0; /* non-finite update: leave x unchanged, flag it */
            if (threadIdx.x == 0 && rank == 0 && t == 0) atomicAdd(flags + ERR_DROP_NONFINITE, 1ull);
        } else if (um > 0.0f) {
            int ex;
            frexp((double)um * (double)smax[b], &ex); /* max|u| * max s_j < 2^ex */
            scale = ldexp(1.0, 29 - (ex > -900 ? ex : -900));
        }
    }
    __syncthreads();
    const int64_t g_begin = seg_bt[(int64_t)b * T.nt + t], g_all_end = seg_bt[(int64_t)b * T.nt + t + 1];
    const int64_t nseg = g_all_end - g_begin;
    const int64_t my0 = g_begin + nseg * rank / BWD_CLUSTER, my1 = g_begin + nseg * (rank + 1) / BWD_CLUSTER;
    const int64_t se = seg_base[b + 1];
    const uint32_t ent_total = (uint32_t)(ent_base[b + 1] - ent_base[b]);
    /* one thread per segment, entries read eight at a time */
    const int64_t eb0 = ent_base[b];
    for (int64_t g = my0 + threadIdx.x; g < my1; g += BWD_THREADS) {
        const int fx = COUNT ? 1 : __double2int_rn((double)u[seg_row[g]] * scale);
        if (fx == 0) continue;
        const int64_t A0 = eb0 + seg_ent[g];
        const int64_t A1 = eb0 + (g + 1 < se ? seg_ent[g + 1] : ent_total);
        for (int64_t a8 = A0 & ~(int64_t)7; a8 < A1; a8 += 8) {
            const uint4 w = *reinterpret_cast<const uint4*>(ent + a8);
            const uint32_t wd[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int64_t idx = a8 + k;
                const uint32_t q = (wd[k >> 1] >> ((k & 1) * 16)) & SEG_LOCAL;
                if (idx >= A0 && idx < A1) atomicAdd(acc + q, fx);
            }
        }
    }
    cluster.sync();
    const int l0 = T.tv * rank / BWD_CLUSTER, l1 = T.tv * (rank + 1) / BWD_CLUSTER;
    int ox, oy, oz;
    tile_origin(T, t, &ox, &oy, &oz);
    unsigned mx = 0;
    for (int l = l0 + threadIdx.x; l < l1; l += BWD_THREADS) {
        int sum = 0;
#pragma unroll
        for (int r = 0; r < BWD_CLUSTER; ++r) sum += cluster.map_shared_rank(acc, r)[l];
        const int v = tile_voxel(T, ox, oy, oz, l);
        if (v < 0) continue;
        if (COUNT) {
            counts[(size_t)b * T.nv + v] = (uint32_t)sum;
            mx = (unsigned)sum > mx ? (unsigned)sum : mx;
        } else if (sum != 0) {
            const uint32_t s = counts[(size_t)b * T.nv + v];
            if (s > 0) x[v] += (float)((double)sum / scale) / (float)s;
        }
    }
    if (COUNT) {
        for (int o = 16; o > 0; o >>= 1) {
            unsigned q = __shfl_xor_sync(0xffffffffu, mx, o);
            mx = q > mx ? q : mx;
        }
        if ((threadIdx.x & 31) == 0 && mx) atomicMax(smax_out + b, mx);
    }
    cluster.sync(); /* keep every CTA's accumulators alive until the cluster has read them */
}

TileGeom tile_geom(const pct_ctx* c) {
    TileGeom T;
    T.C = c->geo.columns;
    T.R = c->geo.rows;
    T.S = c->geo.slices;
    T.nv = c->geo.num_voxels;
    T.tz = T.S < 8 ? T.S : 8;
    T.ntx = (T.C + TX - 1) / TX;
    T.nty = (T.R + TY - 1) / TY;
    T.ntz = (T.S + T.tz - 1) / T.tz;
    T.nt = T.ntx * T.nty * T.ntz;
    T.tv = TX * TY * T.tz;
    T.divC = fast_div((uint32_t)T.C);
    T.divCR = fast_div((uint32_t)(T.C * T.R));
    return T;
}

}  // namespace

/* The tiled form needs per-block entry counts below 2^32, a tile of at most
 * TILE_MAX voxels and the memory for the regrouped rows. */
int pct_drop_tiled_fits(pct_ctx* c) {
    const int64_t n = c->h.n;
    if (n == 0) return 0;
    TileGeom T = tile_geom(c);
    if (T.tv > TILE_MAX || T.C * T.R * (int64_t)T.S >= 2147483647LL) return 0;
    const int64_t max_row = 8 * (int64_t)(c->geo.columns + c->geo.rows + c->geo.slices) + 65;
    if ((double)c->cfg.block_size * (double)max_row >= 4294967295.0) return 0;
    if (max_row > CHUNK_ENTRIES) return 0; /* a segment always fits one staging round */
    /* entries (2 B) + ~1 segment per 8 entries (12 B + 4 B partial) + weights */
    const int64_t nb = (n + c->cfg.block_size - 1) / c->cfg.block_size;
    double need = (double)c->row_capacity * 4.0 + (double)nb * (double)c->geo.num_voxels * 4.0 + (double)n * 16.0;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return 0;
    double have = (double)free_b + (double)c->td.bytes_held();
    return need < 0.8 * have;
}

pct_status pct_drop_tiled_build(pct_ctx* c) {
    TiledDrop& d = c->td;
    const int64_t n = c->h.n;
    const int64_t B = c->cfg.block_size;
    const int nb = (int)((n + B - 1) / B);
    TileGeom T = tile_geom(c);
    const int64_t nbt = (int64_t)nb * T.nt;
    PCT_CUDA(cudaFuncSetAttribute(k_tile_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(sizeof(long long) * TILE_MAX)));
    /* pass 1: counts */
    PCT_TRY(d.row_seg_off.alloc(sizeof(int64_t) * (n + 1)));
    PCT_TRY(d.row_nseg.alloc(sizeof(int64_t) * n));
    const int64_t nbts = nbt * SUBS;
    PCT_TRY(d.bt_cnt.alloc(sizeof(unsigned long long) * nbts));
    PCT_CUDA(cudaMemsetAsync(d.bt_cnt.p, 0, sizeof(unsigned long long) * nbts, c->stream));
    ++c->launches;
    k_tile_count<<<pct_grid_for(n, 128), 128, 0, c->stream>>>(c->dg, n, B, T, c->row_offsets.as<int64_t>(), c->row_len.as<int>(),
                                                             c->rows.as<uint32_t>(), d.row_nseg.as<int64_t>(),
                                                             d.bt_cnt.as<unsigned long long>());
    int64_t total_slots = 0;
    PCT_TRY(pct_scan_lengths(c, d.row_nseg.as<int64_t>(), n, d.row_seg_off.as<int64_t>(), &total_slots));
    std::vector<unsigned long long> cnt(nbts);
    PCT_CUDA(cudaMemcpyAsync(cnt.data(), d.bt_cnt.p, sizeof(unsigned long long) * nbts, cudaMemcpyDeviceToHost, c->stream));
    PCT_CUDA(cudaStreamSynchronize(c->stream));
    /* host: per (block, tile) and per sub-cursor segment and entry offsets, per-block
     * bases, forward work list */
    std::vector<int64_t> seg_bt(nbt + 1), ent_bt(nbt + 1), seg_base(nb + 1), ent_base(nb + 1);
    std::vector<int64_t> seg_sub(nbts), ent_sub(nbts);
    std::vector<int> fw_base(nb + 1);
    std::vector<int4> work;
    int64_t sacc = 0, eacc = 0;
    for (int b = 0; b < nb; ++b) {
        seg_base[b] = sacc;
        ent_base[b] = eacc;
        fw_base[b] = (int)work.size();
        for (int t = 0; t < T.nt; ++t) {
            const int64_t bt = (int64_t)b * T.nt + t;
            int64_t ns = 0, ne = 0;
            for (int q = 0; q < SUBS; ++q) {
                seg_sub[bt * SUBS + q] = sacc + ns;
                ent_sub[bt * SUBS + q] = eacc + ne;
                ns += (int64_t)(cnt[bt * SUBS + q] >> 32);
                ne += (int64_t)(uint32_t)cnt[bt * SUBS + q];
            }
            seg_bt[bt] = sacc;
            ent_bt[bt] = eacc;
            for (int64_t s0 = 0; s0 < ns; s0 += FWD_SEGS) {
                int4 w;
                w.x = t;
                w.y = (int)(sacc + s0 - seg_base[b]);
                w.z = (int)(ns - s0 < FWD_SEGS ? ns - s0 : FWD_SEGS);
                w.w = 0;
                work.push_back(w);
            }
            sacc += ns;
            eacc += ne;
        }
        if (eacc - ent_base[b] >= 4294967295LL || sacc - seg_base[b] >= 2147483647LL)
            return pct_fail(PCT_ERR_OVERFLOW, "drop: block %d has too many row entries for the tiled form", b);
    }
    seg_bt[nbt] = sacc;
    ent_bt[nbt] = eacc;
    seg_base[nb] = sacc;
    ent_base[nb] = eacc;
    fw_base[nb] = (int)work.size();
    if (sacc != total_slots) return pct_fail(PCT_ERR_STATE, "drop: segment count mismatch (%lld vs %lld)",
                                             (long long)sacc, (long long)total_slots);
    if (total_slots >= 4294967295LL) return pct_fail(PCT_ERR_OVERFLOW, "drop: too many row segments for the tiled form");
    PCT_TRY(d.seg_bt.alloc(sizeof(int64_t) * (nbt + 1)));
    PCT_TRY(d.ent_bt.alloc(sizeof(int64_t) * (nbt + 1)));
    PCT_TRY(d.seg_base.alloc(sizeof(int64_t) * (nb + 1)));
    PCT_TRY(d.ent_base.alloc(sizeof(int64_t) * (nb + 1)));
    PCT_TRY(d.work.alloc(sizeof(int4) * (work.size() > 0 ? work.size() : 1)));
    PCT_TRY(d.seg_row.alloc(sizeof(uint32_t) * (sacc > 0 ? sacc : 1)));
    PCT_TRY(d.seg_slot.alloc(sizeof(uint32_t) * (sacc > 0 ? sacc : 1)));
    PCT_TRY(d.seg_ent.alloc(sizeof(uint32_t) * (sacc > 0 ? sacc : 1)));
    PCT_TRY(d.partial.alloc(sizeof(long long) * (sacc > 0 ? sacc : 1)));
    /* padded by 8 entries: the aligned 16-byte loads of the last segment may reach past its end */
    PCT_TRY(d.ent.alloc(sizeof(uint16_t) * (eacc + 8)));
    PCT_TRY(d.u.alloc(sizeof(float) * B));
    PCT_TRY(d.umax.alloc(sizeof(unsigned) * nb));
    PCT_TRY(d.smax.alloc(sizeof(unsigned) * nb));
    PCT_TRY(d.counts.alloc(sizeof(uint32_t) * (size_t)nb * T.nv));
    PCT_TRY(d.cursor.alloc(sizeof(unsigned long long) * nbts));
    PCT_TRY(d.seg_sub.alloc(sizeof(int64_t) * nbts));
    PCT_TRY(d.ent_sub.alloc(sizeof(int64_t) * nbts));
    PCT_CUDA(cudaMemcpyAsync(d.seg_sub.p, seg_sub.data(), sizeof(int64_t) * nbts, cudaMemcpyHostToDevice, c->stream));
    PCT_CUDA(cudaMemcpyAsync(d.ent_sub.p, ent_sub.data(), sizeof(int64_t) * nbts, cudaMemcpyHostToDevice, c->stream));
    PCT_CUDA(cudaMemcpyAsync(d.seg_bt.p, seg_bt.data(), sizeof(int64_t) * (nbt + 1), cudaMemcpyHostToDevice, c->stream));
    PCT_CUDA(cudaMemcpyAsync(d.ent_bt.p, ent_bt.data(), sizeof(int64_t) * (nbt + 1), cudaMemcpyHostToDevice, c->stream));
    PCT_CUDA(cudaMemcpyAsync(d.seg_base.p, seg_base.data(), sizeof(int64_t) * (nb + 1), cudaMemcpyHostToDevice, c->stream));
    PCT_CUDA(cudaMemcpyAsync(d.ent_base.p, ent_base.data(), sizeof(int64_t) * (nb + 1), cudaMemcpyHostToDevice, c->stream));
    if (!work.empty())
        PCT_CUDA(cudaMemcpyAsync(d.work.p, work.data(), sizeof(int4) * work.size(), cudaMemcpyHostToDevice, c->stream));
    PCT_CUDA(cudaMemsetAsync(d.cursor.p, 0, sizeof(unsigned long long) * nbts, c->stream));
    /* pass 2: fill */
    ++c->launches;
    k_tile_fill<<<pct_grid_for(n, 128), 128, 0, c->stream>>>(
        c->dg, n, B, T, c->row_offsets.as<int64_t>(), c->row_len.as<int>(), c->rows.as<uint32_t>(), d.row_seg_off.as<int64_t>(),
        d.seg_sub.as<int64_t>(), d.ent_sub.as<int64_t>(), d.ent_base.as<int64_t>(), d.cursor.as<unsigned long long>(),
        d.seg_row.as<uint32_t>(), d.seg_slot.as<uint32_t>(), d.seg_ent.as<uint32_t>(), d.ent.as<uint16_t>());
    /* diagonal weights */
    PCT_CUDA(cudaMemsetAsync(d.smax.p, 0, sizeof(unsigned) * nb, c->stream));
    for (int b = 0; b < nb; ++b) {
        ++c->launches;
        k_tile_bwd<true><<<T.nt * BWD_CLUSTER, BWD_THREADS, 0, c->stream>>>(
            T, b, d.seg_bt.as<int64_t>(), d.seg_base.as<int64_t>(), d.ent_base.as<int64_t>(), d.seg_row.as<uint32_t>(),
            d.seg_ent.as<uint32_t>(), d.ent.as<uint16_t>(), nullptr, nullptr, nullptr, d.counts.as<uint32_t>(),
            d.smax.as<unsigned>(), nullptr, nullptr);
    }
    PCT_CUDA(cudaGetLastError());
    d.fw_base = fw_base;
    d.num_blocks = nb;
    return PCT_OK;
}

/* Enqueues the three launches of block b. */
void pct_drop_tiled_enqueue(pct_ctx* c, int b, double* resid) {
    TiledDrop& d = c->td;
    const int64_t n = c->h.n;
    const int64_t B = c->cfg.block_size;
    TileGeom T = tile_geom(c);
    const int64_t s = (int64_t)b * B, e = s + B < n ? s + B : n;
    const int nwork = d.fw_base[b + 1] - d.fw_base[b];
    if (nwork > 0)
        k_tile_fwd<<<nwork, FWD_THREADS, sizeof(long long) * T.tv, c->stream>>>(
            T, b, d.fw_base[b], d.work.as<int4>(), d.seg_base.as<int64_t>(), d.ent_base.as<int64_t>(),
            d.seg_slot.as<uint32_t>(), d.seg_ent.as<uint32_t>(), d.ent.as<uint16_t>(), c->x.as<float>(),
            d.partial.as<long long>(), c->err_flags.as<unsigned long long>());
    cudaMemsetAsync(d.umax.as<unsigned>() + b, 0, sizeof(unsigned), c->stream);
    k_tile_rows<<<pct_grid_for(e - s, ROWS_THREADS), ROWS_THREADS, 0, c->stream>>>(
        s, e, d.row_seg_off.as<int64_t>(), d.partial.as<long long>(), c->chord.as<float>(), c->row_scale.as<float>(),
        c->h.wepl.as<float>(), c->cfg.lambda, d.u.as<float>(), d.umax.as<unsigned>() + b, resid);
    k_tile_bwd<false><<<T.nt * BWD_CLUSTER, BWD_THREADS, 0, c->stream>>>(
        T, b, d.seg_bt.as<int64_t>(), d.seg_base.as<int64_t>(), d.ent_base.as<int64_t>(), d.seg_row.as<uint32_t>(),
        d.seg_ent.as<uint32_t>(), d.ent.as<uint16_t>(), d.u.as<float>(), d.umax.as<unsigned>(), d.smax.as<unsigned>(),
        d.counts.as<uint32_t>(), nullptr, c->x.as<float>(), c->err_flags.as<unsigned long long>());
}
