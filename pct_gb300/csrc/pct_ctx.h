/*
 * Reconstruction context: configuration, stream and every device buffer of
 * the path.  Internal to the library.
 *
 * Device data layout (all SoA, one CUDA allocation per array):
 *   history store   capacity H: 10 float coordinates/angles, WEPL (float),
 *                   bin (int32), flags (uint8), first voxel (uint32).  It is
 *                   compacted in place after binning, cuts and endpoints,
 *                   like the reference's *_vector globals.
 *   bins            counts (int32) and the binary32 means / sigmas /
 *                   sinogram (NUM_BINS each); while the cuts run, the store
 *                   order sorted by bin (stable) and each bin's segment of it.
 *   voxels          hull count images (int32), hull masks (uint8), FBP
 *                   image, iterate x, DROP update accumulator (float).
 *   MLP rows        row offsets (int64, R+1), voxel entries (uint32), chord
 *                   length (float) and 1/||a_i||^2 (double) per row; per-block
 *                   diagonal weights for DROP.
 */
#ifndef PCT_CTX_H
#define PCT_CTX_H

#include <cuda_runtime.h>
#include <cstdint>
#include <vector>
#include <cstddef>
#include "pct_internal.h"

#define PCT_CUDA(call)                                                                              \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return pct_fail(PCT_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
    } while (0)

#define PCT_TRY(call)                         \
    do {                                      \
        pct_status s_ = (call);               \
        if (s_ != PCT_OK) return s_;          \
    } while (0)

/* Owning device buffer of bytes. */
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    pct_status alloc(size_t n);           /* reallocates when larger; contents lost */
    pct_status grow_keep(size_t n, cudaStream_t s); /* reallocates keeping the old bytes */
    void release();
    template <class T> T* as() const { return static_cast<T*>(p); }
};

/* Per-history arrays of the resident store. */
struct HistoryStore {
    DevBuf x_entry, y_entry, z_entry, x_exit, y_exit, z_exit;
    DevBuf xy_entry_angle, xz_entry_angle, xy_exit_angle, xz_exit_angle;
    DevBuf wepl, bin_num, bin_valid, failed, first_voxel;
    int64_t n = 0, capacity = 0;
    pct_status reserve(int64_t cap, cudaStream_t s);
    void release();
};

/* Device-side view of the history store for kernels. */
struct HistView {
    float *x_entry, *y_entry, *z_entry, *x_exit, *y_exit, *z_exit;
    float *xy_entry_angle, *xz_entry_angle, *xy_exit_angle, *xz_exit_angle;
    float* wepl;
    int32_t* bin_num;
    uint8_t* bin_valid;
    uint8_t* failed;
    uint32_t* first_voxel;
};

/* Parameters every kernel needs (passed by value). */
struct DevGeom {
    int columns, rows, slices, num_voxels;
    int t_bins, v_bins, angular_bins, num_bins;
    double recon_cyl_radius, recon_cyl_height;
    double voxel_width, voxel_height, voxel_thickness;
    double x_zero, y_zero, z_zero, mlp_u_step;
    double t_bin_size, v_bin_size, angular_bin_size, gantry_angle_interval, source_radius, slice_thickness;
    int brick; /* MLP rows and the DROP iterate use the 4x2x1 brick voxel order (see pct_device.cuh) */
    unsigned long long div_c, div_r; /* ceil(2^64 / COLUMNS), ceil(2^64 / ROWS): q = umulhi64(n, m) */
    /* binary32 copies for the binary32 walks and MLP samples (a conversion in the
     * kernel would run on the FP64 pipe at every use) */
    float fx0, fy0, fz0, fvw, fvh, fvt, fivw, fivh, fivt;
    /* the MLP face margin as a fraction of each voxel size: a binary32 sample
     * whose fractional position along an axis is below flo or above fhi is
     * recomputed in binary64 (rounded outwards from mlp_face_margin / size) */
    float fmlo_x, fmlo_y, fmlo_z, fmhi_x, fmhi_y, fmhi_z;
};

enum Stage {
    ST_EMPTY = 0, ST_BINNED, ST_HULLS_DONE, ST_CUT, ST_FBP, ST_HULL_SELECTED, ST_X0, ST_ENDPOINTS, ST_ROWS
};

/* Rows regrouped per (DROP block, image tile) for the tiled DROP form. */
struct TiledDrop {
    DevBuf row_seg_off, row_nseg, bt_cnt, seg_bt, ent_bt, seg_base, ent_base, work;
    DevBuf seg_row, seg_slot, seg_ent, partial, ent, u, umax, smax, counts, cursor, seg_sub, ent_sub;
    std::vector<int> fw_base;  /* forward work items of each block: [fw_base[b], fw_base[b + 1]) */
    int num_blocks = 0;
    DevBuf* all[20] = {&row_seg_off, &row_nseg, &bt_cnt, &seg_bt, &ent_bt, &seg_base, &ent_base, &work, &seg_row,
                       &seg_slot, &seg_ent, &partial, &ent, &u, &umax, &smax, &counts, &cursor, &seg_sub, &ent_sub};
    size_t bytes_held() const {
        size_t t = 0;
        for (DevBuf* b : all) t += b->bytes;
        return t;
    }
    void release() {
        for (DevBuf* b : all) b->release();
        fw_base.clear();
        num_blocks = 0;
    }
};

struct pct_ctx {
    pct_config cfg;
    pct_geometry geo;
    DevGeom dg;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr; /* hull walks of a chunk, overlapped with its preprocessing */
    int stage = ST_EMPTY;
    int64_t launches = 0;          /* kernels launched, for pct_counts.kernel_launches */
    pct_counts counts{};

    /* chunk staging */
    DevBuf in13[13], in_angle;
    DevBuf tmp_missed, tmp_hist;   /* per-chunk flags and staging for compaction */
    DevBuf scan_tmp;               /* block sums for stream compaction */
    DevBuf pinned_count;           /* host-pinned counters read back after compactions */
    HistoryStore h, h2;            /* h2: scratch store for out-of-place compaction */

    /* bins */
    DevBuf bin_counts, bin_counts_post;
    DevBuf bin_sort, bin_seg;      /* statistics: stable sort of the store by bin, per-bin segments */
    DevBuf mean_wepl, mean_ut, mean_uv, sd_wepl, sd_ut, sd_uv, sinogram, sinogram_filtered;
    DevBuf filter_taps, filter_scale, trig_gantry, trig_bins;
    DevBuf err_flags;              /* device error/overflow counters */

    /* voxels */
    DevBuf sc_hull, msc_counts, sm_counts, msc_hull, sm_hull;
    DevBuf fbp_image, fbp_hull, x_hull, x_hull_filtered, x0, x, x_update;
    DevBuf x_brick;                /* the iterate in brick order while DROP runs */

    /* MLP rows and DROP */
    DevBuf row_offsets, row_len, rows, chord, row_scale, mlp_table;  /* row_offsets: start of each row's slot */
    DevBuf mlp_bound, mlp_rec, mlp_queue, mlp_fix_rows, mlp_order;  /* MLP row generation scratch */
    DevBuf walk_order;                                               /* hull walk launch order + keys */
    DevBuf mlp_tab_trig, mlp_tab_depth;                              /* tables of the tabulated MLP */
    DevBuf block_diag, block_diag_offsets;  /* per DROP block: voxel counts s_j */
    DevBuf block_norm;             /* per DROP block: sum of c^2 per voxel (robust variant) */
    DevBuf robust_norm;            /* robust variant: running per-voxel sum of c^2 since the start (binary64) */
    DevBuf drop_perm, drop_sort;           /* per-block bin order of the rows, sort scratch */
    DevBuf dense_off, dense_rows;  /* CSR view of the rows for pct_get_array */
    int64_t dense_total = 0;
    DevBuf drop_resid;
    DevBuf d64_x, d64_upd, d64_chord, d64_res;  /* binary64 DROP (pct_drop_fp64) */
    /* gather DROP form: rank-ordered row data, slice offsets and slots, column lists, row values */
    DevBuf gather_meta, gather_off, gather_slot, gather_lists, gather_val, gather_tmp, gather_steps;
    int64_t gather_entries = 0;
    cudaGraphExec_t drop_graph_exec = nullptr;  /* one DROP iteration */
    int64_t row_capacity = 0;
    int num_blocks = 0;
    int diag_ready = 0;
    /* sharded DROP: all-reduce callback, this context's shard and the global
     * number of reconstruction histories at pct_select_shard */
    pct_allreduce_fn allreduce = nullptr;
    void* allreduce_user = nullptr;
    int shard = 0, num_shards = 1;
    int64_t shard_total = 0;
    int drop_mode = 0;             /* built DROP form: PCT_DROP_TILED / _SORTED / _SCATTER */
    int drop_launches_per_iter = 0;
    TiledDrop td;

    pct_status set_device() {
        cudaError_t e = cudaSetDevice(device);
        if (e != cudaSuccess) return pct_fail(PCT_ERR_CUDA, "cudaSetDevice(%d): %s", device, cudaGetErrorString(e));
        return PCT_OK;
    }
    HistView view(HistoryStore& s) const;
};

/* The same arrays from entry `off` on. */
inline HistView hv_offset(HistView v, int64_t off) {
    v.x_entry += off; v.y_entry += off; v.z_entry += off; v.x_exit += off; v.y_exit += off; v.z_exit += off;
    v.xy_entry_angle += off; v.xz_entry_angle += off; v.xy_exit_angle += off; v.xz_exit_angle += off;
    v.wepl += off; v.bin_num += off; v.bin_valid += off; v.failed += off; v.first_voxel += off;
    return v;
}

/* Stage implementations (one file each). */
pct_status pct_stage_process_chunk(pct_ctx* c, const float* const data13[13], const float* angle, int64_t n, int on_dev);
pct_status pct_stage_hull_finish(pct_ctx* c);
pct_status pct_stage_cuts(pct_ctx* c);
pct_status pct_stage_fbp(pct_ctx* c);
pct_status pct_stage_hull_selection(pct_ctx* c);
pct_status pct_stage_initial_iterate(pct_ctx* c);
pct_status pct_stage_endpoints(pct_ctx* c);
pct_status pct_stage_mlp_rows(pct_ctx* c);
pct_status pct_stage_mlp_rows_tab(pct_ctx* c);
pct_status pct_stage_drop(pct_ctx* c, int iterations, pct_drop_stats* stats);
/* Iterations whose residual is kept (pct_drop_stats.residual). */
constexpr int PCT_DROP_MAXIT = 64;
pct_status pct_drop_prepare(pct_ctx* c);
pct_status pct_drop_begin(pct_ctx* c);
pct_status pct_drop_end(pct_ctx* c, int done, float ms, pct_drop_stats* stats);
void pct_drop_store_resid(pct_ctx* c, int it);

/* Stable compaction of src[src_off, src_off+n) by a keep flag into dst at dst_off. */
pct_status pct_compact(pct_ctx* c, HistoryStore& src, int64_t src_off, int64_t n, const uint8_t* d_keep,
                       HistoryStore& dst, int64_t dst_off, int64_t* kept);
/* In-place stable compaction of the resident store c->h[0, n). */
pct_status pct_compact_histories(pct_ctx* c, const uint8_t* d_keep, int64_t n, int64_t* kept);

/* Device error counters (indices into err_flags, uint64). */
enum { ERR_WALK_CAPPED = 0, ERR_VOXEL_OUTSIDE = 1, ERR_FIXED_OVERFLOW = 2, ERR_ROW_OVERFLOW = 3,
       ERR_MLP_FP64 = 4, ERR_ROWS_OUTSIDE = 5, ERR_MLP_QUEUED = 6, ERR_MLP_FIXROWS = 7, ERR_DROP_NONFINITE = 8,
       ERR_WALK_FP64 = 9, ERR_COUNT = 16 };

DevGeom pct_make_devgeom(const pct_config& c, const pct_geometry& g);
void pct_drop_release_graph(pct_ctx* c);
void pct_drop_gather_release(pct_ctx* c);
pct_status pct_drop_gather_build(pct_ctx* c);
void pct_drop_gather_enqueue(pct_ctx* c, int block, double* resid);
pct_status pct_scan_lengths(pct_ctx* c, const int64_t* len, int64_t n, int64_t* off, int64_t* total);
pct_status pct_rows_dense(pct_ctx* c, int64_t* total, DevBuf* dense_off, DevBuf* dense);
int pct_drop_tiled_fits(pct_ctx* c);
pct_status pct_drop_tiled_build(pct_ctx* c);
void pct_drop_tiled_enqueue(pct_ctx* c, int block, double* resid);

#endif
