/*
 * Context lifetime, device buffers, array getters and the stable history
 * compaction shared by the stages.
 */
#include <cstring>
#include <utility>
#include "pct_ctx.h"

pct_status DevBuf::alloc(size_t n) {
    if (n <= bytes && p) return PCT_OK;
    release();
    if (n == 0) return PCT_OK;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
        p = nullptr;
        cudaGetLastError();
        return pct_fail(PCT_ERR_ALLOC, "cudaMalloc(%zu bytes): %s", n, cudaGetErrorString(e));
    }
    bytes = n;
    return PCT_OK;
}

pct_status DevBuf::grow_keep(size_t n, cudaStream_t s) {
    if (n <= bytes && p) return PCT_OK;
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, n);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return pct_fail(PCT_ERR_ALLOC, "cudaMalloc(%zu bytes): %s", n, cudaGetErrorString(e));
    }
    if (p && bytes) {
        e = cudaMemcpyAsync(q, p, bytes, cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            cudaFree(q);
            return pct_fail(PCT_ERR_CUDA, "grow_keep copy: %s", cudaGetErrorString(e));
        }
    }
    release();
    p = q;
    bytes = n;
    return PCT_OK;
}

void DevBuf::release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

pct_status HistoryStore::reserve(int64_t cap, cudaStream_t s) {
    if (cap <= capacity) return PCT_OK;
    size_t f = sizeof(float) * (size_t)cap;
    DevBuf* fl[] = {&x_entry, &y_entry, &z_entry, &x_exit, &y_exit, &z_exit,
                    &xy_entry_angle, &xz_entry_angle, &xy_exit_angle, &xz_exit_angle, &wepl, &bin_num, &first_voxel};
    for (DevBuf* b : fl) PCT_TRY(b->grow_keep(f, s));
    PCT_TRY(bin_valid.grow_keep((size_t)cap, s));
    PCT_TRY(failed.grow_keep((size_t)cap, s));
    capacity = cap;
    return PCT_OK;
}

void HistoryStore::release() {
    DevBuf* all[] = {&x_entry, &y_entry, &z_entry, &x_exit, &y_exit, &z_exit, &xy_entry_angle, &xz_entry_angle,
                     &xy_exit_angle, &xz_exit_angle, &wepl, &bin_num, &bin_valid, &failed, &first_voxel};
    for (DevBuf* b : all) b->release();
    n = capacity = 0;
}

HistView pct_ctx::view(HistoryStore& s) const {
    HistView v;
    v.x_entry = s.x_entry.as<float>(); v.y_entry = s.y_entry.as<float>(); v.z_entry = s.z_entry.as<float>();
    v.x_exit = s.x_exit.as<float>(); v.y_exit = s.y_exit.as<float>(); v.z_exit = s.z_exit.as<float>();
    v.xy_entry_angle = s.xy_entry_angle.as<float>(); v.xz_entry_angle = s.xz_entry_angle.as<float>();
    v.xy_exit_angle = s.xy_exit_angle.as<float>(); v.xz_exit_angle = s.xz_exit_angle.as<float>();
    v.wepl = s.wepl.as<float>();
    v.bin_num = s.bin_num.as<int32_t>();
    v.bin_valid = s.bin_valid.as<uint8_t>();
    v.failed = s.failed.as<uint8_t>();
    v.first_voxel = s.first_voxel.as<uint32_t>();
    return v;
}

DevGeom pct_make_devgeom(const pct_config& c, const pct_geometry& g) {
    DevGeom d;
    d.columns = g.columns; d.rows = g.rows; d.slices = g.slices; d.num_voxels = g.num_voxels;
    d.t_bins = g.t_bins; d.v_bins = g.v_bins; d.angular_bins = g.angular_bins; d.num_bins = g.num_bins;
    d.recon_cyl_radius = g.recon_cyl_radius; d.recon_cyl_height = g.recon_cyl_height;
    d.voxel_width = g.voxel_width; d.voxel_height = g.voxel_height; d.voxel_thickness = g.voxel_thickness;
    d.x_zero = g.x_zero; d.y_zero = g.y_zero; d.z_zero = g.z_zero; d.mlp_u_step = g.mlp_u_step;
    d.t_bin_size = c.t_bin_size; d.v_bin_size = c.v_bin_size; d.angular_bin_size = c.angular_bin_size;
    d.gantry_angle_interval = c.gantry_angle_interval; d.source_radius = c.source_radius;
    d.slice_thickness = c.slice_thickness;
    d.brick = (c.voxel_order == PCT_ORDER_AUTO && g.columns % 4 == 0 && g.rows % 2 == 0) ? 1 : 0;
    /* exact for n < 2^31 since 64 >= 31 + log2(d) */
    d.div_c = g.columns > 1 ? (~0ull) / (unsigned long long)g.columns + 1ull : 0ull;
    d.div_r = g.rows > 1 ? (~0ull) / (unsigned long long)g.rows + 1ull : 0ull;
    d.fx0 = (float)g.x_zero; d.fy0 = (float)g.y_zero; d.fz0 = (float)g.z_zero;
    d.fvw = (float)g.voxel_width; d.fvh = (float)g.voxel_height; d.fvt = (float)g.voxel_thickness;
    d.fivw = 1.0f / d.fvw; d.fivh = 1.0f / d.fvh; d.fivt = 1.0f / d.fvt; /* IEEE quotients, as on the device */
    auto up = [](double q) { float f = (float)q; return (double)f < q ? std::nextafter(f, INFINITY) : f; };
    auto down = [](double q) { float f = (float)q; return (double)f > q ? std::nextafter(f, -INFINITY) : f; };
    const double m = c.mlp_face_margin;
    d.fmlo_x = up(m / g.voxel_width); d.fmlo_y = up(m / g.voxel_height); d.fmlo_z = up(m / g.voxel_thickness);
    d.fmhi_x = down(1.0 - m / g.voxel_width); d.fmhi_y = down(1.0 - m / g.voxel_height);
    d.fmhi_z = down(1.0 - m / g.voxel_thickness);
    return d;
}

/* ---- stable compaction ------------------------------------------------------ */
namespace {
constexpr int CT_THREADS = 256;
constexpr int CT_ITEMS = 8;
constexpr int CT_TILE = CT_THREADS * CT_ITEMS;

__global__ void k_tile_counts(const uint8_t* __restrict__ keep, int64_t n, int* __restrict__ tile_counts) {
    int64_t base = (int64_t)blockIdx.x * CT_TILE;
    int c = 0;
    for (int k = 0; k < CT_ITEMS; ++k) {
        int64_t i = base + (int64_t)k * CT_THREADS + threadIdx.x;
        if (i < n && keep[i]) ++c;
    }
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    __shared__ int ws[CT_THREADS / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < CT_THREADS / 32; ++w) t += ws[w];
        tile_counts[blockIdx.x] = t;
    }
}

/* Single-block exclusive scan of the tile counts; writes the total after them. */
__global__ void k_scan_tiles(int* __restrict__ tile_counts, int64_t* __restrict__ tile_offsets, int tiles,
                             int64_t* __restrict__ total) {
    __shared__ int64_t carry;
    __shared__ int64_t ws[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < tiles; base += blockDim.x) {
        int i = base + threadIdx.x;
        int64_t v = i < tiles ? tile_counts[i] : 0;
        int64_t x = v;
        int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        for (int o = 1; o < 32; o <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) ws[w] = x;
        __syncthreads();
        if (w == 0) {
            int64_t s = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                int64_t y = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += y;
            }
            ws[lane] = s;
        }
        __syncthreads();
        int64_t incl = x + (w > 0 ? ws[w - 1] : 0);
        if (i < tiles) tile_offsets[i] = carry + incl - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

struct CompactArgs {
    const void* src[16];
    void* dst[16];
    int size[16];
    int nfields;
};

__global__ void k_scatter(const uint8_t* __restrict__ keep, int64_t n, const int64_t* __restrict__ tile_offsets,
                          CompactArgs a) {
    __shared__ int ws[CT_THREADS / 32 + 1];
    int64_t base = (int64_t)blockIdx.x * CT_TILE;
    int64_t out = tile_offsets[blockIdx.x];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int k = 0; k < CT_ITEMS; ++k) {
        int64_t i = base + (int64_t)k * CT_THREADS + threadIdx.x;
        bool f = i < n && keep[i];
        unsigned m = __ballot_sync(0xffffffffu, f);
        if (lane == 0) ws[w] = __popc(m);
        __syncthreads();
        int before = 0, total = 0;
        for (int j = 0; j < CT_THREADS / 32; ++j) {
            if (j < w) before += ws[j];
            total += ws[j];
        }
        int pos = before + __popc(m & ((1u << lane) - 1));
        if (f) {
            int64_t d = out + pos;
            for (int q = 0; q < a.nfields; ++q) {
                if (a.size[q] == 4) ((uint32_t*)a.dst[q])[d] = ((const uint32_t*)a.src[q])[i];
                else ((uint8_t*)a.dst[q])[d] = ((const uint8_t*)a.src[q])[i];
            }
        }
        out += total;
        __syncthreads();
    }
}
}  // namespace

pct_status pct_compact(pct_ctx* c, HistoryStore& src, int64_t src_off, int64_t n, const uint8_t* d_keep,
                       HistoryStore& dst, int64_t dst_off, int64_t* kept) {
    *kept = 0;
    if (n == 0) return PCT_OK;
    int64_t tiles = (n + CT_TILE - 1) / CT_TILE;
    PCT_TRY(c->scan_tmp.alloc(tiles * (sizeof(int) + sizeof(int64_t)) + 64));
    int* tile_counts = c->scan_tmp.as<int>();
    int64_t* tile_offsets = (int64_t*)((char*)c->scan_tmp.p + ((tiles * sizeof(int) + 15) & ~(size_t)15));
    PCT_TRY(c->pinned_count.alloc(sizeof(int64_t) * 2));
    int64_t* d_total = c->pinned_count.as<int64_t>();
    PCT_TRY(dst.reserve(dst_off + n, c->stream));
    ++c->launches;
    k_tile_counts<<<(unsigned)tiles, CT_THREADS, 0, c->stream>>>(d_keep, n, tile_counts);
    ++c->launches;
    k_scan_tiles<<<1, 1024, 0, c->stream>>>(tile_counts, tile_offsets, (int)tiles, d_total);
    CompactArgs a;
    DevBuf* sf[] = {&src.x_entry, &src.y_entry, &src.z_entry, &src.x_exit, &src.y_exit, &src.z_exit,
                    &src.xy_entry_angle, &src.xz_entry_angle, &src.xy_exit_angle, &src.xz_exit_angle, &src.wepl,
                    &src.bin_num, &src.first_voxel, &src.bin_valid, &src.failed};
    DevBuf* df[] = {&dst.x_entry, &dst.y_entry, &dst.z_entry, &dst.x_exit, &dst.y_exit, &dst.z_exit,
                    &dst.xy_entry_angle, &dst.xz_entry_angle, &dst.xy_exit_angle, &dst.xz_exit_angle, &dst.wepl,
                    &dst.bin_num, &dst.first_voxel, &dst.bin_valid, &dst.failed};
    a.nfields = 15;
    for (int q = 0; q < 15; ++q) {
        int sz = q < 13 ? 4 : 1;
        a.src[q] = (const char*)sf[q]->p + src_off * sz;
        a.dst[q] = (char*)df[q]->p + dst_off * sz;
        a.size[q] = sz;
    }
    ++c->launches;
    k_scatter<<<(unsigned)tiles, CT_THREADS, 0, c->stream>>>(d_keep, n, tile_offsets, a);
    PCT_CUDA(cudaGetLastError());
    int64_t total = 0;
    PCT_CUDA(cudaMemcpyAsync(&total, d_total, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    PCT_CUDA(cudaStreamSynchronize(c->stream));
    *kept = total;
    return PCT_OK;
}

pct_status pct_compact_histories(pct_ctx* c, const uint8_t* d_keep, int64_t n, int64_t* kept) {
    PCT_TRY(pct_compact(c, c->h, 0, n, d_keep, c->h2, 0, kept));
    std::swap(c->h, c->h2);
    c->h.n = *kept;
    return PCT_OK;
}

/* ---- C ABI: lifetime and getters ---------------------------------------------- */
extern "C" pct_status pct_create(const pct_config* cfg, int device, pct_ctx** out) {
    if (!cfg || !out) return pct_fail(PCT_ERR_ARGUMENT, "pct_create: null argument");
    *out = nullptr;
    pct_geometry g;
    int e = pct_geometry_derive(cfg, &g);
    if (e) return pct_fail(PCT_ERR_ARGUMENT, "pct_create: invalid geometry (code %d)", e);
    if (cfg->block_size <= 0) return pct_fail(PCT_ERR_ARGUMENT, "pct_create: block_size must be positive");
    if (cfg->drop_variant < PCT_DROP_STANDARD || cfg->drop_variant > PCT_DROP_ROBUST2)
        return pct_fail(PCT_ERR_ARGUMENT, "pct_create: drop_variant %d", cfg->drop_variant);
    if (cfg->drop_variant != PCT_DROP_STANDARD && (cfg->drop_form == PCT_DROP_TILED || cfg->drop_form == PCT_DROP_GATHER))
        return pct_fail(PCT_ERR_ARGUMENT, "pct_create: the DROP variants run in the scatter or sorted form");
    if (cfg->voxel_order != PCT_ORDER_AUTO && cfg->voxel_order != PCT_ORDER_LINEAR)
        return pct_fail(PCT_ERR_ARGUMENT, "pct_create: voxel_order %d", cfg->voxel_order);
    if (cfg->drop_form < PCT_DROP_SCATTER || cfg->drop_form > PCT_DROP_GATHER)
        return pct_fail(PCT_ERR_ARGUMENT, "pct_create: drop_form %d", cfg->drop_form);
    if (cfg->mlp_hull < 0 || cfg->mlp_hull > 3) return pct_fail(PCT_ERR_ARGUMENT, "pct_create: bad mlp_hull");
    if (cfg->mlp_tabulated != 0 && cfg->mlp_tabulated != 1)
        return pct_fail(PCT_ERR_ARGUMENT, "pct_create: mlp_tabulated %d", cfg->mlp_tabulated);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return pct_fail(PCT_ERR_CUDA, "pct_create: no CUDA device");
    }
    if (device < 0 || device >= ndev) return pct_fail(PCT_ERR_ARGUMENT, "pct_create: device %d of %d", device, ndev);
    pct_ctx* c = new pct_ctx();
    c->cfg = *cfg;
    c->geo = g;
    c->dg = pct_make_devgeom(*cfg, g);
    c->device = device;
    pct_status s = c->set_device();
    if (s == PCT_OK) {
        cudaError_t ce = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        /* the walks' stream outranks the preprocessing stream, so that walk CTAs start as
         * preprocessing CTAs retire and the two share the SMs (binary32 and binary64 pipes) */
        int lo = 0, hi = 0;
        if (ce == cudaSuccess && cudaDeviceGetStreamPriorityRange(&lo, &hi) != cudaSuccess) lo = hi = 0;
        if (ce == cudaSuccess) ce = cudaStreamCreateWithPriority(&c->stream2, cudaStreamNonBlocking, hi);
        if (ce != cudaSuccess) s = pct_fail(PCT_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(ce));
    }
    if (s == PCT_OK) s = c->err_flags.alloc(sizeof(unsigned long long) * ERR_COUNT);
    if (s == PCT_OK && cudaMemsetAsync(c->err_flags.p, 0, c->err_flags.bytes, c->stream) != cudaSuccess)
        s = pct_fail(PCT_ERR_CUDA, "memset err flags");
    if (s != PCT_OK) {
        pct_destroy(c);
        return s;
    }
    *out = c;
    return PCT_OK;
}

extern "C" pct_status pct_destroy(pct_ctx* c) {
    if (!c) return PCT_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->stream2) cudaStreamSynchronize(c->stream2);
    DevBuf* all[] = {&c->dense_off, &c->dense_rows, &c->row_len, &c->in_angle, &c->tmp_missed, &c->tmp_hist, &c->scan_tmp, &c->pinned_count, &c->bin_counts,
                     &c->bin_counts_post, &c->bin_sort, &c->bin_seg, &c->mean_wepl, &c->mean_ut,
                     &c->mean_uv, &c->sd_wepl, &c->sd_ut, &c->sd_uv, &c->sinogram, &c->sinogram_filtered,
                     &c->filter_taps, &c->filter_scale, &c->trig_gantry, &c->trig_bins, &c->err_flags,
                     &c->sc_hull, &c->msc_counts, &c->sm_counts, &c->msc_hull, &c->sm_hull, &c->fbp_image,
                     &c->fbp_hull, &c->x_hull, &c->x_hull_filtered, &c->x0, &c->x, &c->x_update, &c->row_offsets,
                     &c->rows, &c->chord, &c->row_scale, &c->mlp_table, &c->block_diag, &c->block_diag_offsets,
                     &c->drop_resid, &c->mlp_bound, &c->mlp_rec, &c->mlp_queue, &c->mlp_fix_rows, &c->mlp_order, &c->walk_order, &c->mlp_tab_trig, &c->mlp_tab_depth,
                     &c->drop_perm, &c->drop_sort, &c->x_brick, &c->block_norm, &c->robust_norm,
                     &c->d64_x, &c->d64_upd, &c->d64_chord, &c->d64_res,
                     &c->gather_meta, &c->gather_off, &c->gather_slot, &c->gather_lists, &c->gather_val,
                     &c->gather_tmp, &c->gather_steps};
    for (DevBuf* b : all) b->release();
    c->td.release();
    for (auto& b : c->in13) b.release();
    pct_drop_release_graph(c);
    c->h.release();
    c->h2.release();
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->stream2) cudaStreamDestroy(c->stream2);
    delete c;
    return PCT_OK;
}

extern "C" pct_status pct_reserve(pct_ctx* c, int64_t total) {
    if (!c || total < 0) return pct_fail(PCT_ERR_ARGUMENT, "pct_reserve: bad argument");
    PCT_TRY(c->set_device());
    return c->h.reserve(total, c->stream);
}

extern "C" void* pct_stream(pct_ctx* c) { return c ? (void*)c->stream : nullptr; }

extern "C" pct_status pct_get_counts(pct_ctx* c, pct_counts* out) {
    if (!c || !out) return pct_fail(PCT_ERR_ARGUMENT, "pct_get_counts: null argument");
    PCT_TRY(c->set_device());
    unsigned long long f[ERR_COUNT];
    PCT_CUDA(cudaMemcpyAsync(f, c->err_flags.p, sizeof(f), cudaMemcpyDeviceToHost, c->stream));
    PCT_CUDA(cudaStreamSynchronize(c->stream));
    *out = c->counts;
    if (c->stage >= ST_ROWS) {
        DevBuf off;
        int64_t total = 0;
        pct_status st = pct_rows_dense(c, &total, &off, nullptr);
        off.release();
        PCT_TRY(st);
        out->row_entries = total;
    }
    out->drop_list_entries = c->drop_mode == PCT_DROP_GATHER ? c->gather_entries : 0;
    out->walks_capped = (int64_t)f[ERR_WALK_CAPPED];
    out->mlp_fp64_samples = (int64_t)f[ERR_MLP_FP64];
    out->walk_fp64_steps = (int64_t)f[ERR_WALK_FP64];
    out->rows_outside_image = (int64_t)f[ERR_ROWS_OUTSIDE];
    out->kernel_launches = c->launches;
    return PCT_OK;
}

static pct_status array_info(pct_ctx* c, pct_array which, void** p, size_t* bytes) {
    if ((which == PCT_ARR_ROW_OFFSETS || which == PCT_ARR_ROWS) && c->stage >= ST_ROWS) {
        /* rows live in per-row slots; these arrays are the dense (CSR) view */
        PCT_TRY(pct_rows_dense(c, &c->dense_total, &c->dense_off, which == PCT_ARR_ROWS ? &c->dense_rows : nullptr));
        PCT_CUDA(cudaStreamSynchronize(c->stream));
    }
    const size_t V = (size_t)c->geo.num_voxels, B = (size_t)c->geo.num_bins, H = (size_t)c->h.n;
    DevBuf* b = nullptr;
    size_t n = 0;
    switch (which) {
        case PCT_ARR_MSC_COUNTS: b = &c->msc_counts; n = V * 4; break;
        case PCT_ARR_SM_COUNTS: b = &c->sm_counts; n = V * 4; break;
        case PCT_ARR_SC_HULL: b = &c->sc_hull; n = V * 4; break;
        case PCT_ARR_MSC_HULL: b = &c->msc_hull; n = V * 4; break;
        case PCT_ARR_SM_HULL: b = &c->sm_hull; n = V * 4; break;
        case PCT_ARR_BIN_COUNTS_PRE: b = &c->bin_counts; n = B * 4; break;
        case PCT_ARR_MEAN_WEPL: b = &c->mean_wepl; n = B * 4; break;
        case PCT_ARR_MEAN_UT: b = &c->mean_ut; n = B * 4; break;
        case PCT_ARR_MEAN_UV: b = &c->mean_uv; n = B * 4; break;
        case PCT_ARR_SD_WEPL: b = &c->sd_wepl; n = B * 4; break;
        case PCT_ARR_SD_UT: b = &c->sd_ut; n = B * 4; break;
        case PCT_ARR_SD_UV: b = &c->sd_uv; n = B * 4; break;
        case PCT_ARR_BIN_COUNTS_POST: b = &c->bin_counts_post; n = B * 4; break;
        case PCT_ARR_SINOGRAM: b = &c->sinogram; n = B * 4; break;
        case PCT_ARR_SINOGRAM_FILTERED: b = &c->sinogram_filtered; n = B * 4; break;
        case PCT_ARR_FBP_IMAGE: b = &c->fbp_image; n = V * 4; break;
        case PCT_ARR_FBP_HULL: b = &c->fbp_hull; n = V; break;
        case PCT_ARR_X_HULL: b = &c->x_hull; n = V; break;
        case PCT_ARR_X_HULL_FILTERED: b = &c->x_hull_filtered; n = V; break;
        case PCT_ARR_X0: b = &c->x0; n = V * 4; break;
        case PCT_ARR_X: b = &c->x; n = V * 4; break;
        case PCT_ARR_H_BIN_NUM: b = &c->h.bin_num; n = H * 4; break;
        case PCT_ARR_H_WEPL: b = &c->h.wepl; n = H * 4; break;
        case PCT_ARR_H_X_ENTRY: b = &c->h.x_entry; n = H * 4; break;
        case PCT_ARR_H_Y_ENTRY: b = &c->h.y_entry; n = H * 4; break;
        case PCT_ARR_H_Z_ENTRY: b = &c->h.z_entry; n = H * 4; break;
        case PCT_ARR_H_X_EXIT: b = &c->h.x_exit; n = H * 4; break;
        case PCT_ARR_H_Y_EXIT: b = &c->h.y_exit; n = H * 4; break;
        case PCT_ARR_H_Z_EXIT: b = &c->h.z_exit; n = H * 4; break;
        case PCT_ARR_H_XY_ENTRY_ANGLE: b = &c->h.xy_entry_angle; n = H * 4; break;
        case PCT_ARR_H_XZ_ENTRY_ANGLE: b = &c->h.xz_entry_angle; n = H * 4; break;
        case PCT_ARR_H_XY_EXIT_ANGLE: b = &c->h.xy_exit_angle; n = H * 4; break;
        case PCT_ARR_H_XZ_EXIT_ANGLE: b = &c->h.xz_exit_angle; n = H * 4; break;
        case PCT_ARR_H_FIRST_VOXEL: b = &c->h.first_voxel; n = H * 4; break;
        case PCT_ARR_H_FAILED_CUTS: b = &c->h.failed; n = H; break;
        case PCT_ARR_ROW_OFFSETS: b = &c->dense_off; n = c->stage >= ST_ROWS ? (H + 1) * 8 : 0; break;
        case PCT_ARR_ROWS: b = &c->dense_rows; n = c->stage >= ST_ROWS ? (size_t)c->dense_total * 4 : 0; break;
        case PCT_ARR_CHORD: b = &c->chord; n = c->stage >= ST_ROWS ? H * 4 : 0; break;
        default: return pct_fail(PCT_ERR_ARGUMENT, "unknown array %d", (int)which);
    }
    if (n && (!b->p || b->bytes < n)) return pct_fail(PCT_ERR_STATE, "array %d is not available at this stage", (int)which);
    *p = b->p;
    *bytes = n;
    return PCT_OK;
}

extern "C" pct_status pct_array_device_ptr(pct_ctx* c, pct_array which, void** dptr, size_t* bytes) {
    if (!c || !dptr || !bytes) return pct_fail(PCT_ERR_ARGUMENT, "pct_array_device_ptr: null argument");
    return array_info(c, which, dptr, bytes);
}

extern "C" pct_status pct_get_array(pct_ctx* c, pct_array which, void* host_dst, size_t* bytes) {
    if (!c || !bytes) return pct_fail(PCT_ERR_ARGUMENT, "pct_get_array: null argument");
    PCT_TRY(c->set_device());
    void* p = nullptr;
    size_t n = 0;
    PCT_TRY(array_info(c, which, &p, &n));
    if (!host_dst) {
        *bytes = n;
        return PCT_OK;
    }
    if (*bytes < n) return pct_fail(PCT_ERR_ARGUMENT, "pct_get_array: buffer holds %zu bytes, need %zu", *bytes, n);
    if (n) {
        PCT_CUDA(cudaMemcpyAsync(host_dst, p, n, cudaMemcpyDeviceToHost, c->stream));
        PCT_CUDA(cudaStreamSynchronize(c->stream));
    }
    *bytes = n;
    return PCT_OK;
}

extern "C" pct_status pct_set_image(pct_ctx* c, const float* x) {
    if (!c || !x) return pct_fail(PCT_ERR_ARGUMENT, "pct_set_image: null argument");
    PCT_TRY(c->set_device());
    size_t n = sizeof(float) * c->geo.num_voxels;
    PCT_TRY(c->x.alloc(n));
    PCT_TRY(c->x0.alloc(n));
    PCT_CUDA(cudaMemcpyAsync(c->x.p, x, n, cudaMemcpyHostToDevice, c->stream));
    PCT_CUDA(cudaMemcpyAsync(c->x0.p, x, n, cudaMemcpyHostToDevice, c->stream));
    if (c->robust_norm.p)
        PCT_CUDA(cudaMemsetAsync(c->robust_norm.p, 0, sizeof(double) * c->geo.num_voxels, c->stream));
    PCT_CUDA(cudaStreamSynchronize(c->stream));
    return PCT_OK;
}

/* ---- C ABI: stages ------------------------------------------------------------ */
#define STAGE_ENTRY(c)                                                   \
    if (!(c)) return pct_fail(PCT_ERR_ARGUMENT, "null context");         \
    PCT_TRY((c)->set_device())

extern "C" pct_status pct_process_chunk(pct_ctx* c, const float* const data13[13], const float* angle, int64_t n,
                                        int on_dev) {
    STAGE_ENTRY(c);
    if (n < 0 || (n > 0 && (!data13 || !angle))) return pct_fail(PCT_ERR_ARGUMENT, "pct_process_chunk: bad arguments");
    for (int k = 0; n > 0 && k < 13; ++k)
        if (!data13[k]) return pct_fail(PCT_ERR_ARGUMENT, "pct_process_chunk: null array %d", k);
    return pct_stage_process_chunk(c, data13, angle, n, on_dev);
}
extern "C" pct_status pct_hull_detection_finish(pct_ctx* c) { STAGE_ENTRY(c); return pct_stage_hull_finish(c); }
extern "C" pct_status pct_statistical_cuts(pct_ctx* c) {
    STAGE_ENTRY(c);
    if (c->stage == ST_BINNED) PCT_TRY(pct_stage_hull_finish(c));
    return pct_stage_cuts(c);
}
extern "C" pct_status pct_fbp(pct_ctx* c) {
    STAGE_ENTRY(c);
    if (!c->cfg.fbp_on) return PCT_OK;
    return pct_stage_fbp(c);
}
extern "C" pct_status pct_hull_selection(pct_ctx* c) { STAGE_ENTRY(c); return pct_stage_hull_selection(c); }
extern "C" pct_status pct_define_initial_iterate(pct_ctx* c) { STAGE_ENTRY(c); return pct_stage_initial_iterate(c); }
extern "C" pct_status pct_collect_mlp_endpoints(pct_ctx* c) { STAGE_ENTRY(c); return pct_stage_endpoints(c); }
extern "C" pct_status pct_mlp_rows(pct_ctx* c) { STAGE_ENTRY(c); return pct_stage_mlp_rows(c); }
extern "C" pct_status pct_drop(pct_ctx* c, int iterations, pct_drop_stats* stats) {
    STAGE_ENTRY(c);
    return pct_stage_drop(c, iterations, stats);
}
extern "C" pct_status pct_image_reconstruction(pct_ctx* c, pct_drop_stats* stats) {
    STAGE_ENTRY(c);
    PCT_TRY(pct_stage_endpoints(c));
    PCT_TRY(pct_stage_mlp_rows(c));
    return pct_stage_drop(c, c->cfg.iterations, stats);
}

/* ---- sharded DROP ---- */

__global__ void k_shard_keep(int64_t n, int shard, int num_shards, uint8_t* __restrict__ keep) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) keep[i] = (uint8_t)(i % num_shards == shard);
}

extern "C" pct_status pct_set_allreduce(pct_ctx* c, pct_allreduce_fn fn, void* user) {
    if (!c) return pct_fail(PCT_ERR_ARGUMENT, "null context");
    c->allreduce = fn;
    c->allreduce_user = fn ? user : nullptr;
    c->diag_ready = 0; /* the diagonal counts are summed over the ranks when they are built */
    pct_drop_release_graph(c);
    return PCT_OK;
}

extern "C" pct_status pct_select_shard(pct_ctx* c, int shard, int num_shards) {
    STAGE_ENTRY(c);
    if (c->stage != ST_ENDPOINTS) return pct_fail(PCT_ERR_STATE, "pct_select_shard: call it after collect_mlp_endpoints");
    if (c->num_shards != 1) return pct_fail(PCT_ERR_STATE, "pct_select_shard: the histories are already a shard");
    if (num_shards < 1 || shard < 0 || shard >= num_shards)
        return pct_fail(PCT_ERR_ARGUMENT, "pct_select_shard: shard %d of %d", shard, num_shards);
    if (c->cfg.block_size % num_shards != 0)
        return pct_fail(PCT_ERR_ARGUMENT, "pct_select_shard: block size %d is not a multiple of %d shards",
                        c->cfg.block_size, num_shards);
    const int64_t n = c->h.n;
    c->shard_total = n;
    if (num_shards > 1 && n > 0) {
        PCT_TRY(c->tmp_missed.alloc(n));
        uint8_t* keep = c->tmp_missed.as<uint8_t>();
        ++c->launches;
        k_shard_keep<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, shard, num_shards, keep);
        PCT_CUDA(cudaGetLastError());
        int64_t kept = 0;
        PCT_TRY(pct_compact_histories(c, keep, n, &kept));
        c->counts.reconstruction_histories = kept;
    }
    c->shard = shard;
    c->num_shards = num_shards;
    c->cfg.block_size /= num_shards;
    c->diag_ready = 0;
    return PCT_OK;
}

extern "C" pct_status pct_set_block_size(pct_ctx* c, int block_size) {
    if (!c) return pct_fail(PCT_ERR_ARGUMENT, "null context");
    if (block_size < 1) return pct_fail(PCT_ERR_ARGUMENT, "pct_set_block_size: %d", block_size);
    if (c->num_shards != 1) return pct_fail(PCT_ERR_STATE, "pct_set_block_size: the context holds a shard");
    if (block_size != c->cfg.block_size) {
        c->cfg.block_size = block_size;
        c->diag_ready = 0;
        pct_drop_release_graph(c);
        /* sized by the block count: rebuilt for the new size */
        c->block_diag.release();
        c->block_norm.release();
    }
    return PCT_OK;
}

extern "C" pct_status pct_memcpy(void* dst, const void* src, int64_t bytes) {
    if (bytes < 0 || (bytes > 0 && (!dst || !src))) return pct_fail(PCT_ERR_ARGUMENT, "pct_memcpy: bad arguments");
    if (bytes == 0) return PCT_OK;
    PCT_CUDA(cudaMemcpy(dst, src, (size_t)bytes, cudaMemcpyDefault));
    return PCT_OK;
}

extern "C" pct_status pct_reset_iterate(pct_ctx* c) {
    STAGE_ENTRY(c);
    if (!c->x0.p || !c->x.p) return pct_fail(PCT_ERR_STATE, "pct_reset_iterate: no initial iterate");
    PCT_CUDA(cudaMemcpyAsync(c->x.p, c->x0.p, sizeof(float) * c->geo.num_voxels, cudaMemcpyDeviceToDevice, c->stream));
    if (c->robust_norm.p) /* a new reconstruction: the robust variant's running sums restart */
        PCT_CUDA(cudaMemsetAsync(c->robust_norm.p, 0, sizeof(double) * c->geo.num_voxels, c->stream));
    return PCT_OK;
}
