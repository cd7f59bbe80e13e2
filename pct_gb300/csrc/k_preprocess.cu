/*
 * Stages a1-a3 of the path: unit conversion, reconstruction-cylinder
 * intersections and binning, per chunk of histories.
 *
 *   k_preprocess    one thread per history, fused a1+a2+a3 (read_data_chunk_v02
 *                   conversion .cu:1883-1921, recon_volume_intersections_GPU
 *                   .cu:2169-2387, binning_GPU .cu:2507-2578).  SoA in, SoA out;
 *                   the bin counts are integer atomics.  The per-bin sums of
 *                   binning_GPU (.cu:2567-2570) are formed later, in history
 *                   order, with the other statistics (k_binstats.cu).
 * k_preprocess is bound by binary64 arithmetic (a few hundred flops per
 * history on a part with little FP64).
 */
#include "pct_device.cuh"

namespace {

struct In13 {
    const float* p[13];
};

/* calculate_intercepts (.cu:2301-2387); outputs are zero when the line misses. */
__device__ int dev_intercepts(const DevGeom& g, double u, double t, double ut_angle, double* ui, double* ti) {
    int cone = ((ut_angle > PCT_PI_OVER_4) && (ut_angle < PCT_THREE_PI_OVER_4)) ||
               ((ut_angle > PCT_FIVE_PI_OVER_4) && (ut_angle < PCT_SEVEN_PI_OVER_4));
    double tmp;
    *ui = 0.0;
    *ti = 0.0;
    if (cone) {
        tmp = u;
        u = -t;
        t = tmp;
        ut_angle += PCT_PI_OVER_2;
    }
    double m = pct_tan(ut_angle);
    double b_in = t - m * u;
    double a = 1 + m * m;
    double b = 2 * m * b_in;
    double c = b_in * b_in - g.recon_cyl_radius * g.recon_cyl_radius;
    double disc = b * b - (4 * a * c);
    int hit = disc > 0;
    if (hit) {
        double sq = sqrt(disc);
        double u1 = (sq - b) / (2 * a);
        double u2 = (sq + b) / (2 * a);
        double t1 = m * u1 + b_in;
        double t2 = m * u2 - b_in;
        double d1 = (u1 - u) * (u1 - u) + (t1 - t) * (t1 - t);
        double d2 = (u2 + u) * (u2 + u) + (t2 + t) * (t2 + t);
        *ui = u1 * (d1 <= d2) - u2 * (d1 > d2);
        *ti = t1 * (d1 <= d2) - t2 * (d1 > d2);
    }
    if (cone) {
        tmp = *ui;
        *ui = *ti;
        *ti = -tmp;
    }
    return hit;
}

__device__ __forceinline__ int dev_sgn(float z) { return (z >= 0) - (z < 0); }

__global__ void k_trig_table(double2* __restrict__ out, int n, double a, double b) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        double ang = (i * a) * b;
        double s, c;
        pct_sincos_cr(ang, &s, &c); /* the reference's binary64 cos and sin, correctly rounded */
        out[i] = make_double2(c, s);
    }
}

__global__ void __launch_bounds__(256) k_preprocess(DevGeom g, In13 in, const float* __restrict__ proj, int64_t n,
                                                    const double2* __restrict__ trig_gantry,
                                                    const double2* __restrict__ trig_bins, HistView out,
                                                    uint8_t* __restrict__ missed, int* __restrict__ counts) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    /* a1 (.cu:1883-1897, 1921) */
    float t_in_1 = (float)((double)in.p[0][i] * PCT_MM_TO_CM), t_in_2 = (float)((double)in.p[1][i] * PCT_MM_TO_CM);
    float t_out_1 = (float)((double)in.p[2][i] * PCT_MM_TO_CM), t_out_2 = (float)((double)in.p[3][i] * PCT_MM_TO_CM);
    float v_in_1 = (float)((double)in.p[4][i] * PCT_MM_TO_CM), v_in_2 = (float)((double)in.p[5][i] * PCT_MM_TO_CM);
    float v_out_1 = (float)((double)in.p[6][i] * PCT_MM_TO_CM), v_out_2 = (float)((double)in.p[7][i] * PCT_MM_TO_CM);
    float u_in_1 = (float)((double)in.p[8][i] * PCT_MM_TO_CM), u_in_2 = (float)((double)in.p[9][i] * PCT_MM_TO_CM);
    float u_out_1 = (float)((double)in.p[10][i] * PCT_MM_TO_CM), u_out_2 = (float)((double)in.p[11][i] * PCT_MM_TO_CM);
    float w = (float)((double)in.p[12][i] * PCT_MM_TO_CM);
    int ga = ((int)proj[i] + 270) % 360;
    /* a2 (.cu:2198-2298) */
    double rot = ga * PCT_ANGLE_TO_RADIANS;
    double2 cs;
    if (ga >= 0 && ga < 360) {
        cs = trig_gantry[ga];
    } else {
        pct_sincos_cr(rot, &cs.y, &cs.x);
    }
    double cr = cs.x, sr = cs.y;
    double ut_entry = pct_atan2f(t_in_2 - t_in_1, u_in_2 - u_in_1);
    double u_e, t_e, u_x, t_x;
    int entered = dev_intercepts(g, u_in_2, t_in_2, ut_entry, &u_e, &t_e);
    float xy_in = (float)(ut_entry + rot);
    float xe = (float)((cr * u_e) - (sr * t_e));
    float ye = (float)((sr * u_e) + (cr * t_e));
    double ut_exit = pct_atan2f(t_out_2 - t_out_1, u_out_2 - u_out_1);
    int exited = dev_intercepts(g, u_out_1, t_out_1, ut_exit, &u_x, &t_x);
    float xy_out = (float)(ut_exit + rot);
    float xx = (float)((cr * u_x) - (sr * t_x));
    float yx = (float)((sr * u_x) + (cr * t_x));
    double uv_entry_slope = (double)((v_in_2 - v_in_1) / (u_in_2 - u_in_1));
    double uv_exit_slope = (double)((v_out_2 - v_out_1) / (u_out_2 - u_out_1));
    float xz_in = pct_atan2f(v_in_2 - v_in_1, u_in_2 - u_in_1);
    float xz_out = pct_atan2f(v_out_2 - v_out_1, u_out_2 - u_out_1);
    u_e = (cr * xe) + (sr * ye);
    u_x = (cr * xx) + (sr * yx);
    float ze = (float)(v_in_2 + uv_entry_slope * (u_e - u_in_2));
    float zx = (float)(v_out_1 - uv_exit_slope * (u_out_1 - u_x));
    const double H = g.recon_cyl_height;
    if (entered && exited) {
        if ((fabsf(ze) < H * 0.5) && (fabsf(zx) > H * 0.5)) {
            double f = fabs((dev_sgn(zx) * H * 0.5 - ze) / (zx - ze));
            xx = (float)(xe + f * (xx - xe));
            yx = (float)(ye + f * (yx - ye));
            zx = (float)(dev_sgn(zx) * H * 0.5);
        } else if (fabsf(ze) > H * 0.5) {
            entered = 0;
            exited = 0;
        }
        if ((fabsf(ze) > H * 0.5) && (fabsf(zx) < H * 0.5)) {
            double f = fabs((dev_sgn(zx) * H * 0.5 - zx) / (zx - ze));
            xe = (float)(xx + f * (xx - xe));
            ye = (float)(yx + f * (yx - ye));
            ze = (float)(dev_sgn(ze) * H * 0.5);
        }
        if ((fabsf(t_out_1 - t_in_2) > 5) || (fabsf(v_out_1 - v_in_2) > 5)) {
            entered = 0;
            exited = 0;
        }
    }
    uint8_t m = !entered || !exited;
    /* a3 (.cu:2529-2550) */
    double x_mid = (xe + xx) / 2;
    double y_mid = (ye + yx) / 2;
    double z_mid = (ze + zx) / 2;
    double path_angle = pct_atan2f(yx - ye, xx - xe);
    if (path_angle < 0) path_angle += 2 * PCT_PI;
    int angle_bin = pct_d2i((path_angle * PCT_RADIANS_TO_ANGLE / g.angular_bin_size) + 0.5) % g.angular_bins;
    double2 ab;
    if (angle_bin >= 0 && angle_bin < g.angular_bins) {
        ab = trig_bins[angle_bin];
    } else {
        double angle = angle_bin * g.angular_bin_size * PCT_ANGLE_TO_RADIANS;
        pct_sincos_cr(angle, &ab.y, &ab.x);
    }
    double t = y_mid * ab.x - x_mid * ab.y;
    int t_bin = pct_d2i((t / g.t_bin_size) + (g.t_bins / 2));
    int v_bin = pct_d2i((z_mid / g.v_bin_size) + (g.v_bins / 2));
    int valid = (t_bin >= 0) && (v_bin >= 0) && (t_bin < g.t_bins) && (v_bin < g.v_bins);
    int bin = valid ? t_bin + angle_bin * g.t_bins + v_bin * g.t_bins * g.angular_bins : 0;
    /* a negative angle bin (NaN path angle) would index outside the bins */
    if (bin < 0 || bin >= g.num_bins) {
        valid = 0;
        bin = 0;
    }
    out.x_entry[i] = xe; out.y_entry[i] = ye; out.z_entry[i] = ze;
    out.x_exit[i] = xx; out.y_exit[i] = yx; out.z_exit[i] = zx;
    out.xy_entry_angle[i] = xy_in; out.xz_entry_angle[i] = xz_in;
    out.xy_exit_angle[i] = xy_out; out.xz_exit_angle[i] = xz_out;
    out.wepl[i] = w;
    out.bin_num[i] = bin;
    out.bin_valid[i] = (uint8_t)valid;
    out.failed[i] = 0;
    out.first_voxel[i] = 0;
    missed[i] = m;
    /* binning counts (.cu:2551-2567); the sums follow in history order */
    if (!m && valid) atomicAdd(counts + bin, 1);
}

}  // namespace

pct_status pct_hull_images_ready(pct_ctx* c);                                                        /* k_hull.cu */
pct_status pct_hull_walk_range(pct_ctx* c, HistView h, int64_t n, const uint8_t* missed, cudaStream_t st); /* k_hull.cu */

namespace {
__global__ void k_invert(const uint8_t* __restrict__ a, uint8_t* __restrict__ b, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = !a[i];
}
}  // namespace

static pct_status pct_invert_flags(pct_ctx* c, const uint8_t* a, uint8_t* b, int64_t n) {
    ++c->launches;
    k_invert<<<pct_grid_for(n, 256), 256, 0, c->stream>>>(a, b, n);
    PCT_CUDA(cudaGetLastError());
    return PCT_OK;
}

static pct_status ensure_tables(pct_ctx* c) {
    if (c->trig_gantry.p) return PCT_OK;
    PCT_TRY(c->trig_gantry.alloc(sizeof(double2) * 360));
    PCT_TRY(c->trig_bins.alloc(sizeof(double2) * c->geo.angular_bins));
    ++c->launches;
    k_trig_table<<<2, 256, 0, c->stream>>>(c->trig_gantry.as<double2>(), 360, 1.0, PCT_ANGLE_TO_RADIANS);
    ++c->launches;
    k_trig_table<<<pct_grid_for(c->geo.angular_bins, 256), 256, 0, c->stream>>>(
        c->trig_bins.as<double2>(), c->geo.angular_bins, c->cfg.angular_bin_size, PCT_ANGLE_TO_RADIANS);
    PCT_CUDA(cudaGetLastError());
    return PCT_OK;
}

pct_status pct_ensure_bins(pct_ctx* c) {
    if (c->bin_counts.p) return PCT_OK;
    size_t nb = (size_t)c->geo.num_bins;
    PCT_TRY(c->bin_counts.alloc(nb * 4));
    PCT_TRY(c->bin_counts_post.alloc(nb * 4));
    DevBuf* f[] = {&c->mean_wepl, &c->mean_ut, &c->mean_uv, &c->sd_wepl, &c->sd_ut, &c->sd_uv, &c->sinogram,
                   &c->sinogram_filtered};
    for (DevBuf* b : f) PCT_TRY(b->alloc(nb * 4));
    PCT_CUDA(cudaMemsetAsync(c->bin_counts.p, 0, nb * 4, c->stream));
    return PCT_OK;
}

constexpr int PIPE_PARTS = 4;

pct_status pct_stage_process_chunk(pct_ctx* c, const float* const data13[13], const float* angle, int64_t n,
                                   int on_dev) {
    if (c->stage > ST_BINNED) return pct_fail(PCT_ERR_STATE, "process_chunk after hull_detection_finish");
    if (n == 0) {
        c->stage = ST_BINNED;
        return PCT_OK;
    }
    PCT_TRY(ensure_tables(c));
    PCT_TRY(pct_ensure_bins(c));
    PCT_TRY(pct_hull_images_ready(c));
    In13 in;
    const float* d_angle = angle;
    if (!on_dev) {
        for (int k = 0; k < 13; ++k) {
            PCT_TRY(c->in13[k].alloc(sizeof(float) * n));
            in.p[k] = c->in13[k].as<float>();
        }
        PCT_TRY(c->in_angle.alloc(sizeof(float) * n));
        d_angle = c->in_angle.as<float>();
    } else {
        for (int k = 0; k < 13; ++k) in.p[k] = data13[k];
    }
    PCT_TRY(c->h2.reserve(n, c->stream));
    PCT_TRY(c->tmp_missed.alloc(n * 2));
    uint8_t* missed = c->tmp_missed.as<uint8_t>();
    uint8_t* keep = missed + n;
    const HistView stage = c->view(c->h2);
    /* The chunk in PIPE_PARTS parts: the upload and the intersections/binning
     * of a part on the context stream, its hull walks (hull_detection, .cu:100)
     * on the second stream once the part is preprocessed, so that the binary32
     * walks of one part overlap the binary64 preprocessing of the next.  The
     * images and the bin counts are integer counts: the order of the parts
     * does not change them. */
    const int parts = n >= ((int64_t)1 << 22) ? PIPE_PARTS : 1;
    const int64_t part = (n + parts - 1) / parts;
    if (c->cfg.walk_exact == 0 && part <= (int64_t)0xffffffffu)
        PCT_TRY(c->walk_order.alloc(sizeof(uint32_t) * 2 * (size_t)part));
    cudaEvent_t ev[PIPE_PARTS + 1];
    for (int k = 0; k <= parts; ++k) PCT_CUDA(cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming));
    pct_status st = PCT_OK;
    for (int k = 0; k < parts && st == PCT_OK; ++k) {
        const int64_t a = k * part, m = (a + part < n ? a + part : n) - a;
        if (m <= 0) break;
        In13 ink;
        for (int j = 0; j < 13; ++j) ink.p[j] = in.p[j] + a;
        if (!on_dev) {
            for (int j = 0; j < 13 && st == PCT_OK; ++j)
                if (cudaMemcpyAsync(c->in13[j].as<float>() + a, data13[j] + a, sizeof(float) * m,
                                    cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
                    st = pct_fail(PCT_ERR_CUDA, "process_chunk: upload");
            if (st == PCT_OK && cudaMemcpyAsync(c->in_angle.as<float>() + a, angle + a, sizeof(float) * m,
                                                cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
                st = pct_fail(PCT_ERR_CUDA, "process_chunk: upload");
        }
        if (st != PCT_OK) break;
        ++c->launches;
        k_preprocess<<<pct_grid_for(m, 256), 256, 0, c->stream>>>(
            c->dg, ink, d_angle + a, m, c->trig_gantry.as<double2>(), c->trig_bins.as<double2>(),
            hv_offset(stage, a), missed + a, c->bin_counts.as<int>());
        if (cudaGetLastError() != cudaSuccess || cudaEventRecord(ev[k], c->stream) != cudaSuccess ||
            cudaStreamWaitEvent(c->stream2, ev[k], 0) != cudaSuccess) {
            st = pct_fail(PCT_ERR_CUDA, "process_chunk: preprocessing launch");
            break;
        }
        st = pct_hull_walk_range(c, hv_offset(stage, a), m, missed + a, c->stream2);
    }
    /* the context stream waits for the walks before the compaction */
    if (cudaEventRecord(ev[parts], c->stream2) != cudaSuccess ||
        cudaStreamWaitEvent(c->stream, ev[parts], 0) != cudaSuccess)
        st = st == PCT_OK ? pct_fail(PCT_ERR_CUDA, "process_chunk: stream join") : st;
    for (int k = 0; k <= parts; ++k) cudaEventDestroy(ev[k]);
    PCT_TRY(st);
    /* keep = !missed (bin_num >= 0 always holds, .cu:2446) */
    PCT_TRY(pct_invert_flags(c, missed, keep, n));
    int64_t kept = 0;
    PCT_TRY(c->h.reserve(c->h.n + n, c->stream));
    PCT_TRY(pct_compact(c, c->h2, 0, n, keep, c->h, c->h.n, &kept));
    c->h.n += kept;
    c->counts.total_histories += n;
    c->counts.recon_vol_histories += kept;
    c->stage = ST_BINNED;
    return PCT_OK;
}
