/*
 * Stages a10-a12: filtered backprojection, FBP hull, initial iterate.
 *
 *   k_filter_taps / k_filter_scale   the filter value per bin separation and the
 *                  fan-beam weight per (v, t) bin of filter_GPU (.cu:3041-3065),
 *                  precomputed once with the same expressions
 *   k_filter       filter_GPU (.cu:3036-3069): one CTA per (v, angle) sinogram
 *                  row, the row staged in shared memory, one thread per output
 *                  t bin accumulating in binary32 in the reference's order
 *   k_backproject  backprojection_GPU (.cu:3155-3230): one thread per voxel
 *                  column and 16 slices, binary32 accumulation over angle bins
 *                  in order per voxel, per-angle cos/sin table in shared
 *                  memory, divisions from one reciprocal per column and angle
 *                  (pct_div_rn); the sinogram (NUM_BINS floats) stays L2-resident
 *   k_fbp_hull     FBP_image_2_hull_GPU (.cu:3250)
 *   k_initial      define_initial_iterate (.cu:7191-7205)
 * Bound by binary64 throughput (each term of the reference is binary64).
 */
#include "pct_device.cuh"

namespace {

__global__ void k_filter_taps(int T, int filter, double tb, double* __restrict__ taps) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= 2 * T - 1) return;
    int sep = k - (T - 1);
    double f;
    if (filter == PCT_RAM_LAK) {
        double tau = (double)(2 / sqrtf(2.0f)) * tb; /* RAM_LAK_TAU, pCT_data.h:247 */
        if (sep == 0) f = 1.0 / (4.0 * (tau * tau));
        else if (sep % 2 == 0) f = 0;
        else {
            double q = tau * PCT_PI * sep;
            f = -1.0 / (q * q);
        }
    } else if (filter == PCT_SHEPP_LOGAN) {
        f = 1 / ((tb * PCT_PI * tb * PCT_PI) * (1.0 - (2 * sep * 2 * sep)));
    } else {
        /* FILTER NONE leaves the reference's value uninitialised; pass-through here */
        f = sep == 0 ? 1.0 / tb : 0.0;
    }
    taps[k] = f;
}

__global__ void k_filter_scale(int T, int V, double tb, double vb, double sr, double* __restrict__ scale) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= T * V) return;
    int vbin = k / T, tr = k % T;
    double v = (vbin - V / 2) * vb + vb / 2.0;
    double t = (tr - T / 2) * tb + tb / 2.0;
    scale[k] = sr / sqrt(sr * sr + t * t + v * v);
}

__global__ void k_filter(int T, int A, double tb, const float* __restrict__ sino, const double* __restrict__ taps,
                         const double* __restrict__ scale, float* __restrict__ out) {
    extern __shared__ unsigned char smem[];
    double* sscale = (double*)smem;
    double* sw = sscale + T; /* tb * s[tr]: the first product of every term, once per row */
    int vb = blockIdx.x, ab = blockIdx.y;
    int64_t strip = (int64_t)vb * A * T + (int64_t)ab * T;
    for (int k = threadIdx.x; k < T; k += blockDim.x) {
        sw[k] = tb * sino[strip + k];
        sscale[k] = scale[(int64_t)vb * T + k];
    }
    __syncthreads();
    for (int tb_i = threadIdx.x; tb_i < T; tb_i += blockDim.x) {
        float acc = 0.0f;
        const double* tap = taps + (T - 1) + tb_i; /* tap[-tr] = f(sep = tb_i - tr) */
        /* ((tb s) tap) scale, left to right as the reference's product */
        for (int tr = 0; tr < T; ++tr) acc = (float)(acc + sw[tr] * tap[-tr] * sscale[tr]);
        out[strip + tb_i] = acc;
    }
}

/* One thread per voxel column (x, y) and group of BP_SLICES slices: the terms
 * of an angle that do not depend on z (u, t, the t bin, eta and the fan-beam
 * scale) are formed once per column and angle, the z terms per slice; each
 * slice keeps its own binary32 accumulator over the angle bins in order.
 * Every expression is the one of backprojection_GPU, its divisions by SR + u
 * and by the bin sizes formed by pct_div_rn from one reciprocal per column
 * and angle (the same quotients: checked against IEEE division on every
 * quotient of the parity and benchmark grids by tests/test_exact_arith.py),
 * so the image is the same bit for bit. */
constexpr int BP_SLICES = 16;
__global__ void __launch_bounds__(128) k_backproject(DevGeom g, const float* __restrict__ sino,
                                                     const double2* __restrict__ trig, float* __restrict__ image) {
    extern __shared__ double2 strig[];
    for (int k = threadIdx.x; k < g.angular_bins; k += blockDim.x) strig[k] = trig[k];
    __syncthreads();
    const int CR = g.columns * g.rows;
    const int cr = blockIdx.x * blockDim.x + threadIdx.x;
    if (cr >= CR) return;
    const int s_first = blockIdx.y * BP_SLICES;
    const int ns = g.slices - s_first < BP_SLICES ? g.slices - s_first : BP_SLICES;
    const int column = cr % g.columns, row = cr / g.columns;
    const double R = g.recon_cyl_radius, SR = g.source_radius;
    const double delta = g.gantry_angle_interval * PCT_ANGLE_TO_RADIANS;
    const int T = g.t_bins, ATB = g.angular_bins * g.t_bins, NB = g.num_bins;
    const double tbs = g.t_bin_size, vbs = g.v_bin_size, r_tbs = 1.0 / tbs, r_vbs = 1.0 / vbs;
    const double x = -R + (column + 0.5) * g.voxel_width;
    const double y = R - (row + 0.5) * g.voxel_height;
    if ((x * x + y * y) > (R * R)) {
        for (int k = 0; k < ns; ++k) image[(size_t)(s_first + k) * CR + cr] = (float)PCT_RSP_AIR;
        return;
    }
    double z[BP_SLICES];
    float acc[BP_SLICES];
#pragma unroll
    for (int k = 0; k < BP_SLICES; ++k) {
        z[k] = -g.recon_cyl_height / 2.0 + (s_first + k + 0.5) * g.slice_thickness;
        acc[k] = 0.0f;
    }
    for (int ab = 0; ab < g.angular_bins; ++ab) {
        const double ca = strig[ab].x, sa = strig[ab].y;
        const double u = x * ca + y * sa;
        const double t = -x * sa + y * ca;
        const double d = SR + u, rd = 1.0 / d;
        const double dnt = pct_div_rn(t - u * pct_div_rn(t, d, rd), tbs, r_tbs) + T / 2.0;
        int t_bin = pct_d2i(dnt);
        if (t_bin > dnt) t_bin -= 1;
        const double eta = dnt - t_bin;
        const double sf = pct_div_rn(SR, d, rd);
        const double scale = sf * sf;
        const int tbin_ab = t_bin + ab * T;
#pragma unroll
        for (int k = 0; k < BP_SLICES; ++k) {
            if (k >= ns) break;
            const double v = z[k];
            const double dnv = pct_div_rn(v - u * pct_div_rn(v, d, rd), vbs, r_vbs) + g.v_bins / 2.0;
            int v_bin = pct_d2i(dnv);
            if (v_bin > dnv) v_bin -= 1;
            const double eps = dnv - v_bin;
            const int bin = tbin_ab + v_bin * ATB;
            /* bins outside the sinogram read as 0 (the reference reads out of bounds there) */
            const float s0 = (bin >= 0 && bin < NB) ? sino[bin] : 0.0f;
            const float s1 = (bin + 1 >= 0 && bin + 1 < NB) ? sino[bin + 1] : 0.0f;
            if (v_bin == g.v_bins - 1 || (bin < 0)) {
                acc[k] = (float)(acc[k] + scale * (((1 - eta) * s0) + (eta * s1)));
            } else {
                const float s2 = (bin + ATB >= 0 && bin + ATB < NB) ? sino[bin + ATB] : 0.0f;
                const float s3 = (bin + ATB + 1 >= 0 && bin + ATB + 1 < NB) ? sino[bin + ATB + 1] : 0.0f;
                acc[k] = (float)(acc[k] + scale * ((1 - eta) * (1 - eps) * s0 + eta * (1 - eps) * s1 +
                                                   (1 - eta) * eps * s2 + eta * eps * s3));
            }
        }
    }
#pragma unroll
    for (int k = 0; k < BP_SLICES; ++k)
        if (k < ns) image[(size_t)(s_first + k) * CR + cr] = (float)(acc[k] * delta);
}

__global__ void k_trig_bp(int n, double delta, double2* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        double s, c;
        pct_sincos_cr(i * delta, &s, &c); /* the reference's binary64 cos and sin, correctly rounded */
        out[i] = make_double2(c, s);
    }
}

__global__ void k_fbp_hull(DevGeom g, double thr, const float* __restrict__ image, uint8_t* __restrict__ hull) {
    int voxel = blockIdx.x * blockDim.x + threadIdx.x;
    if (voxel >= g.num_voxels) return;
    int column = voxel % g.columns, row = (voxel / g.columns) % g.rows;
    const double R = g.recon_cyl_radius;
    double x = -R + (column + 0.5) * g.voxel_width;
    double y = R - (row + 0.5) * g.voxel_height;
    double d2 = x * x + y * y;
    hull[voxel] = (image[voxel] > thr && d2 < R * R) ? 1 : 0;
}

/* X_HULL: hull as 0/1; FBP_IMAGE: FBP; HYBRID: FBP * hull (std::multiplies<float>, .cu:7199); ZEROS */
__global__ void k_initial(int n, int mode, const float* __restrict__ fbp, const uint8_t* __restrict__ hull,
                          float* __restrict__ x0, float* __restrict__ x) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    float r;
    if (mode == PCT_X_HULL) r = (float)hull[v];
    else if (mode == PCT_FBP_IMAGE) r = fbp[v];
    else if (mode == PCT_HYBRID) r = fbp[v] * (float)hull[v];
    else r = 0.0f;
    x0[v] = r;
    x[v] = r;
}

}  // namespace

pct_status pct_stage_fbp(pct_ctx* c) {
    if (c->stage != ST_CUT) return pct_fail(PCT_ERR_STATE, "FBP needs statistical_cuts first");
    const int T = c->geo.t_bins, A = c->geo.angular_bins, Vb = c->geo.v_bins, V = c->geo.num_voxels;
    PCT_TRY(c->filter_taps.alloc(sizeof(double) * (2 * T - 1)));
    PCT_TRY(c->filter_scale.alloc(sizeof(double) * T * Vb));
    ++c->launches;
    k_filter_taps<<<pct_grid_for(2 * T - 1, 256), 256, 0, c->stream>>>(T, c->cfg.fbp_filter, c->cfg.t_bin_size,
                                                                       c->filter_taps.as<double>());
    ++c->launches;
    k_filter_scale<<<pct_grid_for((int64_t)T * Vb, 256), 256, 0, c->stream>>>(
        T, Vb, c->cfg.t_bin_size, c->cfg.v_bin_size, c->cfg.source_radius, c->filter_scale.as<double>());
    size_t smem = 2 * sizeof(double) * T;
    if (smem > 48 * 1024) PCT_CUDA(cudaFuncSetAttribute(k_filter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int threads = T < 512 ? ((T + 31) / 32) * 32 : 512;
    ++c->launches;
    k_filter<<<dim3(Vb, A), threads, smem, c->stream>>>(T, A, c->cfg.t_bin_size, c->sinogram.as<float>(),
                                                        c->filter_taps.as<double>(), c->filter_scale.as<double>(),
                                                        c->sinogram_filtered.as<float>());
    DevBuf trig;
    PCT_TRY(trig.alloc(sizeof(double2) * A));
    ++c->launches;
    k_trig_bp<<<pct_grid_for(A, 256), 256, 0, c->stream>>>(A, c->cfg.gantry_angle_interval * PCT_ANGLE_TO_RADIANS,
                                                           trig.as<double2>());
    PCT_TRY(c->fbp_image.alloc(sizeof(float) * V));
    PCT_TRY(c->fbp_hull.alloc(V));
    size_t bsm = sizeof(double2) * A;
    if (bsm > 48 * 1024) PCT_CUDA(cudaFuncSetAttribute(k_backproject, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bsm));
    ++c->launches;
    const dim3 bp_grid(pct_grid_for((int64_t)c->geo.columns * c->geo.rows, 128),
                       (unsigned)((c->geo.slices + BP_SLICES - 1) / BP_SLICES));
    k_backproject<<<bp_grid, 128, bsm, c->stream>>>(c->dg, c->sinogram_filtered.as<float>(), trig.as<double2>(),
                                                    c->fbp_image.as<float>());
    ++c->launches;
    k_fbp_hull<<<pct_grid_for(V, 256), 256, 0, c->stream>>>(c->dg, c->cfg.fbp_threshold, c->fbp_image.as<float>(),
                                                            c->fbp_hull.as<uint8_t>());
    cudaError_t e = cudaStreamSynchronize(c->stream);
    trig.release();
    if (e != cudaSuccess) return pct_fail(PCT_ERR_CUDA, "FBP: %s", cudaGetErrorString(e));
    PCT_CUDA(cudaGetLastError());
    c->stage = ST_FBP;
    return PCT_OK;
}

pct_status pct_stage_initial_iterate(pct_ctx* c) {
    if (c->stage != ST_HULL_SELECTED) return pct_fail(PCT_ERR_STATE, "define_initial_iterate needs hull_selection");
    const int V = c->geo.num_voxels;
    if (c->cfg.x_k0 == PCT_IMPORT) {
        if (!c->x0.p) return pct_fail(PCT_ERR_STATE, "X_K0 = IMPORT needs pct_set_image first");
        c->stage = ST_X0;
        return PCT_OK;
    }
    if ((c->cfg.x_k0 == PCT_FBP_IMAGE || c->cfg.x_k0 == PCT_HYBRID) && !c->fbp_image.p)
        return pct_fail(PCT_ERR_STATE, "initial iterate needs the FBP image");
    PCT_TRY(c->x0.alloc(sizeof(float) * V));
    PCT_TRY(c->x.alloc(sizeof(float) * V));
    ++c->launches;
    k_initial<<<pct_grid_for(V, 256), 256, 0, c->stream>>>(V, c->cfg.x_k0, c->fbp_image.as<float>(),
                                                           c->x_hull_filtered.as<uint8_t>(), c->x0.as<float>(),
                                                           c->x.as<float>());
    PCT_CUDA(cudaGetLastError());
    c->stage = ST_X0;
    return PCT_OK;
}
