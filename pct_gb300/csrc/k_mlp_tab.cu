/*
 * Tabulated MLP rows (config mlp_tabulated = 1): the reference's lookup-table
 * variant of the most likely path, find_MLP_path_GPU_tabulated
 * (src/pCT_Reconstruction_Data_Segments.cu:5502-5660), with its tables
 * generate_trig_tables (.cu:4786-4815), generate_scattering_coefficient_table
 * (.cu:4830-4861) and generate_polynomial_tables (.cu:4869-4911), at the
 * reference's table resolutions (pCT_data.h:405-417).  Everything is binary64
 * in the reference's operation order (the tables from the deterministic
 * functions of pct_math.h), so the rows match the oracle's restatement bit
 * for bit.  The tables quantise the entry angle to 0.001 degree and the
 * depths to 0.5 um, so the rows differ from the analytic MLP at a small
 * fraction of samples near voxel faces; this is the reference's alternative
 * path, not a faster one on this part (every sample is binary64).
 *
 *   k_tab_trig / k_tab_depth   the tables (sin, cos; scattering coefficient and
 *                              the five moment polynomials per depth)
 *   k_tab_bound                a row bound per history: (xy distance / step) + 3
 *   k_mlp_tab                  one thread per history, the tabulated loop
 */
#include "pct_device.cuh"

namespace {

/* pCT_data.h:405-417 */
#define TAB_TRIG_MIN (-2 * PCT_PI)
#define TAB_TRIG_STEP (0.001 * PCT_ANGLE_TO_RADIANS)
#define TAB_TRIG_ELEMENTS ((int)((4 * PCT_PI - -2 * PCT_PI) / TAB_TRIG_STEP + 0.5))
#define TAB_DEPTH_STEP 0.00005
#define TAB_DEPTH_ELEMENTS ((int)(40.0 / TAB_DEPTH_STEP + 0.5))

/* The scattering polynomial pieces as the reference's macros expand
 * (pCT_data.h:306-348): a leading A_k_OVER_n is (m_k * p_k) / n, an inner
 * "u * A_k_OVER_n" is ((u * m_k) * p_k) / n. */
#define TAL(k, n) ((PCT_A##k##_M * PCT_A##k##_P) / (n))
#define TAU(u, k, n) ((((u) * PCT_A##k##_M) * PCT_A##k##_P) / (n))
#define TA0 (PCT_A0_M * PCT_A0_P)

enum { TP_1_2 = 0, TP_2_3, TP_3_4, TP_2_6, TP_3_12, TP_SCATTER, TP_COUNT };

__global__ void k_tab_trig(int n, double* __restrict__ sin_t, double* __restrict__ cos_t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    const double val = TAB_TRIG_MIN + i * TAB_TRIG_STEP;
    pct_sincos_cr(val, sin_t + i, cos_t + i); /* sin(val), cos(val) of .cu:4806-4807, correctly rounded */
}

/* depth[k * TP_COUNT + j]: the six depth tables interleaved per depth step */
__global__ void k_tab_depth(int n, double* __restrict__ depth) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > n) return;
    const double du = k * TAB_DEPTH_STEP;
    double* d = depth + (size_t)k * TP_COUNT;
    d[TP_1_2] = du * (TA0 + du * (TAL(1, 2) + du * (TAL(2, 3) + du * (TAL(3, 4) + du * (TAL(4, 5) + TAU(du, 5, 6))))));
    d[TP_2_3] = (du * du) * (TAL(0, 2) + du * (TAL(1, 3) + du * (TAL(2, 4) + du * (TAL(3, 5) + du * (TAL(4, 6) + TAU(du, 5, 7))))));
    d[TP_3_4] = pct_cube(du) * (TAL(0, 3) + du * (TAL(1, 4) + du * (TAL(2, 5) + du * (TAL(3, 6) + du * (TAL(4, 7) + TAU(du, 5, 8))))));
    d[TP_2_6] = (du * du) * (TAL(0, 2) + du * (TAL(1, 6) + du * (TAL(2, 12) + du * (TAL(3, 20) + du * (TAL(4, 30) + TAU(du, 5, 42))))));
    d[TP_3_12] = pct_cube(du) * (TAL(0, 3) + du * (TAL(1, 12) + du * (TAL(2, 30) + du * (TAL(3, 60) + du * (TAL(4, 105) + TAU(du, 5, 168))))));
    /* pow(E_0 (1 + 0.038 log(depth / X0)), 2.0) / X0; depth 0 is never read */
    const double e = PCT_E_0 * (1 + 0.038 * pct_log(du / PCT_X_0));
    d[TP_SCATTER] = k > 0 ? (e * e) / PCT_X_0 : 0.0;
}

/* More entries than the loop can append: u_2 <= the xy distance of the endpoints. */
__global__ void k_tab_bound(DevGeom g, int64_t n, HistView h, int64_t* __restrict__ bound) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double dx = (double)h.x_exit[i] - (double)h.x_entry[i], dy = (double)h.y_exit[i] - (double)h.y_entry[i];
    const double d = sqrt(dx * dx + dy * dy) / g.mlp_u_step;
    bound[i] = d < 1e9 ? (int64_t)d + 3 : 3; /* non-finite endpoints: the loop does not run */
}

__device__ __forceinline__ unsigned tab_trig_index(double angle) {
    return (unsigned)((angle - TAB_TRIG_MIN) / TAB_TRIG_STEP + 0.5);
}

/* find_MLP_path_GPU_tabulated (.cu:5502-5660): the row of one history. */
__global__ void __launch_bounds__(128) k_mlp_tab(DevGeom g, int64_t n, HistView h, const double* __restrict__ sin_t,
                                                 const double* __restrict__ cos_t, int trig_n,
                                                 const double* __restrict__ dt, int depth_n,
                                                 const int64_t* __restrict__ row_start,
                                                 const int64_t* __restrict__ bound, uint32_t* __restrict__ rows,
                                                 int* __restrict__ row_len, unsigned long long* __restrict__ flags) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double STEP = g.mlp_u_step;
    const double x_in = h.x_entry[i], y_in = h.y_entry[i], z_in = h.z_entry[i];
    const double x_out = h.x_exit[i], y_out = h.y_exit[i], z_out = h.z_exit[i];
    double xy_entry = h.xy_entry_angle[i], xz_entry = h.xz_entry_angle[i];
    double xy_exit = h.xy_exit_angle[i], xz_exit = h.xz_exit_angle[i];
    uint32_t* row = rows + row_start[i];
    const int64_t cap = bound[i];
    int len = 0;
    uint32_t prev = h.first_voxel[i];
    row[len++] = dev_to_brick(g, prev);
    unsigned ti = tab_trig_index(xy_entry);
    if (ti > (unsigned)trig_n) { /* entry angle outside the table */
        dev_flag(flags, ERR_ROW_OVERFLOW);
        row_len[i] = len;
        return;
    }
    double sin_term = sin_t[ti], cos_term = cos_t[ti];
    double u_in = cos_term * x_in + sin_term * y_in;
    double u_out = cos_term * x_out + sin_term * y_out;
    if (u_in > u_out) {
        xy_entry += PCT_PI;
        xy_exit += PCT_PI;
        ti = tab_trig_index(xy_entry);
        if (ti > (unsigned)trig_n) {
            dev_flag(flags, ERR_ROW_OVERFLOW);
            row_len[i] = len;
            return;
        }
        sin_term = sin_t[ti];
        cos_term = cos_t[ti];
        u_in = cos_term * x_in + sin_term * y_in;
        u_out = cos_term * x_out + sin_term * y_out;
    }
    const double t_in = cos_term * y_in - sin_term * x_in;
    const double t_out = cos_term * y_out - sin_term * x_out;
    const double T2_1 = xy_exit - xy_entry, V2_1 = xz_exit - xz_entry;
    const double u_2 = fabs(u_out - u_in);
    double depth_2_go = u_2 - STEP;
    double u_shifted = u_in;
    const unsigned step_i = (unsigned)(STEP / TAB_DEPTH_STEP + 0.5);
    unsigned s1 = step_i;
    unsigned s2 = (unsigned)(depth_2_go / TAB_DEPTH_STEP + 0.5);
    unsigned p1 = step_i;
    const unsigned p2 = (unsigned)(u_2 / TAB_DEPTH_STEP + 0.5);
    if (!(u_2 < 40.0) || p2 > (unsigned)depth_n) { /* depth outside the tables */
        dev_flag(flags, ERR_ROW_OVERFLOW);
        row_len[i] = len;
        return;
    }
    const double u2_3_12 = dt[(size_t)p2 * TP_COUNT + TP_3_12];
    const double u2_2_6 = dt[(size_t)p2 * TP_COUNT + TP_2_6];
    const double u2_1_2 = dt[(size_t)p2 * TP_COUNT + TP_1_2];
    const int nv = g.num_voxels;
    int outside = prev >= (uint32_t)nv;
    while (depth_2_go > STEP) {
        const double* d1 = dt + (size_t)p1 * TP_COUNT;
        const double u1_1_2 = d1[TP_1_2], u1_2_3 = d1[TP_2_3];
        const double sigma_t1 = d1[TP_3_12], sigma_t1_theta1 = d1[TP_2_6], sigma_theta1 = u1_1_2;
        const double sigma_t2 = u2_3_12 - (u_2 * u_2) * u1_1_2 + 2 * u_2 * u1_2_3 - d1[TP_3_4];
        const double sigma_t2_theta2 = u2_2_6 - u_2 * u1_1_2 + u1_2_3;
        const double sigma_theta2 = u2_1_2 - u1_1_2;
        const double det1 = dt[(size_t)s1 * TP_COUNT + TP_SCATTER] *
                            (sigma_t1 * sigma_theta1 - (sigma_t1_theta1 * sigma_t1_theta1));
        const double S1I0 = sigma_theta1 / det1, S1I1 = sigma_t1_theta1 / det1, S1I2 = sigma_t1 / det1;
        const double det2 = dt[(size_t)s2 * TP_COUNT + TP_SCATTER] *
                            (sigma_t2 * sigma_theta2 - (sigma_t2_theta2 * sigma_t2_theta2));
        const double S2I0 = sigma_theta2 / det2, S2I1 = sigma_t2_theta2 / det2, S2I2 = sigma_t2 / det2;
        const double ftc = S2I0 * depth_2_go - S2I1;
        const double ft0 = S1I0 + S2I0;
        const double ft1 = ftc - S1I1;
        const double ft2 = depth_2_go * S2I0 - S1I1 - S2I1;
        const double ft3 = S1I2 + S2I2 + depth_2_go * (ftc - S2I1);
        const double detf = ft0 * ft3 - ft1 * ft2;
        (void)ft2;
        double sc = S2I0 * t_out - S2I1 * T2_1;
        double s0 = S1I0 * t_in + sc;
        double s1v = depth_2_go * sc + S2I2 * T2_1 - S2I1 * t_out - S1I1 * t_in;
        const double t_1 = (ft3 * s0 - ft1 * s1v) / detf;
        sc = S2I0 * z_out - S2I1 * V2_1;
        s0 = S1I0 * z_in + sc;
        s1v = depth_2_go * sc + S2I2 * V2_1 - S2I1 * z_out - S1I1 * z_in;
        const double v_1 = (ft3 * s0 - ft1 * s1v) / detf;
        u_shifted += STEP;
        const double x_1 = cos_term * u_shifted - sin_term * t_1;
        const double y_1 = sin_term * u_shifted + cos_term * t_1;
        const int vx = dev_calculate_voxel(g.x_zero, x_1, g.voxel_width);
        const int vy = dev_calculate_voxel(g.y_zero, y_1, g.voxel_height);
        const int vz = dev_calculate_voxel(g.z_zero, v_1, g.voxel_thickness);
        const uint32_t voxel = (uint32_t)(vx + vy * g.columns + vz * g.columns * g.rows);
        if (voxel != prev) {
            if (len >= cap) { /* cannot happen: the bound exceeds the step count */
                dev_flag(flags, ERR_ROW_OVERFLOW);
                break;
            }
            row[len++] = dev_to_brick(g, voxel);
            prev = voxel;
            outside += voxel >= (uint32_t)nv;
        }
        depth_2_go -= STEP;
        s1 += step_i;
        s2 -= step_i;
        p1 += step_i;
    }
    row_len[i] = len;
    if (outside) atomicAdd(flags + ERR_ROWS_OUTSIDE, (unsigned long long)outside);
}

}  // namespace

pct_status pct_stage_row_norms(pct_ctx* c);

/* MLP rows of every reconstruction history from the reference's tables. */
pct_status pct_stage_mlp_rows_tab(pct_ctx* c) {
    const int64_t n = c->h.n;
    PCT_TRY(c->row_offsets.alloc(sizeof(int64_t) * (n + 1)));
    PCT_TRY(c->row_len.alloc(sizeof(int) * (n > 0 ? n : 1)));
    PCT_TRY(c->chord.alloc(sizeof(float) * (n > 0 ? n : 1)));
    PCT_TRY(c->row_scale.alloc(sizeof(float) * (n > 0 ? n : 1)));
    const int trig_n = TAB_TRIG_ELEMENTS, depth_n = TAB_DEPTH_ELEMENTS;
    if (!c->mlp_tab_trig.p) {
        PCT_TRY(c->mlp_tab_trig.alloc(sizeof(double) * 2 * ((size_t)trig_n + 1)));
        PCT_TRY(c->mlp_tab_depth.alloc(sizeof(double) * TP_COUNT * ((size_t)depth_n + 1)));
        c->launches += 2;
        k_tab_trig<<<pct_grid_for((int64_t)trig_n + 1, 256), 256, 0, c->stream>>>(
            trig_n, c->mlp_tab_trig.as<double>(), c->mlp_tab_trig.as<double>() + trig_n + 1);
        k_tab_depth<<<pct_grid_for((int64_t)depth_n + 1, 256), 256, 0, c->stream>>>(depth_n,
                                                                                   c->mlp_tab_depth.as<double>());
    }
    int64_t bound_total = 0;
    HistView h = c->view(c->h);
    unsigned long long* flags = c->err_flags.as<unsigned long long>();
    if (n > 0) {
        PCT_TRY(c->mlp_bound.alloc(sizeof(int64_t) * n));
        ++c->launches;
        k_tab_bound<<<pct_grid_for(n, 256), 256, 0, c->stream>>>(c->dg, n, h, c->mlp_bound.as<int64_t>());
        PCT_TRY(pct_scan_lengths(c, c->mlp_bound.as<int64_t>(), n, c->row_offsets.as<int64_t>(), &bound_total));
        PCT_TRY(c->rows.alloc(sizeof(uint32_t) * (bound_total > 0 ? bound_total : 1)));
        ++c->launches;
        k_mlp_tab<<<pct_grid_for(n, 128), 128, 0, c->stream>>>(
            c->dg, n, h, c->mlp_tab_trig.as<double>(), c->mlp_tab_trig.as<double>() + trig_n + 1, trig_n,
            c->mlp_tab_depth.as<double>(), depth_n, c->row_offsets.as<int64_t>(), c->mlp_bound.as<int64_t>(),
            c->rows.as<uint32_t>(), c->row_len.as<int>(), flags);
        PCT_CUDA(cudaGetLastError());
        PCT_TRY(pct_stage_row_norms(c));
    }
    c->row_capacity = bound_total;
    c->counts.row_entries = -1;
    c->diag_ready = 0;
    pct_drop_release_graph(c);
    c->stage = ST_ROWS;
    return PCT_OK;
}
