/*
 * The reference's host entry points (include/pCT_functions.h) over the pct
 * C ABI; see include/pct_functions_compat.h.
 */
#include <cstdio>
#include <string>
#include "pct_functions_compat.h"

int NUM_FILES_COMPAT = 0;
std::vector<int> histories_per_file;
int total_histories = 0, recon_vol_histories = 0, post_cut_histories = 0;
unsigned int reconstruction_histories = 0;
float* x_h = nullptr;

namespace {

struct Compat {
    pct_ctx* ctx = nullptr;
    pct_config cfg{};
    int device = 0;
    std::vector<std::string> paths;
    std::vector<float> chunk;       /* 13 arrays of chunk_n floats */
    std::vector<float> chunk_angle;
    int64_t chunk_n = 0;
    std::vector<float> image;
    pct_status status = PCT_OK;
};
Compat g;

bool ok() { return g.ctx && g.status == PCT_OK; }

void check(pct_status s, const char* what) {
    if (s != PCT_OK && g.status == PCT_OK) {
        g.status = s;
        fprintf(stderr, "pct compat: %s: %s\n", what, pct_last_error());
    }
}

void refresh_counts() {
    pct_counts c;
    if (pct_get_counts(g.ctx, &c) != PCT_OK) return;
    total_histories = (int)c.total_histories;
    recon_vol_histories = (int)c.recon_vol_histories;
    post_cut_histories = (int)c.post_cut_histories;
    reconstruction_histories = (unsigned int)c.reconstruction_histories;
}

}  // namespace

pct_status pct_compat_setup(const pct_config* cfg, const char* input_directory, const char* input_folder,
                            int device) {
    pct_compat_teardown();
    if (!cfg || !input_directory || !input_folder) return pct_status(PCT_ERR_ARGUMENT);
    g.cfg = *cfg;
    g.device = device;
    g.status = pct_create(cfg, device, &g.ctx);
    if (g.status != PCT_OK) return g.status;
    pct_geometry geo;
    g.status = pct_geometry_from_config(cfg, &geo);
    if (g.status != PCT_OK) return g.status;
    NUM_FILES_COMPAT = geo.gantry_angles;
    g.paths.clear();
    for (int k = 0; k < geo.gantry_angles; ++k) {
        char name[64];
        snprintf(name, sizeof(name), "projection_%03d.bin", (int)(k * cfg->gantry_angle_interval));
        g.paths.push_back(std::string(input_directory) + "/" + input_folder + "/" + name);
    }
    return PCT_OK;
}

pct_status pct_compat_status() { return g.status; }
pct_ctx* pct_compat_context() { return g.ctx; }

void pct_compat_teardown() {
    if (g.ctx) pct_destroy(g.ctx);
    g = Compat();
    histories_per_file.clear();
    NUM_FILES_COMPAT = total_histories = recon_vol_histories = post_cut_histories = 0;
    reconstruction_histories = 0;
    x_h = nullptr;
}

void initializations() {}
void hull_initializations() {}

void count_histories() {
    if (!ok()) return;
    histories_per_file.assign(g.paths.size(), 0);
    int64_t total = 0;
    for (size_t k = 0; k < g.paths.size(); ++k) {
        int64_t n = 0;
        check(pct_pctd_info(g.paths[k].c_str(), &n, nullptr, nullptr), "count_histories");
        if (!ok()) return;
        histories_per_file[k] = (int)n;
        total += n;
    }
    total_histories = (int)total;
}

void reserve_vector_capacity() {
    if (ok()) check(pct_reserve(g.ctx, total_histories), "reserve_vector_capacity");
}

void read_data_chunk(const int num_histories, const int start_file_num, const int end_file_num) {
    if (!ok()) return;
    if (start_file_num < 0 || end_file_num > (int)g.paths.size() || start_file_num > end_file_num) {
        check(PCT_ERR_ARGUMENT, "read_data_chunk: file range");
        return;
    }
    g.chunk.assign((size_t)13 * (size_t)(num_histories > 0 ? num_histories : 1), 0.0f);
    g.chunk_angle.assign((size_t)(num_histories > 0 ? num_histories : 1), 0.0f);
    int64_t at = 0;
    std::vector<float> part;
    for (int f = start_file_num; f < end_file_num; ++f) {
        int64_t n = 0;
        float angle = 0.0f;
        check(pct_pctd_info(g.paths[f].c_str(), &n, &angle, nullptr), "read_data_chunk");
        if (!ok()) return;
        if (at + n > num_histories) {
            check(PCT_ERR_OVERFLOW, "read_data_chunk: more histories in the files than requested");
            return;
        }
        part.assign((size_t)13 * (size_t)(n > 0 ? n : 1), 0.0f);
        float* d13[13];
        for (int k = 0; k < 13; ++k) d13[k] = part.data() + (size_t)k * (size_t)n;
        int64_t got = 0;
        check(pct_pctd_read(g.paths[f].c_str(), d13, n, &got, &angle), "read_data_chunk");
        if (!ok()) return;
        for (int k = 0; k < 13; ++k)
            for (int64_t i = 0; i < got; ++i) g.chunk[(size_t)k * num_histories + at + i] = d13[k][i];
        for (int64_t i = 0; i < got; ++i) g.chunk_angle[at + i] = angle;
        at += got;
    }
    g.chunk_n = at;
}

void recon_volume_intersections(const int) {}
void binning(const int) {}

void hull_detection(const int) {
    if (!ok() || g.chunk_n == 0) return;
    /* the chunk's 13 arrays are strided by the capacity the driver asked for */
    const int64_t cap = (int64_t)(g.chunk.size() / 13);
    const float* c13[13];
    for (int k = 0; k < 13; ++k) c13[k] = g.chunk.data() + (size_t)k * (size_t)cap;
    check(pct_process_chunk(g.ctx, c13, g.chunk_angle.data(), g.chunk_n, 0), "hull_detection");
    g.chunk_n = 0;
    if (ok()) refresh_counts();
}

void hull_detection_finish() {
    if (ok()) check(pct_hull_detection_finish(g.ctx), "hull_detection_finish");
}

void calculate_means() {
    if (!ok()) return;
    check(pct_statistical_cuts(g.ctx), "calculate_means");
    if (ok()) refresh_counts();
}
void initialize_stddev() {}
void sum_squared_deviations(const int, const int) {}
void calculate_standard_deviations() {}
void initialize_sinogram() {}
void statistical_cuts(const int, const int) {}
void construct_sinogram() {}

void FBP() {
    if (ok()) check(pct_fbp(g.ctx), "FBP");
}
void hull_selection() {
    if (ok()) check(pct_hull_selection(g.ctx), "hull_selection");
}
void define_initial_iterate() {
    if (ok()) check(pct_define_initial_iterate(g.ctx), "define_initial_iterate");
}

void image_reconstruction_GPU() {
    if (!ok()) return;
    check(pct_image_reconstruction(g.ctx, nullptr), "image_reconstruction_GPU");
    if (!ok()) return;
    pct_geometry geo;
    pct_geometry_from_config(&g.cfg, &geo);
    g.image.assign((size_t)geo.num_voxels, 0.0f);
    size_t bytes = g.image.size() * sizeof(float);
    check(pct_get_array(g.ctx, PCT_ARR_X, g.image.data(), &bytes), "image_reconstruction_GPU: image");
    x_h = g.image.data();
    refresh_counts();
}
