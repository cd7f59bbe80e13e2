/*
 * A reference-style driver over the compatibility layer: the main() sequence
 * of src/pCT_Reconstruction_Data_Segments.cu:33-238 (chunked reading, hull
 * detection, statistics, cuts, FBP, hull selection, initial iterate, image
 * reconstruction) written against include/pct_functions_compat.h.
 *
 * usage: driver <config.bin> <input_directory> <input_folder> <max_chunk_histories> <image_out>
 * config.bin holds one pct_config as bytes.
 */
#include <cstdio>
#include <cstdlib>
#include "pct_functions_compat.h"

int main(int argc, char** argv) {
    if (argc != 6) {
        fprintf(stderr, "usage: %s config.bin dir folder max_chunk image_out\n", argv[0]);
        return 2;
    }
    pct_config cfg;
    FILE* f = fopen(argv[1], "rb");
    if (!f || fread(&cfg, sizeof(cfg), 1, f) != 1) {
        fprintf(stderr, "cannot read %s\n", argv[1]);
        return 2;
    }
    fclose(f);
    const int max_chunk = atoi(argv[4]);
    if (pct_compat_setup(&cfg, argv[2], argv[3], 0) != PCT_OK) {
        fprintf(stderr, "setup: %s\n", pct_last_error());
        return 1;
    }
    hull_initializations();
    initializations();
    count_histories();
    reserve_vector_capacity();
    int start_file_num = 0, end_file_num = 0, histories_to_process = 0;
    while (start_file_num != NUM_FILES_COMPAT) {
        while (end_file_num < NUM_FILES_COMPAT) {
            if (histories_to_process + histories_per_file[end_file_num] < max_chunk)
                histories_to_process += histories_per_file[end_file_num];
            else
                break;
            end_file_num++;
        }
        if (end_file_num == start_file_num) { /* a single file larger than the chunk limit */
            histories_to_process = histories_per_file[end_file_num];
            end_file_num++;
        }
        read_data_chunk(histories_to_process, start_file_num, end_file_num);
        recon_volume_intersections(histories_to_process);
        binning(histories_to_process);
        hull_detection(histories_to_process);
        start_file_num = end_file_num;
        histories_to_process = 0;
    }
    hull_detection_finish();
    calculate_means();
    initialize_stddev();
    sum_squared_deviations(0, recon_vol_histories);
    calculate_standard_deviations();
    initialize_sinogram();
    statistical_cuts(0, recon_vol_histories);
    construct_sinogram();
    FBP();
    hull_selection();
    define_initial_iterate();
    image_reconstruction_GPU();
    if (pct_compat_status() != PCT_OK || !x_h) {
        fprintf(stderr, "pipeline failed (status %d)\n", (int)pct_compat_status());
        return 1;
    }
    pct_geometry geo;
    pct_geometry_from_config(&cfg, &geo);
    FILE* o = fopen(argv[5], "wb");
    if (!o || fwrite(x_h, sizeof(float), (size_t)geo.num_voxels, o) != (size_t)geo.num_voxels) return 1;
    fclose(o);
    printf("histories %d recon_vol %d post_cut %d reconstruction %u\n", total_histories, recon_vol_histories,
           post_cut_histories, reconstruction_histories);
    pct_compat_teardown();
    return 0;
}
