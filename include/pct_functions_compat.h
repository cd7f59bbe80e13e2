/*
 * Compatibility layer: the reference's host entry points over the C ABI.
 *
 * A driver written against include/pCT_functions.h of the reference
 * (lynch829/pCT) calls these functions in the order of its main()
 * (src/pCT_Reconstruction_Data_Segments.cu:33-238); here they run the
 * pct_gb300 stages on one context.  The reference's compile-time
 * configuration becomes the pct_config given to pct_compat_setup(), and the
 * PCTD input files are found as <directory>/<folder>/projection_<angle>.bin
 * like the reference's INPUT_DIRECTORY/INPUT_FOLDER (.cu:1807-1813).
 *
 * Several reference stages are fused in pct_gb300 (intersections, binning
 * and the hull walks run in hull_detection(); means, deviations, cuts and the
 * sinogram run in calculate_means()); the remaining names of those groups are
 * kept and do no work.  The reference exits on errors; these functions record
 * the first failing status instead (pct_compat_status()) and do nothing after
 * it.  Not thread-safe: one driver thread, as in the reference.
 */
#ifndef PCT_FUNCTIONS_COMPAT_H
#define PCT_FUNCTIONS_COMPAT_H

#include <vector>
#include "pct.h"

/* Set-up and results (no reference counterpart). */
pct_status pct_compat_setup(const pct_config* cfg, const char* input_directory, const char* input_folder,
                            int device);
pct_status pct_compat_status();
pct_ctx* pct_compat_context();
void pct_compat_teardown();

/* Globals the reference driver reads (pCT_data.h): files of the scan, history
 * counts after each stage, and the host image after image_reconstruction_GPU. */
extern int NUM_FILES_COMPAT;
extern std::vector<int> histories_per_file;
extern int total_histories, recon_vol_histories, post_cut_histories;
extern unsigned int reconstruction_histories;
extern float* x_h;

/* The reference's entry points (include/pCT_functions.h). */
void initializations();
void hull_initializations();
void count_histories();
void reserve_vector_capacity();
void read_data_chunk(const int, const int, const int);
void recon_volume_intersections(const int);
void binning(const int);
void hull_detection(const int);
void hull_detection_finish();
void calculate_means();
void initialize_stddev();
void sum_squared_deviations(const int, const int);
void calculate_standard_deviations();
void initialize_sinogram();
void statistical_cuts(const int, const int);
void construct_sinogram();
void FBP();
void hull_selection();
void define_initial_iterate();
void image_reconstruction_GPU();

#endif
