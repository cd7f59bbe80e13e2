/*
 * CPU oracle for the pCT reconstruction path — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference algorithm (lynch829/pCT,
 * src/pCT_Reconstruction_Data_Segments.cu), used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU baseline as the checker.
 * The product never links it.  Each function cites the reference lines it
 * restates.
 *
 * Parity pin: tests/golden/ holds outputs of the reference's own driver
 * sequence (oracle/build_ref.py + oracle/ref/ref_harness.inc) on seeded
 * synthetic scans; tests/test_oracle_golden.py checks this oracle against
 * them stage by stage.
 *
 * Arithmetic: binary64/binary32 operations in the reference's source order,
 * no FMA contraction (built with -ffp-contract=off), elementary functions
 * from pct_gb300/csrc/pct_math.h.  The per-bin statistics and the sinogram
 * are binary32 sums in history order: the order in which a sequential run of
 * the reference's atomicAdd kernels adds them (the golden fixtures' run).
 */
#ifndef PCT_ORACLE_H
#define PCT_ORACLE_H

#include <stdint.h>
#include "pct.h"

#ifdef __cplusplus
extern "C" {
#endif

/* a1-a3: unit conversion, cylinder intersections, bin index; per history. */
int ora_preprocess(const pct_config* cfg, int64_t n, const float* const in13[13], const float* projection_angle,
                   int32_t* gantry_angle, uint8_t* missed, int32_t* bin_num, uint8_t* bin_valid,
                   float* x_entry, float* y_entry, float* z_entry, float* x_exit, float* y_exit, float* z_exit,
                   float* xy_entry_angle, float* xz_entry_angle, float* xy_exit_angle, float* xz_exit_angle,
                   float* wepl_cm);

/* a4: per-bin counts, means and standard deviations over the kept histories. */
int ora_bin_statistics(const pct_config* cfg, int64_t n, const int32_t* bin_num, const uint8_t* bin_valid,
                       const float* wepl, const float* xy_entry_angle, const float* xz_entry_angle,
                       const float* xy_exit_angle, const float* xz_exit_angle,
                       int32_t* counts, float* mean_wepl, float* mean_ut, float* mean_uv,
                       float* sd_wepl, float* sd_ut, float* sd_uv);

/* a5-a6: 3-sigma cuts, post-cut counts and the sinogram (mean WEPL per bin). */
int ora_statistical_cuts(const pct_config* cfg, int64_t n, const int32_t* bin_num, const float* wepl,
                         const float* xy_entry_angle, const float* xz_entry_angle, const float* xy_exit_angle,
                         const float* xz_exit_angle, const float* mean_wepl, const float* mean_ut,
                         const float* mean_uv, const float* sd_wepl, const float* sd_ut, const float* sd_uv,
                         uint8_t* failed, int32_t* counts_post, float* sinogram);

/* a7: hull walks.  kind 0 SC (hull 0/1 image), 1 MSC, 2 SM (count images).
 * The image must be initialised with ora_initialize_hull() first. */
void ora_initialize_hull(const pct_config* cfg, int32_t* image);
int ora_hull_walk(const pct_config* cfg, int kind, int64_t n, const uint8_t* missed, const float* wepl,
                  const float* x_entry, const float* y_entry, const float* z_entry, const float* x_exit,
                  const float* y_exit, const float* z_exit, int32_t* image, int64_t* walk_steps_capped);

/* a8-a9: edge detection, hull selection, averaging filter. */
void ora_msc_edge_detection(const pct_config* cfg, const int32_t* counts, int32_t* hull);
void ora_sm_edge_detection(const pct_config* cfg, const int32_t* counts, int32_t* hull, int32_t* thresholds);
void ora_averaging_filter_bool(const pct_config* cfg, const uint8_t* in, uint8_t* out, int radius, double threshold);

/* a10-a12: FBP filter, backprojection, FBP hull. */
void ora_filter(const pct_config* cfg, const float* sinogram, float* filtered);
void ora_backprojection(const pct_config* cfg, const float* filtered, float* image);
void ora_fbp_hull(const pct_config* cfg, const float* image, uint8_t* hull);

/* a13: hull entry/exit of each history. */
int ora_endpoints(const pct_config* cfg, int64_t n, const uint8_t* hull, const float* x_entry, const float* y_entry,
                  const float* z_entry, const float* xy_entry_angle, const float* xz_entry_angle,
                  const float* x_exit, const float* y_exit, const float* z_exit, const float* xy_exit_angle,
                  const float* xz_exit_angle, uint8_t* intersected, uint32_t* first_voxel,
                  float* x_in, float* y_in, float* z_in, float* x_out, float* y_out, float* z_out);

/* a14-a15: MLP voxel rows.  offsets has n+1 entries; rows holds the voxel
 * indices back to back (capacity entries); chord gets the effective chord
 * length.  Returns the total entries written, or -1 if capacity is too small. */
int64_t ora_mlp_rows(const pct_config* cfg, int64_t n, const float* x_in, const float* y_in, const float* z_in,
                     const float* x_out, const float* y_out, const float* z_out, const float* xy_entry_angle,
                     const float* xz_entry_angle, const float* xy_exit_angle, const float* xz_exit_angle,
                     const uint32_t* first_voxel, int64_t* offsets, uint32_t* rows, int64_t capacity, double* chord);
double ora_effective_chord_length(const pct_config* cfg, double abs_angle_t, double abs_angle_v);

/* a14 tabulated: find_MLP_path_GPU_tabulated (.cu:5502-5660) with the tables
 * of .cu:4786-4911 at the resolutions of pCT_data.h:405-417; same outputs as
 * ora_mlp_rows. */
int64_t ora_mlp_rows_tab(const pct_config* cfg, int64_t n, const float* x_in, const float* y_in, const float* z_in,
                         const float* x_out, const float* y_out, const float* z_out, const float* xy_entry_angle,
                         const float* xz_entry_angle, const float* xy_exit_angle, const float* xz_exit_angle,
                         const uint32_t* first_voxel, int64_t* offsets, uint32_t* rows, int64_t capacity,
                         double* chord);

/* a16-a19: DROP on precomputed rows, FP64 image; iterations over all blocks. */
int ora_drop(const pct_config* cfg, int64_t n, const int64_t* offsets, const uint32_t* rows, const double* chord,
             const float* wepl, int iterations, int block_size, double lambda, double* x);

/* a16-a19 as one shard of a sharded DROP: `n` local rows, this rank's share of
 * every global block in order (local block size block_size, num_blocks global
 * blocks, some possibly empty here); each block's binary64 update and counts
 * are summed over the ranks by fn (PCT_DT_F64 / PCT_DT_U32, host memory,
 * on_device = 0) before x += update / s. */
int ora_drop_shard(const pct_config* cfg, int64_t n, const int64_t* offsets, const uint32_t* rows, const double* chord,
                   const float* wepl, int iterations, int block_size, int num_blocks, double lambda, double* x,
                   pct_allreduce_fn fn, void* user);

/* a16-a19 variants: 1 DROP_blocks_red, 2 DROP_blocks_robust2 + DROP_update_robust2 (0 = ora_drop). */
int ora_drop_variant(const pct_config* cfg, int64_t n, const int64_t* offsets, const uint32_t* rows,
                     const double* chord, const float* wepl, int iterations, int block_size, double lambda,
                     int variant, double eta, int psi_sign, double* x);

/* Same results with `threads` OpenMP threads (per-history parallel rows;
 * per-block parallel DROP with atomic accumulation). */
int64_t ora_mlp_rows_mt(const pct_config* cfg, int64_t n, const float* x_in, const float* y_in, const float* z_in,
                        const float* x_out, const float* y_out, const float* z_out, const float* xy_entry_angle,
                        const float* xz_entry_angle, const float* xy_exit_angle, const float* xz_exit_angle,
                        const uint32_t* first_voxel, int64_t* offsets, uint32_t* rows, int64_t capacity, double* chord,
                        int threads);
int ora_drop_mt(const pct_config* cfg, int64_t n, const int64_t* offsets, const uint32_t* rows, const double* chord,
                const float* wepl, int iterations, int block_size, double lambda, double* x, int threads);

/* Runtime of the library build (so callers can check they loaded the right one). */
int ora_version(void);

#ifdef __cplusplus
}
#endif
#endif
