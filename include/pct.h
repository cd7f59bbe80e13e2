/*
 * pct_gb300 — C ABI of the GB300-native proton-CT reconstruction path.
 *
 * Drop-in boundary for the reconstruction hot path of lynch829/pCT: history
 * preprocessing (binning, statistical cuts, sinogram), SC/MSC/SM hulls, FBP,
 * MLP hull endpoints and voxel rows, and the DROP block solver.  The reference
 * exposes that path as void entry points over global arrays
 * (include/pCT_functions.h:37-237); this ABI carries the same stages over a
 * context that owns all device memory and one CUDA stream.
 *
 * Conventions
 *   - Every call returns pct_status; nothing calls exit().  pct_last_error()
 *     gives a message for the calling thread's last failure.
 *   - Host buffers belong to the caller; device buffers belong to the context.
 *     Entry points that take device pointers say so ("device pointer").
 *   - One context is used by one host thread at a time.  Independent contexts
 *     may run concurrently.
 *   - Units are cm and radians inside the library; the history upload takes
 *     the PCTD file layout (mm, degrees) like read_data_chunk_v02
 *     (src/pCT_Reconstruction_Data_Segments.cu:1769-1933).
 */
#ifndef PCT_H
#define PCT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum pct_status {
    PCT_OK = 0,
    PCT_ERR_ARGUMENT = 1,   /* bad pointer, size or configuration value */
    PCT_ERR_CUDA = 2,       /* a CUDA runtime call failed */
    PCT_ERR_ALLOC = 3,      /* device or host allocation failed */
    PCT_ERR_STATE = 4,      /* stage called out of order */
    PCT_ERR_OVERFLOW = 5,   /* a fixed-capacity buffer or counter would overflow */
    PCT_ERR_TIMEOUT = 6,    /* a bounded device-side wait gave up */
    PCT_ERR_IO = 7,         /* file read/write failed or malformed PCTD data */
    PCT_ERR_NUMERIC = 8     /* non-finite value where the algorithm needs a number */
} pct_status;

/* Hull and initial-iterate choices, same values as the reference enums
 * HULL_TYPES, INITIAL_ITERATE and FILTER_TYPES (include/pCT_data.h:245,292,357). */
enum { PCT_SC_HULL = 0, PCT_MSC_HULL = 1, PCT_SM_HULL = 2, PCT_FBP_HULL = 3 };
enum { PCT_X_HULL = 0, PCT_FBP_IMAGE = 1, PCT_HYBRID = 2, PCT_ZEROS = 3, PCT_IMPORT = 4 };
enum { PCT_RAM_LAK = 0, PCT_SHEPP_LOGAN = 1, PCT_NO_FILTER = 2 };

/*
 * Run-time configuration.  Every field is a compile-time constant of the
 * reference; pct_config_default() returns the reference header values
 * (include/pCT_config.h, include/pCT_data.h:215-420).  Derived sizes
 * (SLICES, T_BINS, NUM_VOXELS, ...) are computed from these exactly as the
 * reference macros do.
 */
typedef struct pct_config {
    /* scanner and binning (pCT_data.h:222-244) */
    double source_radius;          /* SOURCE_RADIUS [cm] */
    double gantry_angle_interval;  /* GANTRY_ANGLE_INTERVAL [deg] */
    double ssd_t_size;             /* SSD_T_SIZE [cm] */
    double ssd_v_size;             /* SSD_V_SIZE [cm] */
    double t_bin_size;             /* T_BIN_SIZE [cm] */
    double v_bin_size;             /* V_BIN_SIZE [cm] */
    double angular_bin_size;       /* ANGULAR_BIN_SIZE [deg] */
    int sigmas_to_keep;            /* SIGMAS_TO_KEEP */
    int sample_std_dev;            /* SAMPLE_STD_DEV (pCT_config.h:18) */
    /* reconstruction volume (pCT_data.h:255-277) */
    double recon_cyl_radius;       /* RECON_CYL_RADIUS [cm] */
    int columns;                   /* COLUMNS */
    int rows;                      /* ROWS */
    double slice_thickness;        /* SLICE_THICKNESS [cm] */
    /* hulls (pCT_config.h:23-26, pCT_data.h:281-293) */
    int sc_on, msc_on, sm_on;      /* SC_ON, MSC_ON, SM_ON */
    int avg_filter_hull;           /* AVG_FILTER_HULL */
    int mlp_hull;                  /* MLP_HULL: PCT_*_HULL */
    int msc_diff_thresh;           /* MSC_DIFF_THRESH */
    double sc_threshold;           /* SC_THRESHOLD [cm] */
    double msc_threshold;          /* MSC_THRESHOLD [cm] */
    double sm_lower_threshold;     /* SM_LOWER_THRESHOLD [cm] */
    double sm_scale_threshold;     /* SM_SCALE_THRESHOLD */
    double hull_filter_threshold;  /* HULL_FILTER_THRESHOLD */
    int hull_filter_radius;        /* HULL_FILTER_RADIUS */
    /* FBP (pCT_data.h:245-251, pCT_config.h:19) */
    int fbp_on;                    /* FBP_ON */
    int fbp_filter;                /* FBP_FILTER: PCT_RAM_LAK / PCT_SHEPP_LOGAN / PCT_NO_FILTER */
    double fbp_threshold;          /* FBP_THRESHOLD */
    /* iterative reconstruction (pCT_config.h:5, pCT_data.h:358-377) */
    int x_k0;                      /* X_K0: PCT_X_HULL ... */
    int iterations;                /* ITERATIONS */
    int block_size;                /* BLOCK_SIZE_RECON */
    float lambda;                  /* LAMBDA */
    /* GB300 extensions (no reference counterpart) */
    double residual_tol;           /* stop DROP early when the FP64 relative data
                                      residual falls below this (0: run all iterations) */
    int chord_bf16;                /* 1: round each row's chord length to bfloat16 (nearest even) before
                                      it enters the row norm and the DROP updates (0: binary32) */
    int mlp_exact;                 /* 1: every MLP sample in binary64 (slow path, for checks) */
    double mlp_face_margin;        /* [cm] binary32 MLP samples closer than this to a voxel face
                                      are recomputed in binary64 (default 2e-5) */
    int drop_form;                 /* DROP block step: PCT_DROP_SCATTER (default), _SORTED, _TILED or _GATHER */
    int walk_exact;                /* 1: every hull-walk step in binary64 (slow path, for checks) */
    int voxel_order;               /* internal voxel order of the MLP rows and the DROP iterate:
                                      PCT_ORDER_AUTO (4x2x1 bricks when COLUMNS % 4 == 0 and ROWS % 2 == 0)
                                      or PCT_ORDER_LINEAR; every array the API returns is linear */
    /* DROP variants of the reference's CPU reconstruction (pCT_data.h:369-371, .cu:329-336) */
    int drop_variant;              /* PCT_DROP_STANDARD, PCT_DROP_RED (DROP_blocks_red .cu:7998) or
                                      PCT_DROP_ROBUST2 (DROP_blocks_robust2 / DROP_update_robust2 .cu:7871-7901) */
    double eta;                    /* ETA (2.5) */
    int psi_sign;                  /* PSI_SIGN (1) */
    int mlp_tabulated;             /* 1: MLP rows from the reference's lookup tables
                                      (find_MLP_path_GPU_tabulated .cu:5502-5660, tables .cu:4786-4910),
                                      binary64; 0: the analytic MLP (default) */
} pct_config;

enum { PCT_DROP_STANDARD = 0, PCT_DROP_RED = 1, PCT_DROP_ROBUST2 = 2 };

enum { PCT_ORDER_AUTO = 0, PCT_ORDER_LINEAR = 1 };

/* DROP block step forms; all compute the same block update.  SCATTER adds
 * every row entry's update with a binary32 reduction in L2.  SORTED is
 * SCATTER with each block's rows visited in sinogram bin order.  TILED
 * regroups each block's rows by image tile once, then gathers and
 * accumulates in shared memory with exact integer sums, so the iterate is
 * reproducible bit for bit (falls back to SCATTER when its memory is not
 * free). */
enum { PCT_DROP_SCATTER = 0, PCT_DROP_SORTED = 1, PCT_DROP_TILED = 2, PCT_DROP_GATHER = 3 };

/* Geometry derived from a pct_config, as the reference macros derive it. */
typedef struct pct_geometry {
    int columns, rows, slices, num_voxels;
    int t_bins, v_bins, angular_bins, num_bins, gantry_angles;
    double recon_cyl_radius, recon_cyl_height;
    double voxel_width, voxel_height, voxel_thickness;
    double x_zero, y_zero, z_zero;
    double mlp_u_step;
} pct_geometry;

/* ---- synthetic phantoms and histories (no reference counterpart) ------- */
enum { PCT_PRIM_CYLINDER = 0, PCT_PRIM_ELLIPSOID = 1 };
/* One phantom primitive; RSP values of overlapping primitives add.
 * Cylinder: axis along z through (cx, cy), radius a, |z - cz| <= c.
 * Ellipsoid: center (cx, cy, cz), semi-axes a, b, c, rotated by phi about z. */
typedef struct pct_phantom_object {
    int kind;
    double cx, cy, cz;
    double a, b, c;
    double phi;
    double rsp;
} pct_phantom_object;

typedef struct pct_scan_params {
    uint64_t seed;
    int num_angles;                /* gantry angles, histories split evenly, angle-major */
    double gantry_angle_interval;  /* [deg] */
    double t_extent, v_extent;     /* half-width / half-height of the field at isocenter [cm] */
    double source_radius;          /* fan divergence source distance [cm] */
    double angular_spread;         /* Gaussian beam spread [rad] */
    double beam_energy_mev;        /* kinetic energy, 200 */
    double wepl_noise;             /* relative Gaussian WEPL noise, 0.02 */
    double outlier_fraction;       /* fraction of object-hitting histories with uniform WEPL */
    double outlier_max;            /* upper bound of the uniform outlier WEPL [cm] */
    double scatter_scale;          /* multiplier on the Highland width */
} pct_scan_params;

/* Fills the 13 PCTD arrays (t0..t3, v0..v3, u0..u3, WEPL; mm) and the
 * per-history projection angle [deg] for n histories. */
pct_status pct_generate_histories(const pct_phantom_object* objs, int n_objs, const pct_scan_params* sp,
                                  float* const out[13], float* projection_angle, int64_t n);
/* RSP of the phantom averaged over supersample^3 points per voxel, in the
 * voxel order of the reconstruction (column fastest, slice 0 at z = +H/2). */
pct_status pct_phantom_voxelize(const pct_phantom_object* objs, int n_objs, const pct_config* cfg,
                                int supersample, float* image);

/* ---- reconstruction context ------------------------------------------- */
typedef struct pct_ctx pct_ctx;

/* History counts after each stage (the reference's total_histories,
 * recon_vol_histories, post_cut_histories, reconstruction_histories;
 * include/pCT_data.h:474-478, 367). */
typedef struct pct_counts {
    int64_t total_histories;
    int64_t recon_vol_histories;
    int64_t post_cut_histories;
    int64_t reconstruction_histories;
    int64_t row_entries;             /* MLP row entries over all recon histories */
    int64_t rows_outside_image;      /* row entries whose voxel index lies outside the image */
    int64_t walks_capped;            /* hull/endpoint walks stopped by the step cap */
    int64_t mlp_fp64_samples;        /* MLP samples recomputed in FP64 near a voxel face */
    int64_t walk_fp64_steps;         /* hull-walk steps taken in FP64 (binary32 could not certify them) */
    int64_t kernel_launches;         /* kernels this context has launched (graph nodes included) */
    int64_t drop_list_entries;       /* gather DROP form: stored column-list entries (padding included) */
} pct_counts;

/* Per-iteration DROP statistics (GB300 extension). */
typedef struct pct_drop_stats {
    int iterations_run;
    double residual[64];             /* FP64 relative data residual ||b - A x|| / ||b|| before each iteration, and after the last */
    double seconds;                  /* device time of the iterations */
    int drop_form;                   /* the DROP form that ran (PCT_DROP_*: a form that does not fit falls back) */
} pct_drop_stats;

/* Arrays readable with pct_get_array().  H_* are per-history arrays of the
 * current history store (compacted in place after binning, cuts and
 * endpoints, like the reference's *_vector globals, pCT_data.h:577-595). */
typedef enum pct_array {
    PCT_ARR_MSC_COUNTS = 0, PCT_ARR_SM_COUNTS, PCT_ARR_SC_HULL, PCT_ARR_MSC_HULL, PCT_ARR_SM_HULL,   /* int32 voxels */
    PCT_ARR_BIN_COUNTS_PRE, PCT_ARR_MEAN_WEPL, PCT_ARR_MEAN_UT, PCT_ARR_MEAN_UV,                    /* bins */
    PCT_ARR_SD_WEPL, PCT_ARR_SD_UT, PCT_ARR_SD_UV, PCT_ARR_BIN_COUNTS_POST, PCT_ARR_SINOGRAM,
    PCT_ARR_SINOGRAM_FILTERED,
    PCT_ARR_FBP_IMAGE, PCT_ARR_FBP_HULL, PCT_ARR_X_HULL, PCT_ARR_X_HULL_FILTERED, PCT_ARR_X0, PCT_ARR_X, /* voxels */
    PCT_ARR_H_BIN_NUM, PCT_ARR_H_WEPL, PCT_ARR_H_X_ENTRY, PCT_ARR_H_Y_ENTRY, PCT_ARR_H_Z_ENTRY,         /* histories */
    PCT_ARR_H_X_EXIT, PCT_ARR_H_Y_EXIT, PCT_ARR_H_Z_EXIT, PCT_ARR_H_XY_ENTRY_ANGLE, PCT_ARR_H_XZ_ENTRY_ANGLE,
    PCT_ARR_H_XY_EXIT_ANGLE, PCT_ARR_H_XZ_EXIT_ANGLE, PCT_ARR_H_FIRST_VOXEL, PCT_ARR_H_FAILED_CUTS,
    PCT_ARR_ROW_OFFSETS, PCT_ARR_ROWS, PCT_ARR_CHORD,                                                  /* MLP rows */
    PCT_ARR_COUNT
} pct_array;

/* Creates a context on CUDA device `device`; every buffer it owns lives there. */
pct_status pct_create(const pct_config* cfg, int device, pct_ctx** out);
pct_status pct_destroy(pct_ctx* ctx);
/* Capacity hint for the history store (total histories to be uploaded). */
pct_status pct_reserve(pct_ctx* ctx, int64_t total_histories);

/* One chunk of PCTD histories: unit conversion, cylinder intersections,
 * binning and the hull walks.  Replaces read_data_chunk + recon_volume_intersections
 * + binning + hull_detection (pCT_functions.h:37,44,45,61;
 * src/pCT_Reconstruction_Data_Segments.cu:97-100).  data13 are the 13 PCTD
 * arrays (t0..t3, v0..v3, u0..u3, WEPL; mm), projection_angle the header
 * angle of each history [deg].  Pointers are host memory unless
 * data_on_device is nonzero (then device pointers on the context's device). */
pct_status pct_process_chunk(pct_ctx* ctx, const float* const data13[13], const float* projection_angle, int64_t n,
                             int data_on_device);
/* hull_detection_finish (pCT_functions.h:62): MSC/SM edge detection. */
pct_status pct_hull_detection_finish(pct_ctx* ctx);
/* calculate_means, sum_squared_deviations, calculate_standard_deviations,
 * statistical_cuts and construct_sinogram (pCT_functions.h:46-52). */
pct_status pct_statistical_cuts(pct_ctx* ctx);
/* FBP (pCT_functions.h:53): filter, backprojection, FBP hull. */
pct_status pct_fbp(pct_ctx* ctx);
/* hull_selection (pCT_functions.h:69) including the averaging filter. */
pct_status pct_hull_selection(pct_ctx* ctx);
/* define_initial_iterate (pCT_functions.h:85).  For PCT_IMPORT, x0 is taken
 * from pct_set_image() beforehand. */
pct_status pct_define_initial_iterate(pct_ctx* ctx);
/* reconstruction_cuts (pCT_functions.h:230): hull entry/exit of each history,
 * compaction to the histories that cross the hull. */
pct_status pct_collect_mlp_endpoints(pct_ctx* ctx);
/* MLP voxel rows of every recon history, kept resident for all iterations
 * (may be called again to regenerate them). */
pct_status pct_mlp_rows(pct_ctx* ctx);
/* DROP iterations on the resident rows (the iteration loop of
 * image_reconstruction_GPU, src/pCT_Reconstruction_Data_Segments.cu:6795-6860).
 * stats may be NULL. */
pct_status pct_drop(pct_ctx* ctx, int iterations, pct_drop_stats* stats);
/* Binary64 DROP on the resident rows: `iterations` iterations of the same
 * block update with every quantity in binary64 (the chord, dot, ||a_i||^2,
 * update accumulator and iterate), as the reference's host DROP_blocks /
 * DROP_update keep them (src/pCT_Reconstruction_Data_Segments.cu:8023-8055).
 * x: host array of NUM_VOXELS doubles (linear voxel order), the start image
 * in and the result out; the context's binary32 iterate is not touched.  For
 * the error of pct_drop against a binary64 run of the same iterations; needs
 * the scatter or sorted form and the standard update.  stats may be NULL. */
pct_status pct_drop_fp64(pct_ctx* ctx, int iterations, double* x, pct_drop_stats* stats);
/* DROP iterations of several scans in one persistent launch per iteration
 * (no reference counterpart: the reference reconstructs one scan per run,
 * src/pCT_Reconstruction_Data_Segments.cu:6795-6844).  `count` distinct
 * contexts on one device, each after pct_mlp_rows, each with its own block
 * size, in the scatter form with the standard update and unsharded.  The
 * blocks of all scans form one queue of work items (rows of a block, or
 * voxels of its relaxation) taken by the CTAs of a cooperative launch;
 * within a scan the blocks run in order, as pct_drop runs them.  At most 64
 * iterations per call.  stats: `count` entries or NULL; every scan's
 * `seconds` is the device time of the whole batch. */
pct_status pct_drop_many(pct_ctx* const* ctxs, int count, int iterations, pct_drop_stats* stats);
/* The MLP rows packed back to back, returning to the device the slack of the
 * per-history slots (sized by the MLP sample count); no reference
 * counterpart.  The rows, their order and the DROP results are unchanged. */
pct_status pct_compact_rows(pct_ctx* ctx);
/* image_reconstruction_GPU (pCT_functions.h:237): endpoints, rows, all
 * cfg->iterations DROP iterations. */
pct_status pct_image_reconstruction(pct_ctx* ctx, pct_drop_stats* stats);

pct_status pct_get_counts(pct_ctx* ctx, pct_counts* counts);
/* Copies an array to host memory; *bytes is the capacity in, the size out. */
pct_status pct_get_array(pct_ctx* ctx, pct_array which, void* host_dst, size_t* bytes);
/* Device pointer and byte size of an array (valid until the next stage call). */
pct_status pct_array_device_ptr(pct_ctx* ctx, pct_array which, void** dptr, size_t* bytes);
/* Sets the current iterate back to the initial iterate x0. */
pct_status pct_reset_iterate(pct_ctx* ctx);
/* Replaces the current iterate (host pointer, num_voxels floats). */
pct_status pct_set_image(pct_ctx* ctx, const float* x);
/* CUDA stream the context runs on (cudaStream_t). */
void* pct_stream(pct_ctx* ctx);

/* DROP without allocation.  No counterpart in the reference (its DROP always
 * allocates per-iteration buffers with cudaMalloc, .cu:6795-6860).
 *
 * For callers that may not allocate during the call: a process on a locked,
 * pre-sized memory pool, or one that must not let cudaMalloc/cudaFree
 * synchronise the device in the middle of its own stream sequence.  The call
 * runs `iterations` DROP iterations in blocks of block_size histories on
 * caller-owned DEVICE arrays (dense CSR rows: row_offsets has n+1 entries,
 * rows holds voxel indices, entries >= num_voxels are skipped) and updates x
 * in place on `stream` (a cudaStream_t; NULL = legacy default stream); it
 * does not synchronise.  residual_sq (device, `iterations` doubles, may be
 * NULL) receives sum_i (b_i - c_i a_i.x)^2 of each sweep.  Per-voxel scratch is
 * a static device array of PCT_NOALLOC_MAX_VOXELS voxels: larger images are
 * rejected with PCT_ERR_ARGUMENT.  Calls that overlap on one device share that
 * scratch and race.  The first call on a device (or pct_noalloc_setup() with
 * that device current) looks the scratch up and may load the module. */
#define PCT_NOALLOC_MAX_VOXELS (1 << 21)
pct_status pct_noalloc_setup(void);
pct_status pct_drop_noalloc(int64_t n, const int64_t* row_offsets, const uint32_t* rows, const float* chord,
                            const float* wepl, int num_voxels, int block_size, float lambda, int iterations,
                            float* x, double* residual_sq, void* stream);

/* PCTD version-0 files (count_histories_v0 .cu:997-1097, read_data_chunk_v02
 * .cu:1769-1933): header query, read into 13 caller host arrays of at least
 * `capacity` floats (t0..t3, v0..v3, u0..u3, WEPL in mm), write, and
 * read+upload of whole files as chunks (one file per gantry angle). */
pct_status pct_pctd_info(const char* path, int64_t* num_histories, float* projection_angle, float* beam_energy);
pct_status pct_pctd_read(const char* path, float* const data13[13], int64_t capacity, int64_t* num_histories,
                         float* projection_angle);
pct_status pct_pctd_write(const char* path, const float* const data13[13], int64_t num_histories,
                          float projection_angle, float beam_energy);
pct_status pct_process_pctd_files(pct_ctx* ctx, const char* const* paths, int num_files);

/* MLP endpoint files (write_MLP_endpoints / read_MLP_endpoints, .cu:4684-4745),
 * MLP path files (the format of the reference's CPU reconstruction,
 * .cu:4746, 7478-7493) and raw float32 image checkpoints (the reference writes
 * its iterates as text, .cu:8092-8134).  Reading endpoints replaces the
 * history store and leaves the context ready for pct_mlp_rows (an iterate of
 * zeros unless one exists or pct_set_image provides one); reading paths
 * replaces the rows of the current endpoints. */
pct_status pct_write_mlp_endpoints(pct_ctx* ctx, const char* path);
pct_status pct_read_mlp_endpoints(pct_ctx* ctx, const char* path);
pct_status pct_write_mlp_paths(pct_ctx* ctx, const char* path);
pct_status pct_read_mlp_paths(pct_ctx* ctx, const char* path);
pct_status pct_write_image(pct_ctx* ctx, pct_array which, const char* path);
pct_status pct_read_image(pct_ctx* ctx, const char* path);

/* Sharded DROP: the rows of every DROP block split over several contexts
 * (ranks), with one elementwise sum over the ranks per block -- the
 * partitioning of a block's histories across GPUs that block_update_GPU's
 * independence within a block allows (.cu:5774-5841, .cu:6803-6844).
 *
 * pct_select_shard (after pct_collect_mlp_endpoints, before pct_mlp_rows)
 * keeps the reconstruction histories i with i % num_shards == shard and makes
 * the block size block_size / num_shards (block_size must be a multiple of
 * num_shards), so that local block k holds this rank's share of global block
 * k; every rank keeps the global number of blocks, some possibly empty.
 *
 * With an all-reduce callback set, pct_drop (scatter or sorted form; the tiled
 * form falls back to scatter) synchronises the context stream and calls
 * fn(user, data, count, dtype, on_device) for: the DROP diagonal counts of
 * all blocks once (PCT_DT_U32, num_blocks * NUM_VOXELS), the sum of squared
 * WEPL once (PCT_DT_F64, 1), then in every iteration each block's update
 * image (PCT_DT_F32, NUM_VOXELS) before it is applied and the iteration's
 * squared residual (PCT_DT_F64, 1); with the ROBUST2 variant also the
 * per-voxel c^2 sums once (PCT_DT_F32, num_blocks * NUM_VOXELS).  `data` is
 * device memory of the context's device (on_device = 1); the callback returns
 * 0 with `data` replaced by the elementwise sum over the ranks and all its
 * own device work complete.  Every rank makes the same sequence of calls.
 * fn = NULL restores the single-context DROP. */
enum { PCT_DT_F32 = 0, PCT_DT_U32 = 1, PCT_DT_F64 = 2 };
typedef int (*pct_allreduce_fn)(void* user, void* data, int64_t count, int dtype, int on_device);
pct_status pct_set_allreduce(pct_ctx* ctx, pct_allreduce_fn fn, void* user);
pct_status pct_select_shard(pct_ctx* ctx, int shard, int num_shards);
/* DROP block size (BLOCK_SIZE_RECON) of an existing context, e.g. for a
 * block-size search; takes effect at the next pct_drop (the diagonal weights
 * are recounted).  Not for a context that holds a shard. */
pct_status pct_set_block_size(pct_ctx* ctx, int block_size);
/* cudaMemcpy with the direction taken from the pointers (for callbacks). */
pct_status pct_memcpy(void* dst, const void* src, int64_t bytes);

pct_status pct_config_default(pct_config* cfg);
pct_status pct_geometry_from_config(const pct_config* cfg, pct_geometry* geo);
const char* pct_last_error(void);
const char* pct_status_string(pct_status s);
/* sizeof of ABI structs (0 config, 1 geometry, 2 phantom object, 3 scan params, 4 counts, 5 drop stats). */
size_t pct_sizeof(int which);

#ifdef __cplusplus
}
#endif
#endif /* PCT_H */
