/*
 * Learned warm start for DROP (GB300 extension, no reference counterpart).
 *
 * A 3D residual CNN (8 convolutions 3x3x3, 32 channels, bf16 weights and
 * activations, fp32 accumulation on the tensor cores) maps the HYBRID initial
 * iterate x0 = FBP x hull and the hull mask to a better DROP start.  It plugs
 * in where the reference chooses the initial iterate: define_initial_iterate
 * (src/pCT_Reconstruction_Data_Segments.cu:7191-7224) with X_K0 = IMPORT
 * (include/pCT_data.h:357), i.e. after pct_define_initial_iterate and before
 * pct_collect_mlp_endpoints / pct_drop.
 *
 * Volumes are [z][y][x] with x extent 128 (the image's COLUMNS), y = ROWS,
 * z = SLICES, in the voxel order of pct_get_array.  Parameters are one fp32
 * vector, layer after layer: weights [27 taps][c_out][c_in] (tap = (dz + 1) * 9
 * + (dy + 1) * 3 + (dx + 1)) then biases [c_out], with (c_in, c_out) = (2, 32),
 * six times (32, 32), (32, 1).  Pointers are host memory unless on_device != 0.
 * Every call returns a status; PCT_ERR_TIMEOUT reports a tensor-core pipeline
 * wait that did not complete (the device stays usable).
 */
#ifndef PCT_CNN_H
#define PCT_CNN_H

#include <stddef.h>
#include <stdint.h>
#include "pct.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pct_cnn pct_cnn;

pct_status pct_cnn_create(int device, int depth, int height, int width, pct_cnn** out);
pct_status pct_cnn_destroy(pct_cnn* net);
size_t pct_cnn_num_params(void);
/* He-uniform initial weights from a seed (the last layer starts at 0: output = x0) */
pct_status pct_cnn_init(pct_cnn* net, uint64_t seed);
pct_status pct_cnn_set_params(pct_cnn* net, const float* params, size_t count);
pct_status pct_cnn_get_params(pct_cnn* net, float* params, size_t count);
/* out = network(x0, hull) */
pct_status pct_cnn_forward(pct_cnn* net, const float* x0, const uint8_t* hull, float* out, int on_device);
/* loss = mean (network(x0, hull) - target)^2 and its gradient for every parameter (grads: host, may be NULL) */
pct_status pct_cnn_gradients(pct_cnn* net, const float* x0, const uint8_t* hull, const float* target, int on_device,
                             double* loss, float* grads);
/* one Adam step (beta 0.9 / 0.999, eps 1e-8) on that loss; *loss before the step */
pct_status pct_cnn_train_step(pct_cnn* net, const float* x0, const uint8_t* hull, const float* target, int on_device,
                              float lr, double* loss);
/* fp32 copy of a stored activation (kind 0: output of layer 0..6, 32 channels) or of an
 * input gradient after the last pct_cnn_gradients / pct_cnn_train_step (kind 1: dY of
 * layer 0..6 (32 channels) or 7 (16 channels, channel 0 used)), [v][C] */
pct_status pct_cnn_inspect(pct_cnn* net, int kind, int layer, float* host, size_t count);
pct_status pct_cnn_counts(pct_cnn* net, int64_t* kernel_launches);
/* x0 and the iterate of a context after pct_define_initial_iterate become
 * network(x0, filtered hull) */
pct_status pct_cnn_warm_start(pct_ctx* ctx, pct_cnn* net);

#ifdef __cplusplus
}
#endif
#endif
