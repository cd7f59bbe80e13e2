/*
 * Measurement aid, not part of the reference interface: the L2 ceiling that
 * bounds the DROP block update (block_update_GPU, src/pCT_Reconstruction_Data_Segments.cu:5774-5841,
 * one float reduction into the update image per row entry), measured on the
 * device at hand.
 */
#ifndef PCT_PROBE_H
#define PCT_PROBE_H

#include "pct.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Pseudo-random float reductions into an 8 MB L2-resident array, one element
 * per 32-byte sector.  mode 0: reductions only; mode 1: before each reduction
 * the same sector of a second 8 MB array is read (the DROP row pass's gather
 * of the iterate and update of x_update).  Returns the
 * sectors reduced per second in *sectors_per_second. */
pct_status pct_probe_l2(int device, int mode, double* sectors_per_second);

#ifdef __cplusplus
}
#endif

#endif
