/*
 * Internal declarations shared by the library's C++/CUDA translation units.
 */
#ifndef PCT_INTERNAL_H
#define PCT_INTERNAL_H

#include "pct.h"
#include "pct_math.h"
#include "pct_geometry.h"

/* Records a message for pct_last_error() and returns the status. */
pct_status pct_fail(pct_status s, const char* fmt, ...);

double pct_phantom_line_integral(const pct_phantom_object* objs, int n_objs, const double p0[3], const double d[3]);
double pct_phantom_rsp_at(const pct_phantom_object* objs, int n_objs, double x, double y, double z);

#endif
