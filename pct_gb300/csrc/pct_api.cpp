/*
 * Error reporting and configuration entry points of the C ABI.
 */
#include <cstdarg>
#include <cstdio>
#include "pct_internal.h"

static thread_local char g_last_error[512] = "";

pct_status pct_fail(pct_status s, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return s;
}

extern "C" const char* pct_last_error(void) { return g_last_error; }

extern "C" const char* pct_status_string(pct_status s) {
    switch (s) {
        case PCT_OK: return "ok";
        case PCT_ERR_ARGUMENT: return "invalid argument";
        case PCT_ERR_CUDA: return "CUDA error";
        case PCT_ERR_ALLOC: return "allocation failed";
        case PCT_ERR_STATE: return "stage called out of order";
        case PCT_ERR_OVERFLOW: return "capacity exceeded";
        case PCT_ERR_TIMEOUT: return "device wait timed out";
        case PCT_ERR_IO: return "I/O or format error";
        case PCT_ERR_NUMERIC: return "non-finite value";
    }
    return "unknown status";
}

extern "C" pct_status pct_config_default(pct_config* cfg) {
    if (!cfg) return pct_fail(PCT_ERR_ARGUMENT, "pct_config_default: null config");
    pct_config_fill_defaults(cfg);
    return PCT_OK;
}

extern "C" pct_status pct_geometry_from_config(const pct_config* cfg, pct_geometry* geo) {
    if (!cfg || !geo) return pct_fail(PCT_ERR_ARGUMENT, "pct_geometry_from_config: null argument");
    int e = pct_geometry_derive(cfg, geo);
    if (e) return pct_fail(PCT_ERR_ARGUMENT, "pct_geometry_from_config: invalid geometry (code %d)", e);
    return PCT_OK;
}

/* Struct sizes, so bindings can check their layout against this build. */
extern "C" size_t pct_sizeof(int which) {
    switch (which) {
        case 0: return sizeof(pct_config);
        case 1: return sizeof(pct_geometry);
        case 2: return sizeof(pct_phantom_object);
        case 3: return sizeof(pct_scan_params);
        case 4: return sizeof(pct_counts);
        case 5: return sizeof(pct_drop_stats);
    }
    return 0;
}
