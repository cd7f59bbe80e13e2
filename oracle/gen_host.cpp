/*
 * Host-only build of the seeded scan generator — TEST INFRASTRUCTURE ONLY.
 *
 * oracle/build_oracle.py links this file with pct_gb300/csrc/phantom.cpp into
 * oracle/_build/libpct_gen.so, so that a caller that must not map the CUDA
 * library (bench.py's CPU reference arm) can make the same seeded histories.
 * phantom.cpp reports errors through pct_fail, defined here.
 */
#include <cstdarg>
#include <cstdio>
#include "pct_internal.h"

static thread_local char g_gen_error[512] = "";

pct_status pct_fail(pct_status s, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_gen_error, sizeof(g_gen_error), fmt, ap);
    va_end(ap);
    return s;
}

extern "C" const char* pct_gen_last_error(void) { return g_gen_error; }
