/* Emulation stub: the real declarations come from pct_ref_prelude.h (test infrastructure only). */
#include "pct_ref_prelude.h"
