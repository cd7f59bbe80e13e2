"""pct_gb300: GB300-native proton-CT reconstruction (binning, cuts, hulls, FBP, MLP, DROP).

The compute path is the CUDA library pct_gb300/_lib/libpct_gb300.so reached
through its C ABI (include/pct.h); this package holds the host-side mirror of
the reference's stage sequence, the PCTD reader/writer and the synthetic
workload generator.
"""
from . import _capi  # noqa: F401
