"""resaxs_gb300: GB300-native (sm_103a) Debye / incremental-recalc / SASA hot
path of resaxslib behind a C ABI (``librsx.so``)."""
