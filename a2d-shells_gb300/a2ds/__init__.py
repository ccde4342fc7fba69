"""Host-side Python access to the GB300 buckling path (ctypes over the C-ABI
declared in include/a2ds.h) plus the synthetic-mesh generators."""
