"""Host-side Python mirror of the GB300 FVM_TVD drop-in (ctypes over libcfd2d_gpu.so)."""
