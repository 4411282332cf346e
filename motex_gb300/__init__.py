"""GB300-native word-based motif extraction (MoTeX hot path).

* ``motex_gb300.native``     -- ctypes binding of the C ABI (include/motex_gpu.h)
* ``motex_gb300.build``      -- in-tree build of libmotex_gpu.so and motexGPU
* ``motex_gb300.workloads``  -- seeded synthetic workloads
"""
__all__ = ["native", "build", "workloads"]
