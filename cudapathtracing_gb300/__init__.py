"""GB300-native path-tracing hot path (LBVH build + trace loop) behind a C ABI.

The compute path is libcpt.so (hand-written sm_103a CUDA, see include/cpt.h); this package
holds its ctypes binding (`_lib`), the data layouts (`abi`), a thin host API (`api`) and
the seeded procedural workloads (`procedural`).
"""
__all__ = ["abi", "procedural"]
