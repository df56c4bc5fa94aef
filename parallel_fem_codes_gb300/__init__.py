"""GB300-native solve path for 2-D stabilised P1 finite elements.

A single-GPU replacement for the MPI solve path of PARALLEL_FEM_CODES:
element-by-element matvecs, preconditioners, restarted GMRES (plain FP64
and FP32-in-FP64 refinement), batched solves and device-side SUPG/CAU
assembly, behind the C ABI declared in include/femgpu.h.

Submodules: ``femgpu`` (ctypes binding of libfemgpu), ``meshgen``
(synthetic meshes and problems), ``build`` (in-tree compilation).
"""
