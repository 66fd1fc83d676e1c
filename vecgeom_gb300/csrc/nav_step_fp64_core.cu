// Plain-FP64 step kernel with the dispatch of the core shape set only (kCoreShapeMask); the
// compile switches are those of kernels_nav_fp64.cu.
#define VG_FP64_INT_COMPARE 0
#define VG_FP64_SHORTCUTS 0
#define VG_INLINE_CONTAINS 1
#define VG_NAV_SET set_core
#define VG_SHAPE_MASK vg::kCoreShapeMask
#include "nav_fp64_step_impl.cuh"
