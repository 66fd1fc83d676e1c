// Transport-stream kernels with the dispatch of the core shape set only (kCoreShapeMask).
#define VG_NAV_SET set_core
#define VG_SHAPE_MASK vg::kCoreShapeMask
#include "nav_transport_impl.cuh"
