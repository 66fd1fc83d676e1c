// Scheduled step kernels with the dispatch of every shape type.
#define VG_NAV_SET set_all
#include "nav_queue_impl.cuh"
