// Transport-stream kernels with the dispatch of every shape type.
#define VG_NAV_SET set_all
#include "nav_transport_impl.cuh"
