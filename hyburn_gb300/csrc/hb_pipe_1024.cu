// Warp-specialised pipeline kernel instantiations, 1024-thread bound: room for eight producer
// threads per node (see hb_resident.cuh).
#include "hb_resident.cuh"

HB_PIPE_UNIT(1024)
