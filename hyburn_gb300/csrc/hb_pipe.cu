// Warp-specialised pipeline kernel instantiations, 512-thread bound (see hb_resident.cuh).
#include "hb_resident.cuh"

HB_PIPE_UNIT(512)
