// Warp-specialised pipeline kernel instantiations (see hb_resident.cuh).
#include "hb_resident.cuh"

HB_PIPE_UNIT
