// Specialised single-projection resident kernel instantiations with launch bound 1024 (see hb_resident.cuh).
#include "hb_resident.cuh"

HB_FAST_UNIT(1024)
