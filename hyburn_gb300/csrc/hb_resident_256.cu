// Point-resident kernel instantiations with launch bound 256 (see hb_resident.cuh).
#include "hb_resident.cuh"

HB_RESIDENT_UNIT(256)
