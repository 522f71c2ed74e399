// Point-resident kernel instantiations for networks of any shape (see hb_resident.cuh).
#include "hb_resident.cuh"

HB_RESIDENT_UNIT(256)
HB_RESIDENT_UNIT(512)
HB_RESIDENT_UNIT(1024)
