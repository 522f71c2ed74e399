// work-queue kernel of grouped launches: 1 node(s) per consumer thread, 512 threads
#include "hb_stream.cuh"
HB_QUEUE_UNIT(1, 512)
