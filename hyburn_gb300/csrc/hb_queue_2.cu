// work-queue kernel of grouped launches: 2 node(s) per consumer thread, 1024 threads
#include "hb_stream.cuh"
HB_QUEUE_UNIT(2, 1024)
