// work-queue kernel of grouped launches: 4 node(s) per consumer thread, 768 threads
#include "hb_stream.cuh"
HB_QUEUE_UNIT(4, 768)
