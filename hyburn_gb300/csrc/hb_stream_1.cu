// streamed-history pipeline kernels: 1 node per consumer thread, 512 threads
#include "hb_stream.cuh"
HB_STREAM_UNIT(1, 512)
