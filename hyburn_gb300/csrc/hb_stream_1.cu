// streamed-history pipeline kernels: 1 node(s) per consumer thread, 512 threads
#include "hb_stream.cuh"
HB_STREAM_UNIT(1, 512)
