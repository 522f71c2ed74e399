// streamed-history pipeline kernels: 4 nodes per consumer thread, 1024 threads
#include "hb_stream.cuh"
HB_STREAM_UNIT(4, 1024)
