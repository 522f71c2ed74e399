// streamed-history pipeline kernels: 2 nodes per consumer thread, 1024 threads
#include "hb_stream.cuh"
HB_STREAM_UNIT(2, 1024)
