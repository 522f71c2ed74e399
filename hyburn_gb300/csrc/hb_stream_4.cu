// streamed-history pipeline kernels: 4 nodes per consumer thread, up to 768 threads (two edge
// windows in flight per producer thread)
#include "hb_stream.cuh"
HB_STREAM_UNIT(4, 768)
