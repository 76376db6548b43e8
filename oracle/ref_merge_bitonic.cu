// Test infrastructure only: the reference's host merge of per-stream top-k lists
// (mergeResBitonic, src/cuknnBitonic.cu:381-417) under a C name, compiled from the
// reference's own source file (the include path is given by oracle/build_ref.py).
// Nothing here is shipped, measured or run on a GPU.
#include "cuknnBitonic.cu"

extern "C" void ref_merge_bitonic(float* data, float* idx, int k, int Q, int numStreams)
{
    mergeResBitonic(data, idx, k, Q, numStreams);
}
