// Test infrastructure only: the reference's host merge of per-stream top-k lists of
// the heap path (mergeResHeap, src/cuknnHeap.cu:26-59) under a C name, compiled from
// the reference's own source file (the include path is given by oracle/build_ref.py).
// Nothing here is shipped, measured or run on a GPU.
#include "cuknnHeap.cu"

extern "C" void ref_merge_heap(float* data, float* idx, int k, int Q, int numStreams)
{
    mergeResHeap(data, idx, k, Q, numStreams);
}
