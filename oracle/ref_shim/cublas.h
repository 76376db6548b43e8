/* Test infrastructure only: stands in for the legacy cuBLAS header when the
 * reference's merges are compiled (oracle/build_ref.py).  The reference includes
 * both cublas.h and cublas_v2.h, which current cuBLAS refuses in one unit; its
 * code uses the v2 API only, so the legacy header is left empty here. */
