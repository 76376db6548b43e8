// knn_test.cpp -- the reference's file-based test driver (src/knnTest.cu) over
// the GB300 libraries, same command line and file formats:
//
//   knn_test <datafile> <queryfile> N Q D k
//
// <datafile> holds N*D and <queryfile> Q*D raw knntype values, each vector's
// D values contiguous (demo/exportData.m writes MATLAB's d x N matrices that
// way); the driver plans (knnsplan), searches (knnsexecute, which prints
// "Time Elapsed: <s>") and writes k*Q values to KNNdist.bin and KNNidx.bin in
// the working directory, k contiguous per query, indices 0-based
// (demo/importData.m reads them as [k Q] matrices).  Built twice: knn_test
// (float, libknngb300.so) and knn_test_double (-D__DOUBLE__,
// libknngb300_double.so), as the reference builds knnTest and knnTestDouble.
// Unlike the reference, a missing or short input file is an error (exit 1)
// instead of a search of uninitialised memory.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "cuknns.h"

static bool load(std::vector<knntype>& a, const char* file, size_t n)
{
    printf("Loading data from file: %s\n", file);
    FILE* f = fopen(file, "rb");
    if (!f) {
        fprintf(stderr, "Can't open input file %s\n", file);
        return false;
    }
    a.resize(n);
    const size_t got = fread(a.data(), sizeof(knntype), n, f);
    fclose(f);
    if (got != n) {
        fprintf(stderr, "%s holds %zu values, %zu expected\n", file, got, n);
        return false;
    }
    return true;
}

static bool save(const std::vector<knntype>& a, const char* file)
{
    printf("Saving data to file: %s\n", file);
    FILE* f = fopen(file, "wb");
    if (!f) {
        fprintf(stderr, "Can't open output file %s\n", file);
        return false;
    }
    const size_t put = fwrite(a.data(), sizeof(knntype), a.size(), f);
    fclose(f);
    return put == a.size();
}

int main(int argc, char** argv)
{
    if (argc != 7) {
        fprintf(stderr, "usage: %s <datafile> <queryfile> N Q D k\n", argv[0]);
        return 2;
    }
    const long N = atol(argv[3]), Q = atol(argv[4]), D = atol(argv[5]), k = atol(argv[6]);
    if (N <= 0 || Q <= 0 || D <= 0 || k <= 0 || k > N) {
        fprintf(stderr, "need N, Q, D >= 1 and 1 <= k <= N\n");
        return 2;
    }
    printf("files: %s %s\n", argv[1], argv[2]);
    std::vector<knntype> data, queries;
    if (!load(data, argv[1], (size_t)N * D) || !load(queries, argv[2], (size_t)Q * D)) return 1;
    std::vector<knntype> dist((size_t)Q * k), idx((size_t)Q * k);
    knnplan plan;
    knnsplan(&plan, N, Q, D, k);
    if (!plan.pt2Function) {
        fprintf(stderr, "knnsplan failed\n");
        return 1;
    }
    knnsexecute(plan, data.data(), queries.data(), dist.data(), idx.data());
    if (!save(dist, "KNNdist.bin") || !save(idx, "KNNidx.bin")) return 1;
    return 0;
}
