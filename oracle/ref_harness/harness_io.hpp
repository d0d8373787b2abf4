// Oracle harness helpers — ORACLE TEST INFRASTRUCTURE ONLY.
//
// The harness programs in this directory include the reference framework's own
// headers (APPFIS_CPU build, single-rank MPI stand-in) and drive its public API
// (Grid / Scatter / Config / Execute*D / Execute*DReduce / Gather) on seeded
// inputs read from raw binary files.  Their outputs pin the C restatement in
// oracle/appfis_oracle.c and provide the golden fixtures under tests/golden/.
#pragma once

#include <chrono>
#include <cmath>
#include <iostream>
#include <limits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace harness {

inline std::vector<char> read_file(const char* path, size_t expect)
{
    std::vector<char> buf(expect);
    FILE* f = std::fopen(path, "rb");
    if (!f) { std::fprintf(stderr, "cannot open %s\n", path); std::exit(2); }
    size_t got = std::fread(buf.data(), 1, expect, f);
    std::fclose(f);
    if (got != expect) { std::fprintf(stderr, "%s: expected %zu bytes, got %zu\n", path, expect, got); std::exit(2); }
    return buf;
}

inline void write_file(const char* path, const void* data, size_t bytes)
{
    FILE* f = std::fopen(path, "wb");
    if (!f) { std::fprintf(stderr, "cannot write %s\n", path); std::exit(2); }
    std::fwrite(data, 1, bytes, f);
    std::fclose(f);
}

struct Clock {
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    double seconds() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

inline int arg_int(int argc, char** argv, int i)
{
    if (i >= argc) { std::fprintf(stderr, "missing argument %d\n", i); std::exit(2); }
    return std::atoi(argv[i]);
}

inline double arg_f(int argc, char** argv, int i)
{
    if (i >= argc) { std::fprintf(stderr, "missing argument %d\n", i); std::exit(2); }
    return std::atof(argv[i]);
}

}  // namespace harness
