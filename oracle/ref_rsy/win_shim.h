// ORACLE — test infrastructure only. The two Windows C runtime names that the
// reference's asset file code (src/Asset/Asset.cpp) uses, so that it compiles
// unchanged with g++ for the golden-file recipe in this directory.
#pragma once
#include <cerrno>
#include <cstdio>

typedef int errno_t;

inline errno_t fopen_s(FILE** file, const char* path, const char* mode) {
    *file = std::fopen(path, mode);
    return *file ? 0 : (errno ? errno : 1);
}
