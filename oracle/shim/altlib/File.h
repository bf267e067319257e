// Compatibility shim (test infrastructure): File::open(...).unwrap(),
// writeAll, close; String::fmt(...).unwrap(), data(), free().
#pragma once
#include <cstdio>
#include <cstdlib>
#include <cstdarg>
#include <cstring>
#include "Vec.h"

template <typename T>
struct ShimResult {
    T value;
    bool ok;
    T unwrap() { if (!ok) { std::fprintf(stderr, "unwrap on error\n"); std::abort(); } return value; }
};

struct String {
    char* buf = nullptr;
    static ShimResult<String> fmt(const char* f, ...) {
        va_list ap;
        va_start(ap, f);
        int n = std::vsnprintf(nullptr, 0, f, ap);
        va_end(ap);
        String s;
        s.buf = (char*)std::malloc((size_t)n + 1);
        va_start(ap, f);
        std::vsnprintf(s.buf, (size_t)n + 1, f, ap);
        va_end(ap);
        return ShimResult<String>{s, s.buf != nullptr};
    }
    const char* data() const { return buf; }
    void free() { std::free(buf); buf = nullptr; }
};

struct File {
    FILE* fp = nullptr;
    static ShimResult<File> open(const char* name, const char* mode) {
        File f;
        f.fp = std::fopen(name, mode);
        return ShimResult<File>{f, f.fp != nullptr};
    }
    void writeAll(const char* s) { std::fputs(s, fp); }
    void close() { if (fp) std::fclose(fp); fp = nullptr; }
};
