// Compatibility shim (test infrastructure): aligned allocation.
#pragma once
#include <stdlib.h>
#include <cstddef>

inline void* aligned_malloc(size_t align, size_t nbytes) {
    void* p = nullptr;
    if (posix_memalign(&p, align < sizeof(void*) ? sizeof(void*) : align, nbytes ? nbytes : align) != 0) return nullptr;
    return p;
}
inline void aligned_free(void* p) { free(p); }
