// Compatibility shim (test infrastructure): the reference includes
// "immintrin.h" unconditionally.  Builds without USE_AVX_SIMD (the
// reference's own `USE_AVX=OFF` configuration, and every non-x86 host)
// take this empty stand-in and compile only the scalar code paths.
#pragma once
