// Compatibility shim (test infrastructure): `defer { ... };` scope guard.
#pragma once
#include <utility>

template <typename F>
struct ShimDeferGuard {
    F f;
    ~ShimDeferGuard() { f(); }
};
struct ShimDeferMaker {
    template <typename F> ShimDeferGuard<F> operator+(F f) { return ShimDeferGuard<F>{std::move(f)}; }
};
#define SHIM_DEFER_CAT2(a, b) a##b
#define SHIM_DEFER_CAT(a, b) SHIM_DEFER_CAT2(a, b)
#define defer auto SHIM_DEFER_CAT(shim_defer_, __LINE__) = ShimDeferMaker() + [&]()
