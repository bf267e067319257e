// Compatibility shim (test infrastructure): growable array with the surface
// the reference simulator uses (create, emptyWithSize, push, resize,
// operator[], public `data`/`size`, free).  Copies are shallow, as the
// simulator passes Vec by value and frees it explicitly.
#pragma once
#include <cstdlib>
#include <cstring>
#include <cstddef>

template <typename T>
struct Vec {
    T* data = nullptr;
    size_t size = 0;
    size_t capacity = 0;

    static Vec create(size_t cap) {
        Vec v;
        v.reserve(cap < 4 ? 4 : cap);
        return v;
    }

    static Vec emptyWithSize(size_t n) {
        Vec v;
        v.reserve(n < 4 ? 4 : n);
        v.size = n;
        return v;
    }

    void reserve(size_t cap) {
        if (cap <= capacity) return;
        T* nd = (T*)std::realloc((void*)data, cap * sizeof(T));
        if (!nd) { std::abort(); }
        std::memset((void*)(nd + capacity), 0, (cap - capacity) * sizeof(T));
        data = nd;
        capacity = cap;
    }

    void push(const T& value) {
        if (size == capacity) reserve(capacity ? capacity * 2 : 4);
        std::memcpy((void*)(data + size), (const void*)&value, sizeof(T));
        size++;
    }

    void resize(size_t n) {
        reserve(n);
        if (n > size) std::memset((void*)(data + size), 0, (n - size) * sizeof(T));
        size = n;
    }

    T& operator[](size_t i) { return data[i]; }
    const T& operator[](size_t i) const { return data[i]; }

    void free() {
        std::free((void*)data);
        data = nullptr;
        size = capacity = 0;
    }
};
