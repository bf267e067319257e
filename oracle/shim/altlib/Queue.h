// Compatibility shim (test infrastructure): fixed-capacity FIFO ring buffer
// (create, enq, deq, public `size`, free) as used by the reference's
// breadth-first velocity extrapolation.
#pragma once
#include <cstdlib>
#include <cstddef>

template <typename T>
struct Queue {
    T* data = nullptr;
    size_t head = 0;
    size_t size = 0;
    size_t capacity = 0;

    static Queue create(size_t cap) {
        Queue q;
        q.capacity = cap ? cap : 1;
        q.data = (T*)std::malloc(q.capacity * sizeof(T));
        if (!q.data) std::abort();
        return q;
    }
    void enq(const T& v) {
        if (size == capacity) std::abort();
        data[(head + size) % capacity] = v;
        size++;
    }
    T deq() {
        T v = data[head];
        head = (head + 1) % capacity;
        size--;
        return v;
    }
    void free() { std::free(data); data = nullptr; size = capacity = 0; }
};
