// Stand-in for the reference's utility/buffer.h, used when compiling reference
// code into the oracle's reference builds (host LBVH, device kernels, record
// layout and host records); "device" buffers are host vectors here. The
// reference header does not compile with g++ 13 (a template parameter that
// shadows another); the code compiled against it needs nothing but these names.
#pragma once
#include <cstddef>
#include <cstdlib>
#include <iostream>
#include <vector>

#define CUDA_CHECK(code)                                                   \
    {                                                                      \
        cudaError_t err__ = (code);                                        \
        if (err__ != cudaSuccess) {                                        \
            std::cerr << "CUDA error " << cudaGetErrorString(err__) << "\n"; \
            std::abort();                                                  \
        }                                                                  \
    }

enum BufferType { HOST_BUFFER, DEVICE_BUFFER };

template <BufferType TYPE, typename T>
class Buffer {
public:
    Buffer(size_t count = 0) : m_host(count) {}
    // copies between buffer kinds (framebuffer.cpp:13-14 reads a device buffer
    // back this way)
    template <BufferType U>
    Buffer(const Buffer<U, T>& other) : m_host(other.data(), other.data() + other.size()) {}
    T operator[](size_t i) const { return m_host[i]; }
    T& operator[](size_t i) { return m_host[i]; }
    // the reference's Buffer hands out a mutable pointer from a const object
    // (environment.cpp:5 relies on it)
    T* data() const { return const_cast<T*>(m_host.data()); }
    size_t size() const { return m_host.size(); }
    void copyFrom(size_t count, BufferType, const T* src) { m_host.assign(src, src + count); }
    void resize(size_t count) { m_host.resize(count); }
    void clear() { m_host.assign(m_host.size(), T()); }

private:
    std::vector<T> m_host;
};
