// Stand-in for the reference's utility/buffer.h, used only when compiling the
// reference's host LBVH (bvh.h) into the oracle's reference build. The
// reference header does not compile with g++ 13 (a template parameter that
// shadows another); the LBVH code needs nothing from it but these names.
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
    T* data() { return m_host.data(); }
    const T* data() const { return m_host.data(); }
    size_t size() const { return m_host.size(); }
    void copyFrom(size_t count, BufferType, const T* src) { m_host.assign(src, src + count); }
    void resize(size_t count) { m_host.resize(count); }
    void clear() { m_host.assign(m_host.size(), T()); }

private:
    std::vector<T> m_host;
};
