// runtime.h — host-side runtime of the C-ABI: error reporting, device buffers,
// temporary workspaces and launch accounting.
#pragma once

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "gbsa.h"

namespace gbsa {

// Exceptions never cross the C-ABI: every entry point catches Error and returns its
// code, with the message stored for gbsa_last_error().
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& msg);

#define GBSA_CUDA(call)                                                                                      \
    do {                                                                                                     \
        cudaError_t _e = (call);                                                                             \
        if (_e != cudaSuccess) {                                                                             \
            throw ::gbsa::Error(_e == cudaErrorMemoryAllocation ? GBSA_ERR_NOMEM : GBSA_ERR_CUDA,            \
                                std::string(#call " failed: ") + cudaGetErrorString(_e) + " at " __FILE__ ":" \
                                    + std::to_string(__LINE__));                                             \
        }                                                                                                    \
    } while (0)

// Counts kernel launches issued by this library (reported by gbsa_launch_count).
extern std::atomic<uint64_t> g_launches;
#define GBSA_LAUNCHED()                                                                                     \
    do {                                                                                                    \
        ::gbsa::g_launches.fetch_add(1, std::memory_order_relaxed);                                         \
        GBSA_CUDA(cudaGetLastError());                                                                      \
    } while (0)

// Owning device buffer.
class DeviceBuffer {
public:
    DeviceBuffer() = default;
    explicit DeviceBuffer(size_t bytes) { resize(bytes); }
    ~DeviceBuffer() { release(); }
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    DeviceBuffer(DeviceBuffer&& o) noexcept : p_(o.p_), n_(o.n_) {
        o.p_ = nullptr;
        o.n_ = 0;
    }
    DeviceBuffer& operator=(DeviceBuffer&& o) noexcept {
        if (this != &o) {
            release();
            p_ = o.p_;
            n_ = o.n_;
            o.p_ = nullptr;
            o.n_ = 0;
        }
        return *this;
    }
    void resize(size_t bytes) {
        if (bytes <= n_) return;
        release();
        void* p = nullptr;
        GBSA_CUDA(cudaMalloc(&p, bytes ? bytes : 16));
        p_ = p;
        n_ = bytes;
    }
    void release() {
        if (p_) cudaFree(p_);
        p_ = nullptr;
        n_ = 0;
    }
    template <class T>
    T* as() const {
        return static_cast<T*>(p_);
    }
    size_t size() const { return n_; }

private:
    void* p_ = nullptr;
    size_t n_ = 0;
};

// Pinned host buffer.
class PinnedBuffer {
public:
    PinnedBuffer() = default;
    ~PinnedBuffer() {
        if (p_) cudaFreeHost(p_);
    }
    PinnedBuffer(const PinnedBuffer&) = delete;
    PinnedBuffer& operator=(const PinnedBuffer&) = delete;
    void resize(size_t bytes) {
        if (bytes <= n_) return;
        if (p_) cudaFreeHost(p_);
        p_ = nullptr;
        n_ = 0;
        GBSA_CUDA(cudaMallocHost(&p_, bytes ? bytes : 16));
        n_ = bytes;
    }
    template <class T>
    T* as() const {
        return static_cast<T*>(p_);
    }
    size_t size() const { return n_; }

private:
    void* p_ = nullptr;
    size_t n_ = 0;
};

// Grow-only pool of temporary device buffers, handed out in order and recycled by
// reset().  Not thread-safe; one per handle.
class Workspace {
public:
    void* get(size_t bytes) {
        bytes = (bytes + 255) & ~size_t(255);
        if (next_ == bufs_.size()) bufs_.emplace_back();
        DeviceBuffer& b = bufs_[next_++];
        b.resize(bytes);
        return b.as<void>();
    }
    template <class T>
    T* get(size_t n) {
        return static_cast<T*>(get(n * sizeof(T)));
    }
    void reset() { next_ = 0; }

private:
    std::vector<DeviceBuffer> bufs_;
    size_t next_ = 0;
};

inline unsigned grid_for(size_t n, unsigned block, unsigned max_blocks = 1u << 30) {
    size_t g = (n + block - 1) / block;
    if (g == 0) g = 1;
    if (g > max_blocks) g = max_blocks;
    return (unsigned)g;
}

int device_sm_count();

// Runs fn(begin, end) over [0, n) in chunks on a process-wide pool of host threads
// (the calling thread takes part); small ranges run inline.  For the per-read host
// loops of the C-ABI (staging offsets, rebasing results).
void host_parallel_for(size_t n, const std::function<void(size_t, size_t)>& fn);

// Runs fn(i) for i in [0, n) as separate tasks on the same pool (one task per
// thread at a time); for a few coarse tasks.
void host_parallel_tasks(size_t n, const std::function<void(size_t)>& fn);

}  // namespace gbsa
