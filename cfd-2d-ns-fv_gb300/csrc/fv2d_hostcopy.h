// Host <-> device transfers of large host buffers.  A page-locked caller buffer is the DMA endpoint
// itself; a pageable one goes through a pinned staging buffer without the single-threaded memcpy
// being the bottleneck: the host copy is split over a pool of threads, and the transfer is cut into
// chunks so chunk k's DMA overlaps chunk k+1's host copy.
#pragma once

#include <algorithm>
#include <condition_variable>
#include <cstddef>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include <unistd.h>

#include <cuda_runtime.h>

namespace fv2d {

// Process-wide pool of copy threads (created on first use, never torn down: the process exit
// reclaims them).  One job at a time; the calling thread takes a share of every job.
class CopyPool {
public:
    static CopyPool& get() {
        static CopyPool* p = new CopyPool();
        return *p;
    }

    void copy(void* dst, const void* src, size_t bytes) {
        if (bytes < kParallelMin || workers_.empty() || getpid() != pid_) {   // a forked child has no workers
            std::memcpy(dst, src, bytes);
            return;
        }
        std::lock_guard<std::mutex> job_lock(job_);
        const int parts = (int)workers_.size() + 1;
        {
            std::lock_guard<std::mutex> lk(m_);
            dst_ = (char*)dst;
            src_ = (const char*)src;
            bytes_ = bytes;
            parts_ = parts;
            pending_ = parts - 1;
            ++gen_;
        }
        cv_.notify_all();
        part(parts - 1);   // the caller's share
        std::unique_lock<std::mutex> lk(m_);
        done_.wait(lk, [&] { return pending_ == 0; });
    }

private:
    static constexpr size_t kParallelMin = size_t(1) << 20;

    CopyPool() : pid_(getpid()) {
        const unsigned hw = std::thread::hardware_concurrency();
        const int n = (int)std::min(15u, hw > 1 ? hw - 1 : 0u);
        for (int i = 0; i < n; i++) workers_.emplace_back([this, i] { loop(i); });
        for (auto& t : workers_) t.detach();
    }

    void part(int i) {
        // 64-byte aligned split points; parts_ x per covers every byte
        const size_t per = (((bytes_ + parts_ - 1) / parts_) + 63) & ~size_t(63);
        const size_t b = std::min(bytes_, per * (size_t)i), e = std::min(bytes_, b + per);
        if (e > b) std::memcpy(dst_ + b, src_ + b, e - b);
    }

    void loop(int i) {
        unsigned long long seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(m_);
                cv_.wait(lk, [&] { return gen_ != seen; });
                seen = gen_;
            }
            part(i);
            std::lock_guard<std::mutex> lk(m_);
            if (--pending_ == 0) done_.notify_one();
        }
    }

    const pid_t pid_;
    std::vector<std::thread> workers_;
    std::mutex job_, m_;
    std::condition_variable cv_, done_;
    char* dst_ = nullptr;
    const char* src_ = nullptr;
    size_t bytes_ = 0;
    int parts_ = 1, pending_ = 0;
    unsigned long long gen_ = 0;
};

constexpr size_t kCopyChunk = size_t(8) << 20;

// Page-locked (cudaMallocHost / cudaHostRegister) host memory can be the DMA endpoint itself.
inline bool host_pinned(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();   // clear the error this query set
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// host (pageable) -> device through `stage` (pinned, >= bytes); returns the first CUDA error.
// `stage_free` is recorded after the last DMA and waited on before the staging buffer is written
// again, so a second upload never overwrites data an earlier one has not transferred yet.
inline cudaError_t staged_h2d(void* dev, const void* host, size_t bytes, void* stage, cudaStream_t s,
                              cudaEvent_t stage_free) {
    if (host_pinned(host)) return cudaMemcpyAsync(dev, host, bytes, cudaMemcpyHostToDevice, s);
    cudaError_t e = cudaEventSynchronize(stage_free);
    for (size_t off = 0; e == cudaSuccess && off < bytes; off += kCopyChunk) {
        const size_t n = std::min(kCopyChunk, bytes - off);
        CopyPool::get().copy((char*)stage + off, (const char*)host + off, n);
        e = cudaMemcpyAsync((char*)dev + off, (char*)stage + off, n, cudaMemcpyHostToDevice, s);
    }
    if (e == cudaSuccess) e = cudaEventRecord(stage_free, s);
    return e;
}

// device -> host (pageable) through `stage`; `events` holds one reusable event per chunk slot.
inline cudaError_t staged_d2h(void* host, const void* dev, size_t bytes, void* stage, cudaStream_t s,
                              std::vector<cudaEvent_t>& events) {
    if (host_pinned(host)) {
        const cudaError_t e = cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, s);
        return e == cudaSuccess ? cudaStreamSynchronize(s) : e;
    }
    const size_t chunks = (bytes + kCopyChunk - 1) / kCopyChunk;
    while (events.size() < chunks) {
        cudaEvent_t ev;
        const cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e != cudaSuccess) return e;
        events.push_back(ev);
    }
    for (size_t k = 0; k < chunks; k++) {
        const size_t off = k * kCopyChunk, n = std::min(kCopyChunk, bytes - off);
        cudaError_t e = cudaMemcpyAsync((char*)stage + off, (const char*)dev + off, n, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaEventRecord(events[k], s);
        if (e != cudaSuccess) return e;
    }
    for (size_t k = 0; k < chunks; k++) {
        const size_t off = k * kCopyChunk, n = std::min(kCopyChunk, bytes - off);
        const cudaError_t e = cudaEventSynchronize(events[k]);
        if (e != cudaSuccess) return e;
        CopyPool::get().copy((char*)host + off, (const char*)stage + off, n);
    }
    return cudaSuccess;
}

}  // namespace fv2d
