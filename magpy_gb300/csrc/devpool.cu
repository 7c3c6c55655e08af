// devpool.cu -- a cache of device blocks for plan buffers.
//
// Creating and destroying a plan per call (the ensemble entry points do) would
// otherwise pay a cudaMalloc / cudaFree per buffer, each of which can cost
// tens of microseconds and cudaFree synchronises the device.  Freed blocks are
// kept per device and size class and handed out again.  A block is returned
// only when no kernel uses it any more: temporaries after their stream has
// been synchronised, plan buffers after the device has been (the plan's
// destructor does it); any other free synchronises the device first, as
// cudaFree does.
#include <map>
#include <mutex>
#include <unordered_map>
#include <vector>
#include <cuda_runtime.h>
#include "plan.hpp"

namespace magpy {

namespace {

constexpr size_t CACHE_LIMIT = (size_t)4 << 30;  // cached bytes per device

struct Pool {
    std::mutex mu;
    std::map<std::pair<int, size_t>, std::vector<void *>> free_blocks;
    std::unordered_map<void *, std::pair<int, size_t>> live;
    std::map<int, size_t> cached;
};

Pool &pool()
{
    static Pool *p = new Pool();  // never destroyed: blocks may be returned at exit
    return *p;
}

size_t size_class(size_t bytes)
{
    if (bytes <= 256) return 256;
    if (bytes <= ((size_t)1 << 20)) {
        size_t c = 512;
        while (c < bytes) c <<= 1;
        return c;
    }
    const size_t g = (size_t)2 << 20;  // 2 MiB granules above 1 MiB
    return (bytes + g - 1) / g * g;
}

}  // namespace

cudaError_t pool_alloc(void **ptr, size_t bytes)
{
    *ptr = nullptr;
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return err;
    const size_t c = size_class(bytes);
    Pool &P = pool();
    {
        std::lock_guard<std::mutex> lock(P.mu);
        auto it = P.free_blocks.find({dev, c});
        if (it != P.free_blocks.end() && !it->second.empty()) {
            *ptr = it->second.back();
            it->second.pop_back();
            P.cached[dev] -= c;
            P.live[*ptr] = {dev, c};
            return cudaSuccess;
        }
    }
    err = cudaMalloc(ptr, c);
    if (err == cudaErrorMemoryAllocation) {
        (void)cudaGetLastError();
        pool_trim(dev);
        err = cudaMalloc(ptr, c);
    }
    if (err != cudaSuccess) { *ptr = nullptr; return err; }
    std::lock_guard<std::mutex> lock(P.mu);
    P.live[*ptr] = {dev, c};
    return cudaSuccess;
}

void pool_free(void *ptr, bool device_synced)
{
    if (!ptr) return;
    // as cudaFree would, wait until no kernel can still be using the block
    if (!device_synced) cudaDeviceSynchronize();
    Pool &P = pool();
    std::unique_lock<std::mutex> lock(P.mu);
    auto it = P.live.find(ptr);
    if (it == P.live.end()) {  // not ours
        lock.unlock();
        cudaFree(ptr);
        return;
    }
    const int dev = it->second.first;
    const size_t c = it->second.second;
    P.live.erase(it);
    if (P.cached[dev] + c > CACHE_LIMIT) {
        lock.unlock();
        cudaFree(ptr);
        return;
    }
    P.free_blocks[{dev, c}].push_back(ptr);
    P.cached[dev] += c;
}

void pool_trim(int dev)
{
    Pool &P = pool();
    std::vector<void *> drop;
    {
        std::lock_guard<std::mutex> lock(P.mu);
        for (auto &kv : P.free_blocks)
            if (kv.first.first == dev) {
                drop.insert(drop.end(), kv.second.begin(), kv.second.end());
                kv.second.clear();
            }
        P.cached[dev] = 0;
    }
    int cur = 0;
    cudaGetDevice(&cur);
    if (cur != dev) cudaSetDevice(dev);
    for (void *p : drop) cudaFree(p);
    if (cur != dev) cudaSetDevice(cur);
}

}  // namespace magpy
