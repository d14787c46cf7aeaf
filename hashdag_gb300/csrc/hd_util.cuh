// Device utilities: exclusive scan, fills, grow-only scratch buffers.
#pragma once

#include <cstdint>
#include <cstdio>
#include <string>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "hd_common.cuh"

namespace hd {

// ---------------------------------------------------------------- errors ---
struct CudaError {
    cudaError_t code;
    std::string where;
};
#define HD_CUDA(call)                                                                  \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess)                                                         \
            throw ::hd::CudaError{e_, std::string(#call) + " @ " + __FILE__ + ":" +    \
                                          std::to_string(__LINE__)};                   \
    } while (0)
#define HD_LAUNCH_CHECK() HD_CUDA(cudaGetLastError())

struct StatusError {
    hd_status status;
    std::string msg;
};

// -------------------------------------------------------------- scratch ---
// Named grow-only device buffers owned by a context.
class Scratch {
public:
    ~Scratch() { release(); }
    void* get(const char* name, size_t bytes)
    {
        auto& b = bufs_[name];
        if (b.bytes < bytes) {
            if (b.ptr)
                cudaFree(b.ptr);
            b.ptr = nullptr;
            b.bytes = 0;
            size_t want = bytes + bytes / 4 + 256;
            if (cudaMalloc(&b.ptr, want) != cudaSuccess) {
                cudaGetLastError();
                throw StatusError{HD_ERR_OOM, std::string("scratch allocation failed: ") + name + " (" +
                                                  std::to_string(want >> 20) + " MiB)"};
            }
            b.bytes = want;
            note_peak();
        }
        return b.ptr;
    }
    template <typename T>
    T* get(const char* name, size_t count)
    {
        return static_cast<T*>(get(name, count * sizeof(T)));
    }
    // frees one buffer (synchronises the device, as cudaFree does)
    void drop(const char* name)
    {
        auto it = bufs_.find(name);
        if (it == bufs_.end())
            return;
        if (it->second.ptr)
            cudaFree(it->second.ptr);
        bufs_.erase(it);
    }
    size_t peak() const { return peak_; }
    void note_peak()
    {
        const size_t t = total();
        peak_ = t > peak_ ? t : peak_;
    }
    void release()
    {
        for (auto& kv : bufs_)
            if (kv.second.ptr)
                cudaFree(kv.second.ptr);
        bufs_.clear();
    }
    size_t total() const
    {
        size_t t = 0;
        for (auto& kv : bufs_)
            t += kv.second.bytes;
        return t;
    }

private:
    struct Buf {
        void* ptr = nullptr;
        size_t bytes = 0;
    };
    std::unordered_map<std::string, Buf> bufs_;
    size_t peak_ = 0;
};

// ----------------------------------------------------------------- scan ---
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8; // per thread
constexpr int kScanTile = kScanThreads * kScanItems;

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T n = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o)
            v += n;
    }
    return v;
}

// Block-wide exclusive scan of one value per thread; returns the block total.
template <typename T>
__device__ __forceinline__ T block_excl_scan(T v, T* total)
{
    __shared__ T warp_sums[kScanThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T inc = warp_incl_scan(v);
    if (lane == 31)
        warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        T s = lane < kScanThreads / 32 ? warp_sums[lane] : T(0);
        s = warp_incl_scan(s);
        if (lane < kScanThreads / 32)
            warp_sums[lane] = s;
    }
    __syncthreads();
    T base = warp ? warp_sums[warp - 1] : T(0);
    *total = warp_sums[kScanThreads / 32 - 1];
    __syncthreads();
    return base + inc - v;
}

template <typename Tin, typename T>
__global__ void k_scan_tiles(const Tin* __restrict__ in, T* __restrict__ out, T* __restrict__ tile_sums, uint64_t n)
{
    const uint64_t base = uint64_t(blockIdx.x) * kScanTile + uint64_t(threadIdx.x) * kScanItems;
    T vals[kScanItems];
    T sum = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        vals[i] = base + i < n ? T(in[base + i]) : T(0);
        sum += vals[i];
    }
    T total;
    T off = block_excl_scan(sum, &total);
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        if (base + i < n)
            out[base + i] = off;
        off += vals[i];
    }
    if (threadIdx.x == 0 && tile_sums)
        tile_sums[blockIdx.x] = total;
}

template <typename T>
__global__ void k_scan_add(T* __restrict__ out, const T* __restrict__ tile_offsets, uint64_t n)
{
    const uint64_t base = uint64_t(blockIdx.x) * kScanTile;
    const T add = tile_offsets[blockIdx.x];
    for (int i = threadIdx.x; i < kScanTile; i += kScanThreads)
        if (base + i < n)
            out[base + i] += add;
}

// out[i] = sum(in[0..i-1]); *d_total (optional, device) = sum(in).  Recursive
// over tile sums.  Tin converts to T per element.
template <typename Tin, typename T>
void exclusive_scan(Scratch& s, const Tin* in, T* out, uint64_t n, T* d_total, cudaStream_t st, int depth = 0)
{
    if (n == 0) {
        if (d_total)
            HD_CUDA(cudaMemsetAsync(d_total, 0, sizeof(T), st));
        return;
    }
    const uint64_t tiles = (n + kScanTile - 1) / kScanTile;
    char name[32];
    snprintf(name, sizeof(name), "scan_sums_%d", depth);
    T* sums = s.get<T>(name, tiles + 1);
    k_scan_tiles<Tin, T><<<uint32_t(tiles), kScanThreads, 0, st>>>(in, out, sums, n);
    HD_LAUNCH_CHECK();
    if (tiles > 1) {
        char name2[32];
        snprintf(name2, sizeof(name2), "scan_offs_%d", depth);
        T* offs = s.get<T>(name2, tiles + 1);
        exclusive_scan<T, T>(s, sums, offs, tiles, d_total, st, depth + 1);
        k_scan_add<T><<<uint32_t(tiles), kScanThreads, 0, st>>>(out, offs, n);
        HD_LAUNCH_CHECK();
    } else if (d_total) {
        HD_CUDA(cudaMemcpyAsync(d_total, sums, sizeof(T), cudaMemcpyDeviceToDevice, st));
    }
}

// ---------------------------------------------------------------- fills ---
template <typename T>
__global__ void k_fill(T* p, T v, uint64_t n)
{
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
        p[i] = v;
}
template <typename T>
void fill(T* p, T v, uint64_t n, cudaStream_t st)
{
    if (!n)
        return;
    uint64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 64)
        blocks = 152 * 64;
    k_fill<T><<<uint32_t(blocks), 256, 0, st>>>(p, v, n);
    HD_LAUNCH_CHECK();
}

inline uint32_t grid_for(uint64_t n, uint32_t block, uint32_t cap = 152 * 32)
{
    uint64_t b = (n + block - 1) / block;
    if (b == 0)
        b = 1;
    return uint32_t(b < cap ? b : cap);
}

#define HD_GRID_STRIDE(i, n) \
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < (n); i += uint64_t(gridDim.x) * blockDim.x)

template <typename T>
T read_scalar(const T* d, cudaStream_t st)
{
    T h;
    HD_CUDA(cudaMemcpyAsync(&h, d, sizeof(T), cudaMemcpyDeviceToHost, st));
    HD_CUDA(cudaStreamSynchronize(st));
    return h;
}

} // namespace hd
