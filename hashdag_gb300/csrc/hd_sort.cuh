// Stable LSD radix sort of (key, value) uint32 pairs, 8-bit digits.
//
// Used to group find-or-add candidates by bucket while keeping their
// depth-first order inside each bucket: every pass is stable, so values that
// enter in increasing order stay in increasing order within equal keys.
#pragma once

#include "hd_util.cuh"

namespace hd {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;

__global__ void __launch_bounds__(kSortThreads)
    k_radix_hist(const uint32_t* __restrict__ keys, uint32_t n, uint32_t shift, uint32_t* __restrict__ hist)
{
    __shared__ uint32_t cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * kSortTile;
    for (int k = 0; k < kSortItems; k++) {
        const uint32_t i = base + k * kSortThreads + threadIdx.x;
        if (i < n)
            atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * gridDim.x + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void __launch_bounds__(kSortThreads)
    k_radix_scatter(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals, uint32_t n, uint32_t shift,
                    const uint32_t* __restrict__ offs, uint32_t* __restrict__ keys_out,
                    uint32_t* __restrict__ vals_out)
{
    __shared__ uint32_t run[256];
    run[threadIdx.x] = 0;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t base = blockIdx.x * kSortTile;
    for (int k = 0; k < kSortItems; k++) {
        const uint32_t i = base + k * kSortThreads + threadIdx.x;
        const bool valid = i < n;
        const uint32_t key = valid ? keys[i] : 0u;
        const uint32_t val = valid ? vals[i] : 0u;
        const uint32_t digit = valid ? (key >> shift) & 255u : 256u + lane; // invalid lanes stay alone
        const uint32_t peers = __match_any_sync(0xffffffffu, digit);
        const uint32_t leader = __ffs(peers) - 1;
        // warps of this round in order: elements keep their input order
        for (uint32_t w = 0; w < kSortThreads / 32; w++) {
            __syncthreads();
            if (warp == w) {
                uint32_t b = 0;
                if (valid && lane == leader) {
                    b = run[digit];
                    run[digit] = b + __popc(peers);
                }
                b = __shfl_sync(0xffffffffu, b, leader);
                if (valid) {
                    const uint32_t pos = offs[digit * gridDim.x + blockIdx.x] + b + __popc(peers & lt);
                    keys_out[pos] = key;
                    vals_out[pos] = val;
                }
            }
        }
    }
}

// Sorts n pairs by the low `bits` bits of the keys.  keys/vals hold the
// input; the result is written back into keys/vals (the scratch buffers
// serve as the ping-pong side).
inline void radix_sort_pairs(Scratch& s, uint32_t* keys, uint32_t* vals, uint32_t n, uint32_t bits, cudaStream_t st)
{
    if (n <= 1)
        return;
    const uint32_t blocks = (n + kSortTile - 1) / kSortTile;
    uint32_t* hist = s.get<uint32_t>("sort_hist", uint64_t(256) * blocks);
    uint32_t* offs = s.get<uint32_t>("sort_offs", uint64_t(256) * blocks);
    uint32_t* k2 = s.get<uint32_t>("sort_keys2", n);
    uint32_t* v2 = s.get<uint32_t>("sort_vals2", n);
    uint32_t *ka = keys, *va = vals, *kb = k2, *vb = v2;
    uint32_t passes = (bits + 7) / 8;
    for (uint32_t p = 0; p < passes; p++) {
        k_radix_hist<<<blocks, kSortThreads, 0, st>>>(ka, n, 8 * p, hist);
        HD_LAUNCH_CHECK();
        exclusive_scan<uint32_t, uint32_t>(s, hist, offs, uint64_t(256) * blocks, nullptr, st);
        k_radix_scatter<<<blocks, kSortThreads, 0, st>>>(ka, va, n, 8 * p, offs, kb, vb);
        HD_LAUNCH_CHECK();
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    if (ka != keys) {
        HD_CUDA(cudaMemcpyAsync(keys, ka, uint64_t(n) * 4, cudaMemcpyDeviceToDevice, st));
        HD_CUDA(cudaMemcpyAsync(vals, va, uint64_t(n) * 4, cudaMemcpyDeviceToDevice, st));
    }
}

} // namespace hd
