// Device helpers shared by the ingest, edit and GC kernels: bucket append
// positions, page mapping, per-bucket work lists.
#pragma once

#include "hd_common.cuh"

namespace hd {

constexpr uint32_t kEmpty = 0xFFFFFFFFu;
// Items one bucket can receive in one pass: a low-level bucket of 4096 words
// holds at most 2048 leaves.
constexpr uint32_t kMaxBucketItems = 2048;

// Position of the next node in a bucket of `size` words, advancing size
// (add_leaf_node / add_interior_node, hash_table.h:359-468): leaves are two
// words and pack pages exactly; an interior node never straddles a page, the
// rest of the page is skipped.
HD_HD uint32_t append_position(uint32_t& size, uint32_t n, bool leaf)
{
    if (!leaf) {
        const uint32_t left = kPage - (size & (kPage - 1));
        if (left != kPage && left < n)
            size += left;
    }
    const uint32_t pos = size;
    size += n;
    return pos;
}

// A physical page for a new virtual page: one a page-releasing GC gave back
// (zeroed, like a never-used page), else poolTop++ (allocate_page,
// hash_table.h:794-809).  0 when the pool is full: a claim past the pool's
// end is given back at once, so poolTop never exceeds the pool (the
// reference, unchecked in release builds, would write past its pool).
// Free-list pops may run concurrently; pushes happen only inside a GC.
HD_D uint32_t claim_page(const Table& t)
{
    uint32_t* free_count = t.pool_top + 1;
    if (__ldcg(free_count) != 0) {
        const uint32_t k = atomicSub(free_count, 1u);
        if (int32_t(k) > 0)
            return __ldcg(t.free_pages + (k - 1));
        atomicAdd(free_count, 1u); // none left: undo
    }
    const uint32_t p = atomicAdd(t.pool_top, 1u);
    if (p >= __ldcg(t.pool_top + 2)) { // the claim limit: the pool less the GC's reserve
        atomicSub(t.pool_top, 1u);
        return 0;
    }
    return p;
}

// Maps every unmapped virtual page that [from, to) of the bucket touches.
// A bucket rebuilt by the default GC keeps its pages; the page-releasing GC
// unmaps those wholly past the bucket's new size.
HD_D bool map_pages(const Table& t, uint32_t level, uint32_t bucket, uint32_t from, uint32_t to)
{
    if (to <= from)
        return true;
    const uint32_t v0 = t.g.make_ptr(level, bucket, from) >> kPageShift;
    const uint32_t v1 = t.g.make_ptr(level, bucket, to - 1) >> kPageShift;
    for (uint32_t vp = v0; vp <= v1; vp++) {
        if (__ldcg(t.page_table + vp) == 0) {
            const uint32_t p = claim_page(t);
            if (!p) {
                set_error(t.error, kErrPoolFull, level, bucket, __ldcg(t.pool_top + 2));
                return false;
            }
            __stcg(t.page_table + vp, p);
        }
    }
    return true;
}

// The filter of the physical page behind virtual word v
HD_D uint32_t* bloom_of(const Table& t, uint32_t v)
{
    return t.bloom + uint64_t(__ldcg(t.page_table + (v >> kPageShift))) * kBloomWords;
}
// Adds a node written at virtual word v to its page's filter
HD_D void bloom_add(const Table& t, uint32_t v, uint32_t bits)
{
    uint32_t* f = bloom_of(t, v);
#pragma unroll
    for (uint32_t i = 0; i < kBloomHashes; i++) {
        const uint32_t b = bloom_pos(bits, i);
        atomicOr(f + (b >> 5), 1u << (b & 31));
    }
}
// Adds a node written into physical page p to the page's filter
HD_D void bloom_add_phys(const Table& t, uint32_t p, uint32_t bits)
{
    uint32_t* f = t.bloom + uint64_t(p) * kBloomWords;
#pragma unroll
    for (uint32_t i = 0; i < kBloomHashes; i++) {
        const uint32_t b = bloom_pos(bits, i);
        atomicOr(f + (b >> 5), 1u << (b & 31));
    }
}
// False when physical page p's filter rules the node out
HD_D bool bloom_may_phys(const Table& t, uint32_t p, uint32_t bits)
{
    const uint32_t* f = t.bloom + uint64_t(p) * kBloomWords;
    bool may = true;
#pragma unroll
    for (uint32_t i = 0; i < kBloomHashes; i++) {
        const uint32_t b = bloom_pos(bits, i);
        may &= ((__ldcg(f + (b >> 5)) >> (b & 31)) & 1u) != 0;
    }
    return may;
}
// False when the page behind virtual word v cannot hold the node
HD_D bool bloom_may(const Table& t, uint32_t v, uint32_t bits)
{
    const uint32_t* f = bloom_of(t, v);
    bool may = true;
#pragma unroll
    for (uint32_t i = 0; i < kBloomHashes; i++) {
        const uint32_t b = bloom_pos(bits, i);
        may &= ((__ldcg(f + (b >> 5)) >> (b & 31)) & 1u) != 0;
    }
    return may;
}

// Pushes item i onto the list of bucket gb; the first item of a bucket also
// records the bucket in `touched`.
HD_D void link_item(uint32_t gb, uint32_t i, uint32_t* head, uint32_t* next, uint32_t* touched, uint32_t* n_touched)
{
    const uint32_t prev = atomicExch(head + gb, i);
    next[i] = prev;
    if (prev == kEmpty)
        touched[atomicAdd(n_touched, 1u)] = gb;
}

// Warp-wide: gathers the items of bucket gb into `items` (shared), sorted
// ascending, resets the list head; returns the count (0 on overflow, with
// the error word set).
HD_D uint32_t collect_sorted(uint32_t gb, uint32_t* head, const uint32_t* next, uint32_t* items, uint32_t* err)
{
    const uint32_t lane = threadIdx.x & 31;
    uint32_t cnt = 0;
    if (lane == 0) {
        uint32_t it = head[gb];
        while (it != kEmpty && cnt < kMaxBucketItems) {
            items[cnt++] = it;
            it = next[it];
        }
        if (it != kEmpty) {
            set_error(err, kErrBucketFull, 0xFFFFFFFFu, gb, cnt);
            cnt = 0;
        }
        head[gb] = kEmpty;
    }
    cnt = __shfl_sync(0xffffffffu, cnt, 0);
    __syncwarp();
    if (cnt <= 1)
        return cnt;
    uint32_t n2 = 2;
    while (n2 < cnt)
        n2 <<= 1;
    for (uint32_t i = cnt + lane; i < n2; i += 32)
        items[i] = kEmpty;
    __syncwarp();
    // bitonic sort, ascending
    for (uint32_t k = 2; k <= n2; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = lane; i < n2; i += 32) {
                const uint32_t ixj = i ^ j;
                if (ixj > i) {
                    const uint32_t a = items[i], b = items[ixj];
                    const bool asc = (i & k) == 0;
                    if ((a > b) == asc) {
                        items[i] = b;
                        items[ixj] = a;
                    }
                }
            }
            __syncwarp();
        }
    }
    return cnt;
}

} // namespace hd
