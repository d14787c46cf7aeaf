// Shared device/host definitions of the hashed-DAG table format.
//
// Format (Phyronnaz/HashDAG): 512-word pages (typedefs.h:201-203); virtual
// address of (level, bucket, position) as make_ptr (hash_table.h:45-63);
// translation pool[pageTable[v / 512] * 512 + v % 512] (get_sys_ptr,
// hash_table.h:155-173); interior nodes [mask | count << 8, children...],
// leaves two words (base_dag.h:6-59); hashes murmurhash64 / murmurhash32xN
// (utils.h:355-396, hash_table.h:80-89).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/hashdag_gb300.h"

#define HD_HD __host__ __device__ __forceinline__
#define HD_D __device__ __forceinline__

namespace hd {

constexpr uint32_t kPage = HD_PAGE_SIZE;
constexpr uint32_t kPageShift = 9;
// Page-table entries allocated per context: one for every page of the 32-bit
// virtual space, so that any node index, even one read from a corrupt or
// foreign table, translates inside the page table (entries past the
// geometry's pages stay 0, the never-used physical page 0).
constexpr uint64_t kPageTableEntries = 1ull << (32 - kPageShift);
constexpr uint32_t kInvalid = HD_INVALID_NODE;
constexpr uint32_t kNotFound = 0xFFFFFFFFu;
// Largest grid.y of a launch: 8x8-pixel tile grids hold at most this many
// rows of tiles (images up to 524,280 pixels high).
constexpr uint32_t kMaxGridRows = 65535;
constexpr uint32_t kEmptyId = 0xFFFFFFFFu; // "no node" in scratch id arrays

// Device-side error word values (first error wins).
enum : uint32_t {
    kErrNone = 0,
    kErrPoolFull = HD_ERR_POOL_FULL,
    kErrBucketFull = HD_ERR_BUCKET_FULL,
    kErrTimeout = HD_ERR_TIMEOUT,
    kErrCapacity = 8, // a scratch array ran out of room
};

// Geometry of one table, passed by value to kernels.
struct Geom {
    uint32_t depth;       // levels; leaves at depth - 2
    uint32_t leaf_level;
    uint32_t T;           // color tree levels
    uint32_t top_levels;
    uint32_t top_bits, low_bits;
    uint32_t top_size, low_size;
    uint32_t ntop;        // min(top_levels, depth)
    uint32_t pool_pages;
    uint64_t total_buckets;
    uint64_t total_vpages;

    HD_HD uint32_t buckets(uint32_t level) const { return level < top_levels ? (1u << top_bits) : (1u << low_bits); }
    HD_HD uint32_t capacity(uint32_t level) const { return level < top_levels ? top_size : low_size; }
    HD_HD uint32_t bucket_global(uint32_t level, uint32_t bucket) const
    {
        return level < top_levels ? level * (1u << top_bits) + bucket
                                  : ntop * (1u << top_bits) + (level - top_levels) * (1u << low_bits) + bucket;
    }
    HD_HD uint32_t level_first_bucket(uint32_t level) const { return bucket_global(level, 0); }
    HD_HD uint32_t make_ptr(uint32_t level, uint32_t bucket, uint32_t pos) const
    {
        uint64_t index;
        if (level < top_levels)
            index = (uint64_t(level) * (1u << top_bits) + bucket) * top_size;
        else
            index = uint64_t(ntop) * (1u << top_bits) * top_size +
                    (uint64_t(level - top_levels) * (1u << low_bits) + bucket) * low_size;
        return uint32_t(index + pos);
    }
};

inline Geom make_geom(const hd_config& c)
{
    Geom g{};
    g.depth = c.depth;
    g.leaf_level = c.depth - 2;
    g.T = c.color_tree_levels;
    g.top_levels = c.top_levels;
    g.top_bits = c.top_bucket_bits;
    g.low_bits = c.low_bucket_bits;
    g.top_size = c.top_bucket_size;
    g.low_size = c.low_bucket_size;
    g.ntop = c.top_levels < c.depth ? c.top_levels : c.depth;
    g.pool_pages = c.pool_pages;
    const uint64_t low = c.depth > c.top_levels ? c.depth - c.top_levels : 0;
    g.total_buckets = uint64_t(g.ntop) * (1u << g.top_bits) + low * (1u << g.low_bits);
    g.total_vpages = (uint64_t(g.ntop) * (1u << g.top_bits) * g.top_size + low * (1u << g.low_bits) * g.low_size) / kPage;
    return g;
}

// Device view of a table (HashDAG passed by value to kernels, as the
// reference's tracer does, tracer.cu:146).
struct Table {
    uint32_t* pool;
    uint32_t* bloom;        // kBloomWords per physical page (see bloom_*)
    uint32_t* page_table;
    uint32_t* bucket_sizes;
    uint32_t* full_nodes;   // [depth]
    uint32_t* pool_top;     // device counters: [0] poolTop, [1] pages in the free list
    uint32_t* free_pages;   // pages a page-releasing GC gave back (pool_pages entries)
    uint32_t* error;        // device error word
    uint64_t* level_nodes;  // stored node count per level
    Geom g;

    // Translation through the read-only data path: for kernels during which
    // neither the page table nor the pool changes (the edit descent, GC
    // gathers, point queries).
    HD_D const uint32_t* sys(uint32_t v) const
    {
        return pool + (uint64_t(__ldg(page_table + (v >> kPageShift))) << kPageShift) + (v & (kPage - 1));
    }
    // Physical word offset of virtual word v in the pool, for the traversal
    // walks, which keep their node by this offset: a node never straddles a
    // page, so the words after a node's first word are at the following
    // physical offsets (32 bits: at most 2^23 pages).  Plain global loads:
    // the read-only path queued on the texture pipe there (tex_throttle).
    HD_D uint32_t phys(uint32_t v) const
    {
        return (page_table[v >> kPageShift] << kPageShift) | (v & (kPage - 1));
    }
    // Translation with an L2-coherent read of the page table, for kernels
    // that map pages while they scan.
    HD_D const uint32_t* sys_cg(uint32_t v) const
    {
        return pool + (uint64_t(__ldcg(page_table + (v >> kPageShift))) << kPageShift) + (v & (kPage - 1));
    }
    // Translation for writers: the page-table entry is read from L2, never
    // from a possibly stale L1 line (pages are mapped inside the same
    // kernels that write through this translation).
    HD_D uint32_t* sys_rw(uint32_t v) const
    {
        return pool + (uint64_t(__ldcg(page_table + (v >> kPageShift))) << kPageShift) + (v & (kPage - 1));
    }
};

// err[0] = first error code; err[1..3] = its detail words.
HD_D void set_error(uint32_t* err, uint32_t code, uint32_t a = 0, uint32_t b = 0, uint32_t c = 0)
{
    if (atomicCAS(err, 0u, code) == 0u) {
        err[1] = a;
        err[2] = b;
        err[3] = c;
    }
}

// ---- hashes (utils.h:355-396) --------------------------------------------
HD_HD uint32_t murmur32(uint32_t h)
{
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}
HD_HD uint64_t murmur64(uint64_t h)
{
    h ^= h >> 33;
    h *= 0xff51afd7ed558ccdull;
    h ^= h >> 33;
    h *= 0xc4ceb9fe1a85ec53ull;
    h ^= h >> 33;
    return h;
}
HD_HD uint32_t hash_leaf(uint64_t leaf) { return uint32_t(murmur64(leaf)); }
HD_HD uint32_t hash_interior(uint32_t n, const uint32_t* node)
{
    uint32_t h = 0;
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t k = node[i];
        k *= 0xcc9e2d51u;
        k = (k << 15) | (k >> 17);
        k *= 0x1b873593u;
        h ^= k;
        h = (h << 13) | (h >> 19);
        h = h * 5u + 0xe6546b64u;
    }
    h ^= n;
    return murmur32(h);
}

HD_HD uint32_t popc32(uint32_t v)
{
#ifdef __CUDA_ARCH__
    return __popc(v);
#else
    return uint32_t(__builtin_popcount(v));
#endif
}
HD_HD uint32_t popc64(uint64_t v)
{
#ifdef __CUDA_ARCH__
    return __popcll(v);
#else
    return uint32_t(__builtin_popcountll(v));
#endif
}
HD_HD uint32_t total_size(uint32_t header) { return popc32(header & 0xffu) + 1; }
HD_HD uint32_t child_offset(uint32_t mask, uint32_t child) { return popc32(mask & ((1u << child) - 1u)) + 1; }

HD_HD uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// ---- per-page Bloom filters (hash_table.h:564-659, USE_BLOOM_FILTER) --------
// Every physical page has a 512-bit filter holding 3 bits of every node
// ever written into it; a bucket scan skips a page whose filter lacks a bit
// of the node it looks for.  The filter can only say "maybe": a page that
// holds the node always passes, so results never change, only the pages
// read.  Bits come from a hash of the node's words independent of the
// bucket hash.
constexpr uint32_t kBloomWords = 16;
constexpr uint32_t kBloomHashes = 3;
HD_HD uint32_t bloom_bits(const uint32_t* q, uint32_t n)
{
    uint64_t h = 0x51ED2701F3A5C9B7ull ^ n;
    for (uint32_t k = 0; k < n; k++)
        h = mix64(h ^ q[k]);
    // three 9-bit positions, packed
    return uint32_t(h & 0x7FFFFFFu);
}
HD_HD uint32_t bloom_pos(uint32_t bits, uint32_t i) { return (bits >> (9 * i)) & 511u; }

// Leaf bit of voxel (x, y, z) inside its 4x4x4 block (dag_utils.h:160-167).
HD_HD uint32_t leaf_bit(uint32_t x, uint32_t y, uint32_t z)
{
    return ((x & 1) ? 4 : 0) | ((y & 1) ? 2 : 0) | ((z & 1) ? 1 : 0) | ((x & 2) ? 32 : 0) | ((y & 2) ? 16 : 0) |
           ((z & 2) ? 8 : 0);
}

inline uint32_t ceil_div(uint64_t a, uint64_t b) { return uint32_t((a + b - 1) / b); }

} // namespace hd
