// Paged hash table on the device: full nodes, bucket-ordered appends and the
// BasicDAG ingest of HashDAGFactory::load_from_DAG.
//
// Reference: HashTable::add_leaf_node / add_interior_node
// (hash_table.h:359-468), allocate_page (:794-809), add_full_node
// (:749-789); HashDAGFactory::load_from_DAG and create_hash_dag
// (hash_dag_factory.cpp:5-99, :152-184).
#include <algorithm>
#include <vector>

#include "hd_ctx.h"
#include "hd_table.cuh"

namespace hd {

// ---------------------------------------------------------------------------
// Full nodes (add_full_node): one thread, levels last..first (descending).
// ---------------------------------------------------------------------------
__global__ void k_add_full_nodes(Table t, uint32_t first_level, uint32_t last_level)
{
    for (int32_t level = int32_t(last_level); level >= int32_t(first_level); level--) {
        uint32_t node[9];
        uint32_t n;
        uint32_t hash;
        const bool leaf = uint32_t(level) == t.g.leaf_level;
        if (leaf) {
            node[0] = node[1] = 0xFFFFFFFFu;
            n = 2;
            hash = hash_leaf(~0ull);
        } else {
            const uint32_t depth = t.g.depth - level;
            const uint32_t voxels = uint32_t(level) < t.g.T ? 0u : (1u << (3 * depth));
            node[0] = (voxels << 8) | 0xffu;
            for (int c = 0; c < 8; c++)
                node[1 + c] = t.full_nodes[level + 1];
            n = 9;
            hash = hash_interior(9, node);
        }
        const uint32_t bucket = hash & (t.g.buckets(level) - 1);
        uint32_t* size_ptr = t.bucket_sizes + t.g.bucket_global(level, bucket);
        uint32_t size = *size_ptr;
        const uint32_t pos = append_position(size, n, leaf);
        if (size > t.g.capacity(level)) {
            set_error(t.error, kErrBucketFull);
            return;
        }
        if (!map_pages(t, level, bucket, pos, size))
            return;
        const uint32_t v = t.g.make_ptr(level, bucket, pos);
        uint32_t* dst = t.sys_rw(v);
        for (uint32_t i = 0; i < n; i++)
            dst[i] = node[i];
        bloom_add(t, v, bloom_bits(node, n));
        *size_ptr = size;
        t.level_nodes[level] += 1;
        t.full_nodes[level] = v;
    }
}

void add_full_nodes(hd_ctx* c, uint32_t first_level, uint32_t last_level)
{
    k_add_full_nodes<<<1, 1, 0, c->stream>>>(c->t, first_level, last_level);
    HD_LAUNCH_CHECK();
}

// The device error word in words: e = {code, detail words} as set_error
// writes them.
static std::string describe_error(const Geom& g, const uint32_t* e)
{
    const std::string level = std::to_string(e[1]), bucket = std::to_string(e[2]);
    switch (e[0]) {
    case kErrPoolFull:
        if (e[3] && e[3] < g.pool_pages)
            return "the pool is full: the " + std::to_string(e[3]) + " pages edits may claim (of " +
                   std::to_string(g.pool_pages) + "; the rest are the GC's reserve) are in use and an append to "
                   "level " + level + ", bucket " + bucket + " needed one more";
        return "the pool is full: all " + std::to_string(g.pool_pages) +
               " pages are in use and an append to level " + level + ", bucket " + bucket + " needed one more";
    case kErrBucketFull:
        if (e[1] == 0xFFFFFFFFu)
            return "global bucket " + bucket + " received more than " + std::to_string(kMaxBucketItems) +
                   " nodes in one pass";
        if (!e[1] && !e[2] && !e[3])
            return "a bucket is full";
        return "bucket " + bucket + " of level " + level + " is full: an append would grow it to " +
               std::to_string(e[3]) + " words, past its capacity of " +
               std::to_string(e[1] < g.depth ? g.capacity(e[1]) : 0) + " words";
    case kErrTimeout:
        return "a bounded device wait gave up";
    default:
        return "error " + std::to_string(e[0]) + ": level " + std::to_string(int32_t(e[1])) + ", bucket " + bucket +
               ", value " + std::to_string(e[3]);
    }
}

uint32_t check_error(hd_ctx* c)
{
    uint32_t e[4];
    HD_CUDA(cudaMemcpyAsync(e, c->t.error, 16, cudaMemcpyDeviceToHost, c->stream));
    HD_CUDA(cudaStreamSynchronize(c->stream));
    if (e[0]) {
        HD_CUDA(cudaMemsetAsync(c->t.error, 0, 16, c->stream));
        c->err_detail = describe_error(c->g, e);
    }
    return e[0];
}

void table_reset(hd_ctx* c)
{
    const Geom& g = c->g;
    HD_CUDA(cudaMemsetAsync(c->t.pool, 0, size_t(g.pool_pages) * kPage * 4 + 64, c->stream));
    HD_CUDA(cudaMemsetAsync(c->t.bloom, 0, size_t(g.pool_pages) * kBloomWords * 4, c->stream));
    HD_CUDA(cudaMemsetAsync(c->t.page_table, 0, kPageTableEntries * 4, c->stream));
    HD_CUDA(cudaMemsetAsync(c->t.bucket_sizes, 0, g.total_buckets * 4, c->stream));
    HD_CUDA(cudaMemsetAsync(c->t.full_nodes, 0, HD_MAX_DEPTH * 4, c->stream));
    HD_CUDA(cudaMemsetAsync(c->t.level_nodes, 0, HD_MAX_DEPTH * 8, c->stream));
    HD_CUDA(cudaMemsetAsync(c->t.error, 0, 16, c->stream));
    const uint32_t top[2] = {1, 0}; // page 0 is the null page; no free pages
    HD_CUDA(cudaMemcpyAsync(c->t.pool_top, top, 8, cudaMemcpyHostToDevice, c->stream));
    set_claim_limit(c, false);
    HD_CUDA(cudaMemsetAsync(c->d_root, 0, 4, c->stream));
}

void set_claim_limit(hd_ctx* c, bool gc)
{
    // the copy reads a local: wait for it
    const uint32_t limit = gc ? c->g.pool_pages : c->g.pool_pages - std::min(c->page_reserve, c->g.pool_pages);
    HD_CUDA(cudaMemcpyAsync(c->t.pool_top + 2, &limit, 4, cudaMemcpyHostToDevice, c->stream));
    HD_CUDA(cudaStreamSynchronize(c->stream));
}

// ---------------------------------------------------------------------------
// BasicDAG ingest.
// 1. Top-down, the depth-first first-visit rank of every node per level:
//    key(child) = min over parents p and slots k of rank(p) * 8 + k; nodes
//    sorted by key are in the order create_hash_dag first reaches them.
// 2. Bottom-up, every level's nodes appended in rank order, bucket by bucket.
// ---------------------------------------------------------------------------
__global__ void k_child_keys(const uint32_t* __restrict__ words, const uint32_t* __restrict__ order, uint32_t n,
                             uint32_t* __restrict__ keyof, uint32_t* __restrict__ list, uint32_t* __restrict__ n_list)
{
    HD_GRID_STRIDE(r, n)
    {
        const uint32_t w = order[r];
        const uint32_t mask = words[w] & 0xffu;
        uint32_t k = 1;
        for (uint32_t c = 0; c < 8; c++) {
            if (!(mask & (1u << c)))
                continue;
            const uint32_t child = words[w + k++];
            const uint32_t key = uint32_t(r) * 8u + c;
            const uint32_t old = atomicMin(keyof + child, key);
            if (old == 0xFFFFFFFFu)
                list[atomicAdd(n_list, 1u)] = child;
        }
    }
}

__global__ void k_scatter_by_key(const uint32_t* __restrict__ list, const uint32_t* __restrict__ n_list,
                                 const uint32_t* __restrict__ keyof, uint32_t* __restrict__ by_key)
{
    const uint32_t n = *n_list;
    HD_GRID_STRIDE(i, n)
    {
        const uint32_t c = list[i];
        by_key[keyof[c]] = c;
    }
}

__global__ void k_flag_valid(const uint32_t* __restrict__ by_key, uint64_t n, uint32_t* __restrict__ flag)
{
    HD_GRID_STRIDE(i, n) flag[i] = by_key[i] != 0xFFFFFFFFu;
}

__global__ void k_compact_valid(const uint32_t* __restrict__ by_key, const uint32_t* __restrict__ pos, uint64_t n,
                                uint32_t* __restrict__ out)
{
    HD_GRID_STRIDE(i, n)
    {
        const uint32_t v = by_key[i];
        if (v != 0xFFFFFFFFu)
            out[pos[i]] = v;
    }
}

// Content of every node of a level in rank order: header (or leaf words)
// and child virtual addresses; hash, bucket and the bucket lists.
__global__ void k_import_content(Table t, uint32_t level, const uint32_t* __restrict__ words,
                                 const uint32_t* __restrict__ order, uint32_t n, const uint32_t* __restrict__ vaddr,
                                 uint32_t* __restrict__ content, uint32_t* __restrict__ head,
                                 uint32_t* __restrict__ next, uint32_t* __restrict__ touched,
                                 uint32_t* __restrict__ n_touched)
{
    const bool leaf = level == t.g.leaf_level;
    HD_GRID_STRIDE(r, n)
    {
        const uint32_t w = order[r];
        uint32_t* out = content + 9 * r;
        uint32_t hash;
        if (leaf) {
            out[0] = words[w];
            out[1] = words[w + 1];
            hash = hash_leaf(uint64_t(out[0]) | (uint64_t(out[1]) << 32));
        } else {
            const uint32_t header = words[w];
            const uint32_t cnt = popc32(header & 0xffu);
            out[0] = header;
            for (uint32_t k = 0; k < cnt; k++)
                out[1 + k] = vaddr[words[w + 1 + k]];
            hash = hash_interior(cnt + 1, out);
        }
        const uint32_t bucket = hash & (t.g.buckets(level) - 1);
        link_item(t.g.bucket_global(level, bucket), uint32_t(r), head, next, touched, n_touched);
    }
}

constexpr uint32_t kAppendWarps = 2;

// One warp per touched bucket: its items, in item order, appended one after
// the other, as the reference's sequential add_*_node calls place them.
// content: 9 words per item; out_addr[item] = the node's virtual address.
__global__ void __launch_bounds__(32 * kAppendWarps)
    k_append_items(Table t, uint32_t level, const uint32_t* __restrict__ content, uint32_t* __restrict__ head,
                   const uint32_t* __restrict__ next, const uint32_t* __restrict__ touched,
                   const uint32_t* __restrict__ n_touched, uint32_t* __restrict__ out_addr)
{
    __shared__ uint32_t items_s[kAppendWarps][kMaxBucketItems];
    __shared__ uint32_t pos_s[kAppendWarps][kMaxBucketItems];
    __shared__ uint32_t ok_s[kAppendWarps];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t* items = items_s[warp];
    uint32_t* pos = pos_s[warp];
    const bool leaf = level == t.g.leaf_level;
    const uint32_t nt = *n_touched;
    for (uint32_t ti = blockIdx.x * kAppendWarps + warp; ti < nt; ti += gridDim.x * kAppendWarps) {
        const uint32_t gb = touched[ti];
        const uint32_t cnt = collect_sorted(gb, head, next, items, t.error);
        if (cnt == 0)
            continue;
        const uint32_t bucket = gb - t.g.level_first_bucket(level);
        if (lane == 0) {
            uint32_t size = t.bucket_sizes[gb];
            const uint32_t start = size;
            uint32_t ok = 1;
            for (uint32_t i = 0; i < cnt; i++) {
                const uint32_t n = leaf ? 2 : total_size(content[9 * uint64_t(items[i])]);
                pos[i] = append_position(size, n, leaf);
            }
            if (size > t.g.capacity(level)) {
                set_error(t.error, kErrBucketFull);
                ok = 0;
            } else if (!map_pages(t, level, bucket, start, size)) {
                ok = 0;
            } else {
                t.bucket_sizes[gb] = size;
                atomicAdd(reinterpret_cast<unsigned long long*>(t.level_nodes + level), cnt);
            }
            ok_s[warp] = ok;
        }
        __syncwarp();
        if (!ok_s[warp])
            continue;
        for (uint32_t i = lane; i < cnt; i += 32) {
            const uint32_t r = items[i];
            const uint32_t* src = content + 9 * uint64_t(r);
            const uint32_t n = leaf ? 2 : total_size(src[0]);
            const uint32_t v = t.g.make_ptr(level, bucket, pos[i]);
            uint32_t* dst = t.sys_rw(v);
            for (uint32_t k = 0; k < n; k++)
                dst[k] = src[k];
            bloom_add(t, v, bloom_bits(src, n));
            out_addr[r] = v;
        }
        __syncwarp();
    }
}

__global__ void k_scatter_addr(const uint32_t* __restrict__ order, uint32_t n, const uint32_t* __restrict__ addr,
                               uint32_t* __restrict__ vaddr)
{
    HD_GRID_STRIDE(r, n) vaddr[order[r]] = addr[r];
}

void append_items(hd_ctx* c, uint32_t level, const uint32_t* content, uint64_t n_items, uint32_t* head,
                  const uint32_t* next, const uint32_t* touched, const uint32_t* n_touched, uint32_t* out_addr)
{
    k_append_items<<<grid_for(n_items * 32, 32 * kAppendWarps, 152 * 16), 32 * kAppendWarps, 0, c->stream>>>(
        c->t, level, content, head, next, touched, n_touched, out_addr);
    HD_LAUNCH_CHECK();
}

__global__ void k_set_root(const uint32_t* __restrict__ vaddr, uint32_t* root) { *root = vaddr[0]; }

void import_basic_dag(hd_ctx* c, const uint32_t* d_words, uint64_t n_words)
{
    cudaStream_t st = c->stream;
    Scratch& s = c->scratch;
    const Geom& g = c->g;
    const uint32_t levels = g.leaf_level + 1;
    if (n_words >= 0xFFFFFFFFull)
        throw StatusError{HD_ERR_INVALID, "BasicDAG larger than 2^32 words"};
    // per-level rank order (word indices)
    uint32_t* keyof = s.get<uint32_t>("imp_keyof", n_words);
    fill<uint32_t>(keyof, 0xFFFFFFFFu, n_words, st);
    std::vector<uint32_t*> order(levels);
    std::vector<uint32_t> count(levels);
    uint32_t* d_n = s.get<uint32_t>("imp_counter", 4);
    order[0] = s.get<uint32_t>("imp_order_0", 1);
    HD_CUDA(cudaMemsetAsync(order[0], 0, 4, st)); // root at word 0
    count[0] = 1;
    for (uint32_t L = 0; L + 1 < levels; L++) {
        const uint32_t nL = count[L];
        uint32_t* list = s.get<uint32_t>("imp_list", uint64_t(nL) * 8 + 1);
        HD_CUDA(cudaMemsetAsync(d_n, 0, 4, st));
        k_child_keys<<<grid_for(nL, 256), 256, 0, st>>>(d_words, order[L], nL, keyof, list, d_n);
        HD_LAUNCH_CHECK();
        const uint64_t nkeys = uint64_t(nL) * 8;
        uint32_t* by_key = s.get<uint32_t>("imp_by_key", nkeys);
        fill<uint32_t>(by_key, 0xFFFFFFFFu, nkeys, st);
        k_scatter_by_key<<<grid_for(nkeys, 256), 256, 0, st>>>(list, d_n, keyof, by_key);
        HD_LAUNCH_CHECK();
        uint32_t* flag = s.get<uint32_t>("imp_flag", nkeys);
        uint32_t* pos = s.get<uint32_t>("imp_pos", nkeys);
        k_flag_valid<<<grid_for(nkeys, 256), 256, 0, st>>>(by_key, nkeys, flag);
        HD_LAUNCH_CHECK();
        exclusive_scan<uint32_t, uint32_t>(s, flag, pos, nkeys, d_n, st);
        const uint32_t nNext = read_scalar(d_n, st);
        char name[32];
        snprintf(name, sizeof(name), "imp_order_%u", L + 1);
        order[L + 1] = s.get<uint32_t>(name, uint64_t(nNext) + 1);
        count[L + 1] = nNext;
        k_compact_valid<<<grid_for(nkeys, 256), 256, 0, st>>>(by_key, pos, nkeys, order[L + 1]);
        HD_LAUNCH_CHECK();
    }
    // full nodes for levels leaf..1 come first (load_from_DAG)
    add_full_nodes(c, 1, g.leaf_level);
    // bottom-up appends; keyof is reused as the word -> virtual address map
    uint32_t* vaddr = keyof;
    uint32_t maxn = 0;
    for (uint32_t L = 0; L < levels; L++)
        maxn = count[L] > maxn ? count[L] : maxn;
    uint32_t* content = s.get<uint32_t>("imp_content", uint64_t(maxn) * 9);
    uint32_t* next = s.get<uint32_t>("imp_next", maxn);
    uint32_t* addr = s.get<uint32_t>("imp_addr", maxn);
    uint32_t* head = s.get<uint32_t>("imp_head", g.total_buckets);
    uint32_t* touched = s.get<uint32_t>("imp_touched", g.total_buckets);
    fill<uint32_t>(head, kEmpty, g.total_buckets, st);
    for (int32_t L = int32_t(levels) - 1; L >= 0; L--) {
        const uint32_t n = count[L];
        HD_CUDA(cudaMemsetAsync(d_n, 0, 4, st));
        k_import_content<<<grid_for(n, 256), 256, 0, st>>>(c->t, uint32_t(L), d_words, order[L], n, vaddr, content,
                                                            head, next, touched, d_n);
        HD_LAUNCH_CHECK();
        append_items(c, uint32_t(L), content, n, head, next, touched, d_n, addr);
        k_scatter_addr<<<grid_for(n, 256), 256, 0, st>>>(order[L], n, addr, vaddr);
        HD_LAUNCH_CHECK();
    }
    k_set_root<<<1, 1, 0, st>>>(vaddr, c->d_root);
    HD_LAUNCH_CHECK();
    const uint32_t e = check_error(c);
    if (e)
        throw StatusError{hd_status(e == kErrCapacity ? HD_ERR_INVALID : e), "BasicDAG ingest failed"};
    c->root = read_scalar(c->d_root, st);
}

// Rebuilds the filters of a table written from outside (imports, snapshots)
// by walking every bucket the way the scans do: leaves two words apart,
// interior nodes by their sizes from each page's start.  Words past a page's
// last node (the gap a node that did not fit leaves) are walked as nodes too,
// which only adds bits, so a filter never misses a node it holds.
__global__ void k_bloom_rebuild(Table t, uint32_t level)
{
    const Geom& g = t.g;
    const bool leaf = level == g.leaf_level;
    HD_GRID_STRIDE(b, uint64_t(g.buckets(level)))
    {
        const uint32_t S = t.bucket_sizes[g.bucket_global(level, uint32_t(b))];
        const uint32_t vbase = g.make_ptr(level, uint32_t(b), 0);
        for (uint32_t pindex = 0; pindex < S; pindex += kPage) {
            const uint32_t used = S - pindex < kPage ? S - pindex : kPage;
            const uint32_t* page = t.sys_cg(vbase + pindex);
            for (uint32_t w = 0; w < used;) {
                const uint32_t n = leaf ? 2 : total_size(page[w]);
                if (w + n > used)
                    break;
                bloom_add(t, vbase + pindex + w, bloom_bits(page + w, n));
                w += n;
            }
        }
    }
}

bool valid_root(const Geom& g, uint32_t root, uint32_t pt_entry)
{
    return (root >> kPageShift) < g.total_vpages && pt_entry != 0;
}

void check_table(const Geom& g, const uint32_t* pt, const uint32_t* bs, uint32_t top, uint32_t root,
                 const std::string& what)
{
    for (uint64_t p = 0; p < g.total_vpages; p++)
        if (pt[p] >= top)
            throw StatusError{HD_ERR_INVALID, what + " maps virtual page " + std::to_string(p) + " to page " +
                                                  std::to_string(pt[p]) + ", past its " + std::to_string(top) +
                                                  " pool pages"};
    if (bs)
        for (uint32_t L = 0; L < g.depth; L++)
            for (uint32_t b = 0; b < g.buckets(L); b++)
                if (bs[g.bucket_global(L, b)] > g.capacity(L))
                    throw StatusError{HD_ERR_INVALID, what + ": bucket " + std::to_string(b) + " of level " +
                                                          std::to_string(L) + " holds more than its capacity"};
    if (!valid_root(g, root, (root >> kPageShift) < g.total_vpages ? pt[root >> kPageShift] : 0))
        throw StatusError{HD_ERR_INVALID, what + ": the root " + std::to_string(root) + " is not on a mapped page"};
}

void bloom_rebuild(hd_ctx* c)
{
    const Geom& g = c->g;
    HD_CUDA(cudaMemsetAsync(c->t.bloom, 0, size_t(g.pool_pages) * kBloomWords * 4, c->stream));
    for (uint32_t L = 0; L <= g.leaf_level; L++) {
        k_bloom_rebuild<<<grid_for(g.buckets(L), 128), 128, 0, c->stream>>>(c->t, L);
        HD_LAUNCH_CHECK();
    }
}

__global__ void k_bloom_clear_level(Table t, uint32_t vp0, uint32_t vp1)
{
    HD_GRID_STRIDE(i, uint64_t(vp1 - vp0))
    {
        const uint32_t p = t.page_table[vp0 + i];
        if (p)
            for (uint32_t k = 0; k < kBloomWords; k++)
                t.bloom[uint64_t(p) * kBloomWords + k] = 0;
    }
}

// Empties the filters of every page of a level (GC rebuilds the level's
// buckets in the same pages).
void bloom_clear_level(hd_ctx* c, uint32_t level)
{
    const Geom& g = c->g;
    const uint32_t vp0 = g.make_ptr(level, 0, 0) >> kPageShift;
    const uint64_t words = uint64_t(g.buckets(level)) * g.capacity(level);
    const uint32_t vp1 = uint32_t((uint64_t(g.make_ptr(level, 0, 0)) + words) >> kPageShift);
    k_bloom_clear_level<<<grid_for(vp1 - vp0, 256), 256, 0, c->stream>>>(c->t, vp0, vp1);
    HD_LAUNCH_CHECK();
}

} // namespace hd
