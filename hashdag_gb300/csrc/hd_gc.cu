// Garbage collection on the device: mark-and-compact of the hash table.
//
// Reference: HashDAG::remove_stale_nodes (hash_dag.h:407-547).  Mark: the
// nodes reachable from the root level by level (here as a bitmap over each
// level's virtual range, so the live list comes out sorted by address).
// Rebuild bottom-up: every live node's content is gathered with its children
// remapped, the level's buckets are emptied, the full node is added first
// (add_full_node) and the live nodes are re-appended without a find, in
// increasing old-address order (the reference uses its hash-set order), so a
// reachable full node is kept twice as in the reference.  Pages stay mapped;
// the words past a bucket's new size keep their old contents.  With
// HD_GC_RELEASE_PAGES (no reference counterpart: its poolTop only grows,
// hash_table.h:794-809), the pages wholly past each bucket's new size are
// unmapped, zeroed and put on the table's free list, from which the next
// page claims draw first.
#include <algorithm>
#include <vector>

#include "hd_ctx.h"
#include "hd_table.cuh"

namespace hd {

__global__ void k_gc_mark(Table t, const uint32_t* __restrict__ live, uint32_t n, uint32_t child_base,
                          uint32_t* __restrict__ bitmap)
{
    HD_GRID_STRIDE(i, n)
    {
        const uint32_t* p = t.sys(live[i]);
        const uint32_t cnt = popc32(p[0] & 0xffu);
        for (uint32_t k = 0; k < cnt; k++) {
            const uint32_t off = p[1 + k] - child_base;
            atomicOr(bitmap + (off >> 5), 1u << (off & 31));
        }
    }
}

__global__ void k_popc_words(const uint32_t* __restrict__ bitmap, uint64_t n, uint32_t* __restrict__ counts)
{
    HD_GRID_STRIDE(i, n) counts[i] = popc32(bitmap[i]);
}

__global__ void k_bitmap_to_list(const uint32_t* __restrict__ bitmap, const uint32_t* __restrict__ pos, uint64_t n,
                                 uint32_t base, uint32_t* __restrict__ list)
{
    HD_GRID_STRIDE(i, n)
    {
        uint32_t b = bitmap[i];
        uint32_t o = pos[i];
        while (b) {
            const uint32_t bit = __ffs(b) - 1;
            b &= b - 1;
            list[o++] = base + uint32_t(i) * 32 + bit;
        }
    }
}

HD_D uint32_t lower_bound(const uint32_t* v, uint32_t n, uint32_t x)
{
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (v[mid] < x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// Gathers the live nodes of a level (children remapped) before the level is
// emptied; hashes and links them into the bucket lists.  A child's index in
// the live list of the level below is its rank in that level's mark bitmap:
// the live count of the bitmap words before it (child_pos) plus the bits
// below it in its word.
__global__ void k_gc_gather(Table t, uint32_t level, const uint32_t* __restrict__ live, uint32_t n,
                            const uint32_t* __restrict__ child_bitmap, const uint32_t* __restrict__ child_pos,
                            uint32_t child_base, const uint32_t* __restrict__ child_new,
                            uint32_t* __restrict__ content,
                            uint32_t* __restrict__ head, uint32_t* __restrict__ next, uint32_t* __restrict__ touched,
                            uint32_t* __restrict__ n_touched)
{
    const bool leaf = level == t.g.leaf_level;
    HD_GRID_STRIDE(i, n)
    {
        const uint32_t* p = t.sys(live[i]);
        uint32_t* c = content + 9 * i;
        uint32_t hash;
        if (leaf) {
            c[0] = p[0];
            c[1] = p[1];
            hash = hash_leaf(uint64_t(c[0]) | (uint64_t(c[1]) << 32));
        } else {
            const uint32_t cnt = popc32(p[0] & 0xffu);
            c[0] = p[0];
            for (uint32_t k = 0; k < cnt; k++) {
                const uint32_t off = p[1 + k] - child_base, w = off >> 5;
                c[1 + k] = child_new[child_pos[w] + popc32(child_bitmap[w] & ((1u << (off & 31)) - 1u))];
            }
            hash = hash_interior(cnt + 1, c);
        }
        const uint32_t bucket = hash & (t.g.buckets(level) - 1);
        link_item(t.g.bucket_global(level, bucket), uint32_t(i), head, next, touched, n_touched);
    }
}

// Pages wholly past a bucket's final size (`sizes`, the level's buckets)
// go to the free list (one thread per bucket, at most capacity / 512 pages
// each).
__global__ void k_gc_release(Table t, uint32_t level, const uint32_t* __restrict__ sizes)
{
    const Geom& g = t.g;
    uint32_t* free_count = t.pool_top + 1;
    HD_GRID_STRIDE(i, g.buckets(level))
    {
        const uint32_t bucket = uint32_t(i);
        const uint32_t size = sizes[bucket], cap = g.capacity(level);
        for (uint32_t off = (size + kPage - 1) & ~(kPage - 1); off < cap; off += kPage) {
            const uint32_t vp = g.make_ptr(level, bucket, off) >> kPageShift;
            const uint32_t p = t.page_table[vp];
            if (p) {
                t.page_table[vp] = 0;
                t.free_pages[atomicAdd(free_count, 1u)] = p;
            }
        }
    }
}

// Zeroes the pages free_pages[from, to) and their Bloom filters.
__global__ void k_zero_pages(Table t, uint32_t from, uint32_t to)
{
    const uint64_t n = uint64_t(to - from) * kPage;
    HD_GRID_STRIDE(i, n)
    {
        const uint32_t p = t.free_pages[from + uint32_t(i / kPage)];
        t.pool[uint64_t(p) * kPage + (i % kPage)] = 0;
        if (i % kPage < kBloomWords)
            t.bloom[uint64_t(p) * kBloomWords + (i % kPage)] = 0;
    }
}

// ---- dry run: the rebuild's page needs, computed before anything changes ----
// The rebuild of a level re-appends its live nodes with a different order
// and so a different padding: a bucket can need a page it never had.  A
// rebuild that runs out of pages half way cannot be undone, so the GC first
// runs every level's rebuild on scratch bucket sizes (the same full node
// first, the same items in the same order, hence the same addresses) and
// counts the pages it would map, and the pages a releasing GC would free.
// A releasing GC frees a level's pages that lie wholly past their bucket's
// final size (kept from the dry run) before it re-appends the level, so the
// appends of the same level can take them: re-hashed parents (children
// remapped) move between buckets, and one bucket's growth is met by
// another's shrinkage.

// The level's full node at the head of its (empty) bucket, on dry sizes.
__global__ void k_gc_dry_full(Table t, uint32_t level, uint32_t* dry_sizes, uint32_t* full_dry)
{
    uint32_t node[9];
    uint32_t n, hash;
    const bool leaf = level == t.g.leaf_level;
    if (leaf) {
        node[0] = node[1] = 0xFFFFFFFFu;
        n = 2;
        hash = hash_leaf(~0ull);
    } else {
        const uint32_t depth = t.g.depth - level;
        const uint32_t voxels = level < t.g.T ? 0u : (1u << (3 * depth));
        node[0] = (voxels << 8) | 0xffu;
        for (int c = 0; c < 8; c++)
            node[1 + c] = full_dry[level + 1];
        n = 9;
        hash = hash_interior(9, node);
    }
    const uint32_t bucket = hash & (t.g.buckets(level) - 1);
    dry_sizes[bucket] = n;
    full_dry[level] = t.g.make_ptr(level, bucket, 0);
}

// The items' addresses and the buckets' final sizes, as k_append_items
// places them, without writing the table.
__global__ void __launch_bounds__(64)
    k_gc_dry_append(Table t, uint32_t level, const uint32_t* __restrict__ content, uint32_t* __restrict__ head,
                    const uint32_t* __restrict__ next, const uint32_t* __restrict__ touched,
                    const uint32_t* __restrict__ n_touched, uint32_t* __restrict__ dry_sizes,
                    uint32_t* __restrict__ out_addr, uint32_t* __restrict__ overflow)
{
    __shared__ uint32_t items_s[2][kMaxBucketItems];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t* items = items_s[warp];
    const bool leaf = level == t.g.leaf_level;
    const uint32_t nt = *n_touched;
    const uint32_t first = t.g.level_first_bucket(level);
    for (uint32_t ti = blockIdx.x * 2 + warp; ti < nt; ti += gridDim.x * 2) {
        const uint32_t gb = touched[ti];
        const uint32_t cnt = collect_sorted(gb, head, next, items, t.error);
        if (cnt == 0)
            continue;
        const uint32_t bucket = gb - first;
        if (lane == 0) {
            uint32_t size = dry_sizes[bucket];
            for (uint32_t i = 0; i < cnt; i++) {
                const uint32_t r = items[i];
                const uint32_t n = leaf ? 2 : total_size(content[9 * uint64_t(r)]);
                out_addr[r] = t.g.make_ptr(level, bucket, append_position(size, n, leaf));
            }
            if (size > t.g.capacity(level))
                atomicExch(overflow, 1u);
            dry_sizes[bucket] = size;
        }
        __syncwarp();
    }
}

// Pages the level's rebuild maps (unmapped pages below a bucket's final
// size) and, releasing, frees (mapped pages wholly past it).
__global__ void k_gc_dry_pages(Table t, uint32_t level, const uint32_t* __restrict__ dry_sizes, uint32_t release,
                               unsigned long long* need, unsigned long long* freed)
{
    const uint32_t cap = t.g.capacity(level);
    unsigned long long a = 0, f = 0;
    HD_GRID_STRIDE(i, t.g.buckets(level))
    {
        const uint32_t bucket = uint32_t(i), size = dry_sizes[bucket];
        for (uint32_t off = 0; off < cap; off += kPage) {
            const bool mapped = t.page_table[t.g.make_ptr(level, bucket, off) >> kPageShift] != 0;
            if (off < size)
                a += !mapped;
            else if (release)
                f += mapped;
        }
    }
    for (int o = 16; o; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        f += __shfl_down_sync(0xffffffffu, f, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(need, a);
        atomicAdd(freed, f);
    }
}

__global__ void k_gc_remap_roots(const uint32_t* __restrict__ live, uint32_t n, const uint32_t* __restrict__ newaddr,
                                 uint32_t* roots, uint32_t n_roots, uint32_t* d_root)
{
    for (uint32_t i = 0; i < n_roots; i++)
        roots[i] = newaddr[lower_bound(live, n, roots[i])];
    *d_root = roots[0];
}

namespace {
// The rebuild may claim the pages other claims leave as the GC's reserve
// (hd_set_page_reserve); the limit comes back however the GC ends.
struct ReserveOpen {
    hd_ctx* c;
    explicit ReserveOpen(hd_ctx* ctx) : c(ctx) { set_claim_limit(c, true); }
    ~ReserveOpen()
    {
        try {
            set_claim_limit(c, false);
        } catch (...) {
        }
    }
};
} // namespace

void gc(hd_ctx* c, std::vector<uint32_t>& roots, bool release_pages)
{
    cudaStream_t st = c->stream;
    Scratch& s = c->scratch;
    const Geom& g = c->g;
    const uint32_t leafl = g.leaf_level;
    ReserveOpen reserve_open(c);
    uint32_t* d_n = s.get<uint32_t>("gc_n", 4);
    // level 0: the roots, sorted unique
    std::vector<uint32_t> r0(roots.begin(), roots.end());
    std::sort(r0.begin(), r0.end());
    r0.erase(std::unique(r0.begin(), r0.end()), r0.end());
    std::vector<uint32_t*> live(leafl + 1), newaddr(leafl + 1);
    std::vector<uint32_t> nlive(leafl + 1);
    live[0] = s.get<uint32_t>("gc_live_0", r0.size());
    HD_CUDA(cudaMemcpyAsync(live[0], r0.data(), r0.size() * 4, cudaMemcpyHostToDevice, st));
    nlive[0] = uint32_t(r0.size());
    // mark; every level's bitmap and word ranks stay for the gathers
    std::vector<uint32_t*> bm(leafl + 1, nullptr), bpos(leafl + 1, nullptr);
    std::vector<uint32_t> bbase(leafl + 1, 0);
    for (uint32_t L = 0; L < leafl; L++) {
        const uint32_t base = g.make_ptr(L + 1, 0, 0);
        const uint64_t range = uint64_t(g.buckets(L + 1)) * g.capacity(L + 1);
        const uint64_t nwords = (range + 31) / 32;
        char bn[32];
        snprintf(bn, sizeof(bn), "gc_bitmap_%u", L + 1);
        uint32_t* bitmap = s.get<uint32_t>(bn, nwords);
        HD_CUDA(cudaMemsetAsync(bitmap, 0, nwords * 4, st));
        k_gc_mark<<<grid_for(nlive[L], 256), 256, 0, st>>>(c->t, live[L], nlive[L], base, bitmap);
        HD_LAUNCH_CHECK();
        uint32_t* counts = s.get<uint32_t>("gc_counts", nwords);
        snprintf(bn, sizeof(bn), "gc_pos_%u", L + 1);
        uint32_t* pos = s.get<uint32_t>(bn, nwords);
        bm[L + 1] = bitmap;
        bpos[L + 1] = pos;
        bbase[L + 1] = base;
        k_popc_words<<<grid_for(nwords, 256), 256, 0, st>>>(bitmap, nwords, counts);
        HD_LAUNCH_CHECK();
        exclusive_scan<uint32_t, uint32_t>(s, counts, pos, nwords, d_n, st);
        nlive[L + 1] = read_scalar(d_n, st);
        char nm[32];
        snprintf(nm, sizeof(nm), "gc_live_%u", L + 1);
        live[L + 1] = s.get<uint32_t>(nm, uint64_t(nlive[L + 1]) + 1);
        k_bitmap_to_list<<<grid_for(nwords, 256), 256, 0, st>>>(bitmap, pos, nwords, base, live[L + 1]);
        HD_LAUNCH_CHECK();
    }
    uint32_t maxn = 1;
    for (uint32_t L = 0; L <= leafl; L++)
        maxn = std::max(maxn, nlive[L]);
    uint32_t* content = s.get<uint32_t>("gc_content", uint64_t(maxn) * 9);
    uint32_t* next = s.get<uint32_t>("gc_next", maxn);
    uint32_t* head = s.get<uint32_t>("gc_head", g.total_buckets);
    uint32_t* touched = s.get<uint32_t>("gc_touched", g.total_buckets);
    fill<uint32_t>(head, kEmpty, g.total_buckets, st);
    // dry run, bottom-up: the pages every level's rebuild needs against the
    // free pages (and those the levels below free when releasing)
    {
        uint32_t top[2];
        HD_CUDA(cudaMemcpyAsync(top, c->t.pool_top, 8, cudaMemcpyDeviceToHost, st));
        uint32_t* dry_all = s.get<uint32_t>("gc_dry_sizes", g.total_buckets);
        uint32_t* full_dry = s.get<uint32_t>("gc_full_dry", HD_MAX_DEPTH);
        uint32_t* dry_addr[2] = {s.get<uint32_t>("gc_dry_addr_a", uint64_t(maxn) + 1),
                                 s.get<uint32_t>("gc_dry_addr_b", uint64_t(maxn) + 1)};
        unsigned long long* cnt = s.get<unsigned long long>("gc_dry_cnt", 2);
        uint32_t* overflow = s.get<uint32_t>("gc_dry_overflow", 1);
        HD_CUDA(cudaMemsetAsync(overflow, 0, 4, st));
        HD_CUDA(cudaStreamSynchronize(st));
        int64_t avail = int64_t(g.pool_pages) - top[0] + top[1];
        for (int32_t L = int32_t(leafl); L >= 0; L--) {
            const uint32_t n = nlive[L];
            uint32_t* addr = dry_addr[L & 1];
            const uint32_t* child_addr = dry_addr[(L + 1) & 1];
            uint32_t* dry_sizes = dry_all + g.level_first_bucket(uint32_t(L));
            HD_CUDA(cudaMemsetAsync(dry_sizes, 0, uint64_t(g.buckets(uint32_t(L))) * 4, st));
            HD_CUDA(cudaMemsetAsync(d_n, 0, 4, st));
            k_gc_dry_full<<<1, 1, 0, st>>>(c->t, uint32_t(L), dry_sizes, full_dry);
            HD_LAUNCH_CHECK();
            k_gc_gather<<<grid_for(n, 256), 256, 0, st>>>(c->t, uint32_t(L), live[L], n,
                                                          L < int32_t(leafl) ? bm[L + 1] : nullptr,
                                                          L < int32_t(leafl) ? bpos[L + 1] : nullptr,
                                                          L < int32_t(leafl) ? bbase[L + 1] : 0u,
                                                          L < int32_t(leafl) ? child_addr : nullptr, content, head,
                                                          next, touched, d_n);
            HD_LAUNCH_CHECK();
            k_gc_dry_append<<<grid_for(uint64_t(n) * 32, 64, 152 * 16), 64, 0, st>>>(
                c->t, uint32_t(L), content, head, next, touched, d_n, dry_sizes, addr, overflow);
            HD_LAUNCH_CHECK();
            HD_CUDA(cudaMemsetAsync(cnt, 0, 16, st));
            k_gc_dry_pages<<<grid_for(g.buckets(uint32_t(L)), 256), 256, 0, st>>>(
                c->t, uint32_t(L), dry_sizes, release_pages ? 1u : 0u, cnt, cnt + 1);
            HD_LAUNCH_CHECK();
            unsigned long long h[2];
            uint32_t ovf = 0;
            HD_CUDA(cudaMemcpyAsync(h, cnt, 16, cudaMemcpyDeviceToHost, st));
            HD_CUDA(cudaMemcpyAsync(&ovf, overflow, 4, cudaMemcpyDeviceToHost, st));
            HD_CUDA(cudaStreamSynchronize(st));
            if (ovf)
                throw StatusError{HD_ERR_BUCKET_FULL, "GC: a rebuilt bucket of level " + std::to_string(L) +
                                                          " would exceed its capacity; the table is unchanged"};
            // releasing: the level's pages past the final sizes are freed
            // before its appends claim
            avail += int64_t(h[1]);
            if (int64_t(h[0]) > avail)
                throw StatusError{HD_ERR_POOL_FULL, "GC: rebuilding level " + std::to_string(L) + " needs " +
                                                        std::to_string(h[0]) + " new pages, " +
                                                        std::to_string(std::max<int64_t>(avail, 0)) +
                                                        " are free; the table is unchanged"};
            avail -= int64_t(h[0]);
        }
        const uint32_t e = check_error(c); // a bucket list over kMaxBucketItems in the dry run
        if (e)
            throw StatusError{hd_status(e), "GC: " + c->err_detail + "; the table is unchanged"};
    }
    // rebuild bottom-up
    const uint32_t* dry_all = s.get<uint32_t>("gc_dry_sizes", g.total_buckets);
    for (int32_t L = int32_t(leafl); L >= 0; L--) {
        const uint32_t n = nlive[L];
        char nm[32];
        snprintf(nm, sizeof(nm), "gc_new_%d", L);
        newaddr[L] = s.get<uint32_t>(nm, uint64_t(n) + 1);
        HD_CUDA(cudaMemsetAsync(d_n, 0, 4, st));
        k_gc_gather<<<grid_for(n, 256), 256, 0, st>>>(c->t, uint32_t(L), live[L], n,
                                                      L < int32_t(leafl) ? bm[L + 1] : nullptr,
                                                      L < int32_t(leafl) ? bpos[L + 1] : nullptr,
                                                      L < int32_t(leafl) ? bbase[L + 1] : 0u,
                                                      L < int32_t(leafl) ? newaddr[L + 1] : nullptr, content, head,
                                                      next, touched, d_n);
        HD_LAUNCH_CHECK();
        // empty the level's buckets and their pages' filters, then the
        // full node first
        HD_CUDA(cudaMemsetAsync(c->t.bucket_sizes + g.level_first_bucket(uint32_t(L)), 0,
                                uint64_t(g.buckets(uint32_t(L))) * 4, st));
        bloom_clear_level(c, uint32_t(L));
        HD_CUDA(cudaMemsetAsync(c->t.level_nodes + L, 0, 8, st));
        if (release_pages) {
            // the level's pages past its final bucket sizes (the dry run's),
            // zeroed, serve this level's appends and the levels above
            uint32_t before[2], after[2];
            HD_CUDA(cudaMemcpyAsync(before, c->t.pool_top, 8, cudaMemcpyDeviceToHost, st));
            k_gc_release<<<grid_for(g.buckets(uint32_t(L)), 256), 256, 0, st>>>(
                c->t, uint32_t(L), dry_all + g.level_first_bucket(uint32_t(L)));
            HD_LAUNCH_CHECK();
            HD_CUDA(cudaMemcpyAsync(after, c->t.pool_top, 8, cudaMemcpyDeviceToHost, st));
            HD_CUDA(cudaStreamSynchronize(st));
            if (after[1] > before[1]) {
                k_zero_pages<<<grid_for(uint64_t(after[1] - before[1]) * kPage, 256), 256, 0, st>>>(c->t, before[1],
                                                                                                   after[1]);
                HD_LAUNCH_CHECK();
            }
        }
        add_full_nodes(c, uint32_t(L), uint32_t(L));
        append_items(c, uint32_t(L), content, n, head, next, touched, d_n, newaddr[L]);
    }
    uint32_t* d_roots = s.get<uint32_t>("gc_roots", roots.size());
    HD_CUDA(cudaMemcpyAsync(d_roots, roots.data(), roots.size() * 4, cudaMemcpyHostToDevice, st));
    k_gc_remap_roots<<<1, 1, 0, st>>>(live[0], nlive[0], newaddr[0], d_roots, uint32_t(roots.size()), c->d_root);
    HD_LAUNCH_CHECK();
    HD_CUDA(cudaMemcpyAsync(roots.data(), d_roots, roots.size() * 4, cudaMemcpyDeviceToHost, st));
    HD_CUDA(cudaStreamSynchronize(st));
    const uint32_t e = check_error(c);
    if (e)
        throw StatusError{hd_status(e), "garbage collection failed on the device"};
    c->root = roots[0];
    c->edit_head_ready = false;
}

} // namespace hd

extern "C" hd_status hd_gc_ex(hd_ctx* c, uint32_t* extra, uint32_t n, uint32_t flags)
{
    if (!c || (n && !extra) || (flags & ~uint32_t(HD_GC_KEEP_HISTORY | HD_GC_RELEASE_PAGES)))
        return HD_ERR_INVALID;
    try {
        std::vector<uint32_t> roots(1 + n);
        roots[0] = hd::read_scalar(c->d_root, c->stream);
        for (uint32_t i = 0; i < n; i++)
            roots[1 + i] = extra[i];
        if (flags & HD_GC_KEEP_HISTORY) {
            // the roots of the undo / redo frames stay alive and are remapped
            for (auto& f : c->undo)
                roots.push_back(f.root);
            for (auto& f : c->redo)
                roots.push_back(f.root);
        } else {
            // the engine frees its undo history with the GC (engine.cpp:178-185)
            c->undo.clear();
            c->redo.clear();
        }
        hd::gc(c, roots, (flags & HD_GC_RELEASE_PAGES) != 0);
        c->needs_gc = false; // the buckets are rebuilt
        // the remapped extra roots go back to the caller
        for (uint32_t i = 0; i < n; i++)
            extra[i] = roots[1 + i];
        size_t k = 1 + n;
        if (flags & HD_GC_KEEP_HISTORY) {
            for (auto& f : c->undo)
                f.root = roots[k++];
            for (auto& f : c->redo)
                f.root = roots[k++];
        }
        return HD_OK;
    } catch (const hd::StatusError& e) {
        c->err = e.msg;
        return e.status;
    } catch (const hd::CudaError& e) {
        c->err = std::string("CUDA error ") + cudaGetErrorString(e.code) + " in " + e.where;
        return HD_ERR_CUDA;
    }
}

extern "C" hd_status hd_gc(hd_ctx* c, uint32_t* extra, uint32_t n) { return hd_gc_ex(c, extra, n, 0); }
