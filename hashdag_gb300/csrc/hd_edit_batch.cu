// Batched edits: a device-driven edit pipeline captured once into a CUDA
// graph and launched once per edit, back to back, with no host round trip
// between edits or between levels.
//
// Same per-entry logic, same order of bucket scans and appends, hence the
// same table, as applying the edits one by one (hd_edit.cu): the edit of
// HashDAG::edit_threads (hash_dag.h:255-405) applied in sequence.  What
// differs is the orchestration:
//  * every kernel reads its level's entry count from a device state block
//    and runs on a fixed grid, so one captured graph serves every edit;
//  * level arrays are sized for the whole batch from the tools' extents (an
//    upper bound of the entries a level can hold); a level that would
//    overflow stops the batch before the edit touches the table, and the
//    host applies that edit with the one-edit path, then resumes;
//  * candidate grouping by bucket is a two-pass stable radix sort on the
//    level-local bucket, and find-or-add warps find their buckets' runs in
//    the sorted keys themselves.
// Tuning (warps per find-or-add block, probe width, grid size) is chosen by
// hd_autotune_batch on a copy of the table.
#include <chrono>
#include <cmath>
#include <vector>

#include "hd_edit.cuh"

namespace hd {

void edit_one(hd_ctx* c, const hd_edit& e, hd_edit_stats* stats); // hd_edit.cu
// hd_edit_persist.cu
void edit_batch_persistent(hd_ctx* c, const hd_edit* edits, uint32_t n, const std::vector<Level>& lv,
                           const std::vector<uint32_t>& caps, uint32_t* keys, uint32_t* vals, uint32_t* keys2,
                           uint32_t* vals2, hd_edit* d_edits, EditCounters* d_ctr, uint32_t* d_roots,
                           std::vector<EditCounters>& ctr, std::vector<float>& dur_ms, std::vector<float>& end_ms,
                           float& device_ms, uint64_t& fallbacks);

enum : uint32_t { kStopNone = 0, kStopCapacity = 1, kStopTableError = 2, kStopEmptyScene = 3 };

struct BatchState {
    uint32_t idx;                  // edit being applied
    uint32_t skip;                 // the rest of this launch does nothing
    uint32_t stop;                 // kStop*: the batch stopped at edit idx
    uint32_t pad;
    uint32_t count[HD_MAX_DEPTH];  // entries of each level of the current edit
    Editor ed;
};

constexpr uint32_t kLevelThreads = kScanThreads; // block_excl_scan wants 512

HD_D uint32_t chunk_of(uint32_t n, uint32_t blocks, uint32_t align)
{
    const uint32_t per = (n + blocks - 1) / blocks;
    return (per + align - 1) / align * align;
}

__global__ void k_b_begin(BatchState* bs, const hd_edit* __restrict__ edits, uint32_t n_edits, Level lv0,
                          const uint32_t* __restrict__ d_root, EditCounters* ctr, const uint32_t* __restrict__ err)
{
    if (threadIdx.x != 0)
        return;
    const uint32_t idx = bs->idx;
    const bool skip = bs->stop != kStopNone || idx >= n_edits || err[0] != 0;
    bs->skip = skip;
    if (skip)
        return;
    bs->ed = make_editor(edits[idx]);
    bs->count[0] = 1;
    for (uint32_t L = 1; L < HD_MAX_DEPTH; L++)
        bs->count[L] = 0;
    lv0.x[0] = 0;
    lv0.y[0] = 0;
    lv0.z[0] = 0;
    lv0.old[0] = *d_root;
    ctr[idx] = EditCounters{};
}

// Top-down, level L: classify a contiguous chunk per block; bsum[block] =
// descended entries of the chunk.
__global__ void __launch_bounds__(kLevelThreads)
    k_b_classify(Table t, const BatchState* bs, uint32_t level, Level lv, EditCounters* ctr, uint32_t* bsum)
{
    if (bs->skip)
        return;
    const uint32_t n = bs->count[level];
    const Editor ed = bs->ed;
    EditCounters* mine = ctr + bs->idx;
    const uint32_t chunk = chunk_of(n, gridDim.x, kLevelThreads);
    const uint32_t i0 = blockIdx.x * chunk, i1 = min(n, i0 + chunk);
    uint32_t flags = 0;
    for (uint32_t i = i0 + threadIdx.x; i < i1; i += kLevelThreads) {
        unsigned long long nodes, voxels;
        classify_entry(t, ed, level, lv, i, nodes, voxels);
        flags += lv.flag[i];
        warp_add(&mine->num_nodes, nodes);
        warp_add(&mine->num_voxels, voxels);
    }
    uint32_t total;
    block_excl_scan(flags, &total);
    if (threadIdx.x == 0)
        bsum[blockIdx.x] = total;
}

// bsum -> exclusive block offsets; the next level's entry count (8 per
// descended entry), checked against its capacity.
__global__ void __launch_bounds__(kScanThreads)
    k_b_scan_blocks(BatchState* bs, uint32_t level, uint32_t* bsum, uint32_t blocks, uint32_t cap_next)
{
    if (bs->skip)
        return;
    const uint32_t per = (blocks + kScanThreads - 1) / kScanThreads;
    const uint32_t b0 = threadIdx.x * per;
    uint32_t s = 0;
    for (uint32_t k = 0; k < per; k++)
        if (b0 + k < blocks)
            s += bsum[b0 + k];
    uint32_t total;
    uint32_t off = block_excl_scan(s, &total);
    for (uint32_t k = 0; k < per; k++)
        if (b0 + k < blocks) {
            const uint32_t v = bsum[b0 + k];
            bsum[b0 + k] = off;
            off += v;
        }
    if (threadIdx.x == 0) {
        const uint64_t next = 8ull * total;
        if (next > cap_next) {
            bs->stop = kStopCapacity;
            bs->skip = 1;
        } else {
            bs->count[level + 1] = uint32_t(next);
        }
    }
}

// Same chunks as k_b_classify: exclusive scan of the flags -> exp, spawn.
__global__ void __launch_bounds__(kLevelThreads)
    k_b_spawn(Table t, const BatchState* bs, uint32_t level, Level lv, Level next, const uint32_t* __restrict__ bsum)
{
    if (bs->skip)
        return;
    const uint32_t n = bs->count[level];
    const uint32_t chunk = chunk_of(n, gridDim.x, kLevelThreads);
    const uint32_t i0 = blockIdx.x * chunk, i1 = min(n, i0 + chunk);
    uint32_t run = bsum[blockIdx.x];
    for (uint32_t base = i0; base < i1; base += kLevelThreads) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t f = i < i1 ? lv.flag[i] : 0u;
        uint32_t total;
        const uint32_t off = block_excl_scan(f, &total);
        if (i < i1) {
            lv.exp[i] = run + off;
            spawn_entry(t, lv, next, i);
        }
        run += total;
    }
}

// Bottom-up, level L: candidates keyed by level-local bucket; resolved
// entries get the key `buckets(L)`, which sorts after every bucket.
__global__ void k_b_candidates(Table t, const BatchState* bs, uint32_t level, Level lv, Level child, uint32_t* keys,
                               uint32_t* vals)
{
    if (bs->skip || __ldcg(t.error) != 0) // after a failed append, levels above are not rebuilt
        return;
    const uint32_t n = bs->count[level];
    const uint32_t empty = t.g.buckets(level);
    HD_GRID_STRIDE(i, n)
    {
        const uint32_t b = candidate_entry(t, level, lv, child, uint32_t(i));
        keys[i] = b == kNoBucket ? empty : b;
        vals[i] = uint32_t(i);
    }
}

constexpr uint32_t kSortBlock = 256;
constexpr uint32_t kMaxDigits = 512;

// The sort uses as many blocks as its input needs (at least kSortBlock keys
// each, at most the grid): a chunk of the input per block.
HD_D uint32_t sort_blocks(uint32_t n, uint32_t grid)
{
    const uint32_t want = (n + kSortBlock - 1) / kSortBlock;
    return want < 1 ? 1 : (want < grid ? want : grid);
}

// Digit histogram of a block's chunk: hist[d * nb + block].
__global__ void __launch_bounds__(kSortBlock)
    k_b_hist(const BatchState* bs, uint32_t level, const uint32_t* __restrict__ keys, uint32_t shift, uint32_t dbits,
             uint32_t* __restrict__ hist)
{
    if (bs->skip)
        return;
    const uint32_t n = bs->count[level];
    const uint32_t nb = sort_blocks(n, gridDim.x);
    if (blockIdx.x >= nb)
        return;
    __shared__ uint32_t cnt[kMaxDigits];
    const uint32_t nd = 1u << dbits;
    for (uint32_t d = threadIdx.x; d < nd; d += kSortBlock)
        cnt[d] = 0;
    __syncthreads();
    const uint32_t chunk = chunk_of(n, nb, kSortBlock);
    const uint32_t i0 = blockIdx.x * chunk, i1 = min(n, i0 + chunk);
    for (uint32_t i = i0 + threadIdx.x; i < i1; i += kSortBlock)
        atomicAdd(&cnt[(keys[i] >> shift) & (nd - 1)], 1u);
    __syncthreads();
    for (uint32_t d = threadIdx.x; d < nd; d += kSortBlock)
        hist[d * nb + blockIdx.x] = cnt[d];
}

// Per digit row of hist: exclusive scan over the blocks in place, and the
// row total.  A warp per row.
__global__ void __launch_bounds__(kScanThreads)
    k_b_hist_rows(const BatchState* bs, uint32_t level, uint32_t* __restrict__ hist, uint32_t grid, uint32_t dbits,
                  uint32_t* __restrict__ row_total)
{
    if (bs->skip)
        return;
    const uint32_t nb = sort_blocks(bs->count[level], grid);
    const uint32_t nd = 1u << dbits;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = gridDim.x * (kScanThreads / 32);
    for (uint32_t d = blockIdx.x * (kScanThreads / 32) + (threadIdx.x >> 5); d < nd; d += warps) {
        uint32_t run = 0;
        for (uint32_t b0 = 0; b0 < nb; b0 += 32) {
            const uint32_t b = b0 + lane;
            const uint32_t x = b < nb ? hist[d * nb + b] : 0u;
            const uint32_t inc = warp_incl_scan(x);
            if (b < nb)
                hist[d * nb + b] = run + inc - x;
            run += __shfl_sync(0xffffffffu, inc, 31);
        }
        if (lane == 0)
            row_total[d] = run;
    }
}

// Stable scatter: a block walks its chunk in order, 256 keys at a time; equal
// digits inside a warp rank by lane, warps take their turn in order.
__global__ void __launch_bounds__(kSortBlock)
    k_b_scatter(const BatchState* bs, uint32_t level, const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                uint32_t shift, uint32_t dbits, const uint32_t* __restrict__ offs,
                const uint32_t* __restrict__ row_total, uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out)
{
    if (bs->skip)
        return;
    const uint32_t n = bs->count[level];
    const uint32_t nb = sort_blocks(n, gridDim.x);
    if (blockIdx.x >= nb)
        return;
    __shared__ uint32_t run[kMaxDigits];
    __shared__ uint32_t wsum[kSortBlock / 32];
    const uint32_t nd = 1u << dbits;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    {
        // digit bases: exclusive scan of the row totals, two digits a thread
        const uint32_t d0 = 2 * threadIdx.x;
        const uint32_t a = d0 < nd ? row_total[d0] : 0u, b = d0 + 1 < nd ? row_total[d0 + 1] : 0u;
        const uint32_t inc = warp_incl_scan(a + b);
        if (lane == 31)
            wsum[warp] = inc;
        __syncthreads();
        uint32_t before = 0;
        for (uint32_t w = 0; w < warp; w++)
            before += wsum[w];
        const uint32_t ex = before + inc - (a + b);
        if (d0 < nd)
            run[d0] = ex + offs[d0 * nb + blockIdx.x];
        if (d0 + 1 < nd)
            run[d0 + 1] = ex + a + offs[(d0 + 1) * nb + blockIdx.x];
    }
    const uint32_t chunk = chunk_of(n, nb, kSortBlock);
    const uint32_t i0 = blockIdx.x * chunk, i1 = min(n, i0 + chunk);
    for (uint32_t base = i0; base < i1; base += kSortBlock) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < i1;
        const uint32_t key = valid ? keys[i] : 0u;
        const uint32_t val = valid ? vals[i] : 0u;
        const uint32_t digit = valid ? (key >> shift) & (nd - 1) : kMaxDigits + lane; // invalid lanes alone
        const uint32_t peers = __match_any_sync(0xffffffffu, digit);
        const uint32_t leader = __ffs(peers) - 1;
        for (uint32_t w = 0; w < kSortBlock / 32; w++) {
            __syncthreads();
            if (warp == w) {
                uint32_t b = 0;
                if (valid && lane == leader) {
                    b = run[digit];
                    run[digit] = b + __popc(peers);
                }
                b = __shfl_sync(0xffffffffu, b, leader);
                if (valid) {
                    const uint32_t pos = b + __popc(peers & lt);
                    keys_out[pos] = key;
                    vals_out[pos] = val;
                }
            }
        }
    }
}

// Find-or-add over the sorted keys: the sorted positions are split into one
// chunk per warp (ceil(n / warps) positions, at least one), and each warp
// resolves every bucket run that starts in its chunk, so that short runs
// spread over all the warps.
template <int PW, uint32_t WARPS>
__global__ void __launch_bounds__(32 * WARPS)
    k_b_find_or_add(Table t, const BatchState* bs, uint32_t level, Level lv, const uint32_t* __restrict__ keys,
                    const uint32_t* __restrict__ vals, EditCounters* ctr)
{
    if (bs->skip || __ldcg(t.error) != 0)
        return;
    __shared__ uint32_t page_s[WARPS][kPage];
    __shared__ uint32_t q_s[WARPS][9];
    __shared__ FoaCache cache_s[WARPS];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t n = bs->count[level];
    const uint32_t empty = t.g.buckets(level);
    unsigned long long foa = 0, added = 0, scanned = 0;
    const uint32_t nw = gridDim.x * WARPS, gw = blockIdx.x * WARPS + warp;
    const uint32_t chunk = n > nw ? (n + nw - 1) / nw : 1u;
    const uint64_t cbeg64 = uint64_t(gw) * chunk;
    const uint32_t cbeg = cbeg64 < n ? uint32_t(cbeg64) : n, cend = n - cbeg < chunk ? n : cbeg + chunk;
    for (uint32_t c0 = cbeg; c0 < cend; c0 += 32) {
        const uint32_t j = c0 + lane;
        const bool in = j < cend;
        const uint32_t key = in ? keys[j] : empty;
        const uint32_t prev = (in && j > 0) ? keys[j - 1] : kNoBucket;
        uint32_t starts = __ballot_sync(0xffffffffu, in && key < empty && key != prev);
        while (starts) {
            const uint32_t s = __ffs(starts) - 1;
            starts &= starts - 1;
            const uint32_t j0 = c0 + s;
            const uint32_t bucket = __shfl_sync(0xffffffffu, key, s);
            // the run ends at the first different key
            uint32_t j1 = j0 + 1;
            for (;;) {
                const uint32_t jj = j1 + lane;
                const uint32_t k = jj < n ? keys[jj] : kNoBucket;
                const uint32_t diff = __ballot_sync(0xffffffffu, k != bucket);
                if (diff) {
                    j1 += __ffs(diff) - 1;
                    break;
                }
                j1 += 32;
            }
            foa_segment<PW>(t, level, lv, vals, j0, j1, bucket, page_s[warp], q_s[warp], cache_s[warp], foa, added,
                            scanned);
        }
    }
    if (lane == 0 && (foa | added | scanned)) {
        EditCounters* mine = ctr + bs->idx;
        atomicAdd(&mine->foa, foa);
        atomicAdd(&mine->added, added);
        atomicAdd(&mine->scanned, scanned);
        atomicAdd(reinterpret_cast<unsigned long long*>(t.level_nodes + level), added);
    }
}

__global__ void k_b_finish(BatchState* bs, const Level lv0, uint32_t* d_root, uint32_t* roots_out,
                           const uint32_t* __restrict__ err)
{
    if (bs->skip)
        return;
    if (err[0] != 0) {
        bs->stop = kStopTableError;
        return;
    }
    const uint32_t r = lv0.res[0];
    if (r == kInvalid || r == kNotFound) {
        bs->stop = kStopEmptyScene;
        return;
    }
    *d_root = r;
    roots_out[bs->idx] = r;
    bs->idx += 1;
}

// ---- host side ------------------------------------------------------------------

// Upper bound of the entries of every level for one edit: 8 per descended
// entry of the level above.  Above C_colorTreeLevels every node the tool's
// box overlaps descends; below, only nodes that cross the tool's surface,
// which lie within 2 node sizes of it.
static void edit_caps(const Geom& g, const hd_edit& e, std::vector<uint64_t>& cap)
{
    const uint32_t D = g.depth, leafl = g.leaf_level;
    const double r = double(e.radius) + 1.0;
    const bool sphere = e.tool == HD_TOOL_SPHERE_ADD || e.tool == HD_TOOL_SPHERE_REMOVE;
    cap[0] = std::max<uint64_t>(cap[0], 1);
    for (uint32_t L = 0; L < leafl; L++) {
        const double s = std::ldexp(1.0, int(D - L));
        const double side = std::ldexp(1.0, int(L));
        double box = 1.0;
        for (int a = 0; a < 3; a++) {
            double lo = std::floor((double(e.center[a]) - r) / s), hi = std::floor((double(e.center[a]) + r) / s);
            lo = std::max(lo, 0.0);
            hi = std::min(hi, side - 1.0);
            box *= std::max(0.0, hi - lo + 1.0);
        }
        double desc = std::min(box, side * side * side);
        if (L >= g.T) {
            double shell;
            if (sphere) {
                const double ro = r + 2.0 * s, ri = std::max(0.0, r - 2.0 * s);
                shell = 4.18879020478639 * (ro * ro * ro - ri * ri * ri) / (s * s * s);
            } else {
                const double ao = 2.0 * r + 4.0 * s, ai = std::max(0.0, 2.0 * r - 4.0 * s);
                shell = (ao * ao * ao - ai * ai * ai) / (s * s * s);
            }
            desc = std::min(desc, std::ceil(shell) + 64.0);
        }
        cap[L + 1] = std::max<uint64_t>(cap[L + 1], uint64_t(8.0 * desc));
    }
}

struct BatchGraph {
    cudaGraphExec_t exec = nullptr;
    std::vector<void*> ptrs; // buffers the graph was captured with
    hd_batch_tuning tuning{};
    std::vector<uint32_t> caps;
    uint32_t edit_cap = 0;
    std::vector<cudaEvent_t> events;
    ~BatchGraph()
    {
        if (exec)
            cudaGraphExecDestroy(exec);
        for (auto e : events)
            cudaEventDestroy(e);
    }
};

struct BatchBuffers {
    std::vector<Level> lv;
    std::vector<uint32_t> caps;
    uint32_t *keys, *vals, *keys2, *vals2, *bsum, *hist, *rows, *roots;
    hd_edit* edits;
    EditCounters* ctr;
    BatchState* bs;
    uint32_t edit_cap;
    std::vector<void*> ptrs() const
    {
        std::vector<void*> p{keys, vals, keys2, vals2, bsum, hist, rows, roots, edits, ctr, bs};
        for (const Level& l : lv)
            p.insert(p.end(), {l.x, l.y, l.z, l.old, l.state, l.res, l.cnt, l.flag, l.exp, l.leaf, l.cand});
        return p;
    }
};

static Level batch_level(Scratch& s, uint32_t L, uint64_t n, bool leaf)
{
    char nm[48];
    auto buf = [&](const char* what, size_t bytes) {
        snprintf(nm, sizeof(nm), "eb_%s_%u", what, L);
        return s.get(nm, bytes);
    };
    Level l{};
    l.x = static_cast<uint32_t*>(buf("x", n * 4));
    l.y = static_cast<uint32_t*>(buf("y", n * 4));
    l.z = static_cast<uint32_t*>(buf("z", n * 4));
    l.old = static_cast<uint32_t*>(buf("old", n * 4));
    l.state = static_cast<uint8_t*>(buf("state", n));
    l.res = static_cast<uint32_t*>(buf("res", n * 4));
    l.cnt = static_cast<uint32_t*>(buf("cnt", n * 4));
    l.flag = static_cast<uint32_t*>(buf("flag", n * 4));
    l.exp = static_cast<uint32_t*>(buf("exp", n * 4));
    l.leaf = leaf ? static_cast<uint64_t*>(buf("leaf", n * 8)) : nullptr;
    l.cand = static_cast<uint32_t*>(buf("cand", n * 36));
    return l;
}

static BatchBuffers batch_buffers(hd_ctx* c, const std::vector<uint64_t>& cap64, uint32_t n_edits)
{
    Scratch& s = c->scratch;
    const Geom& g = c->g;
    const uint32_t levels = g.leaf_level + 1;
    const uint32_t blocks = c->tuning.grid_blocks;
    BatchBuffers b{};
    b.caps.resize(levels);
    uint64_t maxn = 1;
    for (uint32_t L = 0; L < levels; L++) {
        const uint64_t v = std::min<uint64_t>(std::max<uint64_t>(cap64[L], 256), 0xFFFFFFF0ull / 9);
        b.caps[L] = uint32_t(v);
        maxn = std::max(maxn, v);
    }
    b.lv.resize(levels);
    for (uint32_t L = 0; L < levels; L++)
        b.lv[L] = batch_level(s, L, b.caps[L], L == g.leaf_level);
    b.keys = s.get<uint32_t>("eb_keys", maxn);
    b.vals = s.get<uint32_t>("eb_vals", maxn);
    b.keys2 = s.get<uint32_t>("eb_keys2", maxn);
    b.vals2 = s.get<uint32_t>("eb_vals2", maxn);
    b.bsum = s.get<uint32_t>("eb_bsum", blocks);
    b.hist = s.get<uint32_t>("eb_hist", uint64_t(kMaxDigits) * blocks);
    b.rows = s.get<uint32_t>("eb_rows", kMaxDigits);
    b.edit_cap = 64;
    while (b.edit_cap < n_edits)
        b.edit_cap <<= 1;
    b.roots = s.get<uint32_t>("eb_roots", b.edit_cap);
    b.edits = s.get<hd_edit>("eb_edits", b.edit_cap);
    b.ctr = s.get<EditCounters>("eb_ctr", b.edit_cap);
    b.bs = s.get<BatchState>("eb_state", 1);
    return b;
}

constexpr uint32_t kFoaBatchWarps = 152 * 32;

template <int PW, uint32_t WARPS>
static void launch_foa(hd_ctx* c, const BatchBuffers& b, uint32_t L, cudaStream_t st)
{
    // 4864 warps (32 per SM) whatever the block shape
    k_b_find_or_add<PW, WARPS><<<kFoaBatchWarps / WARPS, 32 * WARPS, 0, st>>>(c->t, b.bs, L, b.lv[L], b.keys, b.vals,
                                                                             b.ctr);
}

// The kernel sequence of one edit (read from edits[state.idx]).
static void enqueue_edit(hd_ctx* c, const BatchBuffers& b, uint32_t n_edits, cudaStream_t st)
{
    const Geom& g = c->g;
    const uint32_t leafl = g.leaf_level;
    const uint32_t G = c->tuning.grid_blocks;
    k_b_begin<<<1, 32, 0, st>>>(b.bs, b.edits, n_edits, b.lv[0], c->d_root, b.ctr, c->t.error);
    HD_LAUNCH_CHECK();
    for (uint32_t L = 0; L <= leafl; L++) {
        k_b_classify<<<G, kLevelThreads, 0, st>>>(c->t, b.bs, L, b.lv[L], b.ctr, b.bsum);
        HD_LAUNCH_CHECK();
        if (L == leafl)
            break;
        k_b_scan_blocks<<<1, kScanThreads, 0, st>>>(b.bs, L, b.bsum, G, b.caps[L + 1]);
        HD_LAUNCH_CHECK();
        k_b_spawn<<<G, kLevelThreads, 0, st>>>(c->t, b.bs, L, b.lv[L], b.lv[L + 1], b.bsum);
        HD_LAUNCH_CHECK();
    }
    for (int32_t L = int32_t(leafl); L >= 0; L--) {
        const Level child = uint32_t(L) < leafl ? b.lv[L + 1] : Level{};
        k_b_candidates<<<G, 256, 0, st>>>(c->t, b.bs, uint32_t(L), b.lv[L], child, b.keys, b.vals);
        HD_LAUNCH_CHECK();
        uint32_t key_bits = 1;
        while ((1u << key_bits) <= g.buckets(uint32_t(L)))
            key_bits++;
        const uint32_t dbits = (key_bits + 1) / 2;
        const uint32_t row_blocks = ((1u << dbits) + kScanThreads / 32 - 1) / (kScanThreads / 32);
        k_b_hist<<<G, kSortBlock, 0, st>>>(b.bs, uint32_t(L), b.keys, 0, dbits, b.hist);
        k_b_hist_rows<<<row_blocks, kScanThreads, 0, st>>>(b.bs, uint32_t(L), b.hist, G, dbits, b.rows);
        k_b_scatter<<<G, kSortBlock, 0, st>>>(b.bs, uint32_t(L), b.keys, b.vals, 0, dbits, b.hist, b.rows, b.keys2,
                                               b.vals2);
        k_b_hist<<<G, kSortBlock, 0, st>>>(b.bs, uint32_t(L), b.keys2, dbits, dbits, b.hist);
        k_b_hist_rows<<<row_blocks, kScanThreads, 0, st>>>(b.bs, uint32_t(L), b.hist, G, dbits, b.rows);
        k_b_scatter<<<G, kSortBlock, 0, st>>>(b.bs, uint32_t(L), b.keys2, b.vals2, dbits, dbits, b.hist, b.rows,
                                               b.keys, b.vals);
        HD_LAUNCH_CHECK();
        const hd_batch_tuning& tu = c->tuning;
        if (tu.probe_words == 4) {
            if (tu.foa_warps == 2)
                launch_foa<4, 2>(c, b, uint32_t(L), st);
            else if (tu.foa_warps == 8)
                launch_foa<4, 8>(c, b, uint32_t(L), st);
            else
                launch_foa<4, 4>(c, b, uint32_t(L), st);
        } else if (tu.probe_words == 2) {
            if (tu.foa_warps == 2)
                launch_foa<2, 2>(c, b, uint32_t(L), st);
            else if (tu.foa_warps == 8)
                launch_foa<2, 8>(c, b, uint32_t(L), st);
            else
                launch_foa<2, 4>(c, b, uint32_t(L), st);
        } else {
            if (tu.foa_warps == 2)
                launch_foa<1, 2>(c, b, uint32_t(L), st);
            else if (tu.foa_warps == 8)
                launch_foa<1, 8>(c, b, uint32_t(L), st);
            else
                launch_foa<1, 4>(c, b, uint32_t(L), st);
        }
        HD_LAUNCH_CHECK();
    }
    k_b_finish<<<1, 1, 0, st>>>(b.bs, b.lv[0], c->d_root, b.roots, c->t.error);
    HD_LAUNCH_CHECK();
}

static void capture(hd_ctx* c, BatchGraph& bg, const BatchBuffers& b, uint32_t n_edits)
{
    if (bg.exec) {
        cudaGraphExecDestroy(bg.exec);
        bg.exec = nullptr;
    }
    cudaStream_t cs;
    HD_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    HD_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    try {
        enqueue_edit(c, b, n_edits, cs);
    } catch (...) {
        cudaStreamEndCapture(cs, &graph);
        if (graph)
            cudaGraphDestroy(graph);
        cudaStreamDestroy(cs);
        throw;
    }
    HD_CUDA(cudaStreamEndCapture(cs, &graph));
    const cudaError_t e = cudaGraphInstantiate(&bg.exec, graph, 0);
    cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    HD_CUDA(e);
    bg.ptrs = b.ptrs();
    bg.tuning = c->tuning;
    bg.caps = b.caps;
    bg.edit_cap = b.edit_cap;
}

// Applies edits[0..n) in order; per_edit (optional, n entries) gets each
// edit's counters, its device time (device_ms) and its completion time since
// the batch started (host_ms, device clock).
void edit_batch(hd_ctx* c, const hd_edit* edits, uint32_t n, hd_edit_stats* per_edit, hd_edit_stats* total)
{
    if (c->needs_gc)
        throw StatusError{HD_ERR_STATE, "the table was loaded without bucket sizes; run hd_gc before editing"};
    const auto t0 = std::chrono::steady_clock::now();
    cudaStream_t st = c->stream;
    hd_edit_stats sum{};
    bool plain = c->colors;
    for (uint32_t i = 0; i < n && !plain; i++)
        plain = edits[i].tool > HD_TOOL_BOX_ADD;
    if (plain) {
        // colours, paint and copy take the one-edit path, edit by edit
        float at = 0;
        for (uint32_t i = 0; i < n; i++) {
            hd_edit_stats s{};
            edit_one(c, edits[i], &s);
            at += s.device_ms;
            s.host_ms = at;
            if (per_edit)
                per_edit[i] = s;
            sum.num_voxels += s.num_voxels;
            sum.num_nodes += s.num_nodes;
            sum.find_or_add_calls += s.find_or_add_calls;
            sum.nodes_added += s.nodes_added;
            sum.words_scanned += s.words_scanned;
        }
        sum.device_ms = at;
        sum.host_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (total)
            *total = sum;
        return;
    }
    if (!c->batch)
        c->batch = new BatchGraph();
    BatchGraph& bg = *c->batch;
    std::vector<uint64_t> cap(c->g.leaf_level + 1, 0);
    for (uint32_t i = 0; i < n; i++)
        edit_caps(c->g, edits[i], cap);
    // capacities only grow (powers of two), so that one graph serves many
    // batches; the graph's edit count is the edits buffer's capacity
    for (size_t L = 0; L < cap.size(); L++) {
        uint64_t v = 256;
        while (v < cap[L])
            v <<= 1;
        cap[L] = std::max<uint64_t>(v, L < bg.caps.size() ? bg.caps[L] : 0);
    }
    const BatchBuffers b = batch_buffers(c, cap, std::max<uint32_t>(n, bg.edit_cap));
    if (c->tuning.mode == HD_BATCH_PERSISTENT) {
        std::vector<EditCounters> ctr(n);
        std::vector<float> end_ms(n, 0.0f), dur_ms(n, 0.0f);
        float device_ms = 0.0f;
        bool failed = false;
        StatusError failure{HD_OK, ""};
        try {
            edit_batch_persistent(c, edits, n, b.lv, b.caps, b.keys, b.vals, b.keys2, b.vals2, b.edits, b.ctr,
                                  b.roots, ctr, dur_ms, end_ms, device_ms, c->batch_fallbacks);
        } catch (const StatusError& e) {
            failed = true;
            failure = e;
        }
        c->root = read_scalar(c->d_root, st);
        // the applied edits' counters and times, also when a later one failed
        const uint32_t applied = failed ? c->batch_applied : n;
        for (uint32_t i = 0; i < applied; i++) {
            hd_edit_stats s{};
            s.num_voxels = ctr[i].num_voxels;
            s.num_nodes = ctr[i].num_nodes;
            s.find_or_add_calls = ctr[i].foa;
            s.nodes_added = ctr[i].added;
            s.words_scanned = ctr[i].scanned;
            s.device_ms = dur_ms[i];
            s.host_ms = end_ms[i];
            if (per_edit)
                per_edit[i] = s;
            sum.num_voxels += s.num_voxels;
            sum.num_nodes += s.num_nodes;
            sum.find_or_add_calls += s.find_or_add_calls;
            sum.nodes_added += s.nodes_added;
            sum.words_scanned += s.words_scanned;
        }
        if (failed)
            throw failure;
        sum.device_ms = device_ms;
        sum.host_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (total)
            *total = sum;
        return;
    }
    if (!bg.exec || bg.ptrs != b.ptrs() || bg.caps != b.caps || bg.tuning.foa_warps != c->tuning.foa_warps ||
        bg.tuning.probe_words != c->tuning.probe_words || bg.tuning.grid_blocks != c->tuning.grid_blocks)
        capture(c, bg, b, b.edit_cap);
    while (bg.events.size() < size_t(n) + 1) {
        cudaEvent_t e;
        HD_CUDA(cudaEventCreate(&e));
        bg.events.push_back(e);
    }
    std::vector<EditCounters> ctr(n);
    uint32_t done = 0;
    float elapsed_before = 0.0f; // device ms of earlier rounds (after a fallback edit)
    std::vector<float> end_ms(n, 0.0f), dur_ms(n, 0.0f);
    while (done < n) {
        const uint32_t m = n - done;
        HD_CUDA(cudaMemcpyAsync(b.edits, edits + done, sizeof(hd_edit) * m, cudaMemcpyHostToDevice, st));
        BatchState init{};
        HD_CUDA(cudaMemcpyAsync(b.bs, &init, sizeof(BatchState), cudaMemcpyHostToDevice, st));
        // one launch per edit: the graph reads edits[idx] and advances idx
        HD_CUDA(cudaEventRecord(bg.events[0], st));
        for (uint32_t k = 0; k < m; k++) {
            HD_CUDA(cudaGraphLaunch(bg.exec, st));
            HD_CUDA(cudaEventRecord(bg.events[k + 1], st));
        }
        BatchState fin{};
        HD_CUDA(cudaMemcpyAsync(&fin, b.bs, sizeof(BatchState), cudaMemcpyDeviceToHost, st));
        HD_CUDA(cudaStreamSynchronize(st));
        const uint32_t ok = fin.idx; // edits applied in this round
        if (ok) {
            HD_CUDA(cudaMemcpy(ctr.data() + done, b.ctr, sizeof(EditCounters) * ok, cudaMemcpyDeviceToHost));
            std::vector<uint32_t> roots(ok);
            HD_CUDA(cudaMemcpy(roots.data(), b.roots, 4ull * ok, cudaMemcpyDeviceToHost));
            for (uint32_t k = 0; k < ok; k++) {
                UndoFrame f;
                f.root = c->root;
                push_undo(c, std::move(f));
                c->root = roots[k];
            }
            for (uint32_t k = 0; k < ok; k++) {
                float a = 0, d = 0;
                HD_CUDA(cudaEventElapsedTime(&a, bg.events[0], bg.events[k + 1]));
                HD_CUDA(cudaEventElapsedTime(&d, bg.events[k], bg.events[k + 1]));
                end_ms[done + k] = elapsed_before + a;
                dur_ms[done + k] = d;
            }
            float all = 0;
            HD_CUDA(cudaEventElapsedTime(&all, bg.events[0], bg.events[ok]));
            elapsed_before += all;
        }
        done += ok;
        if (fin.stop == kStopNone)
            break;
        if (fin.stop == kStopTableError || fin.stop == kStopEmptyScene) {
            const uint32_t err = check_error(c);
            c->root = read_scalar(c->d_root, st);
            if (fin.stop == kStopEmptyScene)
                throw StatusError{HD_ERR_STATE, "edit " + std::to_string(done) + " would empty the whole scene"};
            throw StatusError{hd_status(err ? err : HD_ERR_CUDA),
                              "edit " + std::to_string(done) + " failed on the device (" + c->err_detail + ")"};
        }
        // capacity: this edit with the one-edit path, then resume
        c->root = read_scalar(c->d_root, st);
        hd_edit_stats s{};
        edit_one(c, edits[done], &s);
        ctr[done].num_voxels = s.num_voxels;
        ctr[done].num_nodes = s.num_nodes;
        ctr[done].foa = s.find_or_add_calls;
        ctr[done].added = s.nodes_added;
        ctr[done].scanned = s.words_scanned;
        dur_ms[done] = s.device_ms;
        elapsed_before += s.device_ms;
        end_ms[done] = elapsed_before;
        done++;
        c->batch_fallbacks++;
    }
    c->root = read_scalar(c->d_root, st);
    for (uint32_t i = 0; i < n; i++) {
        hd_edit_stats s{};
        s.num_voxels = ctr[i].num_voxels;
        s.num_nodes = ctr[i].num_nodes;
        s.find_or_add_calls = ctr[i].foa;
        s.nodes_added = ctr[i].added;
        s.words_scanned = ctr[i].scanned;
        s.device_ms = dur_ms[i];
        s.host_ms = end_ms[i];
        if (per_edit)
            per_edit[i] = s;
        sum.num_voxels += s.num_voxels;
        sum.num_nodes += s.num_nodes;
        sum.find_or_add_calls += s.find_or_add_calls;
        sum.nodes_added += s.nodes_added;
        sum.words_scanned += s.words_scanned;
    }
    sum.device_ms = elapsed_before;
    sum.host_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (total)
        *total = sum;
}

void batch_release(hd_ctx* c)
{
    delete c->batch;
    c->batch = nullptr;
}

} // namespace hd

namespace {

using namespace hd;

template <typename F>
hd_status guarded_call(hd_ctx* c, F&& f)
{
    try {
        f();
        return HD_OK;
    } catch (const StatusError& e) {
        c->err = e.msg;
        return e.status;
    } catch (const CudaError& e) {
        c->err = std::string("CUDA error ") + cudaGetErrorString(e.code) + " in " + e.where;
        return HD_ERR_CUDA;
    }
}

bool valid_edits(const hd_edit* edits, uint32_t n)
{
    for (uint32_t i = 0; i < n; i++)
        if (edits[i].tool > HD_TOOL_FILL || !(edits[i].radius >= 0.0f))
            return false;
    return true;
}

bool valid_tuning(const hd_batch_tuning& t)
{
    return (t.foa_warps == 2 || t.foa_warps == 4 || t.foa_warps == 8) &&
           (t.probe_words == 1 || t.probe_words == 2 || t.probe_words == 4) && t.grid_blocks >= 64 &&
           t.grid_blocks <= 2048 && t.grid_blocks % 8 == 0 && (t.mode == HD_BATCH_GRAPH || t.mode == HD_BATCH_PERSISTENT);
}

// Copies the table of `from` into `to` (same configuration); pages that `to`
// mapped past the copied pool are zeroed first, as fresh pages are.
void copy_table(hd_ctx* to, hd_ctx* from)
{
    cudaStream_t st = from->stream;
    HD_CUDA(cudaStreamSynchronize(to->stream));
    const uint32_t top_from = read_scalar(from->t.pool_top, st);
    const uint32_t top_to = read_scalar(to->t.pool_top, to->stream);
    if (top_to > top_from)
        HD_CUDA(cudaMemsetAsync(to->t.pool + uint64_t(top_from) * kPage, 0, uint64_t(top_to - top_from) * kPage * 4,
                                st));
    HD_CUDA(cudaMemcpyAsync(to->t.pool, from->t.pool, uint64_t(top_from) * kPage * 4, cudaMemcpyDeviceToDevice, st));
    if (top_to > top_from)
        HD_CUDA(cudaMemsetAsync(to->t.bloom + uint64_t(top_from) * kBloomWords, 0,
                                uint64_t(top_to - top_from) * kBloomWords * 4, st));
    HD_CUDA(cudaMemcpyAsync(to->t.bloom, from->t.bloom, uint64_t(top_from) * kBloomWords * 4, cudaMemcpyDeviceToDevice,
                            st));
    HD_CUDA(cudaMemcpyAsync(to->t.page_table, from->t.page_table, from->g.total_vpages * 4, cudaMemcpyDeviceToDevice,
                            st));
    HD_CUDA(cudaMemcpyAsync(to->t.bucket_sizes, from->t.bucket_sizes, from->g.total_buckets * 4,
                            cudaMemcpyDeviceToDevice, st));
    HD_CUDA(cudaMemcpyAsync(to->t.full_nodes, from->t.full_nodes, HD_MAX_DEPTH * 4, cudaMemcpyDeviceToDevice, st));
    HD_CUDA(cudaMemcpyAsync(to->t.level_nodes, from->t.level_nodes, HD_MAX_DEPTH * 8, cudaMemcpyDeviceToDevice, st));
    HD_CUDA(cudaMemcpyAsync(to->t.pool_top, from->t.pool_top, 8, cudaMemcpyDeviceToDevice, st));
    uint32_t counters[2];
    HD_CUDA(cudaMemcpyAsync(counters, from->t.pool_top, 8, cudaMemcpyDeviceToHost, st));
    HD_CUDA(cudaStreamSynchronize(st));
    if (counters[1])
        HD_CUDA(cudaMemcpyAsync(to->t.free_pages, from->t.free_pages, uint64_t(counters[1]) * 4,
                                cudaMemcpyDeviceToDevice, st));
    HD_CUDA(cudaMemcpyAsync(to->d_root, from->d_root, 4, cudaMemcpyDeviceToDevice, st));
    HD_CUDA(cudaStreamSynchronize(st));
    to->root = from->root;
}

} // namespace

extern "C" {

hd_status hd_edit_batch_ex(hd_ctx* c, const hd_edit* edits, uint32_t n, hd_edit_stats* per_edit, hd_edit_stats* total)
{
    if (!c || (n && !edits) || !valid_edits(edits, n))
        return HD_ERR_INVALID;
    if (n == 0) {
        if (total)
            *total = hd_edit_stats{};
        return HD_OK;
    }
    return guarded_call(c, [&] { edit_batch(c, edits, n, per_edit, total); });
}

hd_status hd_edit_batch(hd_ctx* c, const hd_edit* edits, uint32_t n, hd_edit_stats* stats)
{
    return hd_edit_batch_ex(c, edits, n, nullptr, stats);
}

hd_status hd_set_batch_tuning(hd_ctx* c, const hd_batch_tuning* t)
{
    if (!c || !t || !valid_tuning(*t))
        return HD_ERR_INVALID;
    c->tuning = *t;
    return HD_OK;
}

hd_status hd_get_batch_tuning(hd_ctx* c, hd_batch_tuning* t)
{
    if (!c || !t)
        return HD_ERR_INVALID;
    *t = c->tuning;
    return HD_OK;
}

hd_status hd_batch_fallbacks(hd_ctx* c, uint64_t* count)
{
    if (!c || !count)
        return HD_ERR_INVALID;
    *count = c->batch_fallbacks;
    return HD_OK;
}

hd_status hd_autotune_batch(hd_ctx* c, const hd_edit* sample, uint32_t n, hd_batch_tuning* best, float* best_ms)
{
    if (!c || !sample || n == 0 || !valid_edits(sample, n))
        return HD_ERR_INVALID;
    hd_ctx* k = nullptr;
    hd_status st = hd_create(&c->cfg, &k);
    if (st != HD_OK)
        return st;
    hd_set_stream(k, c->stream);
    hd_batch_tuning chosen = c->tuning;
    float chosen_ms = -1.0f;
    st = guarded_call(c, [&] {
        const uint32_t sms = 152;
        const uint32_t grids[3] = {sms * 2, sms * 4, sms * 8};
        const uint32_t warps[3] = {2, 4, 8};
        const uint32_t probes[3] = {1, 2, 4};
        for (uint32_t P : probes) {
            // the persistent form (its launch shape is fixed: one CTA per SM)
            k->tuning = hd_batch_tuning{4, P, 304, HD_BATCH_PERSISTENT};
            hd_edit_stats tot{};
            copy_table(k, c);
            edit_batch(k, sample, n, nullptr, &tot);
            copy_table(k, c);
            edit_batch(k, sample, n, nullptr, &tot);
            if (chosen_ms < 0.0f || tot.device_ms < chosen_ms) {
                chosen_ms = tot.device_ms;
                chosen = k->tuning;
            }
        }
        for (uint32_t G : grids)
            for (uint32_t W : warps)
                for (uint32_t P : probes) {
                    k->tuning = hd_batch_tuning{W, P, G, HD_BATCH_GRAPH};
                    hd_edit_stats tot{};
                    // first run captures the graph; the second is timed
                    copy_table(k, c);
                    edit_batch(k, sample, n, nullptr, &tot);
                    copy_table(k, c);
                    edit_batch(k, sample, n, nullptr, &tot);
                    if (chosen_ms < 0.0f || tot.device_ms < chosen_ms) {
                        chosen_ms = tot.device_ms;
                        chosen = k->tuning;
                    }
                }
    });
    hd_destroy(k);
    if (st != HD_OK)
        return st;
    c->tuning = chosen;
    if (best)
        *best = chosen;
    if (best_ms)
        *best_ms = chosen_ms;
    return HD_OK;
}

} // extern "C"
