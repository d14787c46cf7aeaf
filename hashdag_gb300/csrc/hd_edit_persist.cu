// Batched edits in one persistent launch: every edit of a batch, level by
// level, in a single cooperative kernel whose CTAs (one per SM) move through
// the levels together, with no host round trip and no kernel boundary.
//
// Same per-entry logic, same order of bucket scans and appends, hence the
// same table, as applying the edits one by one (hd_edit.cu): the edit of
// HashDAG::edit_threads (hash_dag.h:255-405) applied in sequence.  The work
// queue is ordered by level: for each edit, top-down levels (classify,
// spawn), then bottom-up levels (candidates, grouping by bucket,
// find-or-add).
//
//  * Levels are small near the root.  A level of at most kSmall entries is
//    processed by CTA 0 alone while the other CTAs wait at the next grid
//    barrier: consecutive small levels, the end of one edit and the start of
//    the next cost one barrier in all.  A bottom-up small level whose
//    candidates fall in more buckets than CTA 0 has warps hands its
//    find-or-add to the whole grid.
//  * A big level top-down is one grid phase: each CTA scans the descend
//    flags of its chunk (offsets of the chunks before it: sums of per-chunk
//    flag counts gathered while the level was classified), spawns the
//    children of its descended entries and classifies them.
//  * A big level bottom-up is six phases: candidates with their pass-1 digit
//    counts, two stable radix passes on the level-local bucket (digit rows
//    scanned across the grid between them; pass-2 counts gathered while
//    pass 1 scatters), then find-or-add, one warp per bucket run.
//  * Grid barriers are bounded waits: a wait longer than kWaitNs sets
//    HD_ERR_TIMEOUT and every CTA returns; the host reports the error.
//  * Nodes and pages that an edit appends are read by the following edits in
//    the same launch: every table read uses L2-coherent loads.
// The graph-per-edit form (hd_edit_batch.cu) stays as the other batch mode.
#include <vector>

#include "hd_edit.cuh"

namespace hd {

namespace {

constexpr uint32_t kPT = 1024;             // threads per CTA (one CTA per SM)
constexpr uint32_t kPWarps = kPT / 32;
constexpr uint32_t kSmall = kPT;           // entries of a level CTA 0 handles alone
constexpr uint32_t kDigits = 512;          // radix digits per pass at most (9 bits)
constexpr unsigned long long kWaitNs = 2000000000ull;

enum : uint32_t { kRun = 0, kDone = 1, kCapacity = 2, kTableError = 3, kEmptyScene = 4, kAborted = 5 };

// What CTA 0 asks of the grid at a barrier.
struct Cmd {
    uint32_t stop, phase, level, deepest, idx, pad[3];
};

// Control block in global memory, reset by the host before a launch.
// stop / idx / phase / level / deepest are CTA 0's own state (stop and idx
// also read by the host after the launch); the other CTAs read the copy CTA 0
// publishes in cmd[k & 1] before barrier k.  CTA 0 runs ahead as soon as it
// leaves a barrier, so it must not change what the others are still about to
// read: it writes the slot of the next barrier, which no CTA reads until
// every CTA has left this one.
struct Ctl {
    uint32_t arrived, abort, stop; // arrived: grid barrier arrivals of the launch
    uint32_t idx;       // edit being applied
    uint32_t phase;     // the grid step CTA 0 asks for (kPh*)
    uint32_t level;     // its level
    uint32_t deepest;   // deepest level of the current edit
    Cmd cmd[2];
    uint32_t count[HD_MAX_DEPTH];
    // where a wait ran out: the CTA, its barrier count, the arrivals then and
    // the count it waited for, CTA 0's barrier count, phase, level and edit
    uint32_t diag[8];
    uint32_t bars0; // barriers CTA 0 has passed
    // tests of the timeout path (hd_set_test_barrier_skip): CTA skip_cta - 1
    // returns at once, never arriving (0: none); wait_ns bounds every
    // barrier wait (0: kWaitNs)
    uint32_t skip_cta;
    unsigned long long wait_ns;
    Editor ed;
};

struct PArgs {
    Ctl* ctl;
    const hd_edit* edits;
    uint32_t n_edits;
    const Level* lv;     // device array: one Level per depth
    uint32_t cap[HD_MAX_DEPTH];
    uint32_t *keys, *vals, *keys2, *vals2;
    uint32_t* bsum;      // 3 x G: per-chunk descend-flag counts, by level parity
    uint32_t *hist, *hist2, *rows, *rows2; // kDigits x G, kDigits
    EditCounters* ctr;
    uint32_t* roots;
    unsigned long long* t_begin;
    unsigned long long* t_end;
    uint32_t* d_root;
};

HD_D unsigned long long now_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
HD_D uint32_t ld_acquire(const uint32_t* p)
{
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid barrier of the cooperative launch with a bounded wait; false when a
// wait ran out or another CTA gave up (the caller returns).  The arrival
// count only grows (the control block starts at zero every launch), so the
// k-th barrier is passed once k x CTAs have arrived: no reset, and no
// generation word for the last CTA to publish after its arrival.
HD_D bool grid_sync(Ctl* ctl, uint32_t* err, uint32_t& nbar)
{
    __shared__ uint32_t ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        nbar++;
        if (blockIdx.x == 0)
            __stcg(&ctl->bars0, nbar);
        const uint32_t target = nbar * gridDim.x;
        __threadfence();
        if (atomicAdd(&ctl->arrived, 1u) + 1u != target) {
            const unsigned long long t0 = now_ns();
            const unsigned long long set_ns = __ldcg(&ctl->wait_ns);
            const unsigned long long limit = set_ns ? set_ns : kWaitNs;
            uint32_t spins = 0;
            while (int32_t(ld_acquire(&ctl->arrived) - target) < 0) {
                if (ld_acquire(&ctl->abort)) {
                    ok = 0;
                    break;
                }
                if ((++spins & 255u) == 0 && now_ns() - t0 > limit) {
                    if (atomicExch(&ctl->abort, 1u) == 0) {
                        ctl->diag[0] = blockIdx.x;
                        ctl->diag[1] = nbar;
                        ctl->diag[2] = ld_acquire(&ctl->arrived);
                        ctl->diag[3] = target;
                        ctl->diag[4] = ld_acquire(&ctl->bars0);
                        ctl->diag[5] = ld_acquire(&ctl->phase);
                        ctl->diag[6] = ld_acquire(&ctl->level);
                        ctl->diag[7] = ld_acquire(&ctl->idx);
                    }
                    set_error(err, kErrTimeout, 0xFFFFFFFEu, blockIdx.x, 0);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

HD_D uint32_t chunk_len(uint32_t n, uint32_t parts, uint32_t align)
{
    const uint32_t per = (n + parts - 1) / parts;
    return (per + align - 1) / align * align;
}

// Grid phases split a level into one chunk per CTA, a multiple of the warp
// width long (so that a warp's 32 consecutive slots fall in at most two
// chunks): every CTA gets work once a level holds 32 entries per CTA.
constexpr uint32_t kChunkAlign = 32;

// Chunk of level entries a descend flag is counted in (the grid's top-down
// chunking of that level).
HD_D uint32_t td_chunk(uint32_t i, uint32_t n, uint32_t G) { return i / chunk_len(n, G, kChunkAlign); }

// Block-wide exclusive scan (kPT threads) of v; *total = the block's sum.
HD_D uint32_t cta_scan(uint32_t v, uint32_t* total, uint32_t* sm32)
{
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t inc = warp_incl_scan(v);
    if (lane == 31)
        sm32[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const uint32_t s = warp_incl_scan(sm32[lane]);
        sm32[lane] = s;
    }
    __syncthreads();
    const uint32_t base = warp ? sm32[warp - 1] : 0u;
    *total = sm32[kPWarps - 1];
    __syncthreads();
    return base + inc - v;
}

// Top-down: entries [i0, i1) of level L (classified, their descend flags
// set): exclusive positions from `prefix` (descended entries before i0),
// then every child of every descended entry spawned at 8 * exp + c and
// classified; children's descend flags are counted per top-down chunk of
// level L + 1 into cnt_next.  CTA-wide.
HD_D void td_range(const Table& t, const Editor& ed, const Level* lvs, uint32_t L, uint32_t i0, uint32_t i1,
                   uint32_t prefix, uint32_t n_next, uint32_t G, uint32_t* cnt_next, EditCounters* ctr,
                   uint32_t* sm32, uint32_t* list)
{
    const Level lv = lvs[L], nx = lvs[L + 1];
    const uint32_t lane = threadIdx.x & 31;
    uint32_t run = prefix;
    unsigned long long nodes = 0, voxels = 0;
    for (uint32_t base = i0; base < i1; base += kPT) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t f = i < i1 ? lv.flag[i] : 0u;
        uint32_t total;
        const uint32_t off = cta_scan(f, &total, sm32);
        if (f) {
            lv.exp[i] = run + off;
            list[off] = i;
        }
        __syncthreads();
        // the tile's children, spread over the CTA, warps in lockstep
        const uint32_t nchild = 8 * total;
        for (uint32_t k0 = threadIdx.x & ~31u; k0 < nchild; k0 += kPT) {
            const uint32_t k = k0 + lane;
            const bool act = k < nchild;
            uint32_t fl = 0, ch = 0xFFFFFFFFu;
            if (act) {
                const uint32_t parent = list[k >> 3], c = k & 7;
                const uint32_t at = 8 * (run + (k >> 3)) + c;
                uint32_t x, y, z, old;
                spawn_child(t, lv, nx, parent, c, at, x, y, z, old);
                unsigned long long nn, vv;
                classify_values<true>(t, ed, L + 1, nx, at, x, y, z, old, nn, vv);
                nodes += nn;
                voxels += vv;
                fl = nx.flag[at];
                ch = td_chunk(at, n_next, G);
            }
            // the warp's children are 32 consecutive slots (at = 8 run + k),
            // so they fall in at most two chunks (chunks hold >= 32 slots):
            // one atomic per chunk; flags are 0 or 1
            const uint32_t ch0 = __shfl_sync(0xffffffffu, ch, 0);
            const uint32_t b0 = __ballot_sync(0xffffffffu, act && fl && ch == ch0);
            const uint32_t b1 = __ballot_sync(0xffffffffu, act && fl && ch != ch0);
            if (lane == 0 && b0)
                atomicAdd(cnt_next + ch0, uint32_t(__popc(b0)));
            if (b1 && lane == uint32_t(__ffs(b1) - 1))
                atomicAdd(cnt_next + ch, uint32_t(__popc(b1)));
        }
        run += total;
        __syncthreads();
    }
    warp_add(&ctr->num_nodes, nodes);
    warp_add(&ctr->num_voxels, voxels);
}

// The grid's top-down step of a big level, in two phases so that the
// children (8 per descended entry, and the work of classifying them) spread
// evenly over the CTAs whatever chunks the descended entries fall in.
// Phase 1: entries [i0, i1) get their positions (prefix: the descended
// entries before i0) and are listed by position in dlist.
HD_D void td_positions(const Level& lv, uint32_t i0, uint32_t i1, uint32_t prefix, uint32_t* dlist, uint32_t* sm32)
{
    uint32_t run = prefix;
    for (uint32_t base = i0; base < i1; base += kPT) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t f = i < i1 ? lv.flag[i] : 0u;
        uint32_t total;
        const uint32_t off = cta_scan(f, &total, sm32);
        if (f) {
            lv.exp[i] = run + off;
            dlist[run + off] = i;
        }
        run += total;
    }
}

// Phase 2: children [k0, k1) of the level (child k of descended entry
// dlist[k / 8], slot k % 8) spawned and classified; their descend flags
// counted per top-down chunk of the next level into cnt_next.  k0 is a
// multiple of 32, so each warp's 32 consecutive children fall in at most two
// chunks.
HD_D void td_children(const Table& t, const Editor& ed, const Level* lvs, uint32_t L, uint32_t k0, uint32_t k1,
                      uint32_t n_next, uint32_t G, const uint32_t* dlist, uint32_t* cnt_next, EditCounters* ctr)
{
    const Level lv = lvs[L], nx = lvs[L + 1];
    const uint32_t lane = threadIdx.x & 31;
    unsigned long long nodes = 0, voxels = 0;
    for (uint32_t kb = k0 + (threadIdx.x & ~31u); kb < k1; kb += kPT) {
        const uint32_t k = kb + lane;
        const bool act = k < k1;
        uint32_t fl = 0, ch = 0xFFFFFFFFu;
        if (act) {
            uint32_t x, y, z, old;
            spawn_child(t, lv, nx, __ldcg(dlist + (k >> 3)), k & 7, k, x, y, z, old);
            unsigned long long nn, vv;
            classify_values<true>(t, ed, L + 1, nx, k, x, y, z, old, nn, vv);
            nodes += nn;
            voxels += vv;
            fl = nx.flag[k];
            ch = td_chunk(k, n_next, G);
        }
        const uint32_t ch0 = __shfl_sync(0xffffffffu, ch, 0);
        const uint32_t b0 = __ballot_sync(0xffffffffu, act && fl && ch == ch0);
        const uint32_t b1 = __ballot_sync(0xffffffffu, act && fl && ch != ch0);
        if (lane == 0 && b0)
            atomicAdd(cnt_next + ch0, uint32_t(__popc(b0)));
        if (b1 && lane == uint32_t(__ffs(b1) - 1))
            atomicAdd(cnt_next + ch, uint32_t(__popc(b1)));
    }
    warp_add(&ctr->num_nodes, nodes);
    warp_add(&ctr->num_voxels, voxels);
}

// Top-down, one warp of CTA 0 alone: consecutive levels of at most 32
// entries (the levels near the root), as td_range does them for a whole
// level (positions, children spawned and classified, the next level's
// per-chunk descend counts) but with warp votes in place of CTA scans and
// barriers.  Returns the first level it did not descend from; status 0: that
// level holds more than 32 entries (or is the leaf level), 1: it had no
// descended entry (it is the deepest), 2: its children would exceed their
// level's capacity.
HD_D uint32_t td_tiny(const Table& t, const Editor& ed, const PArgs& a, uint32_t L, uint32_t n, EditCounters* ctr,
                      uint32_t* list, uint32_t& status)
{
    const uint32_t lane = threadIdx.x & 31, G = gridDim.x, leafl = t.g.leaf_level;
    unsigned long long nodes = 0, voxels = 0;
    status = 0;
    while (L < leafl && n <= 32) {
        const Level lv = a.lv[L], nx = a.lv[L + 1];
        const uint32_t f = lane < n ? lv.flag[lane] : 0u;
        const uint32_t fb = __ballot_sync(0xffffffffu, f != 0);
        const uint32_t total = __popc(fb);
        if (total == 0) {
            status = 1;
            break;
        }
        const uint32_t n_next = 8 * total;
        if (n_next > a.cap[L + 1]) {
            status = 2;
            break;
        }
        uint32_t* zero = a.bsum + ((L + 2) % 3) * G;
        for (uint32_t k = lane; k < G; k += 32)
            zero[k] = 0;
        uint32_t* cnt_next = a.bsum + ((L + 1) % 3) * G;
        if (f) {
            const uint32_t off = __popc(fb & ((1u << lane) - 1u));
            lv.exp[lane] = off;
            list[off] = lane;
        }
        __syncwarp();
        for (uint32_t k0 = 0; k0 < n_next; k0 += 32) {
            const uint32_t k = k0 + lane;
            const bool act = k < n_next;
            uint32_t fl = 0, ch = 0xFFFFFFFFu;
            if (act) {
                uint32_t x, y, z, old;
                spawn_child(t, lv, nx, list[k >> 3], k & 7, k, x, y, z, old);
                unsigned long long nn, vv;
                classify_values<true>(t, ed, L + 1, nx, k, x, y, z, old, nn, vv);
                nodes += nn;
                voxels += vv;
                fl = nx.flag[k];
                ch = td_chunk(k, n_next, G);
            }
            const uint32_t ch0 = __shfl_sync(0xffffffffu, ch, 0);
            const uint32_t b0 = __ballot_sync(0xffffffffu, act && fl && ch == ch0);
            const uint32_t b1 = __ballot_sync(0xffffffffu, act && fl && ch != ch0);
            if (lane == 0 && b0)
                atomicAdd(cnt_next + ch0, uint32_t(__popc(b0)));
            if (b1 && lane == uint32_t(__ffs(b1) - 1))
                atomicAdd(cnt_next + ch, uint32_t(__popc(b1)));
        }
        if (lane == 0)
            a.ctl->count[L + 1] = n_next;
        __syncwarp(); // the next level reads the flags other lanes wrote
        n = n_next;
        L++;
    }
    warp_add(&ctr->num_nodes, nodes);
    warp_add(&ctr->num_voxels, voxels);
    return L;
}

// Bottom-up candidates of entries [i0, i1) of level L: key = level-local
// bucket, or buckets(L) (sorts last) for entries resolved at once.
HD_D void candidates_range(const Table& t, const Level* lvs, uint32_t L, uint32_t deepest, uint32_t i0, uint32_t i1,
                           uint32_t* keys, uint32_t* vals)
{
    const Level lv = lvs[L];
    const Level child = L < deepest ? lvs[L + 1] : Level{};
    const uint32_t empty = t.g.buckets(L);
    for (uint32_t i = i0 + threadIdx.x; i < i1; i += kPT) {
        const uint32_t b = candidate_entry<true>(t, L, lv, child, i);
        keys[i] = b == kNoBucket ? empty : b;
        vals[i] = i;
    }
}

// Find-or-add over sorted keys [0, n) (runs of one bucket in entry order):
// the positions are split into one chunk per warp (ceil(n / nw), at least
// one) and warp w of nw resolves every run that starts in its chunk, so that
// short runs spread over all the warps.
// SH: keys / vals in the CTA's shared memory (CTA 0's small levels), read
// with plain loads; else global arrays another phase wrote, read from L2.
template <int PW, bool SH = false>
HD_D void foa_sorted(const Table& t, uint32_t L, const Level& lv, const uint32_t* keys, const uint32_t* vals,
                     uint32_t n, uint32_t w, uint32_t nw, uint32_t* page, uint32_t* q, FoaCache& cache,
                     EditCounters* ctr)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t empty = t.g.buckets(L);
    unsigned long long foa = 0, added = 0, scanned = 0;
    const uint32_t chunk = n > nw ? (n + nw - 1) / nw : 1u;
    const uint64_t cbeg64 = uint64_t(w) * chunk;
    const uint32_t cbeg = cbeg64 < n ? uint32_t(cbeg64) : n, cend = n - cbeg < chunk ? n : cbeg + chunk;
    for (uint32_t c0 = cbeg; c0 < cend; c0 += 32) {
        const uint32_t j = c0 + lane;
        const bool in = j < cend;
        const uint32_t key = in ? (SH ? keys[j] : __ldcg(keys + j)) : empty;
        const uint32_t prev = (in && j > 0) ? (SH ? keys[j - 1] : __ldcg(keys + j - 1)) : kNoBucket;
        uint32_t starts = __ballot_sync(0xffffffffu, in && key < empty && key != prev);
        while (starts) {
            const uint32_t s = __ffs(starts) - 1;
            starts &= starts - 1;
            const uint32_t j0 = c0 + s;
            const uint32_t bucket = __shfl_sync(0xffffffffu, key, s);
            uint32_t j1 = j0 + 1;
            for (;;) {
                const uint32_t jj = j1 + lane;
                const uint32_t k = jj < n ? (SH ? keys[jj] : __ldcg(keys + jj)) : kNoBucket;
                const uint32_t diff = __ballot_sync(0xffffffffu, k != bucket);
                if (diff) {
                    j1 += __ffs(diff) - 1;
                    break;
                }
                j1 += 32;
            }
            foa_segment<PW>(t, L, lv, vals, j0, j1, bucket, page, q, cache, foa, added, scanned);
        }
    }
    if (lane == 0 && (foa | added | scanned)) {
        atomicAdd(&ctr->foa, foa);
        atomicAdd(&ctr->added, added);
        atomicAdd(&ctr->scanned, scanned);
        atomicAdd(reinterpret_cast<unsigned long long*>(t.level_nodes + L), added);
    }
}

// CTA 0 alone: stable sort of the n (<= kPT) candidates of a small level by
// (bucket, entry) in shared memory, written back to keys / vals (visible to
// the CTA after its barriers, to the grid after the next grid barrier);
// returns the number of bucket runs.
HD_D uint32_t small_sort(const Table& t, uint32_t L, uint32_t n, uint32_t* keys, uint32_t* vals,
                         unsigned long long* s64, uint32_t* sm32, uint32_t* sk, uint32_t* sv)
{
    const uint32_t empty = t.g.buckets(L);
    if (n <= 32) {
        // one warp, in registers: a bitonic network over the lanes on the
        // (bucket, entry) pairs (entries are distinct: the order is total)
        if (threadIdx.x < 32) {
            const uint32_t lane = threadIdx.x;
            unsigned long long x = lane < n ? (uint64_t(keys[lane]) << 32) | vals[lane] : ~0ull;
            for (uint32_t k = 2; k <= 32; k <<= 1)
                for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                    const unsigned long long y = __shfl_xor_sync(0xffffffffu, x, j);
                    const bool up = (lane & k) == 0, low = (lane & j) == 0;
                    x = (low == up) ? (x < y ? x : y) : (x < y ? y : x);
                }
            const uint32_t key = uint32_t(x >> 32);
            const uint32_t prev = __shfl_up_sync(0xffffffffu, key, 1);
            if (lane < n) {
                keys[lane] = key;
                vals[lane] = uint32_t(x);
                sk[lane] = key;
                sv[lane] = uint32_t(x);
            }
            const uint32_t runs = __popc(__ballot_sync(0xffffffffu, lane < n && key < empty && (lane == 0 || prev != key)));
            if (lane == 0)
                sm32[0] = runs;
        }
        __syncthreads();
        const uint32_t runs = sm32[0];
        __syncthreads();
        return runs;
    }
    // n <= kPT: a rank sort, one element per thread: the (bucket, entry)
    // pairs are distinct, so an element's rank is the count of smaller ones
    // (every thread reads the same shared word at a time: a broadcast)
    unsigned long long* in = s64;
    unsigned long long* out = s64 + kPT;
    const uint32_t i = threadIdx.x;
    const unsigned long long x = i < n ? (uint64_t(keys[i]) << 32) | vals[i] : ~0ull;
    in[i] = x;
    __syncthreads();
    if (i < n) {
        uint32_t rank = 0;
        for (uint32_t k = 0; k < n; k++)
            rank += in[k] < x;
        out[rank] = x;
    }
    __syncthreads();
    uint32_t runs = 0;
    if (i < n) {
        const uint32_t key = uint32_t(out[i] >> 32);
        keys[i] = key;
        vals[i] = uint32_t(out[i]);
        sk[i] = key;
        sv[i] = uint32_t(out[i]);
        runs = key < empty && (i == 0 || uint32_t(out[i - 1] >> 32) != key);
    }
    uint32_t total;
    cta_scan(runs, &total, sm32);
    return total;
}

// Per digit row of a [kDigits][nb] count table: exclusive scan over the
// chunks in place, the row total into rows.  Warps of the whole grid.
HD_D void scan_rows(uint32_t* hist, uint32_t nb, uint32_t nd, uint32_t* rows)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gw = blockIdx.x * kPWarps + (threadIdx.x >> 5), nw = gridDim.x * kPWarps;
    for (uint32_t d = gw; d < nd; d += nw) {
        uint32_t run = 0;
        for (uint32_t b0 = 0; b0 < nb; b0 += 32) {
            const uint32_t b = b0 + lane;
            const uint32_t x = b < nb ? __ldcg(hist + d * nb + b) : 0u;
            const uint32_t inc = warp_incl_scan(x);
            if (b < nb)
                hist[d * nb + b] = run + inc - x;
            run += __shfl_sync(0xffffffffu, inc, 31);
        }
        if (lane == 0)
            rows[d] = run;
    }
}

// Stable scatter of chunk `cb` of (keys, vals) by digit (key >> shift) & (nd
// - 1): bases from the row totals and this chunk's row offsets; warps of a
// tile take their turn in order.  With hist_next, counts each element's next
// digit in the chunk its output position falls in.
HD_D void scatter_chunk(const uint32_t* keys, const uint32_t* vals, uint32_t n, uint32_t nb, uint32_t cb,
                        uint32_t shift, uint32_t nd, const uint32_t* hist, const uint32_t* rows,
                        uint32_t* keys_out, uint32_t* vals_out, uint32_t* hist_next, uint32_t next_shift,
                        uint32_t* run, uint32_t* sm32)
{
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t chunk = chunk_len(n, nb, kChunkAlign);
    // digit bases: exclusive scan of the row totals (nd <= kPT)
    {
        const uint32_t d = threadIdx.x;
        const uint32_t r = d < nd ? __ldcg(rows + d) : 0u;
        uint32_t total;
        const uint32_t ex = cta_scan(r, &total, sm32);
        if (d < nd)
            run[d] = ex + __ldcg(hist + d * nb + cb);
        __syncthreads();
    }
    const uint32_t i0 = cb * chunk, i1 = min(n, i0 + chunk);
    for (uint32_t base = i0; base < i1; base += kPT) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < i1;
        const uint32_t key = valid ? __ldcg(keys + i) : 0u;
        const uint32_t val = valid ? __ldcg(vals + i) : 0u;
        const uint32_t digit = valid ? (key >> shift) & (nd - 1) : kDigits + lane;
        const uint32_t peers = __match_any_sync(0xffffffffu, digit);
        const uint32_t leader = __ffs(peers) - 1;
        for (uint32_t w = 0; w < kPWarps; w++) {
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
                    if (hist_next)
                        atomicAdd(hist_next + ((key >> next_shift) & (nd - 1)) * nb + pos / chunk, 1u);
                }
            }
            __syncthreads();
        }
    }
}

// CTA 0's state between grid steps
enum : uint32_t { kLsBegin = 0, kLsTopDown = 1, kLsBottomUp = 2, kLsFinish = 3 };
// the grid step CTA 0 asks for
enum : uint32_t { kPhNone = 0, kPhTopDown = 1, kPhBottomUp = 2, kPhGridFoa = 3 };

// Bytes of the dynamic shared memory the find-or-add buffers and the small
// sort share (a multiple of 16); the small level's sorted keys and entries
// follow.
HD_HD constexpr size_t persist_smem_core()
{
    return (size_t(kPWarps) * kPage * 4 + size_t(kPWarps) * 12 * 4 + size_t(kPWarps) * sizeof(FoaCache) >
                    size_t(kPT) * 8 * 2
                ? size_t(kPWarps) * kPage * 4 + size_t(kPWarps) * 12 * 4 + size_t(kPWarps) * sizeof(FoaCache)
                : size_t(kPT) * 8 * 2) +
           15 & ~size_t(15);
}

struct Smem {
    uint32_t* sk; // a small level's sorted keys and entries (kPT each), past
    uint32_t* sv; // the buffers below (which the find-or-add overwrites)
    uint32_t* page;
    uint32_t* q;
    FoaCache* cache;
    unsigned long long* s64;
    uint32_t* list;
    uint32_t* sm32;
    Editor* ed;
};

// CTA 0: the next edit of the batch (or the stop); level 0 classified.
// False when the batch stops.
HD_D bool begin_edit(const Table& t, const PArgs& a, const Smem& sm)
{
    Ctl* ctl = a.ctl;
    const uint32_t G = gridDim.x;
    if (threadIdx.x == 0) {
        const uint32_t idx = ctl->idx;
        uint32_t stop = ctl->stop;
        if (stop == kRun && __ldcg(t.error) != 0)
            stop = kTableError;
        if (stop == kRun && idx >= a.n_edits)
            stop = kDone;
        ctl->stop = stop;
        if (stop == kRun) {
            a.t_begin[idx] = now_ns();
            *sm.ed = make_editor(a.edits[idx]);
            ctl->ed = *sm.ed;
            for (uint32_t L = 0; L < HD_MAX_DEPTH; L++)
                ctl->count[L] = 0;
            ctl->count[0] = 1;
            const Level l0 = a.lv[0];
            l0.x[0] = 0;
            l0.y[0] = 0;
            l0.z[0] = 0;
            l0.old[0] = __ldcg(a.d_root);
            a.ctr[idx] = EditCounters{};
        }
        sm.sm32[32] = stop;
    }
    for (uint32_t k = threadIdx.x; k < 3 * G; k += kPT)
        a.bsum[k] = 0;
    __syncthreads();
    if (sm.sm32[32] != kRun)
        return false;
    if (threadIdx.x == 0) {
        unsigned long long nn, vv;
        classify_entry<true>(t, *sm.ed, 0, a.lv[0], 0, nn, vv);
        EditCounters* ctr = a.ctr + ctl->idx;
        atomicAdd(&ctr->num_nodes, nn);
        atomicAdd(&ctr->num_voxels, vv);
    }
    __syncthreads();
    return true;
}

// CTA 0, after level 0's find-or-add: the new root, or the stop.
HD_D void finish_edit(const Table& t, const PArgs& a)
{
    Ctl* ctl = a.ctl;
    if (threadIdx.x == 0) {
        const uint32_t idx = ctl->idx;
        if (__ldcg(t.error) != 0) {
            ctl->stop = kTableError;
        } else {
            const uint32_t r = __ldcg(a.lv[0].res);
            if (r == kInvalid || r == kNotFound) {
                ctl->stop = kEmptyScene;
            } else {
                *a.d_root = r;
                a.roots[idx] = r;
                __threadfence();
                a.t_end[idx] = now_ns();
                ctl->idx = idx + 1;
            }
        }
    }
    __syncthreads();
}

// CTA 0: advances the batch alone from state ls at level L (small levels,
// the end of an edit, the start of the next) until the grid is needed
// (ctl->phase / ctl->level) or the batch stops (ctl->stop).
template <int PW>
HD_D void local_advance(const Table& t, const PArgs& a, uint32_t ls, uint32_t L, const Smem& sm)
{
    Ctl* ctl = a.ctl;
    const uint32_t G = gridDim.x, leafl = t.g.leaf_level;
    const uint32_t warp = threadIdx.x >> 5;
    for (;;) {
        if (ls == kLsFinish) {
            // the edit ends; the grid meets once per edit, so that no wait at
            // a barrier spans more than one edit of CTA 0's work
            finish_edit(t, a);
            if (threadIdx.x == 0)
                ctl->phase = kPhNone;
            __syncthreads();
            return;
        }
        if (ls == kLsBegin) {
            if (!begin_edit(t, a, sm))
                return;
            L = 0;
            ls = kLsTopDown;
        }
        const uint32_t idx = ctl->idx;
        EditCounters* ctr = a.ctr + idx;
        if (ls == kLsTopDown) {
            __shared__ uint32_t tiny[2];
            while (L < leafl) {
                uint32_t n = ctl->count[L];
                if (n <= 32) {
                    // the levels of at most 32 entries: warp 0 alone
                    if (warp == 0) {
                        uint32_t st;
                        const uint32_t L2 = td_tiny(t, *sm.ed, a, L, n, ctr, sm.list, st);
                        if ((threadIdx.x & 31) == 0) {
                            tiny[0] = L2;
                            tiny[1] = st;
                        }
                    }
                    __syncthreads();
                    L = tiny[0];
                    const uint32_t st = tiny[1];
                    __syncthreads();
                    if (st == 2) {
                        if (threadIdx.x == 0)
                            ctl->stop = kCapacity;
                        __syncthreads();
                        return;
                    }
                    if (st == 1 || L >= leafl)
                        break;
                    n = ctl->count[L];
                }
                if (n > kSmall) {
                    if (threadIdx.x == 0) {
                        ctl->phase = kPhTopDown;
                        ctl->level = L;
                    }
                    __syncthreads();
                    return;
                }
                uint32_t f = 0;
                for (uint32_t i = threadIdx.x; i < n; i += kPT)
                    f += a.lv[L].flag[i];
                uint32_t total;
                cta_scan(f, &total, sm.sm32);
                if (total == 0)
                    break;
                const uint64_t n_next = 8ull * total;
                if (n_next > a.cap[L + 1]) {
                    if (threadIdx.x == 0)
                        ctl->stop = kCapacity;
                    __syncthreads();
                    return;
                }
                uint32_t* zero = a.bsum + ((L + 2) % 3) * G;
                for (uint32_t k = threadIdx.x; k < G; k += kPT)
                    zero[k] = 0;
                __syncthreads();
                td_range(t, *sm.ed, a.lv, L, 0, n, 0, uint32_t(n_next), G, a.bsum + ((L + 1) % 3) * G, ctr, sm.sm32,
                         sm.list);
                if (threadIdx.x == 0)
                    ctl->count[L + 1] = uint32_t(n_next);
                __syncthreads();
                L++;
            }
            if (threadIdx.x == 0)
                ctl->deepest = L;
            __syncthreads();
            ls = kLsBottomUp;
        }
        if (ls == kLsBottomUp) {
            const uint32_t deepest = ctl->deepest;
            for (;;) {
                if (__ldcg(t.error) != 0)
                    break;
                const uint32_t n = ctl->count[L];
                if (n > kSmall) {
                    if (threadIdx.x == 0) {
                        ctl->phase = kPhBottomUp;
                        ctl->level = L;
                    }
                    __syncthreads();
                    return;
                }
                candidates_range(t, a.lv, L, deepest, 0, n, a.keys, a.vals);
                __syncthreads();
                const uint32_t runs = small_sort(t, L, n, a.keys, a.vals, sm.s64, sm.sm32, sm.sk, sm.sv);
                if (runs > 2 * kPWarps) {
                    // many buckets: the grid resolves them
                    if (threadIdx.x == 0) {
                        ctl->phase = kPhGridFoa;
                        ctl->level = L;
                    }
                    __syncthreads();
                    return;
                }
                foa_sorted<PW, true>(t, L, a.lv[L], sm.sk, sm.sv, n, warp, kPWarps, sm.page + warp * kPage,
                               sm.q + warp * 12, sm.cache[warp], ctr);
                // the CTA barrier makes this level's results (lv.res, appended
                // nodes) visible to CTA 0's next level; the grid barrier
                // (a CTA barrier, then a fence by its thread 0) to the grid
                __syncthreads();
                if (L == 0)
                    break;
                L--;
            }
            ls = kLsFinish;
        }
    }
}

template <int PW>
__global__ void __launch_bounds__(kPT, 1) k_edit_persistent(Table t, PArgs a)
{
    {
        const uint32_t skip = __ldcg(&a.ctl->skip_cta);
        if (skip && blockIdx.x == skip - 1)
            return; // a test of the timeout path: this CTA never arrives
    }
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint32_t sm32[40];
    __shared__ Editor ed_s;
    __shared__ uint32_t cnt[kDigits];
    // the foa buffers (pages, queries, caches); the same bytes serve the
    // small sort, the top-down tile list and the scatter's digit runs
    Smem sm;
    sm.page = reinterpret_cast<uint32_t*>(smem_raw);
    sm.q = sm.page + kPWarps * kPage;
    sm.cache = reinterpret_cast<FoaCache*>(sm.q + kPWarps * 12);
    sm.s64 = reinterpret_cast<unsigned long long*>(smem_raw);
    sm.sk = reinterpret_cast<uint32_t*>(smem_raw + persist_smem_core());
    sm.sv = sm.sk + kPT;
    sm.list = sm.page;
    sm.sm32 = sm32;
    sm.ed = &ed_s;
    uint32_t* run = sm.page;
    Ctl* ctl = a.ctl;
    const uint32_t G = gridDim.x, cta = blockIdx.x;
    const uint32_t warp = threadIdx.x >> 5;
    const uint32_t leafl = t.g.leaf_level;
    uint32_t ls = kLsBegin, L = 0;
    __shared__ uint32_t nbar; // barriers this CTA has passed (thread 0)
    if (threadIdx.x == 0)
        nbar = 0;
    __syncthreads();
    for (;;) {
        if (cta == 0) {
            local_advance<PW>(t, a, ls, L, sm);
            if (threadIdx.x == 0) // the command of the coming barrier
                ctl->cmd[(nbar + 1) & 1] = Cmd{ctl->stop, ctl->phase, ctl->level, ctl->deepest, ctl->idx, {0, 0, 0}};
        }
        if (!grid_sync(ctl, t.error, nbar))
            return;
        // the grid step CTA 0 asked for, decided the same way by every CTA
        __shared__ Cmd cmd;
        if (threadIdx.x == 0) {
            const uint32_t* src = reinterpret_cast<const uint32_t*>(&ctl->cmd[nbar & 1]);
            uint32_t* dst = reinterpret_cast<uint32_t*>(&cmd);
            for (uint32_t k = 0; k < sizeof(Cmd) / 4; k++)
                dst[k] = __ldcg(src + k);
        }
        __syncthreads();
        if (cmd.stop != kRun)
            return;
        uint32_t phase = cmd.phase;
        if (phase == kPhNone) {
            ls = kLsBegin; // an edit ended: CTA 0 starts the next
            continue;
        }
        L = cmd.level;
        uint32_t deepest = cmd.deepest;
        const uint32_t idx = cmd.idx;
        EditCounters* ctr = a.ctr + idx;
        if (threadIdx.x == 0) {
            const uint32_t* src = reinterpret_cast<const uint32_t*>(&ctl->ed);
            uint32_t* dst = reinterpret_cast<uint32_t*>(&ed_s);
            for (uint32_t k = 0; k < sizeof(Editor) / 4; k++)
                dst[k] = __ldcg(src + k);
        }
        __syncthreads();
        if (phase == kPhTopDown) {
            // one phase per level down to the deepest
            for (;;) {
                const uint32_t n = __ldcg(&ctl->count[L]);
                const uint32_t* cnt_cur = a.bsum + (L % 3) * G;
                uint32_t before = 0, all = 0;
                for (uint32_t b = threadIdx.x; b < G; b += kPT) {
                    const uint32_t v = __ldcg(cnt_cur + b);
                    all += v;
                    before += b < cta ? v : 0u;
                }
                uint32_t tb, ta;
                cta_scan(before, &tb, sm32);
                cta_scan(all, &ta, sm32);
                if (ta == 0)
                    break; // nothing descends: L is the deepest level
                const uint64_t n_next = 8ull * ta;
                if (n_next > a.cap[L + 1]) {
                    if (cta == 0 && threadIdx.x == 0)
                        ctl->stop = kCapacity;
                    return; // every CTA decides this alike
                }
                if (threadIdx.x == 0)
                    a.bsum[((L + 2) % 3) * G + cta] = 0;
                // positions and the list of descended entries (keys2 is
                // free until the edit's bottom-up levels), then the children
                // spread evenly over the CTAs
                const uint32_t chunk = chunk_len(n, G, kChunkAlign);
                const uint32_t i0 = min(n, cta * chunk), i1 = min(n, i0 + chunk);
                td_positions(a.lv[L], i0, i1, tb, a.keys2, sm32);
                if (!grid_sync(ctl, t.error, nbar))
                    return;
                const uint32_t cch = chunk_len(uint32_t(n_next), G, kChunkAlign);
                const uint32_t k0 = min(uint32_t(n_next), cta * cch), k1 = min(uint32_t(n_next), k0 + cch);
                td_children(t, ed_s, a.lv, L, k0, k1, uint32_t(n_next), G, a.keys2, a.bsum + ((L + 1) % 3) * G, ctr);
                if (cta == 0 && threadIdx.x == 0)
                    ctl->count[L + 1] = uint32_t(n_next);
                if (!grid_sync(ctl, t.error, nbar))
                    return;
                L++;
                if (L == leafl)
                    break;
            }
            deepest = L;
            if (cta == 0 && threadIdx.x == 0)
                ctl->deepest = L;
            phase = kPhBottomUp;
        }
        if (phase == kPhGridFoa) {
            // a small level's sorted candidates in many buckets
            const uint32_t n = __ldcg(&ctl->count[L]);
            foa_sorted<PW>(t, L, a.lv[L], a.keys, a.vals, n, cta * kPWarps + warp, G * kPWarps,
                           sm.page + warp * kPage, sm.q + warp * 12, sm.cache[warp], ctr);
            if (!grid_sync(ctl, t.error, nbar))
                return;
            if (L == 0) {
                ls = kLsFinish;
                continue;
            }
            L--;
            phase = kPhBottomUp;
        }
        // bottom-up, big levels: six phases each; small ones go back to CTA 0
        while (__ldcg(&ctl->count[L]) > kSmall && __ldcg(t.error) == 0) {
            const uint32_t n = __ldcg(&ctl->count[L]);
            const uint32_t nb = min(G, (n + kChunkAlign - 1) / kChunkAlign);
            const uint32_t chunk = chunk_len(n, nb, kChunkAlign);
            uint32_t key_bits = 1;
            while ((1u << key_bits) <= t.g.buckets(L))
                key_bits++;
            const uint32_t dbits = (key_bits + 1) / 2, nd = 1u << dbits;
            // 1. candidates and their pass-1 digit counts
            if (cta < nb) {
                for (uint32_t d = threadIdx.x; d < nd; d += kPT) {
                    cnt[d] = 0;
                    a.hist2[d * nb + cta] = 0;
                }
                __syncthreads();
                const uint32_t i0 = cta * chunk, i1 = min(n, i0 + chunk);
                candidates_range(t, a.lv, L, deepest, i0, i1, a.keys, a.vals);
                for (uint32_t i = i0 + threadIdx.x; i < i1; i += kPT)
                    atomicAdd(&cnt[a.keys[i] & (nd - 1)], 1u);
                __syncthreads();
                for (uint32_t d = threadIdx.x; d < nd; d += kPT)
                    a.hist[d * nb + cta] = cnt[d];
            }
            if (!grid_sync(ctl, t.error, nbar))
                return;
            // 2. pass-1 rows
            scan_rows(a.hist, nb, nd, a.rows);
            if (!grid_sync(ctl, t.error, nbar))
                return;
            // 3. pass-1 scatter, pass-2 counts
            if (cta < nb)
                scatter_chunk(a.keys, a.vals, n, nb, cta, 0, nd, a.hist, a.rows, a.keys2, a.vals2, a.hist2, dbits,
                              run, sm32);
            if (!grid_sync(ctl, t.error, nbar))
                return;
            // 4. pass-2 rows
            scan_rows(a.hist2, nb, nd, a.rows2);
            if (!grid_sync(ctl, t.error, nbar))
                return;
            // 5. pass-2 scatter
            if (cta < nb)
                scatter_chunk(a.keys2, a.vals2, n, nb, cta, dbits, nd, a.hist2, a.rows2, a.keys, a.vals, nullptr, 0,
                              run, sm32);
            if (!grid_sync(ctl, t.error, nbar))
                return;
            // 6. find-or-add, one warp per bucket run
            foa_sorted<PW>(t, L, a.lv[L], a.keys, a.vals, n, cta * kPWarps + warp, G * kPWarps,
                           sm.page + warp * kPage, sm.q + warp * 12, sm.cache[warp], ctr);
            if (!grid_sync(ctl, t.error, nbar))
                return;
            if (L == 0)
                break; // (level 0 holds one entry: never big)
            L--;
        }
        ls = kLsBottomUp; // CTA 0 continues at L (or finishes the edit on an error)
    }
}

} // namespace

// ---- host side --------------------------------------------------------------------

struct PersistBuffers {
    Ctl* ctl = nullptr;
    Level* d_lv = nullptr;
    size_t smem = 0;
    uint32_t grid = 0;
};

static size_t persist_smem() { return persist_smem_core() + size_t(kPT) * 4 * 2; }

template <int PW>
static const void* persist_kernel()
{
    return reinterpret_cast<const void*>(k_edit_persistent<PW>);
}

// Applies edits[0..n) in one persistent launch per stretch of the batch (a
// level that would outgrow its bound ends the stretch: that edit takes the
// one-edit path and the next stretch starts after it).
void edit_batch_persistent(hd_ctx* c, const hd_edit* edits, uint32_t n, const std::vector<Level>& lv,
                           const std::vector<uint32_t>& caps, uint32_t* keys, uint32_t* vals, uint32_t* keys2,
                           uint32_t* vals2, hd_edit* d_edits, EditCounters* d_ctr, uint32_t* d_roots,
                           std::vector<EditCounters>& ctr, std::vector<float>& dur_ms, std::vector<float>& end_ms,
                           float& device_ms, uint64_t& fallbacks)
{
    cudaStream_t st = c->stream;
    Scratch& s = c->scratch;
    const uint32_t levels = c->g.leaf_level + 1;
    int dev = 0, sms = 0;
    HD_CUDA(cudaGetDevice(&dev));
    HD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const size_t smem = persist_smem();
    const void* kern = c->tuning.probe_words == 4   ? persist_kernel<4>()
                       : c->tuning.probe_words == 2 ? persist_kernel<2>()
                                                    : persist_kernel<1>();
    HD_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    int per_sm = 0;
    HD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPT, smem));
    if (per_sm < 1)
        throw StatusError{HD_ERR_STATE, "the persistent edit kernel does not fit on an SM"};
    const uint32_t G = uint32_t(sms); // one CTA per SM
    Ctl* ctl = s.get<Ctl>("ep_ctl", 1);
    Level* d_lv = s.get<Level>("ep_lv", HD_MAX_DEPTH);
    HD_CUDA(cudaMemcpyAsync(d_lv, lv.data(), sizeof(Level) * levels, cudaMemcpyHostToDevice, st));
    PArgs a{};
    a.ctl = ctl;
    a.lv = d_lv;
    for (uint32_t L = 0; L < levels; L++)
        a.cap[L] = caps[L];
    a.keys = keys;
    a.vals = vals;
    a.keys2 = keys2;
    a.vals2 = vals2;
    a.bsum = s.get<uint32_t>("ep_bsum", 3ull * G);
    a.hist = s.get<uint32_t>("ep_hist", uint64_t(kDigits) * G);
    a.hist2 = s.get<uint32_t>("ep_hist2", uint64_t(kDigits) * G);
    a.rows = s.get<uint32_t>("ep_rows", kDigits);
    a.rows2 = s.get<uint32_t>("ep_rows2", kDigits);
    a.ctr = d_ctr;
    a.roots = d_roots;
    a.t_begin = s.get<unsigned long long>("ep_tbegin", n + 1);
    a.t_end = s.get<unsigned long long>("ep_tend", n + 1);
    a.d_root = c->d_root;
    std::vector<unsigned long long> tb(n), te(n);
    uint32_t done = 0;
    c->batch_applied = 0;
    float elapsed_before = 0.0f;
    unsigned long long first_ns = 0;
    while (done < n) {
        const uint32_t m = n - done;
        a.edits = d_edits;
        a.n_edits = m;
        HD_CUDA(cudaMemcpyAsync(d_edits, edits + done, sizeof(hd_edit) * m, cudaMemcpyHostToDevice, st));
        HD_CUDA(cudaMemsetAsync(ctl, 0, sizeof(Ctl), st));
        if (c->test_skip_cta) {
            // one launch only: the hook switches itself off
            const uint32_t skip = c->test_skip_cta;
            const unsigned long long wait = c->test_wait_ns;
            HD_CUDA(cudaMemcpyAsync(&ctl->skip_cta, &skip, 4, cudaMemcpyHostToDevice, st));
            HD_CUDA(cudaMemcpyAsync(&ctl->wait_ns, &wait, 8, cudaMemcpyHostToDevice, st));
            HD_CUDA(cudaStreamSynchronize(st));
            c->test_skip_cta = 0;
            c->test_wait_ns = 0;
        }
        HD_CUDA(cudaEventRecord(c->ev0, st));
        void* args[] = {&c->t, &a};
        HD_CUDA(cudaLaunchCooperativeKernel(kern, dim3(G), dim3(kPT), args, smem, st));
        HD_CUDA(cudaEventRecord(c->ev1, st));
        Ctl fin{};
        HD_CUDA(cudaMemcpyAsync(&fin, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
        HD_CUDA(cudaStreamSynchronize(st));
        float launch_ms = 0;
        HD_CUDA(cudaEventElapsedTime(&launch_ms, c->ev0, c->ev1));
        const uint32_t ok = fin.idx;
        if (ok) {
            HD_CUDA(cudaMemcpy(ctr.data() + done, d_ctr, sizeof(EditCounters) * ok, cudaMemcpyDeviceToHost));
            std::vector<uint32_t> roots(ok);
            HD_CUDA(cudaMemcpy(roots.data(), d_roots, 4ull * ok, cudaMemcpyDeviceToHost));
            HD_CUDA(cudaMemcpy(tb.data() + done, a.t_begin, 8ull * ok, cudaMemcpyDeviceToHost));
            HD_CUDA(cudaMemcpy(te.data() + done, a.t_end, 8ull * ok, cudaMemcpyDeviceToHost));
            if (!first_ns)
                first_ns = tb[done];
            for (uint32_t k = 0; k < ok; k++) {
                UndoFrame f;
                f.root = c->root;
                push_undo(c, std::move(f));
                c->root = roots[k];
                dur_ms[done + k] = float(double(te[done + k] - tb[done + k]) * 1e-6);
                end_ms[done + k] = elapsed_before + float(double(te[done + k] - tb[done]) * 1e-6);
            }
        }
        elapsed_before += launch_ms;
        done += ok;
        c->batch_applied = done;
        if (fin.abort) {
            check_error(c);
            c->root = read_scalar(c->d_root, st);
            std::string where;
            for (uint32_t k = 0; k < 8; k++)
                where += (k ? " " : "") + std::to_string(fin.diag[k]);
            throw StatusError{HD_ERR_TIMEOUT, "edit " + std::to_string(done) +
                                                  ": a grid barrier of the persistent edit kernel ran out of time "
                                                  "(cta, barriers, arrivals, arrivals awaited, cta0 barriers, phase, level, edit: " +
                                                  where + ")"};
        }
        if (fin.stop == kDone)
            break;
        if (fin.stop == kTableError || fin.stop == kEmptyScene) {
            const uint32_t err = check_error(c);
            c->root = read_scalar(c->d_root, st);
            if (fin.stop == kEmptyScene)
                throw StatusError{HD_ERR_STATE, "edit " + std::to_string(done) + " would empty the whole scene"};
            throw StatusError{hd_status(err ? err : HD_ERR_CUDA),
                              "edit " + std::to_string(done) + " failed on the device (" + c->err_detail + ")"};
        }
        // capacity: this edit with the one-edit path, then resume
        c->root = read_scalar(c->d_root, st);
        hd_edit_stats es{};
        edit_one(c, edits[done], &es);
        ctr[done].num_voxels = es.num_voxels;
        ctr[done].num_nodes = es.num_nodes;
        ctr[done].foa = es.find_or_add_calls;
        ctr[done].added = es.nodes_added;
        ctr[done].scanned = es.words_scanned;
        dur_ms[done] = es.device_ms;
        elapsed_before += es.device_ms;
        end_ms[done] = elapsed_before;
        done++;
        c->batch_applied = done;
        fallbacks++;
    }
    device_ms = elapsed_before;
}

} // namespace hd
