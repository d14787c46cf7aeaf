// Edit pipeline, one edit per call: the host sizes every level from the
// previous one and launches the level kernels (see hd_edit.cuh for the
// design and the reference lines).  The batched, graph-captured form is in
// hd_edit_batch.cu.
#include <chrono>
#include <vector>

#include "hd_edit.cuh"
#include "hd_sort.cuh"

namespace hd {

constexpr uint32_t kFoaWarps = 4;

// the device error word without clearing it
static uint32_t check_error_peek(hd_ctx* c) { return read_scalar(c->t.error, c->stream); }
constexpr int kFoaProbe = 4;

__global__ void k_edit_classify(Table t, Editor ed, uint32_t level, uint32_t n, Level lv, EditCounters* ctr)
{
    HD_GRID_STRIDE(i, n)
    {
        unsigned long long nodes, voxels;
        classify_entry(t, ed, level, lv, uint32_t(i), nodes, voxels);
        warp_add(&ctr->num_nodes, nodes);
        warp_add(&ctr->num_voxels, voxels);
    }
}

__global__ void k_edit_spawn(Table t, uint32_t n, Level lv, Level next)
{
    HD_GRID_STRIDE(i, n) spawn_entry(t, lv, next, uint32_t(i));
}

// Candidates keyed by global bucket index; kEmpty for resolved entries.
__global__ void k_edit_candidates(Table t, uint32_t level, uint32_t n, Level lv, Level child, uint32_t* keys,
                                  uint32_t* vals, uint32_t* n_cand)
{
    // after a failed append below, the levels above are not rebuilt: their
    // children would be unresolved
    if (__ldcg(t.error) != 0)
        return;
    HD_GRID_STRIDE(i, n)
    {
        const uint32_t b = candidate_entry(t, level, lv, child, uint32_t(i));
        vals[i] = uint32_t(i);
        if (b == kNoBucket) {
            keys[i] = kEmpty;
        } else {
            keys[i] = t.g.bucket_global(level, b);
            atomicAdd(n_cand, 1u);
        }
    }
}

// After the stable sort by bucket: the first position of every bucket's run.
__global__ void k_segment_flags(const uint32_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ flag)
{
    HD_GRID_STRIDE(j, n) flag[j] = keys[j] != kEmpty && (j == 0 || keys[j] != keys[j - 1]);
}

__global__ void k_segment_starts(const uint32_t* __restrict__ flag, const uint32_t* __restrict__ pos, uint32_t n,
                                 uint32_t* __restrict__ starts)
{
    HD_GRID_STRIDE(j, n)
    {
        if (flag[j])
            starts[pos[j]] = uint32_t(j);
    }
}

__global__ void __launch_bounds__(32 * kFoaWarps)
    k_edit_find_or_add(Table t, uint32_t level, Level lv, const uint32_t* __restrict__ keys,
                       const uint32_t* __restrict__ vals, const uint32_t* __restrict__ starts,
                       const uint32_t* __restrict__ n_seg, const uint32_t* __restrict__ n_cand, EditCounters* ctr)
{
    __shared__ uint32_t page_s[kFoaWarps][kPage];
    __shared__ uint32_t q_s[kFoaWarps][9];
    __shared__ FoaCache cache_s[kFoaWarps];
    if (__ldcg(t.error) != 0)
        return; // a level below failed (see k_edit_candidates)
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t nseg = *n_seg, ncand = *n_cand;
    const uint32_t first = t.g.level_first_bucket(level);
    unsigned long long foa = 0, added = 0, scanned = 0;
    for (uint32_t si = blockIdx.x * kFoaWarps + warp; si < nseg; si += gridDim.x * kFoaWarps) {
        const uint32_t j0 = starts[si], j1 = si + 1 < nseg ? starts[si + 1] : ncand;
        foa_segment<kFoaProbe>(t, level, lv, vals, j0, j1, keys[j0] - first, page_s[warp], q_s[warp], cache_s[warp],
                               foa, added, scanned);
    }
    if (lane == 0) {
        atomicAdd(&ctr->foa, foa);
        atomicAdd(&ctr->added, added);
        atomicAdd(&ctr->scanned, scanned);
        atomicAdd(reinterpret_cast<unsigned long long*>(t.level_nodes + level), added);
    }
}

__global__ void k_edit_finish(const Level lv0, uint32_t* d_root, uint32_t* err)
{
    if (err[0] != 0)
        return; // the edit failed: the root stays
    const uint32_t r = lv0.res[0];
    if (r == kInvalid || r == kNotFound)
        set_error(err, kErrCapacity);
    else
        *d_root = r;
}

// ---- host orchestration -------------------------------------------------------
struct EditBuffers {
    std::vector<Level> lv;
    std::vector<uint32_t> cap;
};

static Level alloc_level(Scratch& s, uint32_t L, uint64_t n, bool leaf, bool colors)
{
    char nm[48];
    auto buf = [&](const char* what, size_t bytes) {
        snprintf(nm, sizeof(nm), "ed_%s_%u", what, L);
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
    if (colors) {
        l.ocnt = static_cast<uint32_t*>(buf("ocnt", n * 4));
        l.cn = static_cast<uint32_t*>(buf("cn", n * 4));
        l.noff = static_cast<uint32_t*>(buf("noff", n * 4));
        l.ooff = static_cast<uint32_t*>(buf("ooff", n * 4));
        l.task = static_cast<uint32_t*>(buf("task", n * 4));
    }
    return l;
}

void edit_one(hd_ctx* c, const hd_edit& e, hd_edit_stats* stats)
{
    if (c->needs_gc)
        throw StatusError{HD_ERR_STATE, "the table was loaded without bucket sizes; run hd_gc before editing"};
    cudaStream_t st = c->stream;
    Scratch& s = c->scratch;
    const Geom& g = c->g;
    const uint32_t levels = g.leaf_level + 1;
    Editor ed = make_editor(e);
    const bool colors = c->colors;
    const auto t0 = std::chrono::steady_clock::now();
    HD_CUDA(cudaEventRecord(c->ev0, st));
    if (e.tool == HD_TOOL_COPY)
        copy_source(c, ed); // the source region as it is before the edit
    if (e.tool >= HD_TOOL_NOISE_REMOVE)
        tool_buffers(c, ed); // the noise or fill buffer, made before the edit
    UndoFrame frame;
    frame.root = c->root;
    EditCounters* ctr = s.get<EditCounters>("ed_ctr", 1);
    HD_CUDA(cudaMemsetAsync(ctr, 0, sizeof(EditCounters), st));
    uint32_t* d_n = s.get<uint32_t>("ed_n", 4);
    std::vector<Level> lv(levels);
    std::vector<uint32_t> count(levels, 0);
    lv[0] = alloc_level(s, 0, 1, levels == 1, colors);
    if (colors)
        HD_CUDA(cudaMemsetAsync(lv[0].cn, 0, 4, st));
    HD_CUDA(cudaMemsetAsync(lv[0].x, 0, 4, st));
    HD_CUDA(cudaMemsetAsync(lv[0].y, 0, 4, st));
    HD_CUDA(cudaMemsetAsync(lv[0].z, 0, 4, st));
    HD_CUDA(cudaMemcpyAsync(lv[0].old, c->d_root, 4, cudaMemcpyDeviceToDevice, st));
    count[0] = 1;
    // top-down
    uint32_t deepest = 0;
    for (uint32_t L = 0; L < levels; L++) {
        const uint32_t n = count[L];
        deepest = L;
        k_edit_classify<<<grid_for(n, 128), 128, 0, st>>>(c->t, ed, L, n, lv[L], ctr);
        HD_LAUNCH_CHECK();
        if (L + 1 == levels)
            break;
        exclusive_scan<uint32_t, uint32_t>(s, lv[L].flag, lv[L].exp, n, d_n, st);
        const uint32_t ne = read_scalar(d_n, st);
        if (ne == 0)
            break;
        count[L + 1] = 8 * ne;
        lv[L + 1] = alloc_level(s, L + 1, count[L + 1], L + 1 == g.leaf_level, colors);
        k_edit_spawn<<<grid_for(n, 128), 128, 0, st>>>(c->t, n, lv[L], lv[L + 1]);
        HD_LAUNCH_CHECK();
        if (colors && L < g.T) {
            color_spawn(c, L, n, lv[L], lv[L + 1]);
        }
    }
    // bottom-up
    uint32_t maxn = 1;
    for (uint32_t L = 0; L <= deepest; L++)
        maxn = count[L] > maxn ? count[L] : maxn;
    uint32_t* keys = s.get<uint32_t>("ed_keys", maxn);
    uint32_t* vals = s.get<uint32_t>("ed_vals", maxn);
    uint32_t* flag = s.get<uint32_t>("ed_segflag", maxn);
    uint32_t* pos = s.get<uint32_t>("ed_segpos", maxn);
    uint32_t* starts = s.get<uint32_t>("ed_segstart", maxn);
    uint32_t* d_cnt = s.get<uint32_t>("ed_cnt", 4); // [0] candidates, [1] segments
    uint32_t key_bits = 1;
    while ((uint64_t(1) << key_bits) <= g.total_buckets)
        key_bits++;
    for (int32_t L = int32_t(deepest); L >= 0; L--) {
        const uint32_t n = count[L];
        HD_CUDA(cudaMemsetAsync(d_cnt, 0, 8, st));
        const Level child = uint32_t(L) < deepest ? lv[L + 1] : Level{};
        k_edit_candidates<<<grid_for(n, 128), 128, 0, st>>>(c->t, uint32_t(L), n, lv[L], child, keys, vals, d_cnt);
        HD_LAUNCH_CHECK();
        // candidates grouped by bucket, depth-first order kept inside a bucket
        radix_sort_pairs(s, keys, vals, n, key_bits, st);
        k_segment_flags<<<grid_for(n, 256), 256, 0, st>>>(keys, n, flag);
        HD_LAUNCH_CHECK();
        exclusive_scan<uint32_t, uint32_t>(s, flag, pos, n, d_cnt + 1, st);
        k_segment_starts<<<grid_for(n, 256), 256, 0, st>>>(flag, pos, n, starts);
        HD_LAUNCH_CHECK();
        k_edit_find_or_add<<<grid_for(uint64_t(n) * 32, 32 * kFoaWarps, 152 * 8), 32 * kFoaWarps, 0, st>>>(
            c->t, uint32_t(L), lv[L], keys, vals, starts, d_cnt + 1, d_cnt, ctr);
        HD_LAUNCH_CHECK();
    }
    if (colors && !check_error_peek(c))
        edit_colors(c, ed, lv, count, deepest, frame);
    k_edit_finish<<<1, 1, 0, st>>>(lv[0], c->d_root, c->t.error);
    HD_LAUNCH_CHECK();
    HD_CUDA(cudaEventRecord(c->ev1, st));
    EditCounters h{};
    HD_CUDA(cudaMemcpyAsync(&h, ctr, sizeof(h), cudaMemcpyDeviceToHost, st));
    HD_CUDA(cudaStreamSynchronize(st));
    const uint32_t err = check_error(c);
    if (err)
        throw StatusError{err == kErrCapacity ? HD_ERR_STATE : hd_status(err),
                          err == kErrCapacity ? "edit would empty the whole scene"
                                              : "edit failed on the device (" + c->err_detail + ")"};
    c->root = read_scalar(c->d_root, st);
    push_undo(c, std::move(frame));
    if (stats) {
        stats->num_voxels = h.num_voxels;
        stats->num_nodes = h.num_nodes;
        stats->find_or_add_calls = h.foa;
        stats->nodes_added = h.added;
        stats->words_scanned = h.scanned;
        HD_CUDA(cudaEventElapsedTime(&stats->device_ms, c->ev0, c->ev1));
        stats->host_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
}

} // namespace hd

extern "C" {

hd_status hd_edit_apply(hd_ctx* c, const hd_edit* edit, hd_edit_stats* stats)
{
    if (!c || !edit || edit->tool > HD_TOOL_FILL || !(edit->radius >= 0.0f))
        return HD_ERR_INVALID;
    try {
        hd::edit_one(c, *edit, stats);
        return HD_OK;
    } catch (const hd::StatusError& e) {
        c->err = e.msg;
        return e.status;
    } catch (const hd::CudaError& e) {
        c->err = std::string("CUDA error ") + cudaGetErrorString(e.code) + " in " + e.where;
        return HD_ERR_CUDA;
    }
}

} // extern "C"
