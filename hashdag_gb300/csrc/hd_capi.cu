// The C ABI (include/hashdag_gb300.h): status codes instead of aborts, one
// context per table, all work on the context's stream.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <functional>
#include <cstring>
#include <new>

#include "hd_ctx.h"

using namespace hd;

namespace {

bool valid_config(const hd_config& c, std::string& why)
{
    if (c.depth < 4 || c.depth > HD_MAX_DEPTH)
        return why = "depth must be in [4, 20]", false;
    if (c.color_tree_levels > c.depth - 2)
        return why = "color_tree_levels must not exceed the leaf level", false;
    if (c.top_bucket_bits > 20 || c.low_bucket_bits > 24)
        return why = "bucket bits too large", false;
    if (c.top_bucket_size % HD_PAGE_SIZE || c.low_bucket_size % HD_PAGE_SIZE || !c.top_bucket_size ||
        !c.low_bucket_size)
        return why = "bucket sizes must be multiples of the 512-word page", false;
    if (c.color_tree_levels + 7 < c.depth)
        return why = "a full node at color_tree_levels would need more than 24 count bits", false;
    const Geom g = make_geom(c);
    if (g.total_vpages * HD_PAGE_SIZE > 0xFFFFFFFFull)
        return why = "virtual address space exceeds 32 bits", false;
    if (c.pool_pages < 2)
        return why = "pool_pages too small", false;
    return true;
}

void refresh_root(hd_ctx* c) { c->root = read_scalar(c->d_root, c->stream); }

void check_device_error(hd_ctx* c, const char* what)
{
    const uint32_t e = check_error(c);
    if (e)
        throw StatusError{e == kErrCapacity ? HD_ERR_INVALID : hd_status(e),
                          std::string(what) + " failed on the device (" + c->err_detail + ")"};
}

} // namespace

extern "C" {

uint32_t hd_abi_version(void) { return HD_ABI_VERSION; }

void hd_default_config(uint32_t depth, hd_config* out)
{
    out->depth = depth;
    out->color_tree_levels = depth >= 15 ? 10 : (depth > 5 ? depth - 5 : 0);
    out->top_levels = 9;
    out->top_bucket_bits = depth <= 10 ? 10 : (depth <= 15 ? 12 : 14);
    out->low_bucket_bits = depth <= 15 ? 16 : 17;
    out->top_bucket_size = 1024;
    out->low_bucket_size = 4096;
    // enough pages for every bucket of the table
    const Geom g = make_geom(*out);
    uint64_t pages = g.total_vpages + 1;
    if (pages > (1ull << 23))
        pages = 1ull << 23; // 16 GB of pool
    out->pool_pages = uint32_t(pages);
}

hd_status hd_create(const hd_config* cfg, hd_ctx** out)
{
    if (!out)
        return HD_ERR_INVALID;
    *out = nullptr;
    hd_config conf;
    if (cfg)
        conf = *cfg;
    else
        hd_default_config(16, &conf);
    std::string why;
    if (!valid_config(conf, why))
        return HD_ERR_INVALID;
    hd_ctx* c = new (std::nothrow) hd_ctx();
    if (!c)
        return HD_ERR_OOM;
    c->cfg = conf;
    c->g = make_geom(conf);
    hd_status st = guarded(c, [&] {
        Table& t = c->t;
        t.g = c->g;
        // 64 bytes past the last page: a node read at its physical offset
        // stays inside the allocation even in a corrupt table
        HD_CUDA(cudaMalloc(&t.pool, size_t(conf.pool_pages) * HD_PAGE_SIZE * 4 + 64));
        HD_CUDA(cudaMalloc(&t.bloom, size_t(conf.pool_pages) * kBloomWords * 4));
        HD_CUDA(cudaMalloc(&t.page_table, kPageTableEntries * 4));
        HD_CUDA(cudaMalloc(&t.bucket_sizes, c->g.total_buckets * 4));
        HD_CUDA(cudaMalloc(&t.full_nodes, HD_MAX_DEPTH * 4));
        // poolTop, free-list count, claim limit
        HD_CUDA(cudaMalloc(&t.pool_top, 16));
        HD_CUDA(cudaMalloc(&t.free_pages, size_t(conf.pool_pages) * 4));
        HD_CUDA(cudaMalloc(&t.error, 16));
        HD_CUDA(cudaMalloc(&t.level_nodes, HD_MAX_DEPTH * 8));
        HD_CUDA(cudaMalloc(&c->d_root, 4));
        HD_CUDA(cudaEventCreate(&c->ev0));
        HD_CUDA(cudaEventCreate(&c->ev1));
        table_reset(c);
        HD_CUDA(cudaStreamSynchronize(c->stream));
    });
    if (st != HD_OK) {
        hd_destroy(c);
        return st;
    }
    *out = c;
    return HD_OK;
}

hd_status hd_destroy(hd_ctx* c)
{
    if (!c)
        return HD_ERR_INVALID;
    cudaStreamSynchronize(c->stream);
    hd::batch_release(c);
    hd::color_release(c);
    cudaFree(c->t.pool);
    cudaFree(c->t.bloom);
    cudaFree(c->t.page_table);
    cudaFree(c->t.bucket_sizes);
    cudaFree(c->t.full_nodes);
    cudaFree(c->t.pool_top);
    cudaFree(c->t.free_pages);
    cudaFree(c->t.error);
    cudaFree(c->t.level_nodes);
    cudaFree(c->d_root);
    cudaFree(c->d_basic);
    if (c->copy_stream)
        cudaStreamDestroy(c->copy_stream);
    for (cudaEvent_t e : {c->ev_traced[0], c->ev_traced[1], c->ev_copied[0], c->ev_copied[1]})
        if (e)
            cudaEventDestroy(e);
    if (c->ev0)
        cudaEventDestroy(c->ev0);
    if (c->ev1)
        cudaEventDestroy(c->ev1);
    if (c->ev_mid)
        cudaEventDestroy(c->ev_mid);
    c->scratch.release();
    delete c;
    return HD_OK;
}

const char* hd_last_error(const hd_ctx* c) { return c ? c->err.c_str() : "null context"; }

hd_status hd_set_stream(hd_ctx* c, void* stream)
{
    if (!c)
        return HD_ERR_INVALID;
    return guarded(c, [&] {
        HD_CUDA(cudaStreamSynchronize(c->stream));
        c->stream = static_cast<cudaStream_t>(stream);
    });
}

hd_status hd_sync(hd_ctx* c)
{
    if (!c)
        return HD_ERR_INVALID;
    return guarded(c, [&] { HD_CUDA(cudaStreamSynchronize(c->stream)); });
}

hd_status hd_load_basic_dag(hd_ctx* c, const uint32_t* h_words, uint64_t n_words)
{
    if (!c || !h_words || n_words < 2)
        return HD_ERR_INVALID;
    return guarded(c, [&] {
        keep_basic(c, h_words, n_words);
        table_reset(c);
        import_basic_dag(c, c->d_basic, n_words);
        c->needs_gc = false;
    });
}

hd_status hd_generate_scene(hd_ctx* c, uint64_t seed) { return hd_generate_scene_ex(c, seed, 0); }

hd_status hd_generate_scene_ex(hd_ctx* c, uint64_t seed, uint32_t flags)
{
    if (!c || (flags & ~uint32_t(HD_SCENE_SHELL)))
        return HD_ERR_INVALID;
    return guarded(c, [&] {
        uint32_t* words;
        uint64_t n;
        generate_scene(c, seed, flags, &words, &n);
        c->scratch.release(); // the generator's buffers are large; start the ingest clean
        table_reset(c);
        import_basic_dag(c, words, n);
        c->scratch.release();
        c->needs_gc = false;
    });
}

hd_status hd_export_basic_dag(hd_ctx* c, uint32_t* h_words, uint64_t capacity, uint64_t* n_words)
{
    if (!c || !n_words)
        return HD_ERR_INVALID;
    if (!c->d_basic)
        return HD_ERR_STATE;
    *n_words = c->n_basic;
    if (!h_words)
        return HD_OK;
    if (capacity < c->n_basic)
        return HD_ERR_INVALID;
    return guarded(c, [&] {
        HD_CUDA(cudaMemcpyAsync(h_words, c->d_basic, c->n_basic * 4, cudaMemcpyDeviceToHost, c->stream));
        HD_CUDA(cudaStreamSynchronize(c->stream));
    });
}

hd_status hd_set_page_reserve(hd_ctx* c, uint32_t pages)
{
    if (!c || pages >= c->cfg.pool_pages)
        return HD_ERR_INVALID;
    return guarded(c, [&] {
        c->page_reserve = pages;
        set_claim_limit(c, false);
    });
}

hd_status hd_set_test_barrier_skip(hd_ctx* c, uint32_t cta_plus_one, uint32_t wait_ms)
{
    if (!c)
        return HD_ERR_INVALID;
    c->test_skip_cta = cta_plus_one;
    c->test_wait_ns = uint64_t(wait_ms) * 1000000ull;
    return HD_OK;
}

hd_status hd_set_fp_mode(hd_ctx* c, uint32_t mode)
{
    if (!c || mode > 1)
        return HD_ERR_INVALID;
    c->fp_mode = mode;
    return HD_OK;
}

static hd_status timed(hd_ctx* c, float* ms, const std::function<void()>& f)
{
    return guarded(c, [&] {
        HD_CUDA(cudaEventRecord(c->ev0, c->stream));
        f();
        HD_CUDA(cudaEventRecord(c->ev1, c->stream));
        if (ms) {
            HD_CUDA(cudaEventSynchronize(c->ev1));
            HD_CUDA(cudaEventElapsedTime(ms, c->ev0, c->ev1));
        }
    });
}

hd_status hd_trace_primary(hd_ctx* c, const hd_camera* cam, uint32_t w, uint32_t h, uint32_t* d_paths, float* ms)
{
    if (!c || !cam || !d_paths || !w || !h)
        return HD_ERR_INVALID;
    return timed(c, ms, [&] { trace_primary(c, *cam, w, h, d_paths); });
}

hd_status hd_trace_shadow(hd_ctx* c, const hd_camera* cam, uint32_t w, uint32_t h, const uint32_t* d_paths,
                          const float light[3], float bias, uint8_t* d_mask, float* ms)
{
    if (!c || !cam || !d_paths || !d_mask || !light || !w || !h)
        return HD_ERR_INVALID;
    return timed(c, ms, [&] { trace_shadow(c, *cam, w, h, d_paths, light, bias, d_mask); });
}

hd_status hd_trace_views(hd_ctx* c, const hd_camera* cams, uint32_t n_views, uint32_t width, uint32_t height,
                         uint32_t* d_paths, const float* light, float bias, uint8_t* d_mask, float* ms)
{
    if (!c || !cams || !n_views || !width || !height || !d_paths || !light || !d_mask)
        return HD_ERR_INVALID;
    return guarded(c, [&] {
        hd_camera* d_cams = c->scratch.get<hd_camera>("views_cams", n_views);
        HD_CUDA(cudaMemcpyAsync(d_cams, cams, sizeof(hd_camera) * n_views, cudaMemcpyHostToDevice, c->stream));
        if (!c->ev_mid)
            HD_CUDA(cudaEventCreate(&c->ev_mid));
        HD_CUDA(cudaEventRecord(c->ev0, c->stream));
        trace_views(c, d_cams, n_views, width, height, d_paths, light, bias, d_mask, nullptr, nullptr, c->ev_mid);
        HD_CUDA(cudaEventRecord(c->ev1, c->stream));
        HD_CUDA(cudaEventSynchronize(c->ev1));
        if (ms) {
            HD_CUDA(cudaEventElapsedTime(ms, c->ev0, c->ev_mid));
            HD_CUDA(cudaEventElapsedTime(ms + 1, c->ev_mid, c->ev1));
        }
    });
}

hd_status hd_trace_views_host(hd_ctx* c, const hd_camera* cams, uint32_t n_views, uint32_t width, uint32_t height,
                              uint32_t* h_paths, const float* light, float bias, uint8_t* h_mask,
                              uint32_t chunk_views, float* ms)
{
    if (!c || !cams || !n_views || !width || !height || !h_paths || !light || !h_mask)
        return HD_ERR_INVALID;
    return guarded(c, [&] {
        const auto t0 = std::chrono::steady_clock::now();
        const uint64_t frame = uint64_t(width) * height;
        // Pinned host memory the device can address (Grace's NVLink-C2C):
        // the primary rays write the paths of most views straight into it;
        // the views view_copied names go to a device buffer that the copy
        // engine moves to host memory during the shadow launch, so the host
        // link carries paths through the whole step (the primary launch
        // alone is shorter than the link needs for every view's paths).
        // The shadow mask is copied at the end.
        cudaPointerAttributes attr{};
        void* direct = nullptr;
        if (cudaPointerGetAttributes(&attr, h_paths) == cudaSuccess && attr.type == cudaMemoryTypeHost &&
            attr.devicePointer)
            direct = attr.devicePointer;
        cudaGetLastError();
        if (direct && !chunk_views) {
            if (frame * n_views >= 0xFFFFFFFFull)
                throw StatusError{HD_ERR_INVALID, "views x width x height must stay below 2^32 pixels"};
            hd_camera* d_cams = c->scratch.get<hd_camera>("views_cams", n_views);
            uint8_t* d_mask = c->scratch.get<uint8_t>("vh_mask_direct", frame * n_views);
            const uint32_t n_copied = copied_views(n_views);
            uint32_t* d_copied = nullptr;
            if (n_copied) {
                d_copied = c->scratch.get<uint32_t>("vh_paths_copied", frame * n_copied * 4);
                if (!c->copy_stream)
                    HD_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
                if (!c->ev_traced[0])
                    HD_CUDA(cudaEventCreateWithFlags(&c->ev_traced[0], cudaEventDisableTiming));
            }
            HD_CUDA(cudaMemcpyAsync(d_cams, cams, sizeof(hd_camera) * n_views, cudaMemcpyHostToDevice, c->stream));
            trace_views(c, d_cams, n_views, width, height, static_cast<uint32_t*>(direct), light, bias, d_mask,
                        c->stream, nullptr, n_copied ? c->ev_traced[0] : nullptr, nullptr, nullptr, d_copied);
            if (n_copied) {
                // after the primary launch, beside the shadow launch
                HD_CUDA(cudaStreamWaitEvent(c->copy_stream, c->ev_traced[0], 0));
                uint64_t slot = 0;
                for (uint32_t v = 0; v < n_views; v++)
                    if (view_copied(v))
                        HD_CUDA(cudaMemcpyAsync(h_paths + uint64_t(v) * frame * 4, d_copied + slot++ * frame * 4,
                                                frame * 16, cudaMemcpyDeviceToHost, c->copy_stream));
            }
            HD_CUDA(cudaMemcpyAsync(h_mask, d_mask, frame * n_views, cudaMemcpyDeviceToHost, c->stream));
            if (n_copied)
                HD_CUDA(cudaStreamSynchronize(c->copy_stream));
            HD_CUDA(cudaStreamSynchronize(c->stream));
            if (ms)
                *ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
            return;
        }
        const uint32_t chunk = std::min(n_views, chunk_views ? chunk_views : std::max(1u, (n_views + 1) / 2));
        if (frame * chunk >= 0xFFFFFFFFull)
            throw StatusError{HD_ERR_INVALID, "views x width x height must stay below 2^32 pixels per chunk"};
        if (!c->copy_stream)
            HD_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
        for (auto* e : {&c->ev_traced[0], &c->ev_traced[1], &c->ev_copied[0], &c->ev_copied[1]})
            if (!*e)
                HD_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
        // two sets of device buffers: chunk k traces into set k % 2 while the
        // copy stream brings chunk k - 1 back
        uint32_t* d_paths[2];
        uint8_t* d_mask[2];
        uint32_t* d_list[2];
        hd_camera* d_cams[2];
        for (int b = 0; b < 2; b++) {
            char nm[32];
            snprintf(nm, sizeof(nm), "vh_paths_%d", b);
            d_paths[b] = c->scratch.get<uint32_t>(nm, frame * chunk * 4);
            snprintf(nm, sizeof(nm), "vh_mask_%d", b);
            d_mask[b] = c->scratch.get<uint8_t>(nm, frame * chunk);
            snprintf(nm, sizeof(nm), "vh_list_%d", b);
            d_list[b] = c->scratch.get<uint32_t>(nm, shadow_list_words(frame * chunk));
            snprintf(nm, sizeof(nm), "vh_cams_%d", b);
            d_cams[b] = c->scratch.get<hd_camera>(nm, chunk);
        }
        uint32_t k = 0;
        for (uint32_t v0 = 0; v0 < n_views; v0 += chunk, k++) {
            const uint32_t nv = std::min(chunk, n_views - v0);
            const int b = int(k & 1);
            if (k >= 2) // the copies out of this buffer set are done
                HD_CUDA(cudaStreamWaitEvent(c->stream, c->ev_copied[b], 0));
            HD_CUDA(cudaMemcpyAsync(d_cams[b], cams + v0, sizeof(hd_camera) * nv, cudaMemcpyHostToDevice, c->stream));
            trace_views(c, d_cams[b], nv, width, height, d_paths[b], light, bias, d_mask[b], c->stream, d_list[b]);
            HD_CUDA(cudaEventRecord(c->ev_traced[b], c->stream));
            HD_CUDA(cudaStreamWaitEvent(c->copy_stream, c->ev_traced[b], 0));
            HD_CUDA(cudaMemcpyAsync(h_paths + uint64_t(v0) * frame * 4, d_paths[b], frame * nv * 16,
                                    cudaMemcpyDeviceToHost, c->copy_stream));
            HD_CUDA(cudaMemcpyAsync(h_mask + uint64_t(v0) * frame, d_mask[b], frame * nv, cudaMemcpyDeviceToHost,
                                    c->copy_stream));
            HD_CUDA(cudaEventRecord(c->ev_copied[b], c->copy_stream));
        }
        HD_CUDA(cudaStreamSynchronize(c->copy_stream));
        HD_CUDA(cudaStreamSynchronize(c->stream));
        if (ms)
            *ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    });
}

hd_status hd_trace_frame(hd_ctx* c, const hd_camera* cam, uint32_t w, uint32_t h, const float light[3], float bias,
                         uint32_t* d_paths, uint8_t* d_mask, float* ms_primary, float* ms_shadow)
{
    // one view of hd_trace_views; ms_primary covers the primary rays with
    // the shadow-ray list they build
    float ms[2] = {0, 0};
    const hd_status s = hd_trace_views(c, cam, 1, w, h, d_paths, light, bias, d_mask, ms);
    if (ms_primary)
        *ms_primary = ms[0];
    if (ms_shadow)
        *ms_shadow = ms[1];
    return s;
}

hd_status hd_trace_counters(hd_ctx* c, const hd_camera* cam, uint32_t w, uint32_t h, const float light[3],
                            float bias, uint32_t* d_paths, uint8_t* d_mask, uint64_t out[6])
{
    if (!c || !cam || !d_paths || !d_mask || !light || !out || !w || !h)
        return HD_ERR_INVALID;
    return guarded(c, [&] {
        unsigned long long* d = c->scratch.get<unsigned long long>("trace_counters", 6);
        HD_CUDA(cudaMemsetAsync(d, 0, 6 * 8, c->stream));
        trace_primary(c, *cam, w, h, d_paths, d);
        trace_shadow(c, *cam, w, h, d_paths, light, bias, d_mask, d + 3);
        HD_CUDA(cudaMemcpyAsync(out, d, 6 * 8, cudaMemcpyDeviceToHost, c->stream));
        HD_CUDA(cudaStreamSynchronize(c->stream));
    });
}

hd_status hd_get_values(hd_ctx* c, const uint32_t* d_xyz, uint64_t n, uint8_t* d_out)
{
    if (!c || (n && (!d_xyz || !d_out)))
        return HD_ERR_INVALID;
    return guarded(c, [&] { get_values(c, d_xyz, n, d_out); });
}

hd_status hd_get_root(hd_ctx* c, uint32_t* root)
{
    if (!c || !root)
        return HD_ERR_INVALID;
    return guarded(c, [&] {
        refresh_root(c);
        *root = c->root;
    });
}

hd_status hd_set_root(hd_ctx* c, uint32_t root)
{
    if (!c)
        return HD_ERR_INVALID;
    return guarded(c, [&] {
        uint32_t entry = 0;
        if ((root >> kPageShift) < c->g.total_vpages) {
            HD_CUDA(cudaMemcpyAsync(&entry, c->t.page_table + (root >> kPageShift), 4, cudaMemcpyDeviceToHost,
                                    c->stream));
            HD_CUDA(cudaStreamSynchronize(c->stream));
        }
        if (!valid_root(c->g, root, entry))
            throw StatusError{HD_ERR_INVALID, "root " + std::to_string(root) + " is not on a mapped page"};
        HD_CUDA(cudaMemcpyAsync(c->d_root, &root, 4, cudaMemcpyHostToDevice, c->stream));
        HD_CUDA(cudaStreamSynchronize(c->stream));
        c->root = root;
    });
}

hd_status hd_get_config(hd_ctx* c, hd_config* cfg)
{
    if (!c || !cfg)
        return HD_ERR_INVALID;
    *cfg = c->cfg;
    return HD_OK;
}

__global__ void k_level_words(Table t, uint64_t* out)
{
    // one block per level
    const uint32_t level = blockIdx.x;
    if (level >= t.g.depth)
        return;
    const uint32_t nb = t.g.buckets(level), first = t.g.level_first_bucket(level);
    unsigned long long sum = 0;
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x)
        sum += t.bucket_sizes[first + b];
    for (int o = 16; o; o >>= 1)
        sum += __shfl_down_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31) == 0)
        atomicAdd(reinterpret_cast<unsigned long long*>(out + level), sum);
}

hd_status hd_get_level_stats(hd_ctx* c, hd_level_stats* out)
{
    if (!c || !out)
        return HD_ERR_INVALID;
    return guarded(c, [&] {
        std::memset(out, 0, sizeof(*out));
        uint64_t* d = c->scratch.get<uint64_t>("stats_words", HD_MAX_DEPTH);
        HD_CUDA(cudaMemsetAsync(d, 0, HD_MAX_DEPTH * 8, c->stream));
        const uint32_t levels = c->g.leaf_level + 1;
        k_level_words<<<levels, 256, 0, c->stream>>>(c->t, d);
        HD_LAUNCH_CHECK();
        HD_CUDA(cudaMemcpyAsync(out->words, d, levels * 8, cudaMemcpyDeviceToHost, c->stream));
        HD_CUDA(cudaMemcpyAsync(out->nodes, c->t.level_nodes, levels * 8, cudaMemcpyDeviceToHost, c->stream));
        uint32_t top[2] = {0, 0};
        HD_CUDA(cudaMemcpyAsync(top, c->t.pool_top, 8, cudaMemcpyDeviceToHost, c->stream));
        HD_CUDA(cudaMemcpyAsync(&c->root, c->d_root, 4, cudaMemcpyDeviceToHost, c->stream));
        HD_CUDA(cudaStreamSynchronize(c->stream));
        out->pages_used = top[0] - 1 - top[1]; // pages a GC released are not in use
        out->root = c->root;
        out->levels = c->cfg.depth;
    });
}

hd_status hd_memory_stats(hd_ctx* c, uint64_t* out)
{
    if (!c || !out)
        return HD_ERR_INVALID;
    out[0] = uint64_t(c->cfg.pool_pages) * HD_PAGE_SIZE * 4 + kPageTableEntries * 4 + c->g.total_buckets * 4 +
             uint64_t(c->cfg.pool_pages) * kBloomWords * 4;
    const ColorTable& ct = c->ct;
    out[1] = ct.cap_nodes * 4 + ct.cap_leaves * sizeof(LeafDesc) + ct.cap_blocks * 8 + ct.cap_macros * 8 +
             ct.cap_weights * 4;
    out[2] = c->scratch.total();
    out[3] = c->gen_scratch_peak;
    return HD_OK;
}

hd_status hd_table_sizes(hd_ctx* c, uint64_t* n_buckets, uint64_t* n_vpages, uint64_t* n_pool_pages_used)
{
    if (!c)
        return HD_ERR_INVALID;
    return guarded(c, [&] {
        if (n_buckets)
            *n_buckets = c->g.total_buckets;
        if (n_vpages)
            *n_vpages = c->g.total_vpages;
        if (n_pool_pages_used)
            *n_pool_pages_used = read_scalar(c->t.pool_top, c->stream) - 1;
    });
}

hd_status hd_export_table(hd_ctx* c, uint32_t* bs, uint32_t* pt, uint32_t* pool, uint64_t pool_cap, uint32_t* full)
{
    if (!c)
        return HD_ERR_INVALID;
    return guarded(c, [&] {
        cudaStream_t st = c->stream;
        if (bs)
            HD_CUDA(cudaMemcpyAsync(bs, c->t.bucket_sizes, c->g.total_buckets * 4, cudaMemcpyDeviceToHost, st));
        if (pt)
            HD_CUDA(cudaMemcpyAsync(pt, c->t.page_table, c->g.total_vpages * 4, cudaMemcpyDeviceToHost, st));
        if (pool) {
            const uint64_t top = read_scalar(c->t.pool_top, st);
            uint64_t words = top * HD_PAGE_SIZE;
            if (words > pool_cap)
                words = pool_cap;
            HD_CUDA(cudaMemcpyAsync(pool, c->t.pool, words * 4, cudaMemcpyDeviceToHost, st));
        }
        if (full)
            HD_CUDA(cudaMemcpyAsync(full, c->t.full_nodes, c->cfg.depth * 4, cudaMemcpyDeviceToHost, st));
        HD_CUDA(cudaStreamSynchronize(st));
    });
}

hd_status hd_import_table(hd_ctx* c, const uint32_t* bs, const uint32_t* pt, const uint32_t* pool, uint64_t pool_words,
                          const uint32_t* full, uint32_t root)
{
    if (!c || !bs || !pt || !pool || !full || pool_words % HD_PAGE_SIZE ||
        pool_words > uint64_t(c->cfg.pool_pages) * HD_PAGE_SIZE)
        return HD_ERR_INVALID;
    return guarded(c, [&] {
        cudaStream_t st = c->stream;
        check_table(c->g, pt, bs, uint32_t(pool_words / HD_PAGE_SIZE), root, "the imported table");
        table_reset(c);
        HD_CUDA(cudaMemcpyAsync(c->t.bucket_sizes, bs, c->g.total_buckets * 4, cudaMemcpyHostToDevice, st));
        HD_CUDA(cudaMemcpyAsync(c->t.page_table, pt, c->g.total_vpages * 4, cudaMemcpyHostToDevice, st));
        HD_CUDA(cudaMemcpyAsync(c->t.pool, pool, pool_words * 4, cudaMemcpyHostToDevice, st));
        HD_CUDA(cudaMemcpyAsync(c->t.full_nodes, full, c->cfg.depth * 4, cudaMemcpyHostToDevice, st));
        const uint32_t top[2] = {uint32_t(pool_words / HD_PAGE_SIZE), 0};
        HD_CUDA(cudaMemcpyAsync(c->t.pool_top, top, 8, cudaMemcpyHostToDevice, st));
        HD_CUDA(cudaMemcpyAsync(c->d_root, &root, 4, cudaMemcpyHostToDevice, st));
        bloom_rebuild(c);
        HD_CUDA(cudaStreamSynchronize(st));
        c->root = root;
        c->needs_gc = false;
    });
}

hd_status hd_device_table(hd_ctx* c, uint32_t** pool, uint32_t** pt, uint32_t** bs)
{
    if (!c)
        return HD_ERR_INVALID;
    if (pool)
        *pool = c->t.pool;
    if (pt)
        *pt = c->t.page_table;
    if (bs)
        *bs = c->t.bucket_sizes;
    return HD_OK;
}

} // extern "C"
