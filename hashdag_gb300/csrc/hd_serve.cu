// Serving loop: a stream of edit and render requests against one resident
// DAG (table, colours, undo history on the device).
//
// The reference's interactive engine applies one edit per frame and renders
// in between (Engine::tick, engine.cpp:575-720).  Here requests arrive on
// their own clock and two policies run the same trace:
//  * sequential: one request at a time in arrival order, each finished
//    before the next starts (the plain GPU path);
//  * continuous: renders are admitted into up to max_renders slots, each on
//    its own stream, reading the root of the moment they are admitted;
//    edits run in arrival order on the context stream while renders are in
//    flight (a render's colour pass completes before a later edit replaces
//    colour leaves).  Without colours and with batch_edits, the edits queued
//    at that moment run as one batch: one persistent launch (hd_edit_batch)
//    while the renders in flight go on on their own streams.
// Both policies gate edits on free physical pages (never-claimed pages plus
// pages on the free list): below gc_free_fraction of the pool, the renders
// drain and a GC runs that keeps the undo history and, with release_pages,
// gives emptied pages back.  An edit that still finds the pool full is
// retried once after a GC, then refused (status HD_ERR_POOL_FULL; the
// table's root is unchanged).
// Every render produces paths, a shadow mask and (with colours) RGBA, and a
// checksum of them that does not depend on node addresses, so a render can
// be compared with the same render made alone on the same state.
#include <algorithm>
#include <chrono>
#include <deque>
#include <thread>
#include <vector>

#include "hd_color.cuh"
#include "hd_ctx.h"

namespace hd {

void edit_one(hd_ctx* c, const hd_edit& e, hd_edit_stats* stats);
void edit_batch(hd_ctx* c, const hd_edit* edits, uint32_t n, hd_edit_stats* per_edit, hd_edit_stats* total);

// order-independent checksum of a rendered frame: sum over pixels of a mix of
// (pixel, path, shadow, colour)
__global__ void k_frame_checksum(const uint4* __restrict__ paths, const uint8_t* __restrict__ mask,
                                 const uint32_t* __restrict__ rgba, uint64_t n, unsigned long long* out)
{
    unsigned long long acc = 0;
    HD_GRID_STRIDE(i, n)
    {
        const uint4 p = paths[i];
        uint64_t h = mix64(i ^ (uint64_t(p.x) << 21) ^ (uint64_t(p.y) << 42));
        h = mix64(h ^ p.z ^ (uint64_t(mask[i]) << 32) ^ (rgba ? uint64_t(rgba[i]) << 24 : 0));
        acc += h;
    }
    for (int o = 16; o; o >>= 1)
        acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0)
        atomicAdd(out, acc);
}

namespace {

struct Slot {
    cudaStream_t stream = nullptr;
    uint32_t* paths = nullptr;
    uint8_t* mask = nullptr;
    uint32_t* rgba = nullptr;
    uint32_t* root = nullptr;
    uint32_t* list = nullptr; // the shadow-ray list
    hd_camera* cam = nullptr; // the frame's camera on the device
    double* tables = nullptr; // its camera tables
    unsigned long long* sum = nullptr;
    unsigned long long* h_sum = nullptr; // pinned
    cudaEvent_t colors_done = nullptr, done = nullptr;
    int64_t req = -1;
    uint64_t pixels = 0;
};

struct Clock {
    std::chrono::steady_clock::time_point t0;
    cudaEvent_t ev0 = nullptr;
    double now() const { return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count(); }
    double at(cudaEvent_t e) const
    {
        float ms = 0;
        HD_CUDA(cudaEventElapsedTime(&ms, ev0, e));
        return ms;
    }
};

// Physical pages an edit can still claim: never-claimed pages of the pool
// plus the pages a releasing GC put on the free list.
uint64_t free_pages(hd_ctx* c)
{
    uint32_t top[2];
    HD_CUDA(cudaMemcpyAsync(top, c->t.pool_top, 8, cudaMemcpyDeviceToHost, c->stream));
    HD_CUDA(cudaStreamSynchronize(c->stream));
    return uint64_t(c->cfg.pool_pages) - top[0] + top[1];
}

} // namespace

void serve(hd_ctx* c, const hd_request* reqs, uint32_t n, const hd_serve_config& cfg, hd_request_result* res,
           hd_serve_stats* stats)
{
    cudaStream_t st = c->stream;
    const uint32_t R = cfg.continuous ? (cfg.max_renders ? cfg.max_renders : 1) : 1;
    uint64_t max_pixels = 1, max_table = 1;
    for (uint32_t i = 0; i < n; i++)
        if (reqs[i].kind == HD_REQ_RENDER) {
            max_pixels = std::max<uint64_t>(max_pixels, uint64_t(reqs[i].width) * reqs[i].height);
            max_table = std::max<uint64_t>(max_table, camera_table_words(reqs[i].width, reqs[i].height));
        }
    std::vector<Slot> slots(R);
    for (uint32_t k = 0; k < R; k++) {
        Slot& s = slots[k];
        char nm[32];
        if (cfg.continuous)
            HD_CUDA(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking));
        else
            s.stream = st;
        snprintf(nm, sizeof(nm), "serve_paths_%u", k);
        s.paths = c->scratch.get<uint32_t>(nm, max_pixels * 4);
        snprintf(nm, sizeof(nm), "serve_mask_%u", k);
        s.mask = c->scratch.get<uint8_t>(nm, max_pixels);
        snprintf(nm, sizeof(nm), "serve_rgba_%u", k);
        s.rgba = c->scratch.get<uint32_t>(nm, max_pixels);
        snprintf(nm, sizeof(nm), "serve_root_%u", k);
        s.root = c->scratch.get<uint32_t>(nm, 1);
        snprintf(nm, sizeof(nm), "serve_list_%u", k);
        s.list = c->scratch.get<uint32_t>(nm, shadow_list_words(max_pixels));
        snprintf(nm, sizeof(nm), "serve_cam_%u", k);
        s.cam = c->scratch.get<hd_camera>(nm, 1);
        snprintf(nm, sizeof(nm), "serve_tables_%u", k);
        s.tables = c->scratch.get<double>(nm, max_table);
        snprintf(nm, sizeof(nm), "serve_sum_%u", k);
        s.sum = c->scratch.get<unsigned long long>(nm, 1);
        HD_CUDA(cudaMallocHost(&s.h_sum, 8));
        HD_CUDA(cudaEventCreateWithFlags(&s.colors_done, cudaEventDisableTiming));
        HD_CUDA(cudaEventCreate(&s.done));
    }
    const uint32_t saved_reserve = c->page_reserve;
    auto cleanup = [&] {
        for (Slot& s : slots) {
            if (s.stream && s.stream != st) {
                cudaStreamSynchronize(s.stream);
                cudaStreamDestroy(s.stream);
            }
            if (s.h_sum)
                cudaFreeHost(s.h_sum);
            if (s.colors_done)
                cudaEventDestroy(s.colors_done);
            if (s.done)
                cudaEventDestroy(s.done);
        }
        c->color_fences.clear();
        if (c->page_reserve != saved_reserve) {
            c->page_reserve = saved_reserve;
            try {
                set_claim_limit(c, false);
            } catch (...) {
            }
        }
    };
    try {
        // with GCs in the loop, pages kept back from edits for the GC's
        // rebuild (an edit that fills the pool would otherwise leave the GC
        // none)
        if (cfg.gc_free_fraction > 0 && c->page_reserve < c->cfg.pool_pages / 64) {
            c->page_reserve = c->cfg.pool_pages / 64;
            set_claim_limit(c, false);
        }
        Clock clk;
        HD_CUDA(cudaEventCreate(&clk.ev0));
        HD_CUDA(cudaStreamSynchronize(st));
        HD_CUDA(cudaEventRecord(clk.ev0, st));
        HD_CUDA(cudaEventSynchronize(clk.ev0));
        clk.t0 = std::chrono::steady_clock::now();
        uint32_t edits_done = 0, gcs = 0, completed = 0, refused = 0;
        uint64_t free_after_gc = ~0ull; // free pages right after the last GC
        uint64_t voxels = 0;
        std::deque<uint32_t> edits, renders;
        uint32_t next = 0;
        cudaEvent_t edit_ev;
        HD_CUDA(cudaEventCreate(&edit_ev));

        auto launch_render = [&](Slot& s, uint32_t i) {
            const hd_request& r = reqs[i];
            res[i].start_ms = clk.now();
            res[i].root = c->root;
            res[i].edits_before = edits_done;
            HD_CUDA(cudaMemcpyAsync(s.root, &c->root, 4, cudaMemcpyHostToDevice, s.stream));
            HD_CUDA(cudaMemcpyAsync(s.cam, &r.camera, sizeof(hd_camera), cudaMemcpyHostToDevice, s.stream));
            // the frame as a one-view hd_trace_views: persistent primary
            // warps building the shadow-ray list, then the shadow walks
            trace_views(c, s.cam, 1, r.width, r.height, s.paths, cfg.light, cfg.shadow_bias, s.mask, s.stream, s.list,
                        nullptr, s.root, s.tables);
            if (c->colors)
                trace_colors(c, s.paths, r.width, r.height, s.rgba, s.stream, s.root);
            HD_CUDA(cudaEventRecord(s.colors_done, s.stream));
            const uint64_t px = uint64_t(r.width) * r.height;
            HD_CUDA(cudaMemsetAsync(s.sum, 0, 8, s.stream));
            k_frame_checksum<<<grid_for(px, 256, 152 * 8), 256, 0, s.stream>>>(
                reinterpret_cast<const uint4*>(s.paths), s.mask, c->colors ? s.rgba : nullptr, px, s.sum);
            HD_LAUNCH_CHECK();
            HD_CUDA(cudaMemcpyAsync(s.h_sum, s.sum, 8, cudaMemcpyDeviceToHost, s.stream));
            HD_CUDA(cudaEventRecord(s.done, s.stream));
            s.req = i;
            s.pixels = px;
        };
        auto finish_render = [&](Slot& s) {
            const uint32_t i = uint32_t(s.req);
            res[i].end_ms = clk.at(s.done);
            res[i].checksum = *s.h_sum;
            res[i].status = HD_OK;
            s.req = -1;
            completed++;
        };
        auto drain = [&] {
            for (Slot& s : slots)
                if (s.req >= 0) {
                    HD_CUDA(cudaEventSynchronize(s.done));
                    finish_render(s);
                }
        };
        // a GC; false when it refused to start (its rebuild would not fit the
        // free pages; the table is unchanged)
        auto run_gc = [&] {
            drain();
            uint32_t dummy = 0;
            const uint32_t flags = HD_GC_KEEP_HISTORY | (cfg.release_pages ? HD_GC_RELEASE_PAGES : 0u);
            const hd_status g = hd_gc_ex(c, &dummy, 0, flags);
            free_after_gc = free_pages(c);
            if (g == HD_ERR_POOL_FULL || g == HD_ERR_BUCKET_FULL)
                return false;
            if (g != HD_OK)
                throw StatusError{g, "GC inside the serving loop failed: " + c->err};
            gcs++;
            return true;
        };
        // admission: free pages above the threshold, or a GC first (again
        // only once something was claimed since the last one)
        auto admit = [&] {
            if (cfg.gc_free_fraction <= 0)
                return;
            const uint64_t f = free_pages(c);
            if (double(f) < cfg.gc_free_fraction * double(c->cfg.pool_pages) && f < free_after_gc)
                run_gc();
        };
        auto fence_renders = [&] {
            c->color_fences.clear();
            for (Slot& s : slots)
                if (s.req >= 0)
                    c->color_fences.push_back(s.colors_done);
        };
        auto commit = [&](uint32_t i, double end_ms, uint64_t vox) {
            res[i].end_ms = end_ms;
            res[i].root = c->root;
            res[i].num_voxels = vox;
            res[i].checksum = vox;
            res[i].edits_before = edits_done;
            res[i].status = HD_OK;
            voxels += vox;
            edits_done++;
            completed++;
        };
        auto run_edit = [&](uint32_t i) {
            admit();
            res[i].start_ms = clk.now();
            hd_edit_stats es{};
            for (int attempt = 0;; attempt++) {
                fence_renders();
                try {
                    edit_one(c, reqs[i].edit, &es);
                    break;
                } catch (const StatusError& e) {
                    c->color_fences.clear();
                    if (e.status != HD_ERR_POOL_FULL)
                        throw;
                    if (attempt == 1 || cfg.gc_free_fraction <= 0 || !run_gc()) {
                        // refused: the pool stays full; the root is unchanged
                        res[i].end_ms = clk.now();
                        res[i].root = c->root;
                        res[i].status = HD_ERR_POOL_FULL;
                        res[i].edits_before = edits_done;
                        refused++;
                        completed++;
                        return;
                    }
                }
            }
            HD_CUDA(cudaEventRecord(edit_ev, st));
            HD_CUDA(cudaEventSynchronize(edit_ev));
            c->color_fences.clear();
            commit(i, clk.at(edit_ev), es.num_voxels);
        };
        // the queued edits as one batch (no colours): one persistent launch
        auto run_batch = [&](std::deque<uint32_t>& q) {
            admit();
            std::vector<uint32_t> idx(q.begin(), q.end());
            q.clear();
            std::vector<hd_edit> eds(idx.size());
            std::vector<hd_edit_stats> per(idx.size());
            for (size_t k = 0; k < idx.size(); k++) {
                eds[k] = reqs[idx[k]].edit;
                res[idx[k]].start_ms = clk.now();
            }
            const hd_batch_tuning saved = c->tuning;
            c->tuning.mode = HD_BATCH_PERSISTENT;
            HD_CUDA(cudaEventRecord(edit_ev, st));
            uint32_t applied = uint32_t(idx.size());
            bool full = false;
            try {
                edit_batch(c, eds.data(), uint32_t(idx.size()), per.data(), nullptr);
            } catch (const StatusError& e) {
                c->tuning = saved;
                if (e.status != HD_ERR_POOL_FULL)
                    throw;
                applied = c->batch_applied;
                full = true;
            }
            c->tuning = saved;
            const double base = clk.at(edit_ev);
            for (uint32_t k = 0; k < applied; k++)
                commit(idx[k], base + per[k].host_ms, per[k].num_voxels);
            if (full) // the rest one by one, with a GC first
                for (size_t k = applied; k < idx.size(); k++)
                    run_edit(idx[k]);
        };

        while (completed < n) {
            const double now = clk.now();
            while (next < n && (!cfg.realtime || reqs[next].arrival_ms <= now)) {
                (reqs[next].kind == HD_REQ_RENDER ? renders : edits).push_back(next);
                next++;
            }
            if (!cfg.continuous) {
                // one request at a time, in arrival order
                if (!edits.empty() || !renders.empty()) {
                    const bool edit_first =
                        renders.empty() || (!edits.empty() && edits.front() < renders.front());
                    if (edit_first) {
                        const uint32_t i = edits.front();
                        edits.pop_front();
                        run_edit(i);
                    } else {
                        const uint32_t i = renders.front();
                        renders.pop_front();
                        launch_render(slots[0], i);
                        HD_CUDA(cudaEventSynchronize(slots[0].done));
                        finish_render(slots[0]);
                    }
                    continue;
                }
            } else {
                bool progress = false;
                for (Slot& s : slots)
                    if (s.req >= 0 && cudaEventQuery(s.done) == cudaSuccess) {
                        finish_render(s);
                        progress = true;
                    }
                for (Slot& s : slots)
                    if (s.req < 0 && !renders.empty()) {
                        launch_render(s, renders.front());
                        renders.pop_front();
                        progress = true;
                    }
                if (!edits.empty()) {
                    if (cfg.batch_edits && !c->colors && edits.size() > 1) {
                        run_batch(edits);
                    } else {
                        const uint32_t i = edits.front();
                        edits.pop_front();
                        run_edit(i);
                    }
                    progress = true;
                }
                if (progress)
                    continue;
            }
            // idle: wait for the next arrival or a render
            std::this_thread::sleep_for(std::chrono::microseconds(50));
        }
        drain();
        HD_CUDA(cudaStreamSynchronize(st));
        const double wall = clk.now();
        std::vector<double> el, fr;
        for (uint32_t i = 0; i < n; i++)
            if (res[i].status == HD_OK)
                (reqs[i].kind == HD_REQ_RENDER ? fr : el).push_back(res[i].end_ms - reqs[i].arrival_ms);
        auto pct = [](std::vector<double> v, double q) {
            if (v.empty())
                return 0.0;
            std::sort(v.begin(), v.end());
            const double pos = q / 100.0 * double(v.size() - 1);
            const size_t lo = size_t(pos);
            const size_t hi = std::min(lo + 1, v.size() - 1);
            return v[lo] + (v[hi] - v[lo]) * (pos - double(lo));
        };
        if (stats) {
            *stats = hd_serve_stats{};
            stats->wall_ms = wall;
            stats->edits = uint32_t(el.size());
            stats->renders = uint32_t(fr.size());
            stats->gcs = gcs;
            stats->refused = refused;
            stats->edit_p50_ms = pct(el, 50);
            stats->edit_p99_ms = pct(el, 99);
            stats->frame_p50_ms = pct(fr, 50);
            stats->frame_p99_ms = pct(fr, 99);
            stats->voxels_per_s = double(voxels) / (wall * 1e-3);
            stats->num_voxels = voxels;
        }
        cudaEventDestroy(edit_ev);
        cudaEventDestroy(clk.ev0);
    } catch (...) {
        cleanup();
        throw;
    }
    cleanup();
}

} // namespace hd

extern "C" hd_status hd_serve(hd_ctx* c, const hd_request* reqs, uint32_t n, const hd_serve_config* cfg,
                              hd_request_result* results, hd_serve_stats* stats)
{
    if (!c || !cfg || (n && (!reqs || !results)))
        return HD_ERR_INVALID;
    for (uint32_t i = 0; i < n; i++) {
        if (reqs[i].kind > HD_REQ_RENDER || (i && reqs[i].arrival_ms < reqs[i - 1].arrival_ms))
            return HD_ERR_INVALID;
        if (reqs[i].kind == HD_REQ_RENDER && (!reqs[i].width || !reqs[i].height))
            return HD_ERR_INVALID;
        if (reqs[i].kind == HD_REQ_EDIT && (reqs[i].edit.tool > HD_TOOL_FILL || !(reqs[i].edit.radius >= 0.0f)))
            return HD_ERR_INVALID;
    }
    try {
        hd::serve(c, reqs, n, *cfg, results, stats);
        return HD_OK;
    } catch (const hd::StatusError& e) {
        c->err = e.msg;
        return e.status;
    } catch (const hd::CudaError& e) {
        c->err = std::string("CUDA error ") + cudaGetErrorString(e.code) + " in " + e.where;
        return HD_ERR_CUDA;
    }
}
