// The context behind the opaque hd_ctx handle, shared by the .cu files.
#pragma once

#include <deque>
#include <string>
#include <vector>

#include "hd_color.cuh"
#include "hd_common.cuh"
#include "hd_util.cuh"

namespace hd {
struct BatchGraph; // hd_edit_batch.cu
// One undo step (HashDAGUndoRedo::Frame, hash_dag.h:28-45): the root before
// the edit and the colour leaves it replaced.
struct UndoFrame {
    uint32_t root = 0;
    std::vector<uint32_t> leaf;
    std::vector<LeafDesc> prev, next;
};
}

struct hd_ctx {
    hd_config cfg{};
    hd::Geom g{};
    hd::Table t{};           // device pointers of the table
    cudaStream_t stream = nullptr;
    uint32_t* d_root = nullptr;        // firstNodeIndex on the device
    uint32_t root = 0;                 // host copy, refreshed after each call
    uint32_t fp_mode = 0; // every operation rounded on its own: the reference kernel's arithmetic
    std::string err;
    std::string err_detail;           // detail words of the last device error
    hd::Scratch scratch;               // grow-only working buffers
    // BasicDAG of the last generated scene (device), kept for export
    uint32_t* d_basic = nullptr;
    uint64_t n_basic = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev_mid = nullptr;
    // hd_trace_views_host: the stream that copies results to the host and
    // the events that pipeline it with the traversal
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_traced[2] = {nullptr, nullptr}, ev_copied[2] = {nullptr, nullptr};
    // bucket list heads of the edit path stay all-empty between calls
    bool edit_head_ready = false;
    uint32_t* edit_head_ptr = nullptr;
    // batched edits: tuning, the captured graph, edits that took the
    // one-edit path because a level outgrew its bound
    hd_batch_tuning tuning{4, 4, 304, HD_BATCH_PERSISTENT};
    hd::BatchGraph* batch = nullptr;
    uint64_t batch_fallbacks = 0;
    uint32_t batch_applied = 0; // edits of the last batch call that were applied (also when it failed)
    // colours: the table, host mirror of its counters
    bool colors = false;
    uint64_t color_seed = 0;
    hd::ColorTable ct{};
    uint64_t ctop[5] = {0, 0, 0, 0, 0};
    // undo / redo history
    std::deque<hd::UndoFrame> undo, redo;
    size_t undo_capacity = 200;
    // events the colour commit of the next edit waits for (renders in flight
    // that still read the colour leaves the edit replaces)
    std::vector<cudaEvent_t> color_fences;
    size_t gen_scratch_peak = 0; // bytes of scratch the last scene generation held at most
    // a table loaded from a hash-DAG file without bucket sizes: traversal
    // works, edits wait for a GC to rebuild the buckets
    bool needs_gc = false;
    // pages page claims outside a GC leave untouched (hd_set_page_reserve):
    // the GC's rebuild draws on them
    uint32_t page_reserve = 0;
    // hd_set_test_barrier_skip: for the next persistent batch launch only
    uint32_t test_skip_cta = 0;
    unsigned long long test_wait_ns = 0;
};

namespace hd {

// Runs f, turning the errors it throws into a status and the context's
// message.
template <typename F>
hd_status guarded(hd_ctx* c, F&& f)
{
    try {
        f();
        return HD_OK;
    } catch (const StatusError& e) {
        if (c)
            c->err = e.msg;
        return e.status;
    } catch (const CudaError& e) {
        if (c)
            c->err = std::string("CUDA error ") + cudaGetErrorString(e.code) + " in " + e.where;
        return e.code == cudaErrorMemoryAllocation ? HD_ERR_OOM : HD_ERR_CUDA;
    } catch (const std::bad_alloc&) {
        if (c)
            c->err = "host allocation failed";
        return HD_ERR_OOM;
    }
}

// hd_table.cu
void table_reset(hd_ctx* c);
void add_full_nodes(hd_ctx* c, uint32_t first_level, uint32_t last_level);
void import_basic_dag(hd_ctx* c, const uint32_t* d_words, uint64_t n_words);
uint32_t check_error(hd_ctx* c); // reads and clears the device error word
// Appends items (9-word contents) bucket by bucket in item order; the bucket
// lists must have been linked (link_item) for `level`.
void append_items(hd_ctx* c, uint32_t level, const uint32_t* content, uint64_t n_items, uint32_t* head,
                  const uint32_t* next, const uint32_t* touched, const uint32_t* n_touched, uint32_t* out_addr);

// hd_scene.cu
void generate_scene(hd_ctx* c, uint64_t seed, uint32_t flags, uint32_t** d_words, uint64_t* n_words);

// hd_table.cu: Bloom filters of imported tables and of GC-rebuilt levels
void bloom_rebuild(hd_ctx* c);

// hd_table.cu: checks of a table written from outside (host arrays): every
// mapped page lies below `top`, no bucket holds more than its capacity (bs
// may be null) and the root is a node of a mapped page.  Throws
// HD_ERR_INVALID naming `what`.
void check_table(const Geom& g, const uint32_t* pt, const uint32_t* bs, uint32_t top, uint32_t root,
                 const std::string& what);
// The root is an address of a mapped page (pt_entry: its page-table entry)
bool valid_root(const Geom& g, uint32_t root, uint32_t pt_entry);
void bloom_clear_level(hd_ctx* c, uint32_t level);

// hd_io.cu: keeps a copy of the BasicDAG words (host or device pointer)
void keep_basic(hd_ctx* c, const uint32_t* words, uint64_t n);

// hd_edit.cu / hd_edit_batch.cu
void edit_one(hd_ctx* c, const hd_edit& e, hd_edit_stats* stats);
void edit_batch(hd_ctx* c, const hd_edit* edits, uint32_t n, hd_edit_stats* per_edit, hd_edit_stats* total);
void batch_release(hd_ctx* c);

// hd_color.cu
struct Editor;
struct Level;
void color_release(hd_ctx* c);
void colors_from_scene(hd_ctx* c, uint64_t color_seed);
void colors_from_main_leaf(hd_ctx* c, uint32_t top_levels, const std::vector<uint64_t>& enclosed,
                           const std::vector<uint32_t>& weights, const std::vector<uint64_t>& blocks,
                           const std::vector<uint64_t>& macros);
void color_reserve(hd_ctx* c, const uint64_t add[5]);
void get_colors(hd_ctx* c, const uint32_t* d_xyz, uint64_t n, hd_color* d_out);
void trace_colors(hd_ctx* c, const uint32_t* d_paths, uint32_t w, uint32_t h, uint32_t* d_rgba,
                  cudaStream_t stream = nullptr, const uint32_t* d_root = nullptr,
                  const hd_trace_colors_params* params = nullptr);
void copy_source(hd_ctx* c, Editor& ed);
void tool_buffers(hd_ctx* c, Editor& ed); // hd_tools.cu
void color_spawn(hd_ctx* c, uint32_t level, uint32_t n, const Level& lv, const Level& next);
void edit_colors(hd_ctx* c, const Editor& ed, std::vector<Level>& lv, const std::vector<uint32_t>& count,
                 uint32_t deepest, UndoFrame& frame);
bool undo_step(hd_ctx* c, bool redo);
void push_undo(hd_ctx* c, UndoFrame&& f);

// hd_trace.cu
// stream / d_root: nullptr = the context's stream and root
void trace_primary(hd_ctx* c, const hd_camera& cam, uint32_t w, uint32_t h, uint32_t* d_paths,
                   unsigned long long* d_counters = nullptr, cudaStream_t stream = nullptr,
                   const uint32_t* d_root = nullptr);
// d_list: w * h + 1 words for the list of hit pixels (nullptr = context
// scratch, not for concurrent calls)
// 32-bit words of a shadow-ray list buffer for px pixels: 16 bytes per ray
// and a 4-word head (ray count, two work counters).
inline uint64_t shadow_list_words(uint64_t px) { return 4 * px + 4; }
// Doubles of one view's camera tables (trace_views): a column entry per
// column and a row entry per row, 3 doubles each.
__host__ __device__ inline uint64_t camera_table_words(uint32_t w, uint32_t h) { return 3ull * (uint64_t(w) + h); }
void trace_shadow(hd_ctx* c, const hd_camera& cam, uint32_t w, uint32_t h, const uint32_t* d_paths,
                  const float light[3], float bias, uint8_t* d_mask, unsigned long long* d_counters = nullptr,
                  cudaStream_t stream = nullptr, const uint32_t* d_root = nullptr, uint32_t* d_list = nullptr);
void get_values(hd_ctx* c, const uint32_t* d_xyz, uint64_t n, uint8_t* d_out);
// The page claims' limit on poolTop (the table's third pool_top word):
// pool_pages less the reserve, or (gc = true) the whole pool.
void set_claim_limit(hd_ctx* c, bool gc);
// mid (optional): recorded between the primary and the shadow launches;
// d_tables (optional): camera_table_words(w, h) * n_views doubles of
// scratch for the per-view camera tables (default: the context's);
// d_paths_copied (optional): the paths of the views view_copied names go
// there, packed in view order, instead of into d_paths.
void trace_views(hd_ctx* c, const hd_camera* d_cams, uint32_t n_views, uint32_t w, uint32_t h, uint32_t* d_paths,
                 const float light[3], float bias, uint8_t* d_mask, cudaStream_t stream = nullptr,
                 uint32_t* d_list = nullptr, cudaEvent_t mid = nullptr, const uint32_t* d_root = nullptr,
                 double* d_tables = nullptr, uint32_t* d_paths_copied = nullptr);
// Of every 8 views, trace_views sets aside (d_paths_copied) those from the
// kCopiedFrom-th on (counting from 0).
constexpr uint32_t kCopiedFrom = 5;
inline bool view_copied(uint32_t v) { return (v & 7) >= kCopiedFrom; }
// Views of n_views that trace_views sets aside with d_paths_copied.
inline uint32_t copied_views(uint32_t n_views)
{
    return (n_views >> 3) * (8 - kCopiedFrom) + ((n_views & 7) > kCopiedFrom ? (n_views & 7) - kCopiedFrom : 0);
}

} // namespace hd
