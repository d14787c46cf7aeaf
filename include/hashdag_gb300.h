/*
 * hashdag_gb300 — C ABI of the GB300-native hashed sparse voxel DAG hot path.
 *
 * One opaque context (hd_ctx) owns a device-resident HashDAG: the paged
 * per-level hash table (physical page pool, virtual page table, bucket sizes,
 * full-node indices) plus the root index.  Every call runs sm_103a kernels on
 * the context's CUDA stream; there is no CPU fallback.  All entry points
 * return an hd_status and never abort; hd_last_error() gives the message.
 *
 * Each entry point names the reference interface it replaces
 * (Phyronnaz/HashDAG, file:line).  The table format is the reference's
 * (typedefs.h:201-239, hash_dag_globals.h:7-30, hash_table.h:19-77): 512-word
 * pages, virtual address = (level, bucket, position), interior nodes
 * [header, child pointers...] with header = mask | count << 8, leaves = two
 * words {low, high} holding a 4x4x4 voxel block.
 *
 * Pointers named d_* are device pointers owned by the caller and borrowed for
 * the duration of the call; h_* are host pointers.
 */
#ifndef HASHDAG_GB300_H
#define HASHDAG_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HD_ABI_VERSION 8u
#define HD_PAGE_SIZE 512u
#define HD_MAX_DEPTH 20u
/* Sentinel of the edit recursion (hash_dag_edits.h:17). */
#define HD_INVALID_NODE 0xDFFFFFFu

typedef struct hd_ctx hd_ctx;

typedef enum hd_status {
    HD_OK = 0,
    HD_ERR_INVALID = 1,     /* bad argument or configuration            */
    HD_ERR_CUDA = 2,        /* CUDA runtime error                       */
    HD_ERR_POOL_FULL = 3,   /* physical page pool exhausted             */
    HD_ERR_BUCKET_FULL = 4, /* a bucket ran past its virtual range      */
    HD_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up       */
    HD_ERR_OOM = 6,         /* device allocation failed                 */
    HD_ERR_STATE = 7,       /* call not valid in the context's state    */
    HD_ERR_IO = 8           /* a file could not be read or written      */
} hd_status;

/* Table geometry.  The defaults are the reference's compile-time macros
 * (typedefs.h:152-239): 9 top levels with 2^10 buckets of 1024 words, low
 * levels with 2^16 buckets of 4096 words.  color_tree_levels is
 * C_colorTreeLevels (hash_dag_globals.h:7): levels below it keep mask-only
 * headers when edited, levels at or above it carry voxel counts. */
typedef struct hd_config {
    uint32_t depth;             /* SCENE_DEPTH: leaves sit at depth - 2     */
    uint32_t color_tree_levels; /* C_colorTreeLevels                        */
    uint32_t top_levels;        /* BUCKETS_NUM_TOP_LEVELS                   */
    uint32_t top_bucket_bits;   /* BUCKETS_BITS_FOR_TOP_LEVELS              */
    uint32_t low_bucket_bits;   /* BUCKETS_BITS_FOR_LOW_LEVELS              */
    uint32_t top_bucket_size;   /* BUCKETS_SIZE_FOR_TOP_LEVELS (words)      */
    uint32_t low_bucket_size;   /* BUCKETS_SIZE_FOR_LOW_LEVELS (words)      */
    uint32_t pool_pages;        /* physical pages (HashTable::create arg)   */
} hd_config;

/* Camera in voxel space: Tracer::TracePathsParams (tracer.h:81-91) as built
 * by get_trace_params (dag_tracer.cu:71-113).  Pixel (x, y) looks along
 * normalize(ray_min + x * ray_ddx + y * ray_ddy - position). */
typedef struct hd_camera {
    double position[3];
    double ray_min[3];
    double ray_ddx[3];
    double ray_ddy[3];
} hd_camera;

/* Edit tools (hash_dag_editors.h): sphere carve/fill (SphereEditor<bool>,
 * :272-313), box carve/fill (BoxEditor<bool>, :223-270). */
/* The editors of hash_dag_editors.h: SphereEditor<false/true> (:272-313),
 * BoxEditor<false/true> (:223-270), SpherePaintEditor (:315-330) and the
 * copy tool (CopyEditorWithDecompression, :437-609, the reference's
 * CopyEditor with its default build switches). */
typedef enum hd_tool {
    HD_TOOL_SPHERE_REMOVE = 0,
    HD_TOOL_SPHERE_ADD = 1,
    HD_TOOL_BOX_REMOVE = 2,
    HD_TOOL_BOX_ADD = 3,
    HD_TOOL_SPHERE_PAINT = 4,
    HD_TOOL_COPY = 5,
    HD_TOOL_NOISE_REMOVE = 6, /* SphereNoiseEditor(isAdding = false), :712-760 */
    HD_TOOL_NOISE_ADD = 7,    /* SphereNoiseEditor(isAdding = true)           */
    HD_TOOL_FILL = 8          /* FillEditorColors (flood fill), :624-710      */
} hd_tool;

typedef struct hd_edit {
    uint32_t tool;      /* hd_tool */
    float center[3];    /* sphere centre / box centre; copy: centre of the source region */
    float radius;       /* sphere radius, or box half extent */
    uint32_t rgb;       /* paint: target colour r | g << 8 | b << 16 (the reference paints blue, 0xFF0000) */
    float source[3];    /* copy: the region moves by dest - source (CopyEditor's source / dest) */
    float dest[3];
} hd_edit;

/* CompressedColor (variable_weight_size_colors.h:86-155): 32 colour bits
 * (rgb101210 when bits_per_weight == 0, else two rgb565 end points) and a
 * weight of bits_per_weight bits. */
typedef struct hd_color {
    uint32_t color_bits;
    uint8_t weight;
    uint8_t bits_per_weight;
    uint16_t reserved;
} hd_color;

/* Counters of one edit call (or a batch): the reference's EditStats
 * (hash_dag_edits.h:39-49) plus find-or-add work. */
typedef struct hd_edit_stats {
    uint64_t num_voxels;        /* "num voxels" (hash_dag.h:374-378)        */
    uint64_t num_nodes;         /* visited edit nodes ("num nodes")         */
    uint64_t find_or_add_calls; /* leaf + interior find_or_add calls        */
    uint64_t nodes_added;       /* appended nodes                           */
    uint64_t words_scanned;     /* bucket words compared by the probes      */
    float device_ms;            /* device time of the call                  */
    float host_ms;              /* wall time of the call                    */
} hd_edit_stats;

/* Per-level occupancy of the table (HashTable::get_level_size,
 * hash_table.cpp:277-285; get_virtual_used_size, :246-275;
 * get_allocated_pages, hash_table.h:729-744). */
typedef struct hd_level_stats {
    uint64_t words[HD_MAX_DEPTH];   /* sum of bucket sizes (incl. padding)  */
    uint64_t nodes[HD_MAX_DEPTH];   /* stored nodes (walk of every bucket)  */
    uint64_t pages_used;            /* allocated physical pages             */
    uint32_t root;                  /* firstNodeIndex                       */
    uint32_t levels;                /* depth                                */
} hd_level_stats;

/* ---- lifetime (HashTable::create/destroy, hash_table.cpp:5-104) -------- */

void hd_default_config(uint32_t depth, hd_config* out);
/* HashTable::create(poolSizeInPages) on the device; every page of the pool
 * and the page table start at zero. */
hd_status hd_create(const hd_config* cfg, hd_ctx** out);
hd_status hd_destroy(hd_ctx* ctx);
const char* hd_last_error(const hd_ctx* ctx);
uint32_t hd_abi_version(void);
/* Binds the context to a cudaStream_t (NULL = legacy default stream). */
hd_status hd_set_stream(hd_ctx* ctx, void* stream);
hd_status hd_sync(hd_ctx* ctx);

/* ---- scene ingest ------------------------------------------------------ */

/* HashDAGFactory::load_from_DAG (hash_dag_factory.cpp:152-184): full nodes
 * for levels leaf..1 first, then every BasicDAG node appended in depth-first
 * first-visit order (create_hash_dag, :5-99).  h_words is a BasicDAG word
 * array (basic_dag.h:11-40): root at word 0, interior nodes
 * [header, absolute child word indices...], leaves two words. */
hd_status hd_load_basic_dag(hd_ctx* ctx, const uint32_t* h_words, uint64_t n_words);
/* Seeded procedural scene (fractal value-noise height field unioned with
 * 64 spheres) voxelised on the device straight into a BasicDAG, then
 * imported as hd_load_basic_dag does.  The words of the BasicDAG can be read
 * back with hd_export_basic_dag. */
hd_status hd_generate_scene(hd_ctx* ctx, uint64_t seed);
/* flags: HD_SCENE_SHELL keeps only the surface shell of the solid scene
 * (solid voxels with an empty face neighbour; outside the volume counts as
 * empty), the form the coloured scenes use. */
#define HD_SCENE_SHELL 1u
hd_status hd_generate_scene_ex(hd_ctx* ctx, uint64_t seed, uint32_t flags);
hd_status hd_export_basic_dag(hd_ctx* ctx, uint32_t* h_words, uint64_t capacity, uint64_t* n_words);

/* ---- traversal (DAGTracer, dag_tracer.cu:116-219) ---------------------- */

/* Tracer::trace_paths (tracer.cu:145-252): one primary ray per pixel,
 * nearest hit voxel path written as uint4 (x, y, z, 0) at row
 * (height - 1 - y), or (0, 0, 0, 0) on a miss.  d_paths holds
 * width * height * 4 uint32. */
hd_status hd_trace_primary(hd_ctx* ctx, const hd_camera* cam, uint32_t width, uint32_t height,
                           uint32_t* d_paths, float* ms);
/* Tracer::trace_shadows (tracer.cu:589-697) reduced to its hit test: from
 * the exact hit point of each pixel's primary ray (ray_box_intersection,
 * :574-587) plus bias * light, an any-hit ray toward light
 * (intersect_ray_node_out_of_order, :453-543).  d_mask[i] = 1 if shadowed,
 * 0 if lit, 2 if the pixel has no primary hit.  light is normalised on the
 * device as the reference's sun_direction (:546-549). */
hd_status hd_trace_shadow(hd_ctx* ctx, const hd_camera* cam, uint32_t width, uint32_t height,
                          const uint32_t* d_paths, const float light[3], float bias,
                          uint8_t* d_mask, float* ms);
/* n_views frames in one primary launch and one shadow launch (rays from many
 * views batched, so that the long shadow rays of one view overlap the work
 * of the others): view v's paths at d_paths + v * width * height * 4 and its
 * mask at d_mask + v * width * height, each equal to what hd_trace_primary /
 * hd_trace_shadow give for that view.  cams: host array; ms (optional, 2
 * floats): device time of the primary launch and of the shadow pass. */
hd_status hd_trace_views(hd_ctx* ctx, const hd_camera* cams, uint32_t n_views, uint32_t width, uint32_t height,
                         uint32_t* d_paths, const float* light, float bias, uint8_t* d_mask, float* ms);
/* hd_trace_views with host buffers: cameras read from host memory, every
 * view's paths (width * height * 4 uint32 each) and shadow mask written to
 * host memory.  With chunk_views = 0 and h_paths in pinned memory the
 * device can address, the primary rays write the paths of five views in
 * eight straight into host memory (over NVLink-C2C on a Grace host), the
 * other three are copied there while the shadow rays run, and the mask is
 * copied at the end.  Otherwise the views are traced chunk_views at a time (0: half of
 * them) and each chunk's copies run on a second stream while the next
 * chunk is traced.  ms: wall time of the call. */
hd_status hd_trace_views_host(hd_ctx* ctx, const hd_camera* cams, uint32_t n_views, uint32_t width, uint32_t height,
                              uint32_t* h_paths, const float light[3], float bias, uint8_t* h_mask,
                              uint32_t chunk_views, float* ms);
/* Primary + shadow in one call: the per-frame traversal step. */
hd_status hd_trace_frame(hd_ctx* ctx, const hd_camera* cam, uint32_t width, uint32_t height,
                         const float light[3], float bias, uint32_t* d_paths, uint8_t* d_mask,
                         float* ms_primary, float* ms_shadow);
/* hd_trace_frame with work counters, for the roofline's algorithmic bytes:
 * out = {primary rays, primary interior descents, primary leaf fetches,
 * shadow rays, shadow interior descents, shadow leaf fetches}; shadow rays
 * are the pixels with a primary hit. */
hd_status hd_trace_counters(hd_ctx* ctx, const hd_camera* cam, uint32_t width, uint32_t height,
                            const float light[3], float bias, uint32_t* d_paths, uint8_t* d_mask,
                            uint64_t out[6]);
/* hd_trace_counters for callers that cannot call cudaMalloc when they
 * trace: an embedding application (a game engine, a plugin host) that
 * reserves the device memory budget at start-up and forbids allocations
 * afterwards, or a real-time loop in which an allocation, which may
 * synchronise the whole device, would stall other streams.  No counterpart
 * in the reference.  Same outputs as hd_trace_counters; its scratch is a
 * fixed 6 MB device array inside the library (held on every device that
 * loads the library until the process exits), so it allocates nothing.
 * Images are limited to 262144 blocks of 8x8 pixels (16777216 pixels, e.g.
 * 4096x4096) and to 524280 rows; larger ones return HD_ERR_INVALID.  The
 * first call on each device looks up the array's address with that device
 * current.  The call copies the six totals to `out` and waits for the
 * context's stream.  Calls share the array: calls that overlap on the GPU
 * (other streams, other threads) race. */
hd_status hd_trace_counters_noalloc(hd_ctx* ctx, const hd_camera* cam, uint32_t width, uint32_t height,
                                    const float light[3], float bias, uint32_t* d_paths, uint8_t* d_mask,
                                    uint64_t out[6]);
/* Selects the arithmetic of the ray set-up: 0 = every float/double
 * operation rounded on its own, which is what the reference's tracer.cu
 * computes when nvcc compiles it for sm_103a with its build's flags (the
 * library equals that kernel bit for bit on the same GPU, and equals the
 * reference compiled for the host); 1 = fused multiply-adds at the places a
 * contracting build would put them.  Default 0. */
hd_status hd_set_fp_mode(hd_ctx* ctx, uint32_t mode);

/* ---- point queries (DAGUtils::get_value, dag_utils.h:138-172) ---------- */

/* d_xyz: n x 3 uint32 voxel coordinates; d_out: n uint8 occupancy. */
hd_status hd_get_values(hd_ctx* ctx, const uint32_t* d_xyz, uint64_t n, uint8_t* d_out);

/* ---- edits (HashDAG::edit_threads, hash_dag.h:255-405) ----------------- */

/* One edit: the editor's top-down descent with the reference's early exits
 * (should_edit / is_empty / is_full, hash_dag_edits.h:356-444), the 64-voxel
 * leaf rebuild (:451-546), then bottom-up find_or_add of every changed node
 * (hash_table.h:470-560), level by level, in depth-first order. */
hd_status hd_edit_apply(hd_ctx* ctx, const hd_edit* edit, hd_edit_stats* stats);
/* Batched form of HashDAG::edit_threads over a list of edits: the same
 * result as calling hd_edit_apply for each in order (same table, same
 * addresses), run as one CUDA graph per edit launched back to back, with no
 * host round trip between levels or edits.  stats: the sums over the batch
 * (device_ms = device time of the whole batch). */
hd_status hd_edit_batch(hd_ctx* ctx, const hd_edit* edits, uint32_t n, hd_edit_stats* stats);
/* hd_edit_batch with per-edit results: per_edit[i] (n entries, may be NULL)
 * holds edit i's counters, its device time (device_ms) and its completion
 * time since the batch started on the device (host_ms). */
hd_status hd_edit_batch_ex(hd_ctx* ctx, const hd_edit* edits, uint32_t n, hd_edit_stats* per_edit,
                           hd_edit_stats* total);

/* Launch shape of the batched edit kernels (results never depend on it).
 * mode HD_BATCH_GRAPH: one captured CUDA graph of level kernels per edit;
 * mode HD_BATCH_PERSISTENT: the whole batch in one cooperative launch of one
 * CTA per SM (foa_warps and grid_blocks unused). */
#define HD_BATCH_GRAPH 0u
#define HD_BATCH_PERSISTENT 1u
typedef struct hd_batch_tuning {
    uint32_t foa_warps;   /* warps per find-or-add block: 2, 4 or 8            */
    uint32_t probe_words; /* words per lane per bucket-page load: 1, 2 or 4    */
    uint32_t grid_blocks; /* blocks of the level kernels: 64 .. 2048           */
    uint32_t mode;        /* HD_BATCH_GRAPH or HD_BATCH_PERSISTENT             */
} hd_batch_tuning;
hd_status hd_set_batch_tuning(hd_ctx* ctx, const hd_batch_tuning* tuning);
hd_status hd_get_batch_tuning(hd_ctx* ctx, hd_batch_tuning* tuning);
/* Times every launch shape on a device copy of the table with the n sample
 * edits and keeps the fastest for ctx; the table itself is not changed. */
hd_status hd_autotune_batch(hd_ctx* ctx, const hd_edit* sample, uint32_t n, hd_batch_tuning* best, float* best_ms);
/* Edits that the batched path handed to the one-edit path (a level outgrew
 * its bound), since the context was created. */
hd_status hd_batch_fallbacks(hd_ctx* ctx, uint64_t* count);

/* ---- colours (HashDAGColors, hash_dag_colors.h; variable_weight_size_colors.h) */

/* Builds the colour tree of the current scene: one colour node per path above
 * C_colorTreeLevels, one compressed colour leaf per path at
 * C_colorTreeLevels with its voxels' colours in depth-first order (the
 * seeded colour field of color_seed: RGB8 of a value-noise field on an
 * aligned 8^3 grid, stored as set_single_color(rgb / 255)).  From then on
 * every edit rebuilds the colour leaves it touches (all six tools). */
hd_status hd_colors_from_scene(hd_ctx* ctx, uint64_t color_seed);
/* DAGUtils::get_color (dag_utils.h:423-523) for n voxels (d_xyz: 3 uint32
 * per voxel, device); CompressedColor{} for empty voxels outside any leaf. */
hd_status hd_get_colors(hd_ctx* ctx, const uint32_t* d_xyz, uint64_t n, hd_color* d_out);
/* Tracer::trace_colors (tracer.cu:254-451) on the paths of
 * hd_trace_primary, into a headless RGBA8 buffer (the reference writes a
 * GL surface): float3_to_rgb888 of the hit voxel's colour
 * (CompressedColor::get_color); the sky (187, 242, 250) for a miss; 0xFF00FF
 * where the path leaves the DAG; the checker (1, b, 1 - b), b = (x ^ y ^ z)
 * & 1, for a voxel without a valid colour.  hd_trace_colors is the
 * EDebugColors::None view without the tool overlay. */
hd_status hd_trace_colors(hd_ctx* ctx, const uint32_t* d_paths, uint32_t width, uint32_t height,
                          uint32_t* d_rgba);

/* EDebugColors (tracer.h:7-17) */
typedef enum hd_debug_colors {
    HD_DEBUG_NONE = 0,
    HD_DEBUG_INDEX = 1,      /* murmurhash32 of the node index at debug_level  */
    HD_DEBUG_POSITION = 2,   /* grey checker of the voxel position             */
    HD_DEBUG_COLOR_TREE = 3, /* parity of the colour-tree cell                 */
    HD_DEBUG_COLOR_BITS = 4, /* the colour's debug hash: 0 (no COLOR_DEBUG)    */
    HD_DEBUG_MIN_COLOR = 5,
    HD_DEBUG_MAX_COLOR = 6,
    HD_DEBUG_WEIGHT = 7
} hd_debug_colors;

/* ETool (tracer.h:21-29), for the overlay's ToolInfo::strength */
typedef enum hd_overlay_tool {
    HD_OVERLAY_SPHERE = 0,
    HD_OVERLAY_SPHERE_PAINT = 1,
    HD_OVERLAY_SPHERE_NOISE = 2,
    HD_OVERLAY_CUBE = 3,
    HD_OVERLAY_CUBE_COPY = 4,
    HD_OVERLAY_CUBE_FILL = 5
} hd_overlay_tool;

/* ToolInfo (tracer.h:33-77) and TOOL_OVERLAY (typedefs.h:70-71, on in the
 * interactive build): a pixel whose voxel has strength s > 0 moves toward
 * red by clamp(100 s, 0, 0.5). */
typedef struct hd_tool_overlay {
    uint32_t enabled;
    uint32_t tool; /* hd_overlay_tool */
    uint32_t position[3];
    float radius;
    uint32_t copy_source[3];
    uint32_t copy_dest[3];
} hd_tool_overlay;

typedef struct hd_trace_colors_params {
    uint32_t debug_colors; /* hd_debug_colors */
    uint32_t debug_level;  /* debugColorsIndexLevel of HD_DEBUG_INDEX */
    hd_tool_overlay overlay;
} hd_trace_colors_params;

/* Tracer::trace_colors with a debug view and the tool overlay. */
hd_status hd_trace_colors_ex(hd_ctx* ctx, const uint32_t* d_paths, uint32_t width, uint32_t height,
                             uint32_t* d_rgba, const hd_trace_colors_params* params);
/* colour-tree nodes (entries), leaves, blocks, macro words, weight words */
hd_status hd_color_stats(hd_ctx* ctx, uint64_t* out5);

/* ---- undo / redo (HashDAGUndoRedo, hash_dag.h:20-212) ------------------- */

/* Every successful edit records a frame (the root before it and the colour
 * leaves it replaced); undo restores them, redo re-applies; a new edit drops
 * the redo frames.  At most `capacity` undo frames are kept (default 200). */
hd_status hd_undo(hd_ctx* ctx); /* HD_ERR_STATE when there is nothing to undo */
hd_status hd_redo(hd_ctx* ctx);
hd_status hd_set_undo_capacity(hd_ctx* ctx, uint32_t frames);
hd_status hd_history(hd_ctx* ctx, uint32_t* undo_frames, uint32_t* redo_frames);

/* ---- serving loop -------------------------------------------------------- */

#define HD_REQ_EDIT 0u
#define HD_REQ_RENDER 1u

/* One request of a trace: an edit (any tool) or a render (primary rays,
 * shadow rays toward the configured light, colours when the context has
 * them) at width x height from camera. */
typedef struct hd_request {
    uint32_t kind;           /* HD_REQ_EDIT / HD_REQ_RENDER                    */
    uint32_t width, height;  /* render                                         */
    uint32_t reserved;
    double arrival_ms;       /* since the start of the trace, non-decreasing    */
    hd_edit edit;            /* edit                                           */
    hd_camera camera;        /* render                                         */
} hd_request;

typedef struct hd_serve_config {
    uint32_t continuous;     /* 0: one request at a time in arrival order;
                                1: renders in flight on their own streams while
                                   edits run, edits in arrival order           */
    uint32_t max_renders;    /* render slots (continuous)                      */
    uint32_t realtime;       /* 1: a request is available at its arrival time  */
    float gc_free_fraction;  /* GC (keeping the undo history) when the free
                                pool pages fall below this fraction of the
                                pool, and once more when an edit finds the
                                pool full (then the edit is retried); 0 =
                                never.  Above 0 the loop keeps
                                max(hd_set_page_reserve's pages, pool / 64)
                                pages back for its GCs                        */
    float light[3];
    float shadow_bias;
    uint32_t release_pages;  /* the serving GC releases pages (HD_GC_RELEASE_PAGES) */
    uint32_t batch_edits;    /* continuous, no colours: the queued edits run as
                                one batch (hd_edit_batch, persistent launch)   */
} hd_serve_config;

typedef struct hd_request_result {
    double start_ms, end_ms; /* admission and device completion               */
    uint32_t root;           /* edit: the root after it; render: rendered root */
    uint32_t status;
    uint32_t edits_before;   /* edits committed before the request's state     */
    uint32_t reserved;
    uint64_t checksum;       /* render: address-independent checksum of paths,
                                shadow mask and colours; edit: voxels          */
    uint64_t num_voxels;     /* edit                                           */
} hd_request_result;

typedef struct hd_serve_stats {
    double wall_ms;
    uint32_t edits, renders, gcs;
    uint32_t refused;                   /* edits refused: the pool stayed full
                                           after a GC (status HD_ERR_POOL_FULL) */
    double edit_p50_ms, edit_p99_ms;    /* completion - arrival                */
    double frame_p50_ms, frame_p99_ms;
    double voxels_per_s;                /* edited voxels over the wall time    */
    uint64_t num_voxels;
} hd_serve_stats;

/* Runs the trace against the context's DAG (Engine::tick's edit / render
 * interleaving, engine.cpp:575-720, as a request loop). */
hd_status hd_serve(hd_ctx* ctx, const hd_request* requests, uint32_t n, const hd_serve_config* config,
                   hd_request_result* results, hd_serve_stats* stats);

/* ---- garbage collection (HashDAG::remove_stale_nodes, hash_dag.h:407-547) */

/* Marks the nodes reachable from the root and from the n extra roots, then
 * rebuilds every level bottom-up: buckets emptied, full node re-added first,
 * live nodes re-appended in increasing old-address order with children
 * remapped.  Pages stay mapped (the reference never unmaps them).  The root
 * and h_extra_roots (in/out) are rewritten to their new addresses. */
hd_status hd_gc(hd_ctx* ctx, uint32_t* h_extra_roots, uint32_t n_extra);
/* hd_gc with flags: HD_GC_KEEP_HISTORY keeps the undo / redo frames (their
 * roots stay alive and are remapped); without it the history is dropped, as
 * the reference's engine frees its HashDAGUndoRedo after a GC
 * (engine.cpp:178-185). */
#define HD_GC_KEEP_HISTORY 1u
/* HD_GC_RELEASE_PAGES (no reference counterpart: the reference's poolTop only
 * grows, hash_table.h:794-809): the pages wholly past each bucket's new size
 * are unmapped, zeroed and kept on a free list that later page claims draw
 * from first, so a GC raises the free page count (hd_level_stats.pages_used
 * counts the pages in use).  Bucket contents and addresses are the same as
 * without the flag. */
#define HD_GC_RELEASE_PAGES 2u
hd_status hd_gc_ex(hd_ctx* ctx, uint32_t* h_extra_roots, uint32_t n_extra, uint32_t flags);
/* Keeps `pages` pool pages back from every page claim outside a GC (no
 * reference counterpart).  A GC re-appends the live nodes of a level into
 * buckets chosen by their new hashes (children remapped), so a bucket can
 * need a page it never had; with no free page the GC refuses
 * (HD_ERR_POOL_FULL, table unchanged), which is where an edit stream that
 * fills the pool would leave it.  With a reserve, edits fail at
 * pool_pages - pages (HD_ERR_POOL_FULL, as on a full pool) and the GC's
 * rebuild may use the reserve.  Default 0 (the reference: every page is an
 * edit's). */
hd_status hd_set_page_reserve(hd_ctx* ctx, uint32_t pages);

/* A test of the persistent batch's failure path: in the next persistent
 * hd_edit_batch launch (only), CTA cta_plus_one - 1 returns at once without
 * ever reaching a grid barrier, and every barrier wait is bounded by wait_ms
 * (0: the default 2 s).  The other CTAs' waits run out, the launch ends and
 * the call returns HD_ERR_TIMEOUT; the edits finished before stay applied
 * (hd_edit_batch_ex fills their per-edit results), the root is the last
 * finished edit's, and the context stays usable.  cta_plus_one 0 clears
 * it. */
hd_status hd_set_test_barrier_skip(hd_ctx* ctx, uint32_t cta_plus_one, uint32_t wait_ms);

/* ---- files (serializer.h:11-121) ---------------------------------------- */

/* DAGInfo (dag_info.h:6-10): the scene's bounding box, carried by the files. */
typedef struct hd_dag_info {
    double aabb_min[3];
    double aabb_max[3];
} hd_dag_info;

/* get_trace_params (dag_tracer.cu:71-113): the camera of a CameraView
 * (camera_view.h:7-28: position, rotation rows right = -row 0, up = row 1,
 * forward = row 2, fov 60 degrees in the reference) for a width x height
 * image of a 2^levels scene whose bounding box is info, in voxel space. */
hd_status hd_camera_from_view(const double position[3], const double rotation[9], double fov_degrees, uint32_t levels,
                              const hd_dag_info* info, uint32_t width, uint32_t height, hd_camera* out);

/* BasicDAGFactory::load_dag_from_file (basic_dag.cpp:105-117) followed by
 * load_from_DAG (as hd_load_basic_dag).  The file's level count must equal
 * the context's depth.  info may be NULL. */
hd_status hd_load_basic_dag_file(hd_ctx* ctx, const char* path, hd_dag_info* info);
/* BasicDAGFactory::save_dag_to_file (basic_dag.cpp:94-103) of the BasicDAG
 * the context last imported or generated (HD_ERR_STATE when there is none).
 * info may be NULL (zeros are written). */
hd_status hd_save_basic_dag_file(hd_ctx* ctx, const char* path, const hd_dag_info* info);
/* BasicDAGFactory::load_compressed_colors_from_file (basic_dag.cpp:49-92)
 * followed by HashDAGFactory::load_colors_from_DAG (hash_dag_factory.cpp:
 * 186-197) on the scene the context holds (loaded from the matching BasicDAG
 * file): one main colour leaf shared by every level-C_colorTreeLevels slot at
 * its running leaves count.  HD_COLORS_ENCLOSED_32 reads an old file whose
 * enclosedLeaves are uint32 (the reference then zeroes them). */
#define HD_COLORS_ENCLOSED_32 1u
hd_status hd_load_colors_file(hd_ctx* ctx, const char* path, uint32_t flags);
/* Snapshot: HashDAGFactory::save_dag_to_file's format (hash_dag_factory.cpp:
 * 199-222: DAGInfo, levels, firstNodeIndex, poolMaxSize, pageTableSize,
 * poolTop, the pool's first poolTop pages, the page table), which the
 * reference's load_dag_from_file reads as is, followed by what that format
 * leaves out: the table geometry, bucket sizes, full-node indices, per-level
 * node counts and the colour table.  Undo history is not saved. */
hd_status hd_save_snapshot(hd_ctx* ctx, const char* path, const hd_dag_info* info);
/* Loads a snapshot, or a hash-DAG file the reference wrote
 * (load_dag_from_file, :224-246).  The page table size must match the
 * context's geometry.  A reference file carries no bucket sizes: the table
 * can be traced, and edits return HD_ERR_STATE until hd_gc has rebuilt the
 * buckets. */
hd_status hd_load_snapshot(hd_ctx* ctx, const char* path, hd_dag_info* info);

/* ---- replays (ReplayManager, replay.h:462-635; replay.cpp:5-100) ------- */

/* EReplayActionType (replay.h:12-25) */
typedef enum hd_replay_type {
    HD_REPLAY_SET_LOCATION = 0,
    HD_REPLAY_SET_ROTATION = 1,
    HD_REPLAY_SET_TOOL_PARAMETERS = 2,
    HD_REPLAY_EDIT_SPHERE = 3,
    HD_REPLAY_EDIT_CUBE = 4,
    HD_REPLAY_EDIT_COPY = 5,
    HD_REPLAY_EDIT_FILL = 6,
    HD_REPLAY_EDIT_PAINT = 7,
    HD_REPLAY_UNDO = 8,
    HD_REPLAY_REDO = 9,
    HD_REPLAY_END_FRAME = 10
} hd_replay_type;

typedef struct hd_replay hd_replay;

/* One parsed action: its float cells and (uint32)stoi integer cells in line
 * order, and the boolean cell (add, or the copy's swirl flag). */
typedef struct hd_replay_action {
    uint32_t type;
    uint32_t flag;
    uint32_t n_floats;
    uint32_t n_ints;
    float floats[20];
    uint32_t ints[10];
} hd_replay_action;

/* replay_depth: REPLAY_DEPTH, the depth the replay was recorded on (positions
 * and radii scale by 2^depth / 2^replay_depth); width, height: the image of
 * the frame cameras; info: the scene's DAGInfo (world to voxel space). */
typedef struct hd_replay_config {
    uint32_t replay_depth;
    uint32_t width;
    uint32_t height;
    uint32_t reserved;
    hd_dag_info info;
} hd_replay_config;

/* ReplayManager::load_csv (replay.h:526-567): HD_ERR_INVALID names the first
 * line that does not parse. */
hd_status hd_replay_load(const char* path, hd_replay** out);
hd_status hd_replay_load_text(const char* text, uint64_t n_bytes, hd_replay** out);
hd_status hd_replay_free(hd_replay* replay);
hd_status hd_replay_info(const hd_replay* replay, uint64_t* n_actions, uint64_t* n_frames, uint64_t* next_action);
hd_status hd_replay_get_action(const hd_replay* replay, uint64_t index, hd_replay_action* out);
/* ReplayManager::write_csv (replay.h:504-520) */
hd_status hd_replay_write(const hd_replay* replay, const char* path);
/* ReplayManager::reset_replay */
hd_status hd_replay_reset(hd_replay* replay);
/* ReplayManager::replay_frame (replay.h:479-495): applies the actions up to
 * and including the next EndFrame to the context (edits, undo / redo, the
 * view) and returns the frame's camera (get_trace_params of the view,
 * dag_tracer.cu:71-113) and the number of edits applied.  HD_ERR_STATE when
 * the replay is at its end. */
hd_status hd_replay_frame(hd_ctx* ctx, hd_replay* replay, const hd_replay_config* config, hd_camera* camera,
                          uint32_t* edits);

/* ---- state and statistics ---------------------------------------------- */

hd_status hd_get_root(hd_ctx* ctx, uint32_t* root);
/* HD_ERR_INVALID unless root is an address on a mapped page of the table. */
hd_status hd_set_root(hd_ctx* ctx, uint32_t root);
hd_status hd_get_config(hd_ctx* ctx, hd_config* cfg);
hd_status hd_get_level_stats(hd_ctx* ctx, hd_level_stats* out);
/* Device bytes held: [0] table (pool, page table for the whole 32-bit
 * virtual space, bucket sizes, per-page Bloom filters), [1] colour
 * table, [2] scratch buffers, [3] the peak scratch of the last scene
 * generation. */
hd_status hd_memory_stats(hd_ctx* ctx, uint64_t* out4);
/* Copies the table to the host.  Arrays sized by hd_table_sizes: bucket
 * sizes (total buckets), page table (virtual pages), pool (pages_used + 1
 * pages of 512 words; page 0 is the reserved null page), full-node indices
 * (depth). Any pointer may be NULL to skip that array. */
hd_status hd_table_sizes(hd_ctx* ctx, uint64_t* n_buckets, uint64_t* n_virtual_pages,
                         uint64_t* n_pool_pages_used);
hd_status hd_export_table(hd_ctx* ctx, uint32_t* h_bucket_sizes, uint32_t* h_page_table,
                          uint32_t* h_pool, uint64_t pool_words_capacity,
                          uint32_t* h_full_nodes);
/* Replaces the table with host copies (pool_words = pages * 512).
 * HD_ERR_INVALID (context unchanged) when a page-table entry points past
 * the given pool, a bucket size exceeds its bucket's capacity or the root is
 * not on a mapped page; node contents are not checked, but every address
 * they hold translates inside the page table, so a corrupt table gives wrong
 * pictures, never out-of-bounds reads of the table. */
hd_status hd_import_table(hd_ctx* ctx, const uint32_t* h_bucket_sizes, const uint32_t* h_page_table,
                          const uint32_t* h_pool, uint64_t pool_words,
                          const uint32_t* h_full_nodes, uint32_t root);
/* Device pointers of the table (for zero-copy consumers): pool, page
 * table, bucket sizes. */
hd_status hd_device_table(hd_ctx* ctx, uint32_t** d_pool, uint32_t** d_page_table,
                          uint32_t** d_bucket_sizes);

#ifdef __cplusplus
}
#endif

#endif /* HASHDAG_GB300_H */
