/*
 * hashdag_gb300.hpp — C++ classes over the C ABI (hashdag_gb300.h) in the
 * shapes of the reference's host interfaces (Phyronnaz/HashDAG), so that
 * the reference's call sites (Engine::edit, engine.h:77-103; the replay
 * actions, replay.cpp:7-100; main's load, main.cpp:46) compile against them
 * with their own argument lists:
 *
 *   HashDAG::edit_threads(editor, colors, undoRedo, statsRecorder)   hash_dag.h:255
 *   HashDAG::remove_stale_nodes(maxLevel)                          hash_dag.h:407
 *   HashDAG::firstNodeIndex, is_valid(), free()                    hash_dag.h:214-236
 *   HashDAGFactory::load_from_DAG / save_dag_to_file / load_dag_from_file
 *                                                                  hash_dag_factory.h:10-23
 *   HashDAGUndoRedo::undo / redo / free                            hash_dag.h:20-212
 *   SphereEditor<bool>, BoxEditor<bool>, SpherePaintEditor, CopyEditor,
 *   SphereNoiseEditor, FillEditorColors                            hash_dag_editors.h:223-808
 *   DAGTracer(headLess); resolve_paths / resolve_colors / resolve_shadows
 *   returning kernel milliseconds; get_path                        dag_tracer.h:9-42
 *   CameraView, DAGInfo, StatsRecorder, EDebugColors, ETool, ToolInfo
 *                                                                  camera_view.h, dag_info.h,
 *                                                                  stats.h, tracer.h
 *
 * Everything runs on the device behind the C ABI; the header adds no
 * computation of its own beyond argument packing.  Errors throw
 * hashdag_gb300::Error (the C status and hd_last_error's message) where the
 * reference would abort.  Differences of shape, each forced by the device-
 * resident design:
 *  * the table, colours and undo history live in the HashDAG's context:
 *    HashDAGColors and HashDAGUndoRedo are views of it (a HashDAGColors is
 *    bound to its HashDAG by HashDAGFactory::load_colors_from_file or
 *    colors_from_scene);
 *  * BasicDAG is its word array (basic_dag.h:11-40) as std::vector<uint32_t>;
 *  * DAGTracer's outputs are device buffers (paths, shadow mask, colours)
 *    instead of GL surfaces; resolve_shadows writes the hit mask
 *    (1 shadowed, 0 lit, 2 no hit) toward `light` (default the reference's
 *    sun, tracer.cu:546-549) instead of shading the colour surface;
 *  * CopyEditor is CopyEditorWithDecompression: the transform and swirl
 *    arguments are accepted and not applied, as that editor does.
 *
 * Needs the CUDA runtime (float3 / uint3, cudaMalloc for the tracer's
 * buffers) and the library: -lhashdag_gb300 -lcudart.
 */
#pragma once

#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include <cuda_runtime_api.h>
#include <vector_functions.h>
#include <vector_types.h>

#include "hashdag_gb300.h"

namespace hashdag_gb300 {

using uint32 = uint32_t;
using uint64 = uint64_t;

class Error : public std::runtime_error {
public:
    Error(hd_status s, const std::string& what) : std::runtime_error(what), status(s) {}
    hd_status status;
};

inline void check(hd_ctx* ctx, hd_status s, const char* call)
{
    if (s != HD_OK) {
        const char* msg = ctx ? hd_last_error(ctx) : nullptr;
        throw Error(s, std::string(call) + ": " + (msg && *msg ? msg : "status " + std::to_string(int(s))));
    }
}

inline void check_cuda(cudaError_t e, const char* call)
{
    if (e != cudaSuccess)
        throw Error(HD_ERR_CUDA, std::string(call) + ": " + cudaGetErrorString(e));
}

// ---- StatsRecorder (stats.h:14-...): named values, frame by frame ----------
class StatsRecorder {
public:
    struct Element {
        int32_t frame;
        std::string name;
        double time;
    };
    void next_frame() { frame++; }
    template <typename T>
    void report(std::string name, T value)
    {
        elements.push_back(Element{frame, std::move(name), double(value)});
    }
    void clear()
    {
        frame = 0;
        elements.clear();
    }
    // the value reported under `name` in the current frame (0 if none)
    double get(const std::string& name) const
    {
        for (auto it = elements.rbegin(); it != elements.rend() && it->frame == frame; ++it)
            if (it->name == name)
                return it->time;
        return 0.0;
    }
    std::vector<Element> elements;

private:
    int32_t frame = 0;
};

// ---- CameraView (camera_view.h:7-28), DAGInfo (dag_info.h:6-10) -----------
struct Vector3 {
    float X = 0.f, Y = 0.f, Z = 0.f;
};
struct Matrix3x3 {
    float D00 = 1, D01 = 0, D02 = 0, D10 = 0, D11 = 1, D12 = 0, D20 = 0, D21 = 0, D22 = 1;
    static Matrix3x3 Identity() { return Matrix3x3{}; }
    bool is_identity() const
    {
        return D00 == 1 && D01 == 0 && D02 == 0 && D10 == 0 && D11 == 1 && D12 == 0 && D20 == 0 && D21 == 0 &&
               D22 == 1;
    }
};
struct CameraView {
    static constexpr float fov = 60.f;
    Vector3 position;
    Matrix3x3 rotation;
    Vector3 right() const { return {-rotation.D00, -rotation.D01, -rotation.D02}; }
    Vector3 up() const { return {rotation.D10, rotation.D11, rotation.D12}; }
    Vector3 forward() const { return {rotation.D20, rotation.D21, rotation.D22}; }
};
struct DAGInfo {
    Vector3 boundsAABBMin;
    Vector3 boundsAABBMax;
};

// get_trace_params (dag_tracer.cu:71-113) for a width x height image
inline hd_camera get_trace_params(const CameraView& camera, uint32 levels, const DAGInfo& info, uint32 width,
                                  uint32 height)
{
    const double p[3] = {camera.position.X, camera.position.Y, camera.position.Z};
    const Matrix3x3& m = camera.rotation;
    const double r[9] = {m.D00, m.D01, m.D02, m.D10, m.D11, m.D12, m.D20, m.D21, m.D22};
    hd_dag_info di{{info.boundsAABBMin.X, info.boundsAABBMin.Y, info.boundsAABBMin.Z},
                   {info.boundsAABBMax.X, info.boundsAABBMax.Y, info.boundsAABBMax.Z}};
    hd_camera cam{};
    check(nullptr, hd_camera_from_view(p, r, double(CameraView::fov), levels, &di, width, height, &cam),
          "get_trace_params");
    return cam;
}

// ---- tracer.h:7-77 -----------------------------------------------------------
enum class EDebugColors : uint32 { None, Index, Position, ColorTree, ColorBits, MinColor, MaxColor, Weight };
enum class ETool : uint32 { Sphere, SpherePaint, SphereNoise, Cube, CubeCopy, CubeFill };
struct ToolInfo {
    ETool tool = ETool::Sphere;
    uint3 position{0, 0, 0};
    float radius = 0.f;
    uint3 copySource{0, 0, 0};
    uint3 copyDest{0, 0, 0};
    bool enabled = false;
    ToolInfo() = default;
    ToolInfo(ETool t, uint3 pos, float r, uint3 src, uint3 dst)
        : tool(t), position(pos), radius(r), copySource(src), copyDest(dst), enabled(true)
    {
    }
};

class HashDAG;
class HashDAGColors;

// ---- editors (hash_dag_editors.h) ----------------------------------------------
// Each editor is the C ABI's hd_edit for its tool.
struct EditorBase {
    hd_edit edit{};

protected:
    EditorBase(hd_tool tool, float3 center, float radius)
    {
        edit.tool = tool;
        edit.center[0] = center.x;
        edit.center[1] = center.y;
        edit.center[2] = center.z;
        edit.radius = radius;
        edit.rgb = 0xFF0000u; // blue: the reference's paint colour (hash_dag_editors.h:327)
    }
};

template <bool isAdding>
struct SphereEditor final : EditorBase {
    SphereEditor(float3 center, float radius)
        : EditorBase(isAdding ? HD_TOOL_SPHERE_ADD : HD_TOOL_SPHERE_REMOVE, center, radius)
    {
    }
};

template <bool isAdding>
struct BoxEditor final : EditorBase {
    BoxEditor(float3 center, float radius)
        : EditorBase(isAdding ? HD_TOOL_BOX_ADD : HD_TOOL_BOX_REMOVE, center, radius)
    {
    }
};

// rgb: r | g << 8 | b << 16 (the reference paints blue, the default)
struct SpherePaintEditor final : EditorBase {
    SpherePaintEditor(float3 center, float radius, uint32 rgb = 0xFF0000u)
        : EditorBase(HD_TOOL_SPHERE_PAINT, center, radius)
    {
        edit.rgb = rgb;
    }
};

struct CopyEditor final : EditorBase {
    CopyEditor(const HashDAG&, const HashDAGColors&, float3 source, float3 dest, float3 center, float radius,
               const Matrix3x3& /*transform*/, StatsRecorder& /*statsRecorder*/, bool /*withSwirl*/,
               float /*swirlPeriod*/)
        : EditorBase(HD_TOOL_COPY, center, radius)
    {
        edit.source[0] = source.x;
        edit.source[1] = source.y;
        edit.source[2] = source.z;
        edit.dest[0] = dest.x;
        edit.dest[1] = dest.y;
        edit.dest[2] = dest.z;
    }
};

struct SphereNoiseEditor final : EditorBase {
    SphereNoiseEditor(const HashDAG&, float3 center, float radius, bool isAdding)
        : EditorBase(isAdding ? HD_TOOL_NOISE_ADD : HD_TOOL_NOISE_REMOVE, center, radius)
    {
    }
};

struct FillEditorColors final : EditorBase {
    FillEditorColors(const HashDAG&, HashDAGColors&, float3 center, float radius)
        : EditorBase(HD_TOOL_FILL, center, radius)
    {
    }
};

// ---- HashDAG (hash_dag.h:214-636) -------------------------------------------------
class HashDAG {
public:
    // the root (firstNodeIndex): refreshed after every call that moves it
    uint32 firstNodeIndex = 0;
    uint32 levels = 0;

    HashDAG() = default;
    explicit HashDAG(uint32 depth)
    {
        hd_config cfg;
        hd_default_config(depth, &cfg);
        create(cfg);
    }
    explicit HashDAG(const hd_config& cfg) { create(cfg); }
    ~HashDAG() { free(); }
    HashDAG(const HashDAG&) = delete;
    HashDAG& operator=(const HashDAG&) = delete;
    HashDAG(HashDAG&& o) noexcept { *this = std::move(o); }
    HashDAG& operator=(HashDAG&& o) noexcept
    {
        if (this != &o) {
            free();
            ctx_ = o.ctx_;
            firstNodeIndex = o.firstNodeIndex;
            levels = o.levels;
            o.ctx_ = nullptr;
        }
        return *this;
    }

    void create(const hd_config& cfg)
    {
        free();
        check(nullptr, hd_create(&cfg, &ctx_), "HashTable::create");
        levels = cfg.depth;
    }
    bool is_valid() const { return ctx_ != nullptr; }
    uint32 get_first_node_index() const { return firstNodeIndex; }
    void free()
    {
        if (ctx_)
            hd_destroy(ctx_);
        ctx_ = nullptr;
    }
    hd_ctx* context() const { return ctx_; }

    // HashDAG::edit_threads: the edit with the reference's stats names
    // ("edits" ms, "num nodes", "num voxels"; stats.h report) plus the
    // library's find-or-add counters.
    template <typename T>
    void edit_threads(const T& editor, HashDAGColors&, class HashDAGUndoRedo&, StatsRecorder& statsRecorder)
    {
        hd_edit_stats s{};
        check(ctx_, hd_edit_apply(ctx_, &editor.edit, &s), "HashDAG::edit_threads");
        refresh();
        statsRecorder.report("edits", s.device_ms);
        statsRecorder.report("num nodes", s.num_nodes);
        statsRecorder.report("num voxels", s.num_voxels);
        statsRecorder.report("find or add", s.find_or_add_calls);
        statsRecorder.report("nodes added", s.nodes_added);
    }
    // The batched form (no reference counterpart): edits in order, same
    // result as one edit_threads per edit.
    void edit_batch(const std::vector<hd_edit>& edits, hd_edit_stats* total = nullptr)
    {
        check(ctx_, hd_edit_batch(ctx_, edits.data(), uint32(edits.size()), total), "HashDAG::edit_batch");
        refresh();
    }
    // HashDAG::remove_stale_nodes: every level is collected (maxLevel, the
    // reference's last level to rebuild, is always levels - 2 at its call
    // sites, engine.cpp:178-185); the undo history is dropped as the engine
    // does after a GC.
    void remove_stale_nodes(uint32 /*maxLevel*/ = 0)
    {
        check(ctx_, hd_gc(ctx_, nullptr, 0), "HashDAG::remove_stale_nodes");
        refresh();
    }
    hd_level_stats level_stats() const
    {
        hd_level_stats s{};
        check(ctx_, hd_get_level_stats(ctx_, &s), "HashTable::get_level_size");
        return s;
    }
    void refresh() { check(ctx_, hd_get_root(ctx_, &firstNodeIndex), "HashDAG::firstNodeIndex"); }

private:
    hd_ctx* ctx_ = nullptr;
};

// ---- HashDAGColors (hash_dag_colors.h): the colours of a HashDAG's context -----
class HashDAGColors {
public:
    HashDAGColors() = default;
    bool is_valid() const { return dag_ != nullptr; }
    // the seeded colour field of the generated scenes
    void colors_from_scene(HashDAG& dag, uint64 seed)
    {
        check(dag.context(), hd_colors_from_scene(dag.context(), seed), "HashDAGColors::colors_from_scene");
        dag_ = &dag;
    }
    void bind(HashDAG& dag) { dag_ = &dag; }
    HashDAG* dag() const { return dag_; }

private:
    HashDAG* dag_ = nullptr;
};

// ---- HashDAGUndoRedo (hash_dag.h:20-212) -----------------------------------------
class HashDAGUndoRedo {
public:
    void undo(HashDAG& dag, HashDAGColors&) { step(dag, hd_undo, "HashDAGUndoRedo::undo"); }
    void redo(HashDAG& dag, HashDAGColors&) { step(dag, hd_redo, "HashDAGUndoRedo::redo"); }
    // drops every frame (the capacity stays)
    void free(HashDAG& dag, uint32 capacity = 200)
    {
        check(dag.context(), hd_set_undo_capacity(dag.context(), 0), "HashDAGUndoRedo::free");
        check(dag.context(), hd_set_undo_capacity(dag.context(), capacity), "HashDAGUndoRedo::free");
    }

private:
    static void step(HashDAG& dag, hd_status (*f)(hd_ctx*), const char* what)
    {
        const hd_status s = f(dag.context());
        if (s == HD_ERR_STATE) // nothing to undo / redo: the reference returns
            return;
        check(dag.context(), s, what);
        dag.refresh();
    }
};

// ---- HashDAGFactory (hash_dag_factory.h:10-23) -----------------------------------
struct HashDAGFactory {
    // BasicDAG = its words (basic_dag.h:11-40); numPages: the pool's pages
    // (0 = the library default for the depth)
    static void load_from_DAG(HashDAG& outDag, const std::vector<uint32>& inDag, uint32 depth, uint32 numPages = 0)
    {
        hd_config cfg;
        hd_default_config(depth, &cfg);
        if (numPages)
            cfg.pool_pages = numPages;
        outDag.create(cfg);
        check(outDag.context(), hd_load_basic_dag(outDag.context(), inDag.data(), inDag.size()),
              "HashDAGFactory::load_from_DAG");
        outDag.refresh();
    }
    static void load_colors_from_file(HashDAGColors& outColors, HashDAG& dag, const std::string& path)
    {
        check(dag.context(), hd_load_colors_file(dag.context(), path.c_str(), 0),
              "HashDAGFactory::load_colors_from_DAG");
        outColors.bind(dag);
    }
    static void save_dag_to_file(const DAGInfo& info, const HashDAG& dag, const std::string& path)
    {
        const hd_dag_info di = to_info(info);
        check(dag.context(), hd_save_snapshot(dag.context(), path.c_str(), &di), "HashDAGFactory::save_dag_to_file");
    }
    static void load_dag_from_file(DAGInfo& info, HashDAG& dag, const std::string& path)
    {
        hd_dag_info di{};
        check(dag.context(), hd_load_snapshot(dag.context(), path.c_str(), &di), "HashDAGFactory::load_dag_from_file");
        info.boundsAABBMin = {float(di.aabb_min[0]), float(di.aabb_min[1]), float(di.aabb_min[2])};
        info.boundsAABBMax = {float(di.aabb_max[0]), float(di.aabb_max[1]), float(di.aabb_max[2])};
        dag.refresh();
    }

private:
    static hd_dag_info to_info(const DAGInfo& i)
    {
        return hd_dag_info{{i.boundsAABBMin.X, i.boundsAABBMin.Y, i.boundsAABBMin.Z},
                           {i.boundsAABBMax.X, i.boundsAABBMax.Y, i.boundsAABBMax.Z}};
    }
};

// ---- DAGTracer (dag_tracer.h:9-42), headless ------------------------------------
class DAGTracer {
public:
    const bool headLess;
    const uint32 imageWidth, imageHeight;
    float light[3] = {0.3f, 1.0f, 0.5f}; // sun_direction() (tracer.cu:546-549), normalised on the device

    explicit DAGTracer(bool headLess_, uint32 width = 1920, uint32 height = 1080)
        : headLess(headLess_), imageWidth(width), imageHeight(height)
    {
        const size_t px = size_t(width) * height;
        check_cuda(cudaMalloc(reinterpret_cast<void**>(&paths_), px * 16), "cudaMalloc paths");
        check_cuda(cudaMalloc(reinterpret_cast<void**>(&mask_), px), "cudaMalloc shadow mask");
        check_cuda(cudaMalloc(reinterpret_cast<void**>(&colors_), px * 4), "cudaMalloc colours");
        check_cuda(cudaEventCreate(&ev0_), "cudaEventCreate");
        check_cuda(cudaEventCreate(&ev1_), "cudaEventCreate");
    }
    ~DAGTracer()
    {
        cudaFree(paths_);
        cudaFree(mask_);
        cudaFree(colors_);
        cudaEventDestroy(ev0_);
        cudaEventDestroy(ev1_);
    }
    DAGTracer(const DAGTracer&) = delete;
    DAGTracer& operator=(const DAGTracer&) = delete;

    float resolve_paths(const CameraView& camera, const DAGInfo& dagInfo, const HashDAG& dag)
    {
        return resolve_paths(get_trace_params(camera, dag.levels, dagInfo, imageWidth, imageHeight), dag);
    }
    float resolve_paths(const hd_camera& cam, const HashDAG& dag)
    {
        float ms = 0.f;
        check(dag.context(), hd_trace_primary(dag.context(), &cam, imageWidth, imageHeight, paths_, &ms),
              "DAGTracer::resolve_paths");
        return ms;
    }
    float resolve_colors(const HashDAG& dag, const HashDAGColors&, EDebugColors debugColors,
                         uint32 debugColorsIndexLevel, const ToolInfo& toolInfo)
    {
        hd_trace_colors_params p{};
        p.debug_colors = uint32(debugColors);
        p.debug_level = debugColorsIndexLevel;
        p.overlay.enabled = toolInfo.enabled ? 1u : 0u;
        p.overlay.tool = uint32(toolInfo.tool);
        p.overlay.position[0] = toolInfo.position.x;
        p.overlay.position[1] = toolInfo.position.y;
        p.overlay.position[2] = toolInfo.position.z;
        p.overlay.radius = toolInfo.radius;
        p.overlay.copy_source[0] = toolInfo.copySource.x;
        p.overlay.copy_source[1] = toolInfo.copySource.y;
        p.overlay.copy_source[2] = toolInfo.copySource.z;
        p.overlay.copy_dest[0] = toolInfo.copyDest.x;
        p.overlay.copy_dest[1] = toolInfo.copyDest.y;
        p.overlay.copy_dest[2] = toolInfo.copyDest.z;
        // timed like the reference (dag_tracer.cu:167-172), on the context's
        // default stream
        check_cuda(cudaEventRecord(ev0_, nullptr), "cudaEventRecord");
        check(dag.context(), hd_trace_colors_ex(dag.context(), paths_, imageWidth, imageHeight, colors_, &p),
              "DAGTracer::resolve_colors");
        check_cuda(cudaEventRecord(ev1_, nullptr), "cudaEventRecord");
        check_cuda(cudaEventSynchronize(ev1_), "cudaEventSynchronize");
        float ms = 0.f;
        check_cuda(cudaEventElapsedTime(&ms, ev0_, ev1_), "cudaEventElapsedTime");
        return ms;
    }
    float resolve_shadows(const CameraView& camera, const DAGInfo& dagInfo, const HashDAG& dag, float shadowBias,
                          float /*fogDensity*/)
    {
        return resolve_shadows(get_trace_params(camera, dag.levels, dagInfo, imageWidth, imageHeight), dag,
                               shadowBias);
    }
    float resolve_shadows(const hd_camera& cam, const HashDAG& dag, float shadowBias)
    {
        float ms = 0.f;
        check(dag.context(),
              hd_trace_shadow(dag.context(), &cam, imageWidth, imageHeight, paths_, light, shadowBias, mask_, &ms),
              "DAGTracer::resolve_shadows");
        return ms;
    }
    // DAGTracer::get_path: the hit voxel of pixel (posX, posY) in output rows
    uint3 get_path(uint32 posX, uint32 posY) const
    {
        uint32 v[4] = {0, 0, 0, 0};
        check_cuda(cudaMemcpy(v, paths_ + (size_t(posY) * imageWidth + posX) * 4, 16, cudaMemcpyDeviceToHost),
                   "DAGTracer::get_path");
        return uint3{v[0], v[1], v[2]};
    }
    // device buffers: paths (uint4 per pixel), shadow mask, rgba colours
    uint32* paths() const { return paths_; }
    uint8_t* shadows() const { return mask_; }
    uint32* colors() const { return colors_; }

private:
    uint32* paths_ = nullptr;
    uint8_t* mask_ = nullptr;
    uint32* colors_ = nullptr;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
};

} // namespace hashdag_gb300
