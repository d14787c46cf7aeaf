// ORACLE — test infrastructure only.
//
// Builds the reference's own host-side hot path (HashTable, HashDAGFactory,
// HashDagEdits, editors, remove_stale_nodes) from its unmodified sources and
// exposes a small C API used to generate the golden fixtures that pin the
// C restatement (oracle/hd_oracle.c).  Compiled by oracle/build_ref.py into
// oracle/_ref/libhdref_d<depth>.so; never shipped, never linked by the
// product.
//
// Compile-time configuration (command line): BENCHMARK=1 (single-threaded,
// no undo), USE_BLOOM_FILTER=0, EDITS_ENABLE_COLORS=0, EDITS_COUNTERS=1,
// HARNESS_DEPTH, BUCKETS_BITS_FOR_TOP_LEVELS, and
// C_colorTreeLevels="CTL_VALUE = <T>, CTL_IGNORED" which turns the
// reference's `constexpr uint32 C_colorTreeLevels = 10;`
// (hash_dag_globals.h:7) into `constexpr uint32 CTL_VALUE = <T>, CTL_IGNORED
// = 10;` so that the colour-tree depth can follow the scene depth.

// Standard headers first: the harness opens the reference's classes for
// reading (private -> public) and the library headers must not see that.
#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cinttypes>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <iomanip>
#include <iostream>
#include <limits>
#include <memory>
#include <mutex>
#include <random>
#include <set>
#include <sstream>
#include <string>
#include <thread>
#include <type_traits>
#include <unordered_map>
#include <unordered_set>
#include <utility>
#include <vector>
#include <cuda_runtime.h>
#define private public
#define protected public

#include "typedefs.h"
// script_definitions.h forces USE_VIDEO=1 and with it SCENE_DEPTH=17; every
// use of the depth goes through MAX_LEVELS -> SCENE_DEPTH later on.
#undef SCENE_DEPTH
#define SCENE_DEPTH HARNESS_DEPTH
#include "dags/hash_dag/hash_dag_globals.h"
#undef C_colorTreeLevels
#define C_colorTreeLevels CTL_VALUE

#include "camera_view.h"
#include "dags/hash_dag/hash_dag.h"
#include "dags/hash_dag/hash_dag_editors.h"
#include "dags/hash_dag/hash_dag_factory.h"

// The reference's translation units, compiled here as one unit so the
// overrides above apply everywhere.
#include "hash_table.cpp"
#include "stats.cpp"
#include "hash_dag_factory.cpp"
#include "FastNoise.cpp"
#if EDITS_ENABLE_COLORS
// the BasicDAG / compressed-colour file writers and readers, replays
#include "dags/basic_dag/basic_dag.cpp"
#include "replay.h"
#endif

#include <algorithm>
#include <cstdlib>
#include <cstring>

// ---------------------------------------------------------------------------
// Host-memory stand-ins for Memory (memory.h:15-117) and the few CUDA runtime
// calls the host path makes: device allocations become host allocations and
// host<->device copies become memcpy, so the table the reference "uploads"
// is simply left in host memory.
// ---------------------------------------------------------------------------
Memory Memory::singleton;
Memory::~Memory() {}
void* Memory::malloc_impl(size_t size, const char*, EMemoryType)
{
    void* p = std::calloc(1, size ? size : 1);
    Element e;
    e.size = size;
    allocations[p] = e;
    return p;
}
void Memory::free_impl(void* ptr)
{
    allocations.erase(ptr);
    std::free(ptr);
}
void Memory::realloc_impl(void*& ptr, size_t newSize)
{
    size_t old = allocations.count(ptr) ? allocations[ptr].size : 0;
    void* p = std::calloc(1, newSize ? newSize : 1);
    if (ptr)
        std::memcpy(p, ptr, std::min(old, newSize));
    allocations.erase(ptr);
    std::free(ptr);
    Element e;
    e.size = newSize;
    allocations[p] = e;
    ptr = p;
}
void Memory::cuda_memcpy_impl(uint8* dst, const uint8* src, uint64 size, cudaMemcpyKind)
{
    std::memmove(dst, src, size);
}
const char* Memory::get_alloc_name_impl(void*) const { return "harness"; }
std::string Memory::get_stats_string_impl() const { return {}; }

extern "C" {
cudaError_t cudaMemcpyAsync(void* dst, const void* src, size_t count, cudaMemcpyKind, cudaStream_t)
{
    std::memmove(dst, src, count);
    return cudaSuccess;
}
cudaError_t cudaMemcpy(void* dst, const void* src, size_t count, cudaMemcpyKind)
{
    std::memmove(dst, src, count);
    return cudaSuccess;
}
cudaError_t cudaDeviceSynchronize(void) { return cudaSuccess; }
cudaError_t cudaGetLastError(void) { return cudaSuccess; }
const char* cudaGetErrorString(cudaError_t) { return "harness"; }
}

// ---------------------------------------------------------------------------
// Harness state: one scene per process (the reference's HashTable keeps its
// host data in a static singleton, hash_table.h:862).
// ---------------------------------------------------------------------------
static HashDAG g_dag;
static HashDAGColors g_colors;
static StatsRecorder* g_recorder = nullptr;
static bool g_loaded = false;

extern "C" uint32 ref_depth() { return MAX_LEVELS; }
extern "C" uint32 ref_color_tree_levels() { return C_colorTreeLevels; }
extern "C" uint32 ref_total_buckets() { return C_totalNumberOfBuckets; }
extern "C" uint32 ref_total_pages() { return C_totalPages; }

// HashDAGFactory::load_from_DAG on a BasicDAG word array.
extern "C" int ref_load(const uint32* words, uint64 nWords, uint32 poolPages)
{
    if (g_loaded)
        return 1;
    BasicDAG basic;
    basic.data = StaticArray<uint32>::allocate("basic dag", nWords, EMemoryType::CPU);
    std::memcpy(basic.data.data(), words, nWords * sizeof(uint32));
    HashDAGFactory::load_from_DAG(g_dag, basic, poolPages);
    // A colour tree whose root has no children: the edit recursion reads it
    // (hash_dag_edits.h:168-173) but, with colours off, never fills it.
    HashColorsBuilder builder;
    builder.nodes.assign(8, 0);
    builder.build(g_colors, CompressedColorLeaf{});
    g_recorder = new StatsRecorder();
    g_loaded = true;
    return 0;
}

extern "C" uint32 ref_root() { return g_dag.firstNodeIndex; }
extern "C" uint32 ref_pool_top() { return uint32(g_dag.data.get_allocated_pages() + 1); }

// Copies the reference's own table: bucket sizes, page table, pool
// (poolTop pages), full-node indices.
extern "C" void ref_export(uint32* bucketSizes, uint32* pageTable, uint32* pool, uint64 poolWords, uint32* fullNodes)
{
    auto& cpu = HashTable::cpuData;
    std::memcpy(bucketSizes, cpu.bucketsSizes, C_totalNumberOfBuckets * sizeof(uint32));
    std::memcpy(pageTable, cpu.cpuPageTable, C_totalPages * sizeof(uint32));
    const uint64 words = std::min<uint64>(poolWords, uint64(g_dag.data.poolTop) * C_pageSize);
    std::memcpy(pool, cpu.cpuPool, words * sizeof(uint32));
    for (uint32 level = 0; level < C_maxNumberOfLevels; level++)
        fullNodes[level] = level <= C_leafLevel ? cpu.fullNodeIndices[level] : 0;
}

extern "C" uint32 ref_read_word(uint32 level, uint32 vptr) { return *g_dag.data.get_sys_ptr(level, vptr); }

static uint64 morton(uint3 p, uint32 bits)
{
    uint64 key = 0;
    for (int32 b = int32(bits) - 1; b >= 0; b--)
        key = (key << 3) | (uint64((p.x >> b) & 1) << 2) | (uint64((p.y >> b) & 1) << 1) | uint64((p.z >> b) & 1);
    return key;
}

// HashDAG::edit_threads (hash_dag.h:255-405) with its task list run in
// depth-first order of the tasks' level-C_colorTreeLevels paths instead of
// unordered_map iteration order; colours and undo off (BENCHMARK).
template<typename TEditor>
static void run_edit(const TEditor& editor, uint64* stats)
{
    HashDagEdits::ThreadedEditParameters parameters{ g_dag.data, g_colors, *g_recorder };
    HashDagEdits::edit_threaded<true>(0, g_dag.firstNodeIndex, 0, Path(0, 0, 0), editor, parameters);
    std::vector<std::pair<uint64, HashDagEdits::Thread*>> tasks;
    for (auto& it : parameters.threads)
        tasks.emplace_back(morton(it.first, C_colorTreeLevels), it.second.get());
    std::sort(tasks.begin(), tasks.end(),
              [](const std::pair<uint64, HashDagEdits::Thread*>& a, const std::pair<uint64, HashDagEdits::Thread*>& b) {
                  return a.first < b.first;
              });
    for (auto& task : tasks)
        task.second->lambda();
    for (auto& it : parameters.threads)
        parameters.stats += it.second->stats;
    g_dag.firstNodeIndex =
        HashDagEdits::edit_threaded<false>(0, g_dag.firstNodeIndex, 0, Path(0, 0, 0), editor, parameters).nodeIndex;
    stats[0] = parameters.stats.numVoxels;
    stats[1] = parameters.stats.numNodes;
}

// tool: 0 sphere remove, 1 sphere add, 2 box remove, 3 box add
extern "C" int ref_edit(uint32 tool, float cx, float cy, float cz, float radius, uint64* stats)
{
    const float3 c = make_float3(cx, cy, cz);
    switch (tool) {
    case 0: run_edit(SphereEditor<false>(c, radius), stats); break;
    case 1: run_edit(SphereEditor<true>(c, radius), stats); break;
    case 2: run_edit(BoxEditor<false>(c, radius), stats); break;
    case 3: run_edit(BoxEditor<true>(c, radius), stats); break;
    default: return 1;
    }
    return 0;
}

// HashDAG::remove_stale_nodes(levels - 2) (hash_dag.h:407-547), which also
// re-uploads the whole table (a host copy here).
extern "C" void ref_gc() { g_dag.remove_stale_nodes(C_leafLevel); }

// DAGUtils::get_value (dag_utils.h:138-172)
extern "C" int ref_get_value(uint32 x, uint32 y, uint32 z) { return DAGUtils::get_value(g_dag, Path(x, y, z)) ? 1 : 0; }

// HashTable::get_level_size (hash_table.cpp:277-285)
extern "C" uint32 ref_level_size(uint32 level) { return g_dag.data.get_level_size(level); }

// FastNoise known answers: GetPerlinFractal with the seed, frequency and
// octaves SphereNoiseEditor sets (hash_dag_editors.h:724-727).
extern "C" float ref_perlin_fractal(int seed, float frequency, int octaves, float x, float y, float z)
{
    FastNoise noise;
    noise.SetSeed(seed);
    noise.SetFrequency(frequency);
    noise.SetFractalOctaves(octaves);
    return noise.GetPerlinFractal(x, y, z);
}

// Hash known-answer vectors (hash_table.h:80-89).
extern "C" uint32 ref_hash_leaf(uint64 leaf) { return HashDagUtils::hash_leaf(leaf); }
extern "C" uint32 ref_hash_interior(uint32 n, const uint32* node) { return HashDagUtils::hash_interior(n, node); }

#if EDITS_ENABLE_COLORS
// ---------------------------------------------------------------------------
// Colours (built with EDITS_ENABLE_COLORS=1): the scene's voxel colours come
// from the oracle's colour field (the test input, like the scene), packed
// by the reference's own ColorLeafBuilder into a BasicDAGCompressedColors
// main leaf and imported with HashDAGFactory::load_colors_from_DAG.
// ---------------------------------------------------------------------------
extern "C" hd_color or_voxel_color(uint64_t seed, uint32_t x, uint32_t y, uint32_t z);

static void add_voxel_colors(const BasicDAG& dag, uint32 level, uint32 index, uint3 path, uint64 seed,
                             ColorLeafBuilder& builder)
{
    if (level == C_leafLevel) {
        const uint64 leaf = dag.get_leaf(index).to_64();
        for (uint32 bit = 0; bit < 64; bit++) {
            if (!((leaf >> bit) & 1))
                continue;
            const uint32 c1 = bit >> 3, c2 = bit & 7;
            const uint32 x = (path.x << 2) | (((c1 >> 2) & 1) << 1) | ((c2 >> 2) & 1);
            const uint32 y = (path.y << 2) | (((c1 >> 1) & 1) << 1) | ((c2 >> 1) & 1);
            const uint32 z = (path.z << 2) | ((c1 & 1) << 1) | (c2 & 1);
            const hd_color k = or_voxel_color(seed, x, y, z);
            CompressedColor color;
            color.colorBits = k.color_bits;
            color.weight = k.weight;
            color.bitsPerWeight = k.bits_per_weight;
            builder.add(color);
        }
        return;
    }
    const uint32 node = dag.get_node(level, index);
    const uint8 mask = Utils::child_mask(node);
    for (uint8 c = 0; c < 8; c++)
        if (mask & (1u << c))
            add_voxel_colors(dag, level + 1, dag.get_child_index(level, index, mask, c),
                             make_uint3((path.x << 1) | ((c >> 2) & 1), (path.y << 1) | ((c >> 1) & 1),
                                        (path.z << 1) | (c & 1)),
                             seed, builder);
}

// HashDAGFactory::load_from_DAG + load_colors_from_DAG (hash_dag_factory.cpp:
// 150-197) on a BasicDAG and the colour field of `colorSeed`.
// The BasicDAG and its compressed colours of the last ref_load_colored.
static BasicDAG g_basic;
static BasicDAGCompressedColors g_basic_colors;

extern "C" int ref_load_colored(const uint32* words, uint64 nWords, uint32 poolPages, uint64 colorSeed)
{
    if (g_loaded)
        return 1;
    BasicDAG& basic = g_basic;
    basic.data = StaticArray<uint32>::allocate("basic dag", nWords, EMemoryType::CPU);
    std::memcpy(basic.data.data(), words, nWords * sizeof(uint32));
    HashDAGFactory::load_from_DAG(g_dag, basic, poolPages);
    // enclosedLeaves: indexed by the upper header bits of the top levels
    uint32 maxIndex = 0;
    {
        std::vector<std::pair<uint32, uint32>> stack{{0u, 0u}};
        std::unordered_set<uint64> seen;
        while (!stack.empty()) {
            auto [level, index] = stack.back();
            stack.pop_back();
            if (level >= C_colorTreeLevels || !seen.insert((uint64(level) << 32) | index).second)
                continue;
            const uint32 node = basic.get_node(level, index);
            maxIndex = std::max(maxIndex, node >> 8);
            const uint8 mask = Utils::child_mask(node);
            for (uint8 c = 0; c < 8; c++)
                if (mask & (1u << c))
                    stack.push_back({level + 1, basic.get_child_index(level, index, mask, c)});
        }
    }
    BasicDAGCompressedColors& colors = g_basic_colors;
    colors.topLevels = C_colorTreeLevels;
    colors.enclosedLeaves = StaticArray<EnclosedLeavesType>::allocate("enclosed leaves", maxIndex + 1, EMemoryType::CPU);
    std::memset(colors.enclosedLeaves.data(), 0, (maxIndex + 1) * sizeof(EnclosedLeavesType));
    DAGUtils::fix_enclosed_leaves(basic, colors.enclosedLeaves, C_colorTreeLevels);
    ColorLeafBuilder builder;
    add_voxel_colors(basic, 0, 0, make_uint3(0, 0, 0), colorSeed, builder);
    builder.build(colors.leaf, true);
    HashDAGFactory::load_colors_from_DAG(g_colors, basic, colors);
    g_recorder = new StatsRecorder();
    g_loaded = true;
    return 0;
}

// HashDAG::edit_threads with colours (hash_dag.h:255-405), task order as in
// run_edit, colour leaves rebuilt at the end (BENCHMARK: no undo frame).
template<typename TEditor>
static void run_edit_colored(const TEditor& editor, uint64* stats)
{
    HashDagEdits::ThreadedEditParameters parameters{ g_dag.data, g_colors, *g_recorder };
    HashDagEdits::edit_threaded<true>(0, g_dag.firstNodeIndex, 0, Path(0, 0, 0), editor, parameters);
    std::vector<std::pair<uint64, HashDagEdits::Thread*>> tasks;
    for (auto& it : parameters.threads)
        tasks.emplace_back(morton(it.first, C_colorTreeLevels), it.second.get());
    std::sort(tasks.begin(), tasks.end(),
              [](const std::pair<uint64, HashDagEdits::Thread*>& a, const std::pair<uint64, HashDagEdits::Thread*>& b) {
                  return a.first < b.first;
              });
    for (auto& task : tasks)
        task.second->lambda();
    for (auto& it : parameters.threads)
        parameters.stats += it.second->stats;
    g_dag.firstNodeIndex =
        HashDagEdits::edit_threaded<false>(0, g_dag.firstNodeIndex, 0, Path(0, 0, 0), editor, parameters).nodeIndex;
    for (auto& colorToBuild : parameters.colorsToBuild) {
        auto& leaf = g_colors.get_leaf_ref(colorToBuild.newLeafIndex);
        colorToBuild.builder->build(leaf, true);
    }
    g_colors.upload_to_gpu(false);
    stats[0] = parameters.stats.numVoxels;
    stats[1] = parameters.stats.numNodes;
}

// tool: 0..3 as ref_edit, 4 SpherePaintEditor (blue), 5 CopyEditor
// (identity transform, no swirl) moving center +- radius by dest - source,
// 6 / 7 SphereNoiseEditor (isAdding false / true), 8 FillEditorColors
extern "C" int ref_edit_colored(uint32 tool, const float* center, float radius, const float* source,
                                const float* dest, uint64* stats)
{
    const float3 c = make_float3(center[0], center[1], center[2]);
    switch (tool) {
    case 0: run_edit_colored(SphereEditor<false>(c, radius), stats); break;
    case 1: run_edit_colored(SphereEditor<true>(c, radius), stats); break;
    case 2: run_edit_colored(BoxEditor<false>(c, radius), stats); break;
    case 3: run_edit_colored(BoxEditor<true>(c, radius), stats); break;
    case 4: run_edit_colored(SpherePaintEditor(c, radius), stats); break;
    case 5: {
        const Matrix3x3 identity = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        run_edit_colored(CopyEditor(g_dag, g_colors, make_float3(source[0], source[1], source[2]),
                                    make_float3(dest[0], dest[1], dest[2]), c, radius, identity, *g_recorder, false,
                                    0.0f),
                         stats);
        break;
    }
    case 6: run_edit_colored(SphereNoiseEditor(g_dag, c, radius, false), stats); break;
    case 7: run_edit_colored(SphereNoiseEditor(g_dag, c, radius, true), stats); break;
    case 8: run_edit_colored(FillEditorColors(g_dag, g_colors, c, radius), stats); break;
    default: return 1;
    }
    return 0;
}

// The reference's own file writers on the state of ref_load_colored (and the
// edits since, for the hash-DAG file): BasicDAGFactory::save_dag_to_file,
// save_compressed_colors_to_file (basic_dag.cpp:34-103) and
// HashDAGFactory::save_dag_to_file (hash_dag_factory.cpp:199-222).  The
// DAGInfo is the scene's cube [0, 2^depth].
extern "C" int ref_save_files(const char* dagPath, const char* colorsPath, const char* hashPath)
{
    if (!g_loaded)
        return 1;
    DAGInfo info;
    info.boundsAABBMin = Vector3(0, 0, 0);
    info.boundsAABBMax = Vector3(double(1u << MAX_LEVELS), double(1u << MAX_LEVELS), double(1u << MAX_LEVELS));
    if (dagPath)
        BasicDAGFactory::save_dag_to_file(info, g_basic, dagPath);
    if (colorsPath)
        BasicDAGFactory::save_compressed_colors_to_file(g_basic_colors, colorsPath);
    if (hashPath)
        HashDAGFactory::save_dag_to_file(info, g_dag, hashPath);
    return 0;
}

// The reference's loaders: BasicDAGFactory::load_dag_from_file and
// load_compressed_colors_from_file, then load_from_DAG and
// load_colors_from_DAG (a fresh process: the table is a singleton).
extern "C" int ref_load_files(const char* dagPath, const char* colorsPath, uint32 poolPages)
{
    if (g_loaded)
        return 1;
    DAGInfo info;
    BasicDAGFactory::load_dag_from_file(info, g_basic, dagPath);
    BasicDAGFactory::load_compressed_colors_from_file(g_basic_colors, colorsPath);
    HashDAGFactory::load_from_DAG(g_dag, g_basic, poolPages);
    HashDAGFactory::load_colors_from_DAG(g_colors, g_basic, g_basic_colors);
    g_recorder = new StatsRecorder();
    g_loaded = true;
    return 0;
}

// ---------------------------------------------------------------------------
// Replays: the reference's ReplayManager (replay.h, header only) reading and
// writing CSV.  The actions' apply() bodies live in replay.cpp with the
// engine; parsing and writing never call them, so they are empty here.
// ---------------------------------------------------------------------------
void ReplayActionUndo::apply() {}
void ReplayActionRedo::apply() {}
void ReplayActionSetLocation::apply() {}
void ReplayActionSetRotation::apply() {}
void ReplayActionSetToolParameters::apply() {}
void ReplayActionSphere::apply() {}
void ReplayActionCube::apply() {}
void ReplayActionCopy::apply() {}
void ReplayActionFill::apply() {}
void ReplayActionPaint::apply() {}
static ReplayManager g_replay;

extern "C" int ref_replay_load(const char* path)
{
    g_replay.load_csv(path);
    return 0;
}
extern "C" int ref_replay_write(const char* path)
{
    std::ofstream os(path, std::ios::binary);
    g_replay.write_csv(os);
    return os.good() ? 0 : 1;
}
extern "C" uint64 ref_replay_count() { return g_replay.actions.size(); }
extern "C" uint64 ref_replay_frames() { return g_replay.numFrames; }
// Action i as its type and its fields as doubles in declaration order
// (booleans as 0 / 1, uint3 and uint32 fields as their values).
extern "C" uint32 ref_replay_action(uint64 i, double* v, uint32* n)
{
    IReplayAction* a = g_replay.actions[i].get();
    uint32 k = 0;
    auto put = [&](double x) { v[k++] = x; };
    switch (a->type) {
    case EReplayActionType::SetLocation: {
        auto& b = static_cast<ReplayActionSetLocation&>(*a);
        put(b.location.X), put(b.location.Y), put(b.location.Z);
        break;
    }
    case EReplayActionType::SetRotation: {
        auto& b = static_cast<ReplayActionSetRotation&>(*a);
        const Matrix3x3& m = b.rotation;
        put(m.D00), put(m.D01), put(m.D02), put(m.D10), put(m.D11), put(m.D12), put(m.D20), put(m.D21), put(m.D22);
        break;
    }
    case EReplayActionType::SetToolParameters: {
        auto& b = static_cast<ReplayActionSetToolParameters&>(*a);
        put(b.path.x), put(b.path.y), put(b.path.z), put(b.copySourcePath.x), put(b.copySourcePath.y),
            put(b.copySourcePath.z), put(b.copyDestPath.x), put(b.copyDestPath.y), put(b.copyDestPath.z),
            put(b.radius), put(b.tool);
        break;
    }
    case EReplayActionType::EditSphere: {
        auto& b = static_cast<ReplayActionSphere&>(*a);
        put(b.location.x), put(b.location.y), put(b.location.z), put(b.radius), put(b.add);
        break;
    }
    case EReplayActionType::EditCube: {
        auto& b = static_cast<ReplayActionCube&>(*a);
        put(b.location.x), put(b.location.y), put(b.location.z), put(b.radius), put(b.add);
        break;
    }
    case EReplayActionType::EditCopy: {
        auto& b = static_cast<ReplayActionCopy&>(*a);
        put(b.location.x), put(b.location.y), put(b.location.z), put(b.src.x), put(b.src.y), put(b.src.z),
            put(b.dest.x), put(b.dest.y), put(b.dest.z), put(b.radius);
        const Matrix3x3& m = b.transform;
        put(m.D00), put(m.D01), put(m.D02), put(m.D10), put(m.D11), put(m.D12), put(m.D20), put(m.D21), put(m.D22);
        put(b.enableSwirl), put(b.swirlPeriod);
        break;
    }
    case EReplayActionType::EditFill: {
        auto& b = static_cast<ReplayActionFill&>(*a);
        put(b.location.x), put(b.location.y), put(b.location.z), put(b.radius);
        break;
    }
    case EReplayActionType::EditPaint: {
        auto& b = static_cast<ReplayActionPaint&>(*a);
        put(b.location.x), put(b.location.y), put(b.location.z), put(b.radius);
        break;
    }
    default:
        break;
    }
    *n = k;
    return uint32(a->type);
}

// DAGUtils::get_color (dag_utils.h:423-523): colour bits, weight, bits per weight
extern "C" void ref_get_color(uint32 x, uint32 y, uint32 z, uint32* out)
{
    const CompressedColor k = DAGUtils::get_color(g_dag, g_colors, Path(x, y, z));
    out[0] = k.colorBits;
    out[1] = k.weight;
    out[2] = k.bitsPerWeight;
}
#endif
