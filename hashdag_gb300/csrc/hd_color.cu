// Colours: the colour table of a context, its construction from a generated
// scene, queries (DAGUtils::get_color, dag_utils.h:423-523), the colour pass
// over traced paths (the colour lookup of Tracer::trace_colors,
// tracer.cu:254-451), and the colour phase of an edit.
//
// Colour phase of an edit (HashDagEdits::edit_leaf's colour side,
// hash_dag_edits.h:335-643, and the rebuild in HashDAG::edit_threads,
// hash_dag.h:380-400): every level-C_colorTreeLevels entry the tool touches is
// a task whose new colour sequence (the voxels of its subtree in depth-first
// order) is assembled from the old leaf (untouched subtrees and unchanged
// voxels), the tool's colour (filled subtrees and edited voxels) and nothing
// (carved subtrees); the sequence is then packed as ColorLeafBuilder packs it
// (a block at every colour change and macro-block start, MSB-first weights,
// byte-swapped words) into a leaf, new slots get colour nodes and leaves
// as edit_threaded allocates them, and the replaced leaves go to an undo
// frame (HashDAGUndoRedo, hash_dag.h:20-212).
#include <functional>
#include <vector>

#include "hd_color.cuh"
#include "hd_edit.cuh"

namespace hd {

// ---- table storage --------------------------------------------------------------

static void grow_buffer(void** ptr, uint64_t old_bytes, uint64_t new_bytes, cudaStream_t st)
{
    void* p = nullptr;
    if (cudaMalloc(&p, new_bytes) != cudaSuccess) {
        cudaGetLastError();
        throw StatusError{HD_ERR_OOM, "colour pool allocation failed"};
    }
    HD_CUDA(cudaMemsetAsync(p, 0, new_bytes, st));
    if (*ptr && old_bytes)
        HD_CUDA(cudaMemcpyAsync(p, *ptr, old_bytes, cudaMemcpyDeviceToDevice, st));
    HD_CUDA(cudaStreamSynchronize(st));
    if (*ptr)
        cudaFree(*ptr);
    *ptr = p;
}

// Makes room for `add` more entries of each pool (host mirror of the device
// counters in c->ctop).
void color_reserve(hd_ctx* c, const uint64_t add[5])
{
    ColorTable& ct = c->ct;
    cudaStream_t st = c->stream;
    uint64_t* caps[5] = {&ct.cap_nodes, &ct.cap_leaves, &ct.cap_blocks, &ct.cap_macros, &ct.cap_weights};
    void** ptrs[5] = {reinterpret_cast<void**>(&ct.nodes), reinterpret_cast<void**>(&ct.leaves),
                      reinterpret_cast<void**>(&ct.blocks), reinterpret_cast<void**>(&ct.macros),
                      reinterpret_cast<void**>(&ct.weights)};
    const uint64_t elem[5] = {4, sizeof(LeafDesc), 8, 8, 4};
    for (int k = 0; k < 5; k++) {
        const uint64_t need = c->ctop[k] + add[k] + 8; // + padding: extract_bits reads a byte past the end
        if (need <= *caps[k] && *ptrs[k])
            continue;
        uint64_t cap = *caps[k] ? *caps[k] : 1024;
        while (cap < need)
            cap = cap + cap / 2 + 1024;
        grow_buffer(ptrs[k], *caps[k] * elem[k], cap * elem[k], st);
        *caps[k] = cap;
    }
    if (!ct.top) {
        HD_CUDA(cudaMalloc(&ct.top, 8 * sizeof(unsigned long long)));
        HD_CUDA(cudaMemsetAsync(ct.top, 0, 8 * sizeof(unsigned long long), st));
    }
}

void color_release(hd_ctx* c)
{
    ColorTable& ct = c->ct;
    cudaFree(ct.nodes);
    cudaFree(ct.leaves);
    cudaFree(ct.blocks);
    cudaFree(ct.macros);
    cudaFree(ct.weights);
    cudaFree(ct.top);
    ct = ColorTable{};
    for (auto& v : c->ctop)
        v = 0;
    c->colors = false;
}

static void sync_tops(hd_ctx* c)
{
    unsigned long long t[8];
    HD_CUDA(cudaMemcpyAsync(t, c->ct.top, sizeof(t), cudaMemcpyDeviceToHost, c->stream));
    HD_CUDA(cudaStreamSynchronize(c->stream));
    for (int k = 0; k < 5; k++)
        c->ctop[k] = t[k];
}

// ---- import from a scene ------------------------------------------------------

struct PathLevel {
    uint32_t* node; // DAG node index
    uint32_t* x;
    uint32_t* y;
    uint32_t* z;
    uint32_t* nkids; // present children
    uint32_t* first; // exclusive scan of nkids
    uint64_t* base;  // leavesCount of create_hash_dag_colors at the path (file import only)
};

// Leaves under a node (BasicDAGColorsBase::get_leaves_count, basic_dag.h:
// 60-74): an index into enclosedLeaves above topLevels, the count itself
// below.  An index past the array sets *bad.
struct LeavesCount {
    const uint64_t* enclosed;
    uint64_t n_enclosed;
    uint32_t top_levels;
    uint32_t* bad;
    HD_D uint64_t operator()(uint32_t level, uint32_t header) const
    {
        const uint32_t upper = header >> 8;
        if (level >= top_levels)
            return upper;
        if (upper >= n_enclosed) {
            atomicExch(bad, 1u);
            return 0;
        }
        return enclosed[upper];
    }
};

__global__ void k_path_children(Table t, PathLevel lv, uint32_t n)
{
    HD_GRID_STRIDE(i, n) lv.nkids[i] = popc32(t.sys(lv.node[i])[0] & 0xffu);
}

// children of the level's paths, in child order; colour-tree entries of the
// level: nodes[8 * (node_base + i) + c] = child's colour node, or at level
// T - 1 the leaf of the child (leaf_base + its index at level T)
// With leaves counts (the file import), each child also gets its base: the
// path's base plus the leaves of its earlier siblings (the running
// leavesCount of create_hash_dag_colors, hash_dag_factory.cpp:100-147).
__global__ void k_path_expand(Table t, ColorTable ct, PathLevel lv, uint32_t n, PathLevel next, uint64_t node_base,
                              uint64_t next_node_base, bool last_tree_level, uint32_t level, LeavesCount count)
{
    HD_GRID_STRIDE(i, n)
    {
        const uint32_t* p = t.sys(lv.node[i]);
        const uint32_t mask = p[0] & 0xffu;
        uint32_t o = lv.first[i], k = 1;
        uint64_t running = lv.base ? lv.base[i] : 0;
        for (uint32_t c = 0; c < 8; c++) {
            if (!(mask & (1u << c)))
                continue;
            next.node[o] = p[k++];
            if (lv.base) {
                next.base[o] = running;
                running += count(level + 1, t.sys(next.node[o])[0]);
            }
            next.x[o] = (lv.x[i] << 1) | ((c >> 2) & 1);
            next.y[o] = (lv.y[i] << 1) | ((c >> 1) & 1);
            next.z[o] = (lv.z[i] << 1) | (c & 1);
            ct.nodes[8 * (node_base + i) + c] =
                last_tree_level ? (kLeafFlag | o) : uint32_t(8 * (next_node_base + o));
            o++;
        }
    }
}

// Depth-first voxels of one level-T subtree, in the reference's colour order
// (children in order, leaf bits in index order); calls f(x, y, z).
template <typename F>
HD_D void for_each_voxel(const Table& t, uint32_t node, uint32_t px, uint32_t py, uint32_t pz, F&& f)
{
    const uint32_t T = t.g.T, leafl = t.g.leaf_level;
    struct Frame {
        uint32_t node, x, y, z, next;
    } stack[HD_MAX_DEPTH];
    int sp = 0;
    stack[sp++] = Frame{node, px, py, pz, 0};
    while (sp) {
        Frame& fr = stack[sp - 1];
        const uint32_t level = T + uint32_t(sp) - 1;
        const uint32_t* p = t.sys(fr.node);
        if (level == leafl) {
            const uint64_t leaf = uint64_t(p[0]) | (uint64_t(p[1]) << 32);
            for (uint32_t bit = 0; bit < 64; bit++) {
                if (!((leaf >> bit) & 1))
                    continue;
                const uint32_t c1 = bit >> 3, c2 = bit & 7;
                f((fr.x << 2) | (((c1 >> 2) & 1) << 1) | ((c2 >> 2) & 1),
                  (fr.y << 2) | (((c1 >> 1) & 1) << 1) | ((c2 >> 1) & 1), (fr.z << 2) | ((c1 & 1) << 1) | (c2 & 1));
            }
            sp--;
            continue;
        }
        const uint32_t mask = p[0] & 0xffu;
        while (fr.next < 8 && !(mask & (1u << fr.next)))
            fr.next++;
        if (fr.next == 8) {
            sp--;
            continue;
        }
        const uint32_t c = fr.next++;
        stack[sp++] = Frame{p[child_offset(mask, c)], (fr.x << 1) | ((c >> 2) & 1), (fr.y << 1) | ((c >> 1) & 1),
                            (fr.z << 1) | (c & 1), 0};
    }
}

// pass 1: blocks of each slot leaf
__global__ void k_slot_count(Table t, PathLevel lv, uint32_t n, uint64_t seed, uint32_t* nb, uint32_t* nm)
{
    HD_GRID_STRIDE(i, n)
    {
        uint32_t k = 0, blocks = 0;
        uint64_t last = ~0ull;
        for_each_voxel(t, lv.node[i], lv.x[i], lv.y[i], lv.z[i], [&](uint32_t x, uint32_t y, uint32_t z) {
            const uint64_t col = voxel_color(seed, x, y, z);
            if (k % kColorsPerMacro == 0 || col != last)
                blocks++;
            last = col;
            k++;
        });
        nb[i] = blocks;
        nm[i] = 2 * ((k + kColorsPerMacro - 1) / kColorsPerMacro);
    }
}

// pass 2: blocks, macro blocks and descriptor of each slot leaf
__global__ void k_slot_write(Table t, ColorTable ct, PathLevel lv, uint32_t n, uint64_t seed, const uint32_t* bo,
                             const uint32_t* mo, const uint32_t* nb, const uint32_t* nm, uint64_t block_base,
                             uint64_t macro_base)
{
    HD_GRID_STRIDE(i, n)
    {
        uint64_t* blocks = ct.blocks + block_base + bo[i];
        uint64_t* macros = ct.macros + macro_base + mo[i];
        uint32_t k = 0, b = 0;
        uint64_t last = ~0ull;
        for_each_voxel(t, lv.node[i], lv.x[i], lv.y[i], lv.z[i], [&](uint32_t x, uint32_t y, uint32_t z) {
            const uint64_t col = voxel_color(seed, x, y, z);
            if (k % kColorsPerMacro == 0) {
                macros[2 * (k / kColorsPerMacro)] = b;
                macros[2 * (k / kColorsPerMacro) + 1] = 0;
            }
            if (k % kColorsPerMacro == 0 || col != last)
                blocks[b++] = (uint64_t(pc_bits(col)) << 32) | make_block_header(0, 0, k % kColorsPerMacro);
            last = col;
            k++;
        });
        LeafDesc d{};
        d.blocks = block_base + bo[i];
        d.macros = macro_base + mo[i];
        d.weights = 0;
        d.nb = nb[i];
        d.nm = nm[i];
        d.nw = 0;
        ct.leaves[i] = d;
    }
}

// The colour tree above C_colorTreeLevels of the context's current scene: one
// colour node per path (layout of create_hash_dag_colors,
// hash_dag_factory.cpp:100-147, in breadth-first order) whose level T - 1
// entries name the leaves 0.. of the level-T paths, returned in lv[T] (with
// their bases when `count` has leaves counts).
static uint64_t color_tree(hd_ctx* c, std::vector<PathLevel>& lv, std::vector<uint32_t>& n, const LeavesCount& count)
{
    cudaStream_t st = c->stream;
    Scratch& s = c->scratch;
    const uint32_t T = c->g.T;
    const bool with_base = count.bad != nullptr;
    lv.assign(T + 1, PathLevel{});
    n.assign(T + 1, 0);
    uint32_t* d_n = s.get<uint32_t>("col_n", 4);
    auto alloc = [&](uint32_t L, uint64_t cnt) {
        char a[32];
        PathLevel p{};
        uint32_t** f[6] = {&p.node, &p.x, &p.y, &p.z, &p.nkids, &p.first};
        const char* names[6] = {"node", "x", "y", "z", "nk", "first"};
        for (int k = 0; k < 6; k++) {
            snprintf(a, sizeof(a), "col_%s_%u", names[k], L);
            *f[k] = s.get<uint32_t>(a, cnt + 1);
        }
        if (with_base) {
            snprintf(a, sizeof(a), "col_base_%u", L);
            p.base = s.get<uint64_t>(a, cnt + 1);
        }
        return p;
    };
    lv[0] = alloc(0, 1);
    const uint32_t zero = 0, root = c->root;
    HD_CUDA(cudaMemcpyAsync(lv[0].node, &root, 4, cudaMemcpyHostToDevice, st));
    HD_CUDA(cudaMemcpyAsync(lv[0].x, &zero, 4, cudaMemcpyHostToDevice, st));
    HD_CUDA(cudaMemcpyAsync(lv[0].y, &zero, 4, cudaMemcpyHostToDevice, st));
    HD_CUDA(cudaMemcpyAsync(lv[0].z, &zero, 4, cudaMemcpyHostToDevice, st));
    if (with_base)
        HD_CUDA(cudaMemsetAsync(lv[0].base, 0, 8, st));
    n[0] = 1;
    std::vector<uint64_t> node_base(T + 1, 0);
    for (uint32_t L = 0; L < T; L++) {
        k_path_children<<<grid_for(n[L], 256), 256, 0, st>>>(c->t, lv[L], n[L]);
        HD_LAUNCH_CHECK();
        exclusive_scan<uint32_t, uint32_t>(s, lv[L].nkids, lv[L].first, n[L], d_n, st);
        n[L + 1] = read_scalar(d_n, st);
        lv[L + 1] = alloc(L + 1, n[L + 1]);
        node_base[L + 1] = node_base[L] + n[L];
        // the colour nodes of this level's paths, then the next level's paths
        const uint64_t add[5] = {8 * node_base[L + 1], L + 1 == T ? n[T] : 0, 0, 0, 0};
        color_reserve(c, add);
        k_path_expand<<<grid_for(n[L], 256), 256, 0, st>>>(c->t, c->ct, lv[L], n[L], lv[L + 1], node_base[L],
                                                            node_base[L + 1], L + 1 == T, L, count);
        HD_LAUNCH_CHECK();
    }
    return node_base[T];
}

// The colour tree of the context's current scene with one leaf per path at
// C_colorTreeLevels holding its voxels' colours from the colour field.
void colors_from_scene(hd_ctx* c, uint64_t color_seed)
{
    cudaStream_t st = c->stream;
    Scratch& s = c->scratch;
    const Geom& g = c->g;
    const uint32_t T = g.T;
    if (T == 0 || T >= g.leaf_level)
        throw StatusError{HD_ERR_INVALID, "colours need 0 < C_colorTreeLevels < leaf level"};
    if (c->root == kInvalid)
        throw StatusError{HD_ERR_STATE, "empty scene"};
    color_release(c);
    std::vector<PathLevel> lv;
    std::vector<uint32_t> n;
    const uint64_t tree_nodes = color_tree(c, lv, n, LeavesCount{});
    // slot leaves
    const uint32_t ns = n[T];
    uint32_t* nb = s.get<uint32_t>("col_nb", uint64_t(ns) + 1);
    uint32_t* nm = s.get<uint32_t>("col_nm", uint64_t(ns) + 1);
    uint32_t* bo = s.get<uint32_t>("col_bo", uint64_t(ns) + 1);
    uint32_t* mo = s.get<uint32_t>("col_mo", uint64_t(ns) + 1);
    k_slot_count<<<grid_for(ns, 128), 128, 0, st>>>(c->t, lv[T], ns, color_seed, nb, nm);
    HD_LAUNCH_CHECK();
    uint32_t* d_tot = s.get<uint32_t>("col_tot", 4);
    exclusive_scan<uint32_t, uint32_t>(s, nb, bo, ns, d_tot, st);
    exclusive_scan<uint32_t, uint32_t>(s, nm, mo, ns, d_tot + 1, st);
    uint32_t tot[2];
    HD_CUDA(cudaMemcpyAsync(tot, d_tot, 8, cudaMemcpyDeviceToHost, st));
    HD_CUDA(cudaStreamSynchronize(st));
    const uint64_t add1[5] = {8 * tree_nodes, ns, tot[0], tot[1], 0};
    color_reserve(c, add1);
    k_slot_write<<<grid_for(ns, 128), 128, 0, st>>>(c->t, c->ct, lv[T], ns, color_seed, bo, mo, nb, nm, 0, 0);
    HD_LAUNCH_CHECK();
    const unsigned long long tops[5] = {8 * tree_nodes, ns, tot[0], tot[1], 0};
    HD_CUDA(cudaMemcpyAsync(c->ct.top, tops, sizeof(tops), cudaMemcpyHostToDevice, st));
    HD_CUDA(cudaStreamSynchronize(st));
    for (int k = 0; k < 5; k++)
        c->ctop[k] = tops[k];
    c->colors = true;
    c->color_seed = color_seed;
}

// Slot leaves as views of the main leaf: colour i of slot k is colour
// base[k] + i of the main leaf.
__global__ void k_slot_shared(ColorTable ct, PathLevel lv, uint32_t n, uint32_t nb, uint32_t nm, uint32_t nw)
{
    HD_GRID_STRIDE(i, n)
    {
        LeafDesc d{};
        d.base = lv.base[i];
        d.nb = nb;
        d.nm = nm;
        d.nw = nw;
        ct.leaves[i] = d;
    }
}

// HashDAGFactory::load_colors_from_DAG (hash_dag_factory.cpp:186-197) for a
// BasicDAGCompressedColors main leaf (weights already byte-swapped as the
// leaf decoder reads them) and its enclosedLeaves, on the table imported from
// the same BasicDAG: the colour tree, and at C_colorTreeLevels a view of the
// main leaf per path at the running leaves count.
void colors_from_main_leaf(hd_ctx* c, uint32_t top_levels, const std::vector<uint64_t>& enclosed,
                           const std::vector<uint32_t>& weights, const std::vector<uint64_t>& blocks,
                           const std::vector<uint64_t>& macros)
{
    cudaStream_t st = c->stream;
    Scratch& s = c->scratch;
    const uint32_t T = c->g.T;
    if (T == 0 || T >= c->g.leaf_level)
        throw StatusError{HD_ERR_INVALID, "colours need 0 < C_colorTreeLevels < leaf level"};
    if (top_levels > T)
        throw StatusError{HD_ERR_INVALID, "C_colorTreeLevels is lower than the file's topLevels"};
    if (c->root == kInvalid)
        throw StatusError{HD_ERR_STATE, "empty scene"};
    if (blocks.size() >= (1ull << 32) || macros.size() >= (1ull << 32) || weights.size() >= (1ull << 32))
        throw StatusError{HD_ERR_INVALID, "colour leaf too large"};
    color_release(c);
    uint64_t* d_enc = s.get<uint64_t>("col_enclosed", enclosed.size() + 1);
    if (!enclosed.empty())
        HD_CUDA(cudaMemcpyAsync(d_enc, enclosed.data(), enclosed.size() * 8, cudaMemcpyHostToDevice, st));
    uint32_t* bad = s.get<uint32_t>("col_bad", 1);
    HD_CUDA(cudaMemsetAsync(bad, 0, 4, st));
    std::vector<PathLevel> lv;
    std::vector<uint32_t> n;
    const uint64_t tree_nodes = color_tree(c, lv, n, LeavesCount{d_enc, enclosed.size(), top_levels, bad});
    uint32_t h_bad = 0;
    HD_CUDA(cudaMemcpyAsync(&h_bad, bad, 4, cudaMemcpyDeviceToHost, st));
    HD_CUDA(cudaStreamSynchronize(st));
    if (h_bad)
        throw StatusError{HD_ERR_INVALID, "a node's enclosedLeaves index is past the file's array"};
    const uint32_t ns = n[T];
    const uint64_t add[5] = {8 * tree_nodes, ns, blocks.size(), macros.size(), weights.size()};
    color_reserve(c, add);
    if (!blocks.empty())
        HD_CUDA(cudaMemcpyAsync(c->ct.blocks, blocks.data(), blocks.size() * 8, cudaMemcpyHostToDevice, st));
    if (!macros.empty())
        HD_CUDA(cudaMemcpyAsync(c->ct.macros, macros.data(), macros.size() * 8, cudaMemcpyHostToDevice, st));
    if (!weights.empty())
        HD_CUDA(cudaMemcpyAsync(c->ct.weights, weights.data(), weights.size() * 4, cudaMemcpyHostToDevice, st));
    k_slot_shared<<<grid_for(ns, 256), 256, 0, st>>>(c->ct, lv[T], ns, uint32_t(blocks.size()),
                                                     uint32_t(macros.size()), uint32_t(weights.size()));
    HD_LAUNCH_CHECK();
    const unsigned long long tops[5] = {8 * tree_nodes, ns, blocks.size(), macros.size(), weights.size()};
    HD_CUDA(cudaMemcpyAsync(c->ct.top, tops, sizeof(tops), cudaMemcpyHostToDevice, st));
    HD_CUDA(cudaStreamSynchronize(st));
    for (int k = 0; k < 5; k++)
        c->ctop[k] = tops[k];
    c->colors = true;
    c->color_seed = 0;
}

// ---- queries ----------------------------------------------------------------------

__global__ void k_get_colors(Table t, ColorTable ct, const uint32_t* __restrict__ root, const uint32_t* xyz,
                             uint64_t n, hd_color* out)
{
    const uint32_t r = *root;
    HD_GRID_STRIDE(i, n)
    {
        const uint64_t col = get_color(t, ct, r, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
        hd_color k;
        k.color_bits = pc_bits(col);
        k.weight = uint8_t(pc_weight(col));
        k.bits_per_weight = uint8_t(pc_bpw(col));
        k.reserved = 0;
        out[i] = k;
    }
}

void get_colors(hd_ctx* c, const uint32_t* d_xyz, uint64_t n, hd_color* d_out)
{
    if (!c->colors)
        throw StatusError{HD_ERR_STATE, "the context has no colours"};
    if (!n)
        return;
    k_get_colors<<<grid_for(n, 256), 256, 0, c->stream>>>(c->t, c->ct, c->d_root, d_xyz, n, d_out);
    HD_LAUNCH_CHECK();
}

// ToolInfo::strength (tracer.h:51-77): how close the pixel's voxel is to
// the tool (> 0 inside)
HD_D float sphere_strength(const uint32_t pos[3], uint4 p, float radius)
{
    const float dx = float(pos[0]) - float(p.x), dy = float(pos[1]) - float(p.y), dz = float(pos[2]) - float(p.z);
    return 1 - sqrtf(dx * dx + dy * dy + dz * dz) / radius;
}
HD_D float cube_strength(const uint32_t pos[3], uint4 p, float radius)
{
    const float dx = fabsf(float(pos[0]) - float(p.x)), dy = fabsf(float(pos[1]) - float(p.y)),
                dz = fabsf(float(pos[2]) - float(p.z));
    const float m = dx > (dy > dz ? dy : dz) ? dx : (dy > dz ? dy : dz);
    return 1 - m / radius;
}
HD_D float tool_strength(const hd_tool_overlay& o, uint4 p)
{
    switch (o.tool) {
    case HD_OVERLAY_SPHERE:
    case HD_OVERLAY_SPHERE_PAINT:
    case HD_OVERLAY_SPHERE_NOISE:
        return sphere_strength(o.position, p, o.radius);
    case HD_OVERLAY_CUBE:
        return cube_strength(o.position, p, o.radius);
    default: {
        const float a = sphere_strength(o.copy_source, p, 3), b = sphere_strength(o.copy_dest, p, 3);
        const float m = a > b ? a : b, c = cube_strength(o.position, p, o.radius);
        return m > c ? m : c;
    }
    }
}

// Tracer::trace_colors (tracer.cu:254-451) for one pixel of the paths image:
// the sky for a miss, 0xFF00FF where the path leaves the DAG, a checker for
// a voxel without a valid colour, else the voxel's colour (or the debug
// view), pulled toward red under the tool when the overlay is on.
HD_D uint32_t trace_color(const Table& t, const ColorTable& ct, uint32_t root, uint4 p,
                          const hd_trace_colors_params& q)
{
    if (!(p.x | p.y | p.z))
        return f3_to_rgb888(F3{187 / 255.f, 242 / 255.f, 250 / 255.f});
    const float strength = q.overlay.enabled ? tool_strength(q.overlay, p) : 0.f;
    auto out = [&](uint32_t color) {
        if (q.overlay.enabled && strength > 0) {
            const F3 a = F3{float((color >> 0) & 0xFF) / 255.0f, float((color >> 8) & 0xFF) / 255.0f,
                            float((color >> 16) & 0xFF) / 255.0f};
            const float f = clampf(100 * strength, 0.f, .5f);
            color = f3_to_rgb888(F3{a.x * (1 - f) + 1 * f, a.y * (1 - f) + 0 * f, a.z * (1 - f) + 0 * f});
        }
        return color;
    };
    auto invalid = [&]() {
        const float b = float((p.x ^ p.y ^ p.z) & 1u);
        return out(f3_to_rgb888(F3{1, b, 1.f - b}));
    };
    const uint32_t D = t.g.depth, T = t.g.T, leafl = t.g.leaf_level;
    const bool tree_debug = q.debug_colors == HD_DEBUG_INDEX || q.debug_colors == HD_DEBUG_POSITION ||
                            q.debug_colors == HD_DEBUG_COLOR_TREE;
    uint64_t nof = 0;
    uint32_t debug_index = 0, cn = 0;
    const LeafDesc* leaf = nullptr;
    uint32_t index = root;
    for (uint32_t level = 0; level < leafl;) {
        level++;
        const uint32_t* node = t.sys(index);
        const uint32_t mask = node[0] & 0xffu;
        const uint32_t sh = D - level;
        const uint32_t child = (((p.x >> sh) & 1) << 2) | (((p.y >> sh) & 1) << 1) | ((p.z >> sh) & 1);
        if (!(mask & (1u << child)))
            return out(0xFF00FFu);
        if (level - 1 < T) {
            cn = ct.nodes[cn + child];
            if (level == T)
                leaf = (cn & kLeafFlag) ? ct.leaves + (cn & ~kLeafFlag) : nullptr;
            else if (!cn)
                return invalid();
        }
        if (tree_debug) {
            if (q.debug_colors == HD_DEBUG_INDEX && q.debug_level == level - 1)
                debug_index = index;
            if (level == leafl) {
                if (q.debug_level == leafl)
                    debug_index = node[child_offset(mask, child)];
                if (q.debug_colors == HD_DEBUG_INDEX)
                    return out(murmur32(debug_index)); // Utils::murmurhash32 (utils.h:68-76)
                if (q.debug_colors == HD_DEBUG_POSITION) {
                    float c = float((p.x ^ p.y ^ p.z) & 0x7FFu) / float(0x7FF);
                    c = float((double(c) + 0.5) / 2);
                    return out(f3_to_rgb888((index & kLeafFlag) ? F3{c, 0, 0} : F3{c, c, c}));
                }
                const uint32_t off = D - T;
                const float c = float(((p.x >> off) ^ (p.y >> off) ^ (p.z >> off)) & 1u);
                return out(f3_to_rgb888(F3{c, c, c}));
            }
            index = node[child_offset(mask, child)];
            continue;
        }
        if (level == leafl) {
            for (uint32_t cb = 0; cb < child; cb++)
                if (mask & (1u << cb)) {
                    const uint32_t* lp = t.sys(node[child_offset(mask, cb)]);
                    nof += popc32(lp[0]) + popc32(lp[1]);
                }
            const uint32_t* lp = t.sys(node[child_offset(mask, child)]);
            const uint64_t bits = uint64_t(lp[0]) | (uint64_t(lp[1]) << 32);
            const uint32_t bi = ((p.x & 1) ? 4 : 0) | ((p.y & 1) ? 2 : 0) | ((p.z & 1) ? 1 : 0) | ((p.x & 2) ? 32 : 0) |
                                ((p.y & 2) ? 16 : 0) | ((p.z & 2) ? 8 : 0);
            nof += popc64(bits & ((1ull << bi) - 1));
            break;
        }
        if (level > T)
            for (uint32_t cb = 0; cb < child; cb++)
                if (mask & (1u << cb))
                    nof += t.sys(node[child_offset(mask, cb)])[0] >> 8;
        index = node[child_offset(mask, child)];
    }
    if (!leaf || !leaf_valid_index(*leaf, nof))
        return invalid();
    const uint64_t col = leaf_color(ct, *leaf, nof);
    switch (q.debug_colors) {
    case HD_DEBUG_COLOR_BITS:
        return out(0u); // get_debug_hash: 0 without COLOR_DEBUG (the benchmark build)
    case HD_DEBUG_MIN_COLOR:
        return out(f3_to_rgb888(rgb565_to_f3(pc_bits(col) & 0xFFFF)));
    case HD_DEBUG_MAX_COLOR:
        return out(f3_to_rgb888(rgb565_to_f3((pc_bits(col) >> 16) & 0xFFFF)));
    case HD_DEBUG_WEIGHT: {
        const float w = pc_bpw(col) ? float(pc_weight(col)) / float((1 << pc_bpw(col)) - 1) : 0.f;
        return out(f3_to_rgb888(F3{w, w, w}));
    }
    default:
        return out(f3_to_rgb888(color_value(col)));
    }
}

__global__ void k_trace_colors(Table t, ColorTable ct, const uint32_t* __restrict__ root, const uint4* paths,
                               uint64_t n, uint32_t* rgba, hd_trace_colors_params q)
{
    const uint32_t r = *root;
    HD_GRID_STRIDE(i, n) rgba[i] = trace_color(t, ct, r, paths[i], q);
}

void trace_colors(hd_ctx* c, const uint32_t* d_paths, uint32_t w, uint32_t h, uint32_t* d_rgba, cudaStream_t stream,
                  const uint32_t* d_root, const hd_trace_colors_params* params)
{
    if (!c->colors)
        throw StatusError{HD_ERR_STATE, "the context has no colours"};
    const uint64_t n = uint64_t(w) * h;
    const hd_trace_colors_params q = params ? *params : hd_trace_colors_params{};
    k_trace_colors<<<grid_for(n, 256), 256, 0, stream ? stream : c->stream>>>(
        c->t, c->ct, d_root ? d_root : c->d_root, reinterpret_cast<const uint4*>(d_paths), n, d_rgba, q);
    HD_LAUNCH_CHECK();
}

// ---- the copy tool's source region -------------------------------------------------

// values / colours of the box [start, start + size)^3 before the edit; as
// DAGUtils::get_values (dag_utils.h:264-283) a voxel whose x, y or z equals
// the start is never written (its inclusive-bounds overlap test) and stays 0.
__global__ void k_copy_source(Table t, ColorTable ct, bool colors, const uint32_t* __restrict__ root, uint32_t sx,
                              uint32_t sy, uint32_t sz, uint32_t size, uint8_t* values, uint64_t* cols)
{
    const uint32_t r = *root;
    const uint64_t n = uint64_t(size) * size * size;
    const uint32_t D = t.g.depth;
    HD_GRID_STRIDE(i, n)
    {
        const uint32_t x = uint32_t(i % size), y = uint32_t((i / size) % size), z = uint32_t(i / (uint64_t(size) * size));
        uint8_t v = 0;
        uint64_t col = 0;
        if (x && y && z && r != kInvalid) {
            const uint32_t px = sx + x, py = sy + y, pz = sz + z;
            // DAGUtils::get_value
            uint32_t index = r;
            bool ok = true;
            for (uint32_t level = 0; level < t.g.leaf_level && ok; level++) {
                const uint32_t* p = t.sys(index);
                const uint32_t sh = D - level - 1;
                const uint32_t cidx = (((px >> sh) & 1) << 2) | (((py >> sh) & 1) << 1) | ((pz >> sh) & 1);
                const uint32_t mask = p[0] & 0xffu;
                if (!(mask & (1u << cidx)))
                    ok = false;
                else
                    index = p[child_offset(mask, cidx)];
            }
            if (ok) {
                const uint32_t* lp = t.sys(index);
                const uint32_t bi = ((px & 1) ? 4 : 0) | ((py & 1) ? 2 : 0) | ((pz & 1) ? 1 : 0) | ((px & 2) ? 32 : 0) |
                                    ((py & 2) ? 16 : 0) | ((pz & 2) ? 8 : 0);
                v = uint8_t(((bi < 32 ? lp[0] >> bi : lp[1] >> (bi - 32)) & 1));
            }
            if (v && colors)
                col = get_color(t, ct, r, px, py, pz);
        }
        values[i] = v;
        cols[i] = col;
    }
}

void copy_source(hd_ctx* c, Editor& ed)
{
    const uint64_t n = uint64_t(ed.size) * ed.size * ed.size;
    if (n > (uint64_t(1) << 34))
        throw StatusError{HD_ERR_INVALID, "copy region too large"};
    uint8_t* values = c->scratch.get<uint8_t>("copy_values", n + 1);
    uint64_t* cols = c->scratch.get<uint64_t>("copy_colors", n + 1);
    k_copy_source<<<grid_for(n, 256), 256, 0, c->stream>>>(c->t, c->ct, c->colors, c->d_root, uint32_t(ed.minx),
                                                            uint32_t(ed.miny), uint32_t(ed.minz), ed.size, values,
                                                            cols);
    HD_LAUNCH_CHECK();
    ed.values = values;
    ed.colors = cols;
}

// ---- the colour phase of an edit -------------------------------------------------

// Top-down: colour nodes of the next level's entries (levels < T), the slot
// reference at level T.
__global__ void k_col_spawn(ColorTable ct, uint32_t level, uint32_t n, Level lv, Level next)
{
    HD_GRID_STRIDE(i, n)
    {
        if (!lv.flag[i])
            continue;
        const uint32_t cn = lv.cn[i];
        const bool has = level == 0 || cn != 0;
        const uint32_t base = 8 * lv.exp[i];
        for (uint32_t k = 0; k < 8; k++)
            next.cn[base + k] = has ? ct.nodes[cn + k] : 0u;
    }
}

void color_spawn(hd_ctx* c, uint32_t level, uint32_t n, const Level& lv, const Level& next)
{
    k_col_spawn<<<grid_for(n, 128), 128, 0, c->stream>>>(c->ct, level, n, lv, next);
    HD_LAUNCH_CHECK();
}

// Level T: the tasks; offsets 0, task = own index.
__global__ void k_col_tasks(uint32_t n, Level lv, uint64_t* len)
{
    HD_GRID_STRIDE(i, n)
    {
        const bool task = lv.state[i] != kSkip;
        lv.noff[i] = 0;
        lv.ooff[i] = 0;
        lv.task[i] = uint32_t(i);
        len[i] = (task && lv.res[i] != kInvalid) ? lv.cnt[i] : 0;
    }
}

// Offsets of the children of descended entries (levels T .. leaf - 1).
__global__ void k_col_offsets(uint32_t n, Level lv, Level next)
{
    HD_GRID_STRIDE(i, n)
    {
        if (lv.state[i] != kDescend)
            continue;
        const uint32_t base = 8 * lv.exp[i];
        uint32_t no = lv.noff[i], oo = lv.ooff[i];
        const uint32_t task = lv.task[i];
        for (uint32_t k = 0; k < 8; k++) {
            const uint32_t j = base + k;
            next.noff[j] = no;
            next.ooff[j] = oo;
            next.task[j] = task;
            no += next.res[j] != kInvalid ? next.cnt[j] : 0u;
            oo += next.ocnt[j];
        }
    }
}

HD_D bool leaf_of_slot(const ColorTable& ct, uint32_t slot, LeafDesc* d)
{
    if (!(slot & kLeafFlag))
        return false;
    *d = ct.leaves[slot & ~kLeafFlag];
    return d->nb != 0;
}

// get_new_color of the tools (hash_dag_editors.h:262-269, :302-312,
// :323-329, :595-608); prev_col: the voxel's old colour (0 if it was empty)
HD_D uint64_t new_color(const Editor& e, float px, float py, float pz, bool prev, bool nv, uint64_t prev_col)
{
    if (e.tool == HD_TOOL_SPHERE_PAINT) {
        const F3 old = color_value(prev_col);
        const float dx = px - e.cx, dy = py - e.cy, dz = pz - e.cz;
        const float len = sqrtf(dx * dx + dy * dy + dz * dz);
        const float f = clampf(1 - len / e.r, 0.f, .1f);
        return single_color(F3{old.x * (1 - f) + e.paint_r * f, old.y * (1 - f) + e.paint_g * f,
                               old.z * (1 - f) + e.paint_b * f});
    }
    if (e.tool == HD_TOOL_COPY) {
        if (prev == nv || !nv)
            return prev_col;
        const int64_t i = copy_index(e, px, py, pz);
        return i < 0 ? prev_col : e.colors[i];
    }
    if (e.tool == HD_TOOL_NOISE_ADD || e.tool == HD_TOOL_NOISE_REMOVE) {
        // SphereNoiseEditor::get_new_color (:745-758): two rgb565 end points,
        // 3-bit weight from the distance over BoxEditorBase::radius
        if (prev == nv)
            return prev_col;
        const uint32_t bits = f3_to_rgb565(F3{94 / 255.f, 30 / 255.f, 0 / 255.f}) |
                              (f3_to_rgb565(F3{125 / 255.f, 100 / 255.f, 89 / 255.f}) << 16);
        const float dx = px - e.cx, dy = py - e.cy, dz = pz - e.cz;
        const float len = sqrtf(dx * dx + dy * dy + dz * dz);
        const int32_t w = int32_t((len / e.buf_r - 0.3f) * float((1 << 3) - 1));
        return pack_color(bits, uint32_t(w < 0 ? 0 : w > 7 ? 7 : w), 3);
    }
    if (e.tool == HD_TOOL_FILL) {
        // FillEditorColors::get_new_color (:693-709)
        if (nv && !prev) {
            const int64_t i = buffer_index(e, px, py, pz);
            if (i >= 0 && (e.values[i] & kBufSet))
                return e.colors[i];
        }
        return prev_col;
    }
    return single_color(e.sphere() ? F3{1, 0, 0} : F3{1, 0, 1});
}

// Emission of one level's colours into out[base[task] + offset ...]; a warp
// per entry.
__global__ void k_col_emit(Table t, ColorTable ct, Editor ed, uint32_t level, uint32_t n, Level lv, Level lvT,
                           const uint64_t* __restrict__ base, uint64_t* out)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t D = t.g.depth, leafl = t.g.leaf_level;
    const uint64_t warps = uint64_t(gridDim.x) * (blockDim.x / 32);
    for (uint64_t i = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32; i < n; i += warps) {
        const uint8_t st = lv.state[i];
        if (st == kSkip || st == kEmptied || st == kDescend)
            continue;
        const uint32_t task = lv.task[i];
        if (lvT.res[task] == kInvalid)
            continue;
        uint64_t* dst = out + base[task] + lv.noff[i];
        LeafDesc old{};
        const bool has_old = leaf_of_slot(ct, lvT.cn[task], &old);
        const uint32_t ooff = lv.ooff[i];
        if (st == kKeep) {
            const uint32_t cnt = lv.cnt[i];
            for (uint32_t k = lane; k < cnt; k += 32)
                dst[k] = (has_old && leaf_valid_index(old, ooff + k)) ? leaf_color(ct, old, ooff + k) : 0ull;
        } else if (st == kFilled) {
            const uint32_t cnt = lv.cnt[i];
            const uint64_t col = single_color(ed.sphere() ? F3{1, 0, 0} : F3{1, 0, 1});
            for (uint32_t k = lane; k < cnt; k += 32)
                dst[k] = col;
        } else if (st == kLeafEval && level == leafl) {
            uint64_t oldmask = 0;
            if (lv.old[i] != kInvalid) {
                const uint32_t* p = t.sys(lv.old[i]);
                oldmask = uint64_t(p[0]) | (uint64_t(p[1]) << 32);
            }
            const uint64_t newmask = lv.leaf[i];
            const uint32_t x0 = lv.x[i] << 2, y0 = lv.y[i] << 2, z0 = lv.z[i] << 2;
            for (uint32_t b = lane; b < 64; b += 32) {
                const uint64_t bit = 1ull << b;
                if (!(newmask & bit))
                    continue;
                const uint32_t c1 = b >> 3, c2 = b & 7;
                const float px = float(x0 + ((c1 >> 2) & 1) * 2 + ((c2 >> 2) & 1));
                const float py = float(y0 + ((c1 >> 1) & 1) * 2 + ((c2 >> 1) & 1));
                const float pz = float(z0 + (c1 & 1) * 2 + (c2 & 1));
                const bool prev = (oldmask & bit) != 0;
                const uint32_t oi = ooff + popc64(oldmask & (bit - 1));
                const uint64_t prev_col =
                    (prev && has_old && leaf_valid_index(old, oi)) ? leaf_color(ct, old, oi) : 0ull;
                const bool se = should_edit_impl(ed, px, py, pz, px + 1.0f, py + 1.0f, pz + 1.0f);
                dst[popc64(newmask & (bit - 1))] = se ? new_color(ed, px, py, pz, prev, true, prev_col) : prev_col;
            }
        }
        (void)D;
    }
}

// Leaf packing, pass 1 (a warp per task): blocks, macro words, weight bits.
__global__ void k_col_count(uint32_t n, const uint64_t* __restrict__ len, const uint64_t* __restrict__ base,
                            const uint64_t* __restrict__ out, uint32_t* nb, uint32_t* nm, uint32_t* nw)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warps = uint64_t(gridDim.x) * (blockDim.x / 32);
    for (uint64_t t = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32; t < n; t += warps) {
        const uint64_t L = len[t];
        const uint64_t* c = out + base[t];
        uint32_t blocks = 0, bits = 0;
        for (uint64_t k0 = 0; k0 < L; k0 += 32) {
            const uint64_t k = k0 + lane;
            bool start = false;
            uint32_t b = 0;
            if (k < L) {
                const uint64_t col = c[k];
                start = k % kColorsPerMacro == 0 || (pc_bits(col) != pc_bits(c[k - 1]) || pc_bpw(col) != pc_bpw(c[k - 1]));
                b = pc_bpw(col);
            }
            blocks += __popc(__ballot_sync(0xffffffffu, start));
            for (int o = 16; o; o >>= 1)
                b += __shfl_xor_sync(0xffffffffu, b, o);
            bits += b;
        }
        if (lane == 0) {
            nb[t] = blocks;
            nm[t] = uint32_t(2 * ((L + kColorsPerMacro - 1) / kColorsPerMacro));
            nw[t] = (bits + 31) / 32;
        }
    }
}

// Leaf packing, pass 2: the ColorLeafBuilder words (blocks, macro blocks,
// MSB-first weights in byte-swapped words) and the new descriptor.
__global__ void k_col_pack(ColorTable ct, uint32_t n, const uint64_t* __restrict__ len,
                           const uint64_t* __restrict__ base, const uint64_t* __restrict__ out,
                           const uint32_t* __restrict__ nb, const uint32_t* __restrict__ nm,
                           const uint32_t* __restrict__ nw, const uint32_t* __restrict__ bo,
                           const uint32_t* __restrict__ mo, const uint32_t* __restrict__ wo, uint64_t block_base,
                           uint64_t macro_base, uint64_t weight_base, LeafDesc* desc)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warps = uint64_t(gridDim.x) * (blockDim.x / 32);
    for (uint64_t t = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32; t < n; t += warps) {
        const uint64_t L = len[t];
        if (!L)
            continue;
        const uint64_t* c = out + base[t];
        uint64_t* blocks = ct.blocks + block_base + bo[t];
        uint64_t* macros = ct.macros + macro_base + mo[t];
        uint32_t* weights = ct.weights + weight_base + wo[t];
        uint32_t blk = 0, bitpos = 0, macro_bits = 0;
        for (uint64_t k0 = 0; k0 < L; k0 += 32) {
            // kColorsPerMacro is a multiple of 32: a macro block starts only
            // at the first lane of a chunk
            if (k0 % kColorsPerMacro == 0)
                macro_bits = bitpos;
            const uint64_t k = k0 + lane;
            bool start = false;
            uint32_t b = 0;
            uint64_t col = 0;
            if (k < L) {
                col = c[k];
                start = k % kColorsPerMacro == 0 || pc_bits(col) != pc_bits(c[k - 1]) || pc_bpw(col) != pc_bpw(c[k - 1]);
                b = pc_bpw(col);
            }
            const uint32_t sb = __ballot_sync(0xffffffffu, start);
            const uint32_t inc = warp_incl_scan(b);
            const uint32_t my_bits = bitpos + inc - b; // weight bit offset of this colour in the leaf
            const uint32_t my_blk = blk + __popc(sb & ((1u << lane) - 1u));
            if (k < L) {
                if (k % kColorsPerMacro == 0) {
                    macros[2 * (k / kColorsPerMacro)] = my_blk;
                    macros[2 * (k / kColorsPerMacro) + 1] = my_bits;
                }
                if (start)
                    blocks[my_blk] = (uint64_t(pc_bits(col)) << 32) |
                                     make_block_header(my_bits - macro_bits, b, uint32_t(k % kColorsPerMacro));
                if (b) {
                    // MSB-first: bits [my_bits, my_bits + b) of the stream
                    const uint32_t w = my_bits / 32, o = my_bits % 32;
                    const uint64_t v = uint64_t(pc_weight(col)) << (64 - b - o);
                    atomicOr(weights + w, uint32_t(v >> 32));
                    if (o + b > 32)
                        atomicOr(weights + w + 1, uint32_t(v));
                }
            }
            blk += __popc(sb);
            bitpos += __shfl_sync(0xffffffffu, inc, 31);
        }
        __syncwarp();
        // byte-swapped words (CFG_COLOR_SWAP_BYTE_ORDER)
        for (uint32_t w = lane; w < nw[t]; w += 32) {
            const uint32_t v = weights[w];
            weights[w] = ((v & 0xffu) << 24) | ((v & 0xff00u) << 8) | ((v & 0xff0000u) >> 8) | ((v & 0xff000000u) >> 24);
        }
        if (lane == 0) {
            LeafDesc d{};
            d.blocks = block_base + bo[t];
            d.macros = macro_base + mo[t];
            d.weights = weight_base + wo[t];
            d.nb = nb[t];
            d.nm = nm[t];
            d.nw = nw[t];
            desc[t] = d;
        }
    }
}

// Slot of each task with colours: the existing unique leaf, or a new leaf
// (need_new = 1).
__global__ void k_col_slots(uint32_t n, Level lvT, const uint64_t* __restrict__ len, uint32_t* need_new)
{
    HD_GRID_STRIDE(i, n) need_new[i] = len[i] > 0 && !(lvT.cn[i] & kLeafFlag);
}

// Descriptors in place; new slots get leaf indices leaf_top + rank; the
// replaced descriptors go to the undo diff.
__global__ void k_col_commit(ColorTable ct, uint32_t n, Level lvT, const uint64_t* __restrict__ len,
                             const uint32_t* __restrict__ need_new, const uint32_t* __restrict__ rank,
                             uint64_t leaf_top, const LeafDesc* __restrict__ desc, uint32_t* slot_out,
                             LeafDesc* prev_out)
{
    HD_GRID_STRIDE(i, n)
    {
        if (!len[i])
            continue;
        uint32_t slot = lvT.cn[i];
        LeafDesc prev{};
        if (need_new[i]) {
            slot = kLeafFlag | uint32_t(leaf_top + rank[i]);
            lvT.cn[i] = slot; // linked into the tree below
        } else {
            prev = ct.leaves[slot & ~kLeafFlag];
        }
        ct.leaves[slot & ~kLeafFlag] = desc[i];
        slot_out[i] = slot;
        prev_out[i] = prev;
    }
}

// Bottom-up colour-node allocation (edit_threaded's allocateColorNode,
// hash_dag_edits.h:152-161): an entry above T whose child got a new leaf or
// node and that has no colour node gets one.
__global__ void k_col_need(uint32_t level, uint32_t T, uint32_t n, Level lv, Level next,
                           const uint32_t* __restrict__ need_new_T, const uint32_t* __restrict__ newnode_next,
                           uint32_t* newnode)
{
    HD_GRID_STRIDE(i, n)
    {
        bool any = false;
        if (lv.flag[i]) {
            const uint32_t base = 8 * lv.exp[i];
            for (uint32_t k = 0; k < 8; k++)
                any |= (level + 1 == T) ? need_new_T[base + k] != 0 : newnode_next[base + k] != 0;
        }
        newnode[i] = any && level > 0 && lv.cn[i] == 0;
    }
}
__global__ void k_col_alloc(uint32_t n, Level lv, const uint32_t* __restrict__ newnode, const uint32_t* __restrict__ rank,
                            uint64_t node_top)
{
    HD_GRID_STRIDE(i, n)
    {
        if (newnode[i])
            lv.cn[i] = uint32_t(node_top + 8ull * rank[i]);
    }
}
__global__ void k_col_link(ColorTable ct, uint32_t level, uint32_t T, uint32_t n, Level lv, Level next,
                           const uint32_t* __restrict__ need_new_T, const uint32_t* __restrict__ newnode_next)
{
    HD_GRID_STRIDE(i, n)
    {
        if (!lv.flag[i])
            continue;
        const uint32_t base = 8 * lv.exp[i];
        for (uint32_t k = 0; k < 8; k++) {
            const bool link = (level + 1 == T) ? need_new_T[base + k] != 0 : newnode_next[base + k] != 0;
            if (link)
                ct.nodes[lv.cn[i] + k] = next.cn[base + k];
        }
    }
}

// The colour phase of an edit, after its geometry: lv / count / deepest as
// edit_one left them (levels T .. deepest hold the tasks' subtrees).  Fills
// frame (replaced leaves) for the undo history.
void edit_colors(hd_ctx* c, const Editor& ed, std::vector<Level>& lv, const std::vector<uint32_t>& count,
                 uint32_t deepest, UndoFrame& frame)
{
    const Geom& g = c->g;
    const uint32_t T = g.T;
    if (!c->colors || deepest < T || count[T] == 0)
        return;
    cudaStream_t st = c->stream;
    Scratch& s = c->scratch;
    const uint32_t nT = count[T];
    uint64_t* len = s.get<uint64_t>("ec_len", uint64_t(nT) + 1);
    uint64_t* base = s.get<uint64_t>("ec_base", uint64_t(nT) + 1);
    uint64_t* d_tot64 = s.get<uint64_t>("ec_tot64", 2);
    k_col_tasks<<<grid_for(nT, 256), 256, 0, st>>>(nT, lv[T], len);
    HD_LAUNCH_CHECK();
    for (uint32_t L = T; L < deepest; L++) {
        k_col_offsets<<<grid_for(count[L], 256), 256, 0, st>>>(count[L], lv[L], lv[L + 1]);
        HD_LAUNCH_CHECK();
    }
    exclusive_scan<uint64_t, uint64_t>(s, len, base, nT, d_tot64, st);
    const uint64_t total = read_scalar(d_tot64, st);
    uint64_t* out = s.get<uint64_t>("ec_out", total + 1);
    for (uint32_t L = T; L <= deepest; L++) {
        const uint64_t threads = uint64_t(count[L]) * 32;
        k_col_emit<<<grid_for(threads, 256, 152 * 16), 256, 0, st>>>(c->t, c->ct, ed, L, count[L], lv[L], lv[T], base,
                                                                     out);
        HD_LAUNCH_CHECK();
    }
    uint32_t* nb = s.get<uint32_t>("ec_nb", uint64_t(nT) + 1);
    uint32_t* nm = s.get<uint32_t>("ec_nm", uint64_t(nT) + 1);
    uint32_t* nw = s.get<uint32_t>("ec_nw", uint64_t(nT) + 1);
    uint32_t* bo = s.get<uint32_t>("ec_bo", uint64_t(nT) + 1);
    uint32_t* mo = s.get<uint32_t>("ec_mo", uint64_t(nT) + 1);
    uint32_t* wo = s.get<uint32_t>("ec_wo", uint64_t(nT) + 1);
    uint32_t* d_tot = s.get<uint32_t>("ec_tot", 4);
    k_col_count<<<grid_for(uint64_t(nT) * 32, 256, 152 * 16), 256, 0, st>>>(nT, len, base, out, nb, nm, nw);
    HD_LAUNCH_CHECK();
    exclusive_scan<uint32_t, uint32_t>(s, nb, bo, nT, d_tot, st);
    exclusive_scan<uint32_t, uint32_t>(s, nm, mo, nT, d_tot + 1, st);
    exclusive_scan<uint32_t, uint32_t>(s, nw, wo, nT, d_tot + 2, st);
    uint32_t need_new_total = 0;
    uint32_t* need_new = s.get<uint32_t>("ec_neednew", uint64_t(nT) + 1);
    uint32_t* rank = s.get<uint32_t>("ec_rank", uint64_t(nT) + 1);
    k_col_slots<<<grid_for(nT, 256), 256, 0, st>>>(nT, lv[T], len, need_new);
    HD_LAUNCH_CHECK();
    exclusive_scan<uint32_t, uint32_t>(s, need_new, rank, nT, d_tot + 3, st);
    uint32_t tot[4];
    HD_CUDA(cudaMemcpyAsync(tot, d_tot, 16, cudaMemcpyDeviceToHost, st));
    HD_CUDA(cudaStreamSynchronize(st));
    need_new_total = tot[3];
    // renders in flight read the leaves about to be replaced: wait for them
    for (cudaEvent_t e : c->color_fences)
        HD_CUDA(cudaStreamWaitEvent(st, e, 0));
    // nodes: at most one per entry above T
    uint64_t max_nodes = 0;
    for (uint32_t L = 1; L < T; L++)
        max_nodes += 8ull * count[L];
    const uint64_t add[5] = {max_nodes, need_new_total, tot[0], tot[1], tot[2]};
    color_reserve(c, add);
    LeafDesc* desc = s.get<LeafDesc>("ec_desc", uint64_t(nT) + 1);
    k_col_pack<<<grid_for(uint64_t(nT) * 32, 256, 152 * 16), 256, 0, st>>>(
        c->ct, nT, len, base, out, nb, nm, nw, bo, mo, wo, c->ctop[2], c->ctop[3], c->ctop[4], desc);
    HD_LAUNCH_CHECK();
    uint32_t* slot_out = s.get<uint32_t>("ec_slot", uint64_t(nT) + 1);
    LeafDesc* prev_out = s.get<LeafDesc>("ec_prev", uint64_t(nT) + 1);
    k_col_commit<<<grid_for(nT, 256), 256, 0, st>>>(c->ct, nT, lv[T], len, need_new, rank, c->ctop[1], desc,
                                                    slot_out, prev_out);
    HD_LAUNCH_CHECK();
    // colour nodes, bottom-up, then the links
    std::vector<uint32_t*> newnode(T + 1, nullptr);
    newnode[T] = need_new;
    uint64_t node_top = c->ctop[0];
    for (uint32_t L = T - 1; L >= 1; L--) {
        char nm_[32];
        snprintf(nm_, sizeof(nm_), "ec_newnode_%u", L);
        newnode[L] = s.get<uint32_t>(nm_, uint64_t(count[L]) + 1);
        k_col_need<<<grid_for(count[L], 256), 256, 0, st>>>(L, T, count[L], lv[L], lv[L + 1], need_new,
                                                            newnode[L + 1], newnode[L]);
        HD_LAUNCH_CHECK();
        uint32_t* r = s.get<uint32_t>("ec_noderank", uint64_t(count[L]) + 1);
        exclusive_scan<uint32_t, uint32_t>(s, newnode[L], r, count[L], d_tot, st);
        const uint32_t k = read_scalar(d_tot, st);
        k_col_alloc<<<grid_for(count[L], 256), 256, 0, st>>>(count[L], lv[L], newnode[L], r, node_top);
        HD_LAUNCH_CHECK();
        node_top += 8ull * k;
    }
    for (uint32_t L = 0; L < T; L++) {
        k_col_link<<<grid_for(count[L], 256), 256, 0, st>>>(c->ct, L, T, count[L], lv[L], lv[L + 1], need_new,
                                                            newnode[L + 1]);
        HD_LAUNCH_CHECK();
    }
    c->ctop[0] = node_top;
    c->ctop[1] += need_new_total;
    c->ctop[2] += tot[0];
    c->ctop[3] += tot[1];
    c->ctop[4] += tot[2];
    const unsigned long long tops[5] = {c->ctop[0], c->ctop[1], c->ctop[2], c->ctop[3], c->ctop[4]};
    HD_CUDA(cudaMemcpyAsync(c->ct.top, tops, sizeof(tops), cudaMemcpyHostToDevice, st));
    // undo diff: replaced leaves (new slots had no leaf: an empty descriptor)
    std::vector<uint64_t> h_len(nT);
    std::vector<uint32_t> h_slot(nT);
    std::vector<LeafDesc> h_prev(nT), h_next(nT);
    HD_CUDA(cudaMemcpyAsync(h_len.data(), len, 8ull * nT, cudaMemcpyDeviceToHost, st));
    HD_CUDA(cudaMemcpyAsync(h_slot.data(), slot_out, 4ull * nT, cudaMemcpyDeviceToHost, st));
    HD_CUDA(cudaMemcpyAsync(h_prev.data(), prev_out, sizeof(LeafDesc) * nT, cudaMemcpyDeviceToHost, st));
    HD_CUDA(cudaMemcpyAsync(h_next.data(), desc, sizeof(LeafDesc) * nT, cudaMemcpyDeviceToHost, st));
    HD_CUDA(cudaStreamSynchronize(st));
    for (uint32_t i = 0; i < nT; i++)
        if (h_len[i]) {
            frame.leaf.push_back(h_slot[i] & ~kLeafFlag);
            frame.prev.push_back(h_prev[i]);
            frame.next.push_back(h_next[i]);
        }
}

__global__ void k_set_leaves(ColorTable ct, const uint32_t* __restrict__ index, const LeafDesc* __restrict__ d,
                             uint32_t n)
{
    HD_GRID_STRIDE(i, n) ct.leaves[index[i]] = d[i];
}

// HashDAGUndoRedo::undo / redo (hash_dag.h:67-120): the root and the
// replaced leaves of the frame go back; the inverted frame goes to the other
// stack.
bool undo_step(hd_ctx* c, bool redo)
{
    auto& from = redo ? c->redo : c->undo;
    auto& to = redo ? c->undo : c->redo;
    if (from.empty())
        return false;
    UndoFrame f = std::move(from.back());
    from.pop_back();
    UndoFrame inv;
    inv.root = c->root;
    inv.leaf = f.leaf;
    inv.prev = f.next;
    inv.next = f.prev;
    cudaStream_t st = c->stream;
    HD_CUDA(cudaMemcpyAsync(c->d_root, &f.root, 4, cudaMemcpyHostToDevice, st));
    if (!f.leaf.empty()) {
        const uint32_t n = uint32_t(f.leaf.size());
        uint32_t* d_i = c->scratch.get<uint32_t>("undo_i", n);
        LeafDesc* d_d = c->scratch.get<LeafDesc>("undo_d", n);
        HD_CUDA(cudaMemcpyAsync(d_i, f.leaf.data(), 4ull * n, cudaMemcpyHostToDevice, st));
        HD_CUDA(cudaMemcpyAsync(d_d, f.prev.data(), sizeof(LeafDesc) * n, cudaMemcpyHostToDevice, st));
        k_set_leaves<<<grid_for(n, 256), 256, 0, st>>>(c->ct, d_i, d_d, n);
        HD_LAUNCH_CHECK();
    }
    HD_CUDA(cudaStreamSynchronize(st));
    c->root = f.root;
    to.push_back(std::move(inv));
    return true;
}

void push_undo(hd_ctx* c, UndoFrame&& f)
{
    c->redo.clear();
    c->undo.push_back(std::move(f));
    while (c->undo.size() > c->undo_capacity)
        c->undo.pop_front();
}

} // namespace hd

extern "C" {

static hd_status color_guard(hd_ctx* c, const std::function<void()>& f)
{
    try {
        f();
        return HD_OK;
    } catch (const hd::StatusError& e) {
        c->err = e.msg;
        return e.status;
    } catch (const hd::CudaError& e) {
        c->err = std::string("CUDA error ") + cudaGetErrorString(e.code) + " in " + e.where;
        return HD_ERR_CUDA;
    }
}

hd_status hd_colors_from_scene(hd_ctx* c, uint64_t color_seed)
{
    if (!c)
        return HD_ERR_INVALID;
    return color_guard(c, [&] { hd::colors_from_scene(c, color_seed); });
}

hd_status hd_get_colors(hd_ctx* c, const uint32_t* d_xyz, uint64_t n, hd_color* d_out)
{
    if (!c || (n && (!d_xyz || !d_out)))
        return HD_ERR_INVALID;
    return color_guard(c, [&] {
        hd::get_colors(c, d_xyz, n, d_out);
        HD_CUDA(cudaStreamSynchronize(c->stream));
    });
}

hd_status hd_trace_colors(hd_ctx* c, const uint32_t* d_paths, uint32_t width, uint32_t height, uint32_t* d_rgba)
{
    if (!c || !d_paths || !d_rgba || !width || !height)
        return HD_ERR_INVALID;
    return color_guard(c, [&] {
        hd::trace_colors(c, d_paths, width, height, d_rgba);
        HD_CUDA(cudaStreamSynchronize(c->stream));
    });
}

hd_status hd_trace_colors_ex(hd_ctx* c, const uint32_t* d_paths, uint32_t width, uint32_t height, uint32_t* d_rgba,
                             const hd_trace_colors_params* params)
{
    if (!c || !d_paths || !d_rgba || !params || params->debug_colors > HD_DEBUG_WEIGHT ||
        params->overlay.tool > HD_OVERLAY_CUBE_FILL)
        return HD_ERR_INVALID;
    return color_guard(c, [&] {
        hd::trace_colors(c, d_paths, width, height, d_rgba, nullptr, nullptr, params);
        HD_CUDA(cudaStreamSynchronize(c->stream));
    });
}

hd_status hd_color_stats(hd_ctx* c, uint64_t* out)
{
    if (!c || !out)
        return HD_ERR_INVALID;
    for (int k = 0; k < 5; k++)
        out[k] = c->ctop[k];
    return HD_OK;
}

hd_status hd_undo(hd_ctx* c)
{
    if (!c)
        return HD_ERR_INVALID;
    bool done = false;
    const hd_status st = color_guard(c, [&] { done = hd::undo_step(c, false); });
    return st != HD_OK ? st : (done ? HD_OK : HD_ERR_STATE);
}

hd_status hd_redo(hd_ctx* c)
{
    if (!c)
        return HD_ERR_INVALID;
    bool done = false;
    const hd_status st = color_guard(c, [&] { done = hd::undo_step(c, true); });
    return st != HD_OK ? st : (done ? HD_OK : HD_ERR_STATE);
}

hd_status hd_set_undo_capacity(hd_ctx* c, uint32_t frames)
{
    if (!c)
        return HD_ERR_INVALID;
    c->undo_capacity = frames;
    while (c->undo.size() > c->undo_capacity)
        c->undo.pop_front();
    return HD_OK;
}

hd_status hd_history(hd_ctx* c, uint32_t* undo_frames, uint32_t* redo_frames)
{
    if (!c)
        return HD_ERR_INVALID;
    if (undo_frames)
        *undo_frames = uint32_t(c->undo.size());
    if (redo_frames)
        *redo_frames = uint32_t(c->redo.size());
    return HD_OK;
}

} // extern "C"
