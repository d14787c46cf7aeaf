// Edit pipeline, per-entry device logic shared by the one-edit-per-call path
// (hd_edit.cu) and the graph-captured batched path (hd_edit_batch.cu).
//
// Reference: HashDAG::edit_threads (hash_dag.h:255-405), which runs
// HashDagEdits::edit_threaded over the levels above C_colorTreeLevels
// (hash_dag_edits.h:106-333) and edit_leaf below (:335-643); editors
// (hash_dag_editors.h:57-127, :223-313); find_or_add_leaf_node /
// find_or_add_interior_node with their bucket scans (hash_table.h:196-357,
// :470-560).
//
// The recursion becomes two level-synchronous sweeps:
//  * top-down, every level's edit entries (a node path and its old index) are
//    classified as in the reference (untouched, carved away, filled, a leaf
//    to rebuild, or an interior node to descend into); descended entries
//    spawn their 8 children, in child order, so each level's entries stay in
//    depth-first (Morton) order;
//  * bottom-up, every rebuilt node is compared with its old self and, when
//    changed, hashed and resolved by find-or-add.  Candidates of a level are
//    grouped by bucket and each bucket is resolved by one warp, candidates in
//    depth-first order one after the other: the same sequence of bucket scans
//    and appends as the reference's single-threaded depth-first recursion,
//    including its scan rules (a node flush with the bucket tail or the page
//    end is invisible to an equal-size query).
#pragma once

#include "hd_ctx.h"
#include "hd_table.cuh"

namespace hd {

constexpr uint32_t kNoBucket = 0xFFFFFFFFu;


// ---- editors ----------------------------------------------------------------
// SphereEditor / BoxEditor (hash_dag_editors.h:223-313), SpherePaintEditor
// (:315-330) and the copy tool (CopyEditorWithDecompression, :437-609).
struct Editor {
    uint32_t tool;
    float cx, cy, cz, r, r2;
    float bminx, bminy, bminz, bmaxx, bmaxy, bmaxz;
    float paint_r, paint_g, paint_b; // paint target colour
    // copy: source / dest, the source region's corner (copyMin) and size,
    // its occupancy and colours read before the edit (x fastest)
    float srcx, srcy, srcz, dstx, dsty, dstz, minx, miny, minz;
    uint32_t size;
    const uint8_t* values;
    const uint64_t* colors;
    // noise and fill (BufferEditor, :129-221): the buffer's corner
    // (BoxEditorBase::min; minx.. above), its radius (1.5 r for the noise)
    // and per voxel kBufNew (the voxel reads true) | kBufSet (set by the
    // tool); the fill's colour of each set voxel in `colors`
    float buf_r;
    HD_HD bool sphere() const
    {
        return tool == HD_TOOL_SPHERE_ADD || tool == HD_TOOL_SPHERE_REMOVE || tool == HD_TOOL_SPHERE_PAINT;
    }
    HD_HD bool adding() const { return tool == HD_TOOL_SPHERE_ADD || tool == HD_TOOL_BOX_ADD; }
    // is_full / is_empty exist for the sphere and box editors only
    HD_HD bool shortcuts() const { return tool <= HD_TOOL_BOX_ADD; }
};

HD_HD Editor make_editor(const hd_edit& e)
{
    Editor ed{};
    ed.tool = e.tool;
    ed.cx = e.center[0];
    ed.cy = e.center[1];
    ed.cz = e.center[2];
    ed.r = e.radius;
    ed.r2 = e.radius * e.radius;
    float bx = e.center[0], by = e.center[1], bz = e.center[2];
    if (e.tool == HD_TOOL_COPY) {
        // BoxEditorBase(center - source + dest, radius)
        ed.srcx = e.source[0];
        ed.srcy = e.source[1];
        ed.srcz = e.source[2];
        ed.dstx = e.dest[0];
        ed.dsty = e.dest[1];
        ed.dstz = e.dest[2];
        bx = e.center[0] - e.source[0] + e.dest[0];
        by = e.center[1] - e.source[1] + e.dest[1];
        bz = e.center[2] - e.source[2] + e.dest[2];
        ed.minx = e.center[0] - e.radius;
        ed.miny = e.center[1] - e.radius;
        ed.minz = e.center[2] - e.radius;
        ed.size = 2 * uint32_t(ceilf(e.radius));
    }
    float br = e.radius;
    if (e.tool == HD_TOOL_NOISE_ADD || e.tool == HD_TOOL_NOISE_REMOVE)
        br = 1.5f * e.radius; // BufferEditor(dag, center, 1.5f * radius) (:716)
    if (e.tool >= HD_TOOL_NOISE_REMOVE) {
        ed.buf_r = br;
        ed.minx = bx - br;
        ed.miny = by - br;
        ed.minz = bz - br;
        ed.size = 2 * uint32_t(ceilf(br));
    }
    ed.bminx = bx - br;
    ed.bminy = by - br;
    ed.bminz = bz - br;
    ed.bmaxx = bx + br;
    ed.bmaxy = by + br;
    ed.bmaxz = bz + br;
    ed.paint_r = float(e.rgb & 0xFF) / 255.0f;
    ed.paint_g = float((e.rgb >> 8) & 0xFF) / 255.0f;
    ed.paint_b = float((e.rgb >> 16) & 0xFF) / 255.0f;
    return ed;
}

// the copy tool's source index of a destination voxel, or -1 (:585-606)
HD_HD int64_t copy_index(const Editor& e, float px, float py, float pz)
{
    const float qx = ((px - e.dstx) + e.srcx) - e.minx, qy = ((py - e.dsty) + e.srcy) - e.miny,
                qz = ((pz - e.dstz) + e.srcz) - e.minz;
    const uint32_t ix = uint32_t(qx < 0 ? 0.0f : qx), iy = uint32_t(qy < 0 ? 0.0f : qy),
                   iz = uint32_t(qz < 0 ? 0.0f : qz);
    if (ix >= e.size || iy >= e.size || iz >= e.size)
        return -1;
    return int64_t(ix) + int64_t(e.size) * iy + int64_t(e.size) * e.size * iz;
}
// Per-voxel flags of the noise and fill buffers
constexpr uint8_t kBufNew = 1; // BufferEditor::get_value reads true (set, or loaded true)
constexpr uint8_t kBufSet = 2; // EValues::SetTrue

// truncate(float3) (cuda_math.h:80) of a float that may be negative, as the
// reference's x86-64 build converts it: to a 64-bit integer toward zero, then
// its low 32 bits ((-1, 0) gives 0, anything below -1 a huge index)
HD_HD uint32_t trunc_u32(float f) { return uint32_t((long long)f); }

// the buffer index of a voxel, or -1 (BufferEditor::get_new_value, :211-220)
HD_HD int64_t buffer_index(const Editor& e, float px, float py, float pz)
{
    const uint32_t x = trunc_u32(px - e.minx), y = trunc_u32(py - e.miny), z = trunc_u32(pz - e.minz);
    if (x >= e.size || y >= e.size || z >= e.size)
        return -1;
    return int64_t(x) + int64_t(e.size) * y + int64_t(e.size) * e.size * z;
}

// get_new_value of each editor
HD_HD bool new_value(const Editor& e, float px, float py, float pz, bool prev)
{
    if (e.tool >= HD_TOOL_NOISE_REMOVE) {
        // `get_value(p) == EValues::Unknown` compares a bool with 0: a
        // voxel reads true when set or loaded true, else keeps its value
        const int64_t i = buffer_index(e, px, py, pz);
        return (i >= 0 && (e.values[i] & kBufNew)) ? true : prev;
    }
    if (e.tool == HD_TOOL_SPHERE_PAINT)
        return prev;
    if (e.tool == HD_TOOL_COPY) {
        if (prev)
            return prev;
        const int64_t i = copy_index(e, px, py, pz);
        return i < 0 ? prev : e.values[i] != 0;
    }
    return e.adding();
}

HD_D float sqr(float f) { return f * f; }
HD_D float fmax_r(float a, float b) { return a > b ? a : b; }

// SphereEditorBase::should_edit_impl (:112-126) / BoxEditorBase (:76-91)
HD_D bool should_edit_impl(const Editor& e, float mnx, float mny, float mnz, float mxx, float mxy, float mxz)
{
    if (e.sphere()) {
        float dist = e.r2;
        if (e.cx < mnx)
            dist -= sqr(e.cx - mnx);
        else if (e.cx > mxx)
            dist -= sqr(e.cx - mxx);
        if (e.cy < mny)
            dist -= sqr(e.cy - mny);
        else if (e.cy > mxy)
            dist -= sqr(e.cy - mxy);
        if (e.cz < mnz)
            dist -= sqr(e.cz - mnz);
        else if (e.cz > mxz)
            dist -= sqr(e.cz - mxz);
        return dist > 0;
    }
    return !(e.bminx >= mxx || e.bminy >= mxy || e.bminz >= mxz || e.bmaxx <= mnx || e.bmaxy <= mny ||
             e.bmaxz <= mnz || mnx >= e.bmaxx || mny >= e.bmaxy || mnz >= e.bmaxz || mxx <= e.bminx ||
             mxy <= e.bminy || mxz <= e.bminz);
}

// is_full_impl / is_empty_impl (:280-295, :233-252): the region lies inside
// the tool.
HD_D bool inside_tool(const Editor& e, float mnx, float mny, float mnz, float mxx, float mxy, float mxz)
{
    if (e.sphere()) {
        const float a = fmax_r(sqr(mnx - e.cx), sqr(mxx - e.cx));
        const float b = fmax_r(sqr(mny - e.cy), sqr(mxy - e.cy));
        const float c = fmax_r(sqr(mnz - e.cz), sqr(mxz - e.cz));
        return (a + b) + c < e.r2;
    }
    return e.bminx <= mnx && e.bminy <= mny && e.bminz <= mnz && e.bmaxx >= mxx && e.bmaxy >= mxy && e.bmaxz >= mxz;
}

// ---- per-level entry state ---------------------------------------------------
enum : uint8_t {
    kSkip = 0,      // level-C_colorTreeLevels child the parent never hands to edit_leaf
    kKeep = 1,      // untouched: result = old
    kEmptied = 2,   // carved away (is_empty)
    kFilled = 3,    // filled (is_full): the level's full node
    kLeafEval = 4,  // leaf rebuilt voxel by voxel
    kDescend = 5,   // interior node rebuilt from its children
};

struct Level {
    uint32_t* x;
    uint32_t* y;
    uint32_t* z;
    uint32_t* old;
    uint8_t* state;
    uint32_t* res;   // new index (kInvalid = empty)
    uint32_t* cnt;   // voxel count of the new node (levels >= T)
    uint32_t* flag;  // 1 = descends
    uint32_t* exp;   // exclusive scan of flag
    uint64_t* leaf;  // new leaf masks (leaf level only)
    uint32_t* cand;  // candidate content, 9 words per entry
    // colours (allocated only when the context has colours)
    uint32_t* ocnt;  // voxel count of the old node (levels >= T)
    uint32_t* cn;    // levels < T: colour node; level T: the slot's leaf reference
    uint32_t* noff;  // offset in the task's new colour sequence (levels >= T)
    uint32_t* ooff;  // offset in the task's old leaf
    uint32_t* task;  // level-T entry the entry belongs to
};

struct EditCounters {
    unsigned long long num_voxels, num_nodes, foa, added, scanned;
};

HD_D void warp_add(unsigned long long* p, unsigned long long v)
{
    // warp-aggregated atomic
    const uint32_t mask = __activemask();
    for (int o = 16; o; o >>= 1)
        v += __shfl_down_sync(mask, v, o);
    if ((threadIdx.x & 31) == __ffs(mask) - 1)
        atomicAdd(p, v);
}

// Reads of a node's words.  CG = false: through the read-only path, for
// kernels during which the table does not change; CG = true: L2-coherent
// loads, for a launch that also appends to the table (the persistent batched
// edits read in one edit the nodes and pages an earlier edit of the same
// launch wrote).
template <bool CG>
struct NodeRead {
    const uint32_t* p;
    HD_D NodeRead(const Table& t, uint32_t v) : p(CG ? t.sys_cg(v) : t.sys(v)) {}
    HD_D uint32_t operator[](uint32_t k) const { return CG ? __ldcg(p + k) : p[k]; }
};

// Top-down classification of entry i of level `level` (edit_threaded /
// edit_leaf early exits); nodes / voxels: its share of the edit counters.
// The entry's path (x, y, z) and old node are given (a caller that has just
// spawned it holds them in registers); classify_entry reads them.
template <bool CG = false>
HD_D void classify_values(const Table& t, const Editor& ed, uint32_t level, const Level& lv, uint32_t i, uint32_t x,
                          uint32_t y, uint32_t z, uint32_t old, unsigned long long& nodes, unsigned long long& voxels)
{
    const uint32_t D = t.g.depth, T = t.g.T, leafl = t.g.leaf_level;
    const uint32_t depth = D - level;
    const float s = float(1u << depth);
    const float mnx = float(x << depth), mny = float(y << depth), mnz = float(z << depth);
    const float mxx = mnx + s, mxy = mny + s, mxz = mnz + s;
    const bool se = should_edit_impl(ed, mnx, mny, mnz, mxx, mxy, mxz);
    uint8_t state;
    uint32_t res = old, cnt = 0;
    nodes = 0;
    voxels = 0;
    if (level < T) {
        // edit_threaded: visited in both passes; no early full/empty exits
        nodes = 2;
        state = se ? kDescend : kKeep;
    } else {
        if (level == T && !se) {
            state = kSkip; // the parent keeps the old child without a visit
        } else {
            nodes = 1;
            if (!se) {
                state = kKeep;
                if (old != kInvalid) {
                    const NodeRead<CG> p(t, old);
                    cnt = level < leafl ? (p[0] >> 8) : popc32(p[0]) + popc32(p[1]);
                }
            } else if (ed.shortcuts() && inside_tool(ed, mnx, mny, mnz, mxx, mxy, mxz)) {
                const uint32_t full_count = 1u << (3 * depth);
                voxels = full_count;
                if (ed.adding()) {
                    state = kFilled;
                    res = t.full_nodes[level];
                    cnt = full_count;
                } else {
                    state = kEmptied;
                    res = kInvalid;
                }
            } else if (level == leafl) {
                state = kLeafEval;
                uint64_t leaf = 0;
                if (old != kInvalid) {
                    const NodeRead<CG> p(t, old);
                    leaf = uint64_t(p[0]) | (uint64_t(p[1]) << 32);
                }
                const uint32_t x0 = x << 2, y0 = y << 2, z0 = z << 2;
                uint32_t edited = 0;
                for (uint32_t c1 = 0; c1 < 8; c1++)
                    for (uint32_t c2 = 0; c2 < 8; c2++) {
                        const float px = float(x0 + ((c1 >> 2) & 1) * 2 + ((c2 >> 2) & 1));
                        const float py = float(y0 + ((c1 >> 1) & 1) * 2 + ((c2 >> 1) & 1));
                        const float pz = float(z0 + (c1 & 1) * 2 + (c2 & 1));
                        if (should_edit_impl(ed, px, py, pz, px + 1.0f, py + 1.0f, pz + 1.0f)) {
                            edited++;
                            const uint64_t bit = 1ull << (c1 * 8 + c2);
                            leaf = new_value(ed, px, py, pz, (leaf & bit) != 0) ? (leaf | bit) : (leaf & ~bit);
                        }
                    }
                voxels = edited;
                lv.leaf[i] = leaf;
            } else {
                state = kDescend;
            }
        }
    }
    lv.state[i] = state;
    lv.res[i] = res;
    lv.cnt[i] = cnt;
    lv.flag[i] = state == kDescend;
    if (lv.ocnt && level >= T) {
        uint32_t oc = 0;
        if (old != kInvalid) {
            const NodeRead<CG> p(t, old);
            oc = level < leafl ? (p[0] >> 8) : popc32(p[0]) + popc32(p[1]);
        }
        lv.ocnt[i] = oc;
    }
}

template <bool CG = false>
HD_D void classify_entry(const Table& t, const Editor& ed, uint32_t level, const Level& lv, uint32_t i,
                         unsigned long long& nodes, unsigned long long& voxels)
{
    classify_values<CG>(t, ed, level, lv, i, lv.x[i], lv.y[i], lv.z[i], lv.old[i], nodes, voxels);
}

// A descended entry spawns its 8 children (child order) at 8 * exp[i] on the
// next level.
HD_D void spawn_entry(const Table& t, const Level& lv, const Level& next, uint32_t i)
{
    if (!lv.flag[i])
        return;
    const uint32_t base = 8 * lv.exp[i];
    const uint32_t old = lv.old[i];
    uint32_t mask = 0;
    const uint32_t* p = nullptr;
    if (old != kInvalid) {
        p = t.sys(old);
        mask = p[0] & 0xffu;
    }
    uint32_t k = 1;
    for (uint32_t c = 0; c < 8; c++) {
        next.x[base + c] = (lv.x[i] << 1) | ((c >> 2) & 1);
        next.y[base + c] = (lv.y[i] << 1) | ((c >> 1) & 1);
        next.z[base + c] = (lv.z[i] << 1) | (c & 1);
        next.old[base + c] = (mask & (1u << c)) ? p[k++] : kInvalid;
    }
}

// Child c of descended entry i, written at slot `at` of the next level
// (spawn_entry for one child, with L2-coherent table reads); its path and
// old node are also returned (for classify_values).
HD_D void spawn_child(const Table& t, const Level& lv, const Level& next, uint32_t i, uint32_t c, uint32_t at,
                      uint32_t& x, uint32_t& y, uint32_t& z, uint32_t& child)
{
    const uint32_t old = lv.old[i];
    child = kInvalid;
    if (old != kInvalid) {
        const NodeRead<true> p(t, old);
        const uint32_t mask = p[0] & 0xffu;
        if (mask & (1u << c))
            child = p[child_offset(mask, c)];
    }
    x = (lv.x[i] << 1) | ((c >> 2) & 1);
    y = (lv.y[i] << 1) | ((c >> 1) & 1);
    z = (lv.z[i] << 1) | (c & 1);
    next.x[at] = x;
    next.y[at] = y;
    next.z[at] = z;
    next.old[at] = child;
}

// Bottom-up: the rebuilt content of entry i (kLeafEval / kDescend).  Unchanged
// and emptied nodes resolve at once (kNoBucket); otherwise the content goes
// to lv.cand and the function returns its bucket for find-or-add.
template <bool CG = false>
HD_D uint32_t candidate_entry(const Table& t, uint32_t level, const Level& lv, const Level& child, uint32_t i)
{
    const uint32_t T = t.g.T;
    const uint8_t state = lv.state[i];
    uint32_t* c = lv.cand + 9 * i;
    uint32_t hash;
    if (state == kLeafEval) {
        const uint64_t leaf = lv.leaf[i];
        const uint32_t old = lv.old[i];
        uint64_t initial = 0;
        if (old != kInvalid) {
            const NodeRead<CG> p(t, old);
            initial = uint64_t(p[0]) | (uint64_t(p[1]) << 32);
        }
        lv.cnt[i] = popc64(leaf);
        if (leaf == initial) {
            lv.res[i] = old;
            return kNoBucket;
        }
        if (!leaf) {
            lv.res[i] = kInvalid;
            lv.cnt[i] = 0;
            return kNoBucket;
        }
        c[0] = uint32_t(leaf);
        c[1] = uint32_t(leaf >> 32);
        hash = hash_leaf(leaf);
    } else if (state == kDescend) {
        const uint32_t base = 8 * lv.exp[i];
        const uint32_t old = lv.old[i];
        uint32_t mask = 0, k = 1, total = 0;
        bool changed = false;
        for (uint32_t s = 0; s < 8; s++) {
            // the old child in slot s: the spawned child's old node (all 8
            // children were spawned; kInvalid where the old node had none),
            // so the old node itself is not read again
            const uint32_t oc = child.old[base + s];
            const uint8_t cs = child.state[base + s];
            const uint32_t nc = cs == kSkip ? oc : child.res[base + s];
            changed |= nc != oc;
            if (nc != kInvalid) {
                mask |= 1u << s;
                c[k++] = nc;
                if (level >= T)
                    total += child.cnt[base + s];
            }
        }
        lv.cnt[i] = total;
        if (!changed) {
            lv.res[i] = old;
            return kNoBucket;
        }
        if (!mask) {
            lv.res[i] = kInvalid;
            lv.cnt[i] = 0;
            return kNoBucket;
        }
        c[0] = (level >= T ? (total << 8) : 0u) | mask;
        hash = hash_interior(k, c);
    } else {
        return kNoBucket;
    }
    const uint32_t bucket = hash & (t.g.buckets(level) - 1);
    lv.res[i] = kNotFound; // resolved by find-or-add
    return bucket;
}

// One warp per bucket: the bucket's candidates, in depth-first order, each
// resolved against the bucket as it stands (earlier candidates' appends
// included) and appended when not found.  A per-warp cache remembers, for
// every content already resolved in this bucket, the positions where a copy
// lies (the first match a scan sees, the bucket's last node when it holds
// the content, and the copies appended since): a repeated content then needs
// no new scan, only the visibility rule on those positions.  Runs of
// identical candidates after a found result take that result at once.
constexpr uint32_t kCache = 32;
constexpr uint32_t kCachePos = 3;

struct FoaCache {
    uint32_t words[kCache][9];
    uint32_t n[kCache];
    uint32_t npos[kCache];
    uint32_t pos[kCache][kCachePos];
};

// A node at bucket position p (a walk position) of size n is compared by the
// reference's interior scan iff p + n < min(S, page end) (leaves: always).
HD_D bool visible(uint32_t p, uint32_t n, uint32_t S, bool leaf)
{
    if (leaf)
        return p + 2 <= S;
    const uint32_t pe = (p & ~(kPage - 1)) + kPage;
    return p + n < (S < pe ? S : pe);
}

// Copies words [0, used) of a page (used <= kPage) into the warp's shared
// buffer, PW words per lane and load (the probe width: 1, 2 or 4).  L2-
// coherent loads: the same kernel appends nodes and maps pages.  Up to PW-1
// words past `used`, still inside the page, are copied too.
template <int PW>
HD_D void stage_page(const uint32_t* src, uint32_t used, uint32_t* page, uint32_t lane)
{
    if constexpr (PW == 4) {
        for (uint32_t w = lane * 4; w < used; w += 128) {
            const uint4 v = __ldcg(reinterpret_cast<const uint4*>(src + w));
            page[w] = v.x;
            page[w + 1] = v.y;
            page[w + 2] = v.z;
            page[w + 3] = v.w;
        }
    } else if constexpr (PW == 2) {
        for (uint32_t w = lane * 2; w < used; w += 64) {
            const uint2 v = __ldcg(reinterpret_cast<const uint2*>(src + w));
            page[w] = v.x;
            page[w + 1] = v.y;
        }
    } else {
        for (uint32_t w = lane; w < used; w += 32)
            page[w] = __ldcg(src + w);
    }
}

// Warp-wide scan of the bucket for the first compared position holding q
// (find_leaf_node_in_bucket / find_interior_node_in_bucket); returns the
// bucket position or kNotFound.  *last_match: for interiors, the bucket's
// last node when it holds q (compared by no scan until something follows).
template <int PW>
HD_D uint32_t scan_bucket(const Table& t, uint32_t vbase, uint32_t S, const uint32_t* q, uint32_t n, bool leaf,
                          uint32_t bloom, uint32_t pt_lane, uint32_t* page, uint32_t* last_match,
                          unsigned long long& scanned)
{
    const uint32_t lane = threadIdx.x & 31;
    uint32_t found = kNotFound;
    *last_match = kNotFound;
    // the filters of the bucket's first 32 pages at once, a lane per page
    // (pt_lane: the physical page behind the bucket's page `lane`, read
    // once per bucket run)
    const uint32_t npages = (S + kPage - 1) / kPage;
    const uint32_t may = __ballot_sync(0xffffffffu, lane < npages && bloom_may_phys(t, pt_lane, bloom));
    for (uint32_t pindex = 0; pindex < S && found == kNotFound; pindex += kPage) {
        const uint32_t page_end = S < pindex + kPage ? S : pindex + kPage;
        if (!leaf && pindex + n >= page_end)
            break; // "return 0xFFFFFFFF" of the reference scan
        const uint32_t pi = pindex / kPage;
        if (pi < 32 ? !((may >> pi) & 1u) : !bloom_may(t, vbase + pindex, bloom))
            continue; // the page cannot hold q
        const uint32_t used = page_end - pindex;
        const uint32_t phys = __shfl_sync(0xffffffffu, pt_lane, pi & 31);
        stage_page<PW>(pi < 32 ? t.pool + (uint64_t(phys) << kPageShift) : t.sys_cg(vbase + pindex), used, page, lane);
        __syncwarp();
        if (leaf) {
            for (uint32_t w0 = 0; w0 < used && found == kNotFound; w0 += 64) {
                const uint32_t w = w0 + 2 * lane;
                const bool m = w < used && page[w] == q[0] && page[w + 1] == q[1];
                const uint32_t b = __ballot_sync(0xffffffffu, m);
                if (b)
                    found = pindex + w0 + 2 * (__ffs(b) - 1);
            }
        } else {
            const uint32_t lim = used - n;
            for (uint32_t w0 = 0; w0 < lim && found == kNotFound; w0 += 32) {
                const uint32_t w = w0 + lane;
                bool m = w < lim && page[w] == q[0];
                if (m)
                    for (uint32_t k = 1; k < n; k++)
                        m &= page[w + k] == q[k];
                uint32_t b = __ballot_sync(0xffffffffu, m);
                while (b && found == kNotFound) {
                    const uint32_t cand = w0 + __ffs(b) - 1;
                    b &= b - 1;
                    uint32_t on_walk = 0;
                    if (lane == 0) {
                        uint32_t p = 0;
                        while (p < cand)
                            p += total_size(page[p]);
                        on_walk = p == cand;
                    }
                    on_walk = __shfl_sync(0xffffffffu, on_walk, 0);
                    if (on_walk)
                        found = pindex + cand;
                }
            }
        }
        scanned += found == kNotFound ? used : (found - pindex + n);
        __syncwarp();
    }
    const uint32_t tail_pi = (S - n) / kPage;
    if (!leaf && found == kNotFound && S >= n && ((S - n) & ~(kPage - 1)) == ((S - 1) & ~(kPage - 1)) &&
        (tail_pi < 32 ? ((may >> tail_pi) & 1u) != 0 : bloom_may(t, vbase + ((S - n) & ~(kPage - 1)), bloom))) {
        // the bucket's last node ends at S; it holds q iff it starts at S - n
        // (nodes never straddle a page, so S - n lies in the tail's page)
        const uint32_t p = S - n;
        const uint32_t pindex = p & ~(kPage - 1);
        const uint32_t phys = __shfl_sync(0xffffffffu, pt_lane, tail_pi & 31);
        stage_page<PW>(tail_pi < 32 ? t.pool + (uint64_t(phys) << kPageShift) : t.sys_cg(vbase + pindex), S - pindex,
                       page, lane); // S - pindex <= kPage
        __syncwarp();
        uint32_t ok = 0;
        if (lane == 0) {
            bool m = true;
            for (uint32_t k = 0; k < n; k++)
                m &= page[p - pindex + k] == q[k];
            if (m) {
                uint32_t w = 0;
                while (w < p - pindex)
                    w += total_size(page[w]);
                ok = w == p - pindex;
            }
        }
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (ok)
            *last_match = p;
        __syncwarp();
    }
    return found;
}

// Resolves the candidates vals[j0..j1) of one bucket (all lanes of a warp):
// each gets its index in lv.res.  page / q / cache: the warp's shared
// buffers.  Returns false when an append failed (the device error word says
// why); the bucket size is written back either way.
template <int PW>
HD_D bool foa_segment(const Table& t, uint32_t level, const Level& lv, const uint32_t* __restrict__ vals, uint32_t j0,
                      uint32_t j1, uint32_t bucket, uint32_t* page, uint32_t* q, FoaCache& cache,
                      unsigned long long& foa, unsigned long long& added, unsigned long long& scanned)
{
    const uint32_t lane = threadIdx.x & 31;
    const bool leaf = level == t.g.leaf_level;
    const uint32_t gb = t.g.bucket_global(level, bucket);
    const uint32_t vbase = t.g.make_ptr(level, bucket, 0);
    uint32_t S = __ldcg(t.bucket_sizes + gb);
    // the bucket's page-table entries, lane p holding page p's (the warp owns
    // the bucket for the run: only its own appends map pages here)
    const uint32_t vpage0 = vbase >> kPageShift, cap_pages = t.g.capacity(level) >> kPageShift;
    uint32_t pt_lane = lane < cap_pages ? __ldcg(t.page_table + vpage0 + lane) : 0u;
    uint32_t used_entries = 0, next_slot = 0;
    bool failed = false;
    uint32_t j = j0;
    // the run's entry indices 32 at a time (lane k: entry of position vb + k)
    // and the next candidate's words loaded while the current one resolves
    uint32_t vb = j0, vreg = j0 + lane < j1 ? vals[j0 + lane] : 0u;
    const uint32_t c0 = __shfl_sync(0xffffffffu, vreg, 0); // every lane: a full-warp shuffle
    uint32_t qj = j0, qw = lane < 9 ? lv.cand[9 * uint64_t(c0) + lane] : 0u;
    while (j < j1 && !failed) {
        if (j - vb >= 32) {
            vb = j;
            vreg = j + lane < j1 ? vals[j + lane] : 0u;
        }
        const uint32_t ci = __shfl_sync(0xffffffffu, vreg, j - vb);
        if (qj != j && lane < 9)
            qw = lv.cand[9 * uint64_t(ci) + lane];
        if (lane < 9)
            q[lane] = qw;
        __syncwarp();
        // prefetch candidate j + 1 (its entry index is in vreg unless it
        // starts the next group of 32)
        qj = j + 1;
        if (qj < j1 && qj - vb < 32) {
            const uint32_t cn = __shfl_sync(0xffffffffu, vreg, qj - vb);
            if (lane < 9)
                qw = lv.cand[9 * uint64_t(cn) + lane];
        } else {
            qj = kNotFound;
        }
        const uint32_t n = leaf ? 2 : total_size(q[0]);
        // cache lookup: lane e checks entry e
        bool hit = lane < used_entries && cache.n[lane] == n;
        if (hit)
            for (uint32_t k = 0; k < n; k++)
                hit &= cache.words[lane][k] == q[k];
        const uint32_t hb = __ballot_sync(0xffffffffu, hit);
        const uint32_t bloom = bloom_bits(q, n);
        uint32_t e;
        if (hb) {
            e = __ffs(hb) - 1;
        } else {
            uint32_t last_match;
            const uint32_t f = scan_bucket<PW>(t, vbase, S, q, n, leaf, bloom, pt_lane, page, &last_match, scanned);
            e = next_slot;
            next_slot = (next_slot + 1) % kCache;
            used_entries = used_entries < kCache ? used_entries + 1 : kCache;
            if (lane < 9)
                cache.words[e][lane] = q[lane];
            if (lane == 0) {
                cache.n[e] = n;
                cache.npos[e] = 0;
                if (f != kNotFound)
                    cache.pos[e][cache.npos[e]++] = f;
                else if (last_match != kNotFound)
                    cache.pos[e][cache.npos[e]++] = last_match;
            }
            __syncwarp();
        }
        // the first visible copy, else append (lane 0)
        uint32_t result = kNotFound, appended = 0, ok = 1;
        const uint32_t S_scan = S;
        // where an append would go, on every lane (S and n are the warp's),
        // and the physical page there when it is already mapped: the pages
        // below the size are, so an append that stays in the size's last
        // page reads no page-table entry
        uint32_t a_size = S;
        const uint32_t a_pos = append_position(a_size, n, leaf);
        const bool a_mapped = S > 0 && a_size <= ((S + kPage - 1) & ~(kPage - 1));
        const uint32_t a_phys = __shfl_sync(0xffffffffu, pt_lane, (a_pos >> kPageShift) & 31);
        if (lane == 0) {
            for (uint32_t k = 0; k < cache.npos[e] && result == kNotFound; k++)
                if (visible(cache.pos[e][k], n, S, leaf))
                    result = cache.pos[e][k];
            if (result == kNotFound) {
                uint32_t size = a_size;
                const uint32_t pos = a_pos;
                if (size > t.g.capacity(level)) {
                    set_error(t.error, kErrBucketFull, level, bucket, size);
                    ok = 0;
                } else if (!a_mapped && !map_pages(t, level, bucket, pos, size)) {
                    ok = 0;
                } else {
                    const uint32_t phys =
                        a_mapped && (pos >> kPageShift) < 32 ? a_phys : __ldcg(t.page_table + vpage0 + (pos >> kPageShift));
                    uint32_t* dst = t.pool + (uint64_t(phys) << kPageShift) + (pos & (kPage - 1));
                    for (uint32_t k = 0; k < n; k++)
                        __stcg(dst + k, q[k]);
                    bloom_add_phys(t, phys, bloom);
                    result = pos;
                    S = size;
                    appended = 1;
                    if (cache.npos[e] == kCachePos) { // keep the newest copies
                        for (uint32_t k = 1; k < kCachePos; k++)
                            cache.pos[e][k - 1] = cache.pos[e][k];
                        cache.npos[e]--;
                    }
                    cache.pos[e][cache.npos[e]++] = pos;
                }
            }
            lv.res[ci] = vbase + result;
        }
        ok = __shfl_sync(0xffffffffu, ok, 0);
        result = __shfl_sync(0xffffffffu, result, 0);
        appended = __shfl_sync(0xffffffffu, appended, 0);
        const uint32_t S_before = __shfl_sync(0xffffffffu, S_scan, 0);
        S = __shfl_sync(0xffffffffu, S, 0);
        // an append that reached a new page mapped it: refresh that lane
        if (appended && lane < cap_pages && lane * kPage < S && lane * kPage + kPage > S_before)
            pt_lane = __ldcg(t.page_table + vpage0 + lane);
        foa++;
        added += appended;
        if (!ok) {
            failed = true;
            break;
        }
        j++;
        // a found result holds for the identical candidates that follow
        if (!appended) {
            for (;;) {
                const uint32_t jj = j + lane;
                bool same = jj < j1;
                if (same) {
                    const uint32_t* c = lv.cand + 9 * uint64_t(vals[jj]);
                    for (uint32_t k = 0; k < n; k++)
                        same &= c[k] == q[k];
                }
                const uint32_t b = __ballot_sync(0xffffffffu, same);
                const uint32_t run = b == 0xffffffffu ? 32u : __ffs(~b) - 1;
                if (lane < run)
                    lv.res[vals[jj]] = vbase + result;
                foa += run;
                j += run;
                if (run < 32)
                    break;
            }
        }
        __syncwarp();
    }
    if (lane == 0)
        __stcg(t.bucket_sizes + gb, S);
    return !failed;
}

} // namespace hd
