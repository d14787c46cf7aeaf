// Seeded procedural scene voxelised on the device into a BasicDAG.
//
// The scene is the integer function of hashdag_gb300/scene.py: a Q16
// fixed-point fractal value-noise height field united with 64 spheres.
// Pipeline (levels of the DAG, root 0 .. leaf depth-2):
//   1. min/max of the height over every node footprint (a quad pyramid);
//   2. top-down, each level's "mixed" nodes (neither entirely solid nor
//      entirely empty by exact height bounds and sphere/box tests) expand
//      into the next level; leaves get their 64-bit masks;
//   3. bottom-up, nodes deduplicated per level by content (mask and child
//      ids) in a device hash set, voxel counts summed;
//   4. top-down depth-first first-visit ranks, then the BasicDAG words
//      (basic_dag.h:11-40) laid out level by level in rank order: headers
//      mask | count << 8 at levels >= C_colorTreeLevels, mask | enclosed
//      index << 8 above (the enclosedLeaves convention, basic_dag.h:47-76).
#include <vector>

#include "hd_ctx.h"

namespace hd {

__constant__ int64_t c_spheres[256];

HD_HD int64_t lattice_value(uint64_t seed, uint32_t octave, uint32_t i, uint32_t j)
{
    const uint64_t k = mix64(seed ^ mix64((uint64_t(octave) << 58) ^ (uint64_t(i) << 29) ^ uint64_t(j)));
    return int64_t(k >> 47) - 65536;
}
HD_HD int64_t smooth_q16(int64_t t) { return (t * t * (3 * 65536 - 2 * t)) >> 32; }
HD_HD int64_t floor_div(int64_t a, int64_t b)
{
    int64_t q = a / b;
    if ((a % b) != 0 && a < 0)
        q -= 1;
    return q;
}
HD_HD int64_t scene_height(uint64_t seed, uint32_t depth, uint32_t x, uint32_t z)
{
    int64_t total = 0;
    for (uint32_t o = 0; o < 5; o++) {
        const uint32_t lp = depth - 2 - o;
        const uint32_t i = x >> lp, j = z >> lp;
        const uint32_t fx = x & ((1u << lp) - 1), fz = z & ((1u << lp) - 1);
        const int64_t sx = smooth_q16(int64_t((uint64_t(fx) << 16) >> lp));
        const int64_t sz = smooth_q16(int64_t((uint64_t(fz) << 16) >> lp));
        const int64_t v00 = lattice_value(seed, o, i, j), v10 = lattice_value(seed, o, i + 1, j);
        const int64_t v01 = lattice_value(seed, o, i, j + 1), v11 = lattice_value(seed, o, i + 1, j + 1);
        const int64_t a = v00 + (((v10 - v00) * sx) >> 16);
        const int64_t b = v01 + (((v11 - v01) * sx) >> 16);
        const int64_t n = a + (((b - a) * sz) >> 16);
        total += n >> o;
    }
    const int64_t e = int64_t(1) << depth;
    return (e >> 1) + floor_div(total * e, 31 * 16384);
}

static void scene_spheres(uint64_t seed, uint32_t depth, int64_t* out)
{
    uint64_t state = seed ^ 0x5EED5EED12345678ull;
    const uint64_t mask = (uint64_t(1) << depth) - 1;
    for (int s = 0; s < 64; s++) {
        state += 0x9E3779B97F4A7C15ull;
        out[4 * s + 0] = int64_t(mix64(state) & mask);
        state += 0x9E3779B97F4A7C15ull;
        out[4 * s + 1] = int64_t(mix64(state) & mask);
        state += 0x9E3779B97F4A7C15ull;
        out[4 * s + 2] = int64_t(mix64(state) & mask);
        state += 0x9E3779B97F4A7C15ull;
        out[4 * s + 3] = 8 + int64_t(mix64(state) % 57);
    }
}

// ---- 1. height bounds ------------------------------------------------------
// hmax: the maximum height over the 4x4 columns of a leaf footprint.  hmin:
// the minimum over the same columns, or with `grown` over the footprint grown
// by one column on every side (6x6; a column outside the volume counts as
// -infinity), which makes the shell scenes' height-field fullness test exact.
__global__ void k_height_leaf(uint64_t seed, uint32_t depth, uint32_t n, bool grown, int32_t* __restrict__ hmin,
                              int32_t* __restrict__ hmax)
{
    const int64_t E = int64_t(1) << depth;
    HD_GRID_STRIDE(idx, uint64_t(n) * n)
    {
        const uint32_t cx = uint32_t(idx / n), cz = uint32_t(idx % n);
        int64_t lo = INT64_MAX, hi = INT64_MIN;
        const int r = grown ? 1 : 0;
        for (int a = -r; a < 4 + r; a++)
            for (int b = -r; b < 4 + r; b++) {
                const int64_t x = int64_t(4 * cx) + a, z = int64_t(4 * cz) + b;
                const bool in = a >= 0 && a < 4 && b >= 0 && b < 4;
                if (x < 0 || z < 0 || x >= E || z >= E) {
                    lo = INT32_MIN;
                    continue;
                }
                const int64_t h = scene_height(seed, depth, uint32_t(x), uint32_t(z));
                lo = h < lo ? h : lo;
                if (in)
                    hi = h > hi ? h : hi;
            }
        hmin[idx] = int32_t(lo);
        hmax[idx] = int32_t(hi);
    }
}

__global__ void k_height_reduce(uint32_t m, const int32_t* __restrict__ cmin, const int32_t* __restrict__ cmax,
                                int32_t* __restrict__ hmin, int32_t* __restrict__ hmax)
{
    HD_GRID_STRIDE(idx, uint64_t(m) * m)
    {
        const uint32_t cx = uint32_t(idx / m), cz = uint32_t(idx % m);
        const uint64_t m2 = 2ull * m;
        int32_t lo = INT32_MAX, hi = INT32_MIN;
        for (uint32_t a = 0; a < 2; a++)
            for (uint32_t b = 0; b < 2; b++) {
                const uint64_t i = (2ull * cx + a) * m2 + 2ull * cz + b;
                lo = cmin[i] < lo ? cmin[i] : lo;
                hi = cmax[i] > hi ? cmax[i] : hi;
            }
        hmin[idx] = lo;
        hmax[idx] = hi;
    }
}

// ---- 2. top-down frontier --------------------------------------------------
// classification of the region of node (x, y, z) at `level`: 0 empty,
// 1 full, 2 mixed; *live = spheres touching it.
HD_D uint32_t classify(uint32_t depth, uint32_t level, uint32_t x, uint32_t y, uint32_t z, const int32_t* hmin,
                       const int32_t* hmax, uint64_t parent_live, uint64_t* live)
{
    const uint32_t shift = depth - level;
    const int64_t s = int64_t(1) << shift;
    const uint64_t cell = (uint64_t(x) << level) | z;
    const int64_t y0 = int64_t(y) << shift;
    const int64_t x0 = int64_t(x) << shift, z0 = int64_t(z) << shift;
    bool full = y0 + s - 1 <= hmin[cell];
    bool touched = y0 <= hmax[cell];
    uint64_t out = 0;
    uint64_t todo = parent_live;
    while (todo) {
        const uint32_t k = __ffsll(todo) - 1;
        todo &= todo - 1;
        const int64_t* sp = c_spheres + 4 * k;
        const int64_t lo[3] = {x0, y0, z0};
        int64_t d2near = 0, d2far = 0;
        for (int a = 0; a < 3; a++) {
            const int64_t c = sp[a], l = lo[a], h = lo[a] + s - 1;
            const int64_t dn = c < l ? l - c : (c > h ? c - h : 0);
            const int64_t df = (c - l) > (h - c) ? (c - l) : (h - c);
            d2near += dn * dn;
            d2far += df * df;
        }
        const int64_t r2 = sp[3] * sp[3];
        if (d2near <= r2) {
            out |= 1ull << k;
            touched = true;
            if (d2far <= r2)
                full = true;
        }
    }
    *live = out;
    if (full)
        return 1;
    if (!touched)
        return 0;
    return 2;
}

// Shell scenes: a node holds no shell voxel when it holds no solid voxel or
// when the node grown by one voxel on every side is solid throughout (single
// source: the height field alone or one sphere alone; conservative).  *live
// = spheres touching the grown node.  Returns 0 (empty) or 2 (mixed).
HD_D uint32_t classify_shell(uint32_t depth, uint32_t level, uint32_t x, uint32_t y, uint32_t z, const int32_t* hmin,
                             const int32_t* hmax, uint64_t parent_live, uint64_t* live)
{
    const uint32_t shift = depth - level;
    const int64_t s = int64_t(1) << shift, E = int64_t(1) << depth;
    const uint64_t m = uint64_t(1) << level;
    const int64_t x0 = int64_t(x) << shift, y0 = int64_t(y) << shift, z0 = int64_t(z) << shift;
    bool touched = y0 <= hmax[(uint64_t(x) << level) | z];
    const bool inside = x0 > 0 && z0 > 0 && y0 > 0 && x0 + s < E && z0 + s < E && y0 + s < E;
    // hmin holds the minimum over the grown footprint in shell scenes
    bool full = inside && y0 + s <= hmin[uint64_t(x) * m + z];
    uint64_t out = 0;
    uint64_t todo = parent_live;
    while (todo) {
        const uint32_t k = __ffsll(todo) - 1;
        todo &= todo - 1;
        const int64_t* sp = c_spheres + 4 * k;
        const int64_t lo3[3] = {x0, y0, z0};
        int64_t d2in = 0, d2near = 0, d2far = 0;
        for (int a = 0; a < 3; a++) {
            const int64_t c = sp[a], l = lo3[a], h = lo3[a] + s - 1;
            const int64_t din = c < l ? l - c : (c > h ? c - h : 0);
            const int64_t dn = c < l - 1 ? l - 1 - c : (c > h + 1 ? c - h - 1 : 0);
            const int64_t df = (c - l + 1) > (h + 1 - c) ? (c - l + 1) : (h + 1 - c);
            d2in += din * din;
            d2near += dn * dn;
            d2far += df * df;
        }
        const int64_t r2 = sp[3] * sp[3];
        if (d2near <= r2)
            out |= 1ull << k;
        if (d2in <= r2)
            touched = true;
        if (inside && d2far <= r2)
            full = true;
    }
    *live = out;
    return (!touched || full) ? 0u : 2u;
}

HD_D uint32_t classify_any(bool shell, uint32_t depth, uint32_t level, uint32_t x, uint32_t y, uint32_t z,
                           const int32_t* hmin, const int32_t* hmax, uint64_t parent_live, uint64_t* live)
{
    return shell ? classify_shell(depth, level, x, y, z, hmin, hmax, parent_live, live)
                 : classify(depth, level, x, y, z, hmin, hmax, parent_live, live);
}

struct Frontier {
    uint32_t* x;
    uint32_t* y;
    uint32_t* z;
    uint64_t* live;
};

__global__ void k_classify_children(bool shell, uint32_t depth, uint32_t level, Frontier f, uint32_t n,
                                    const int32_t* hmin, const int32_t* hmax, uint32_t* __restrict__ cls2,
                                    uint32_t* __restrict__ nmixed)
{
    HD_GRID_STRIDE(i, n)
    {
        uint32_t c2 = 0, nm = 0;
        const uint32_t px = f.x[i], py = f.y[i], pz = f.z[i];
        const uint64_t pl = f.live[i];
        for (uint32_t c = 0; c < 8; c++) {
            uint64_t live;
            const uint32_t cls = classify_any(shell, depth, level + 1, 2 * px + ((c >> 2) & 1),
                                              2 * py + ((c >> 1) & 1), 2 * pz + (c & 1), hmin, hmax, pl, &live);
            c2 |= cls << (2 * c);
            nm += cls == 2;
        }
        cls2[i] = c2;
        nmixed[i] = nm;
    }
}

__global__ void k_expand(bool shell, uint32_t depth, uint32_t level, Frontier f, uint32_t n,
                         const uint32_t* __restrict__ cls2, const uint32_t* __restrict__ coff, const int32_t* hmin,
                         const int32_t* hmax, Frontier out)
{
    HD_GRID_STRIDE(i, n)
    {
        uint32_t o = coff[i];
        const uint32_t c2 = cls2[i];
        for (uint32_t c = 0; c < 8; c++) {
            if (((c2 >> (2 * c)) & 3) != 2)
                continue;
            const uint32_t cx = 2 * f.x[i] + ((c >> 2) & 1), cy = 2 * f.y[i] + ((c >> 1) & 1), cz = 2 * f.z[i] + (c & 1);
            uint64_t live;
            classify_any(shell, depth, level + 1, cx, cy, cz, hmin, hmax, f.live[i], &live);
            out.x[o] = cx;
            out.y[o] = cy;
            out.z[o] = cz;
            out.live[o] = live;
            o++;
        }
    }
}

__global__ void k_leaf_masks(uint64_t seed, uint32_t depth, Frontier f, uint32_t n, uint64_t* __restrict__ masks)
{
    HD_GRID_STRIDE(i, n)
    {
        const uint32_t x0 = f.x[i] << 2, y0 = f.y[i] << 2, z0 = f.z[i] << 2;
        const uint64_t live = f.live[i];
        uint64_t leaf = 0;
        for (uint32_t lx = 0; lx < 4; lx++)
            for (uint32_t lz = 0; lz < 4; lz++) {
                const int64_t h = scene_height(seed, depth, x0 + lx, z0 + lz);
                for (uint32_t ly = 0; ly < 4; ly++) {
                    const int64_t x = x0 + lx, y = y0 + ly, z = z0 + lz;
                    bool solid = y <= h;
                    uint64_t todo = live;
                    while (!solid && todo) {
                        const uint32_t k = __ffsll(todo) - 1;
                        todo &= todo - 1;
                        const int64_t* sp = c_spheres + 4 * k;
                        const int64_t dx = x - sp[0], dy = y - sp[1], dz = z - sp[2];
                        solid = dx * dx + dy * dy + dz * dz <= sp[3] * sp[3];
                    }
                    if (solid) {
                        const uint32_t c1 = ((lx >> 1) << 2) | ((ly >> 1) << 1) | (lz >> 1);
                        const uint32_t c2 = ((lx & 1) << 2) | ((ly & 1) << 1) | (lz & 1);
                        leaf |= 1ull << (c1 * 8 + c2);
                    }
                }
            }
        masks[i] = leaf;
    }
}

// Shell leaves: solid voxels with an empty face neighbour; heights of the
// 6x6 footprint around the leaf, outside the volume empty.
HD_D bool shell_solid(const int64_t* h, uint64_t live, int64_t E, int64_t x0, int64_t z0, int64_t x, int64_t y,
                      int64_t z)
{
    if (x < 0 || y < 0 || z < 0 || x >= E || y >= E || z >= E)
        return false;
    if (y <= h[(x - x0 + 1) * 6 + (z - z0 + 1)])
        return true;
    uint64_t todo = live;
    while (todo) {
        const uint32_t k = __ffsll(todo) - 1;
        todo &= todo - 1;
        const int64_t* sp = c_spheres + 4 * k;
        const int64_t dx = x - sp[0], dy = y - sp[1], dz = z - sp[2];
        if (dx * dx + dy * dy + dz * dz <= sp[3] * sp[3])
            return true;
    }
    return false;
}

__global__ void k_leaf_masks_shell(uint64_t seed, uint32_t depth, Frontier f, uint32_t n, uint64_t* __restrict__ masks)
{
    const int64_t E = int64_t(1) << depth;
    HD_GRID_STRIDE(i, n)
    {
        const int64_t x0 = int64_t(f.x[i]) << 2, y0 = int64_t(f.y[i]) << 2, z0 = int64_t(f.z[i]) << 2;
        const uint64_t live = f.live[i];
        int64_t h[36];
        for (int a = 0; a < 6; a++)
            for (int b = 0; b < 6; b++) {
                const int64_t x = x0 + a - 1, z = z0 + b - 1;
                h[a * 6 + b] = (x < 0 || z < 0 || x >= E || z >= E)
                                   ? -1
                                   : scene_height(seed, depth, uint32_t(x), uint32_t(z));
            }
        uint64_t leaf = 0;
        for (uint32_t lx = 0; lx < 4; lx++)
            for (uint32_t ly = 0; ly < 4; ly++)
                for (uint32_t lz = 0; lz < 4; lz++) {
                    const int64_t x = x0 + lx, y = y0 + ly, z = z0 + lz;
                    if (!shell_solid(h, live, E, x0, z0, x, y, z))
                        continue;
                    if (shell_solid(h, live, E, x0, z0, x + 1, y, z) && shell_solid(h, live, E, x0, z0, x - 1, y, z) &&
                        shell_solid(h, live, E, x0, z0, x, y + 1, z) && shell_solid(h, live, E, x0, z0, x, y - 1, z) &&
                        shell_solid(h, live, E, x0, z0, x, y, z + 1) && shell_solid(h, live, E, x0, z0, x, y, z - 1))
                        continue;
                    const uint32_t c1 = ((lx >> 1) << 2) | ((ly >> 1) << 1) | (lz >> 1);
                    const uint32_t c2 = ((lx & 1) << 2) | ((ly & 1) << 1) | (lz & 1);
                    leaf |= 1ull << (c1 * 8 + c2);
                }
        masks[i] = leaf;
    }
}

// ---- 3. bottom-up dedup ----------------------------------------------------
// Candidate content: 9 words [mask, kid0..kid7] (unused kids 0); leaves use
// words 0-1 for the 64-bit mask and a mask word of 0xFF.
HD_D uint64_t content_hash(const uint32_t* c)
{
    uint64_t h = mix64(c[0]);
    for (int k = 1; k < 9; k++)
        h = mix64(h ^ c[k]);
    return h;
}

__global__ void k_build_leaf_candidates(const uint64_t* __restrict__ masks, uint32_t n, uint32_t* __restrict__ cont,
                                        uint64_t* __restrict__ count, uint64_t* __restrict__ hash)
{
    HD_GRID_STRIDE(i, uint64_t(n) + 1)
    {
        const uint64_t m = i < n ? masks[i] : ~0ull;
        uint32_t* c = cont + 9 * i;
        c[0] = m ? 0xFFu : 0u;
        c[1] = uint32_t(m);
        c[2] = uint32_t(m >> 32);
        for (int k = 3; k < 9; k++)
            c[k] = 0;
        count[i] = popc64(m);
        hash[i] = content_hash(c);
    }
}

__global__ void k_build_interior_candidates(uint32_t depth, uint32_t level, uint32_t n,
                                            const uint32_t* __restrict__ cls2, const uint32_t* __restrict__ coff,
                                            const uint32_t* __restrict__ child_uid,
                                            const uint64_t* __restrict__ child_ucount, uint32_t child_full,
                                            uint32_t* __restrict__ cont, uint64_t* __restrict__ count,
                                            uint64_t* __restrict__ hash)
{
    const uint64_t child_full_count = uint64_t(1) << (3 * (depth - level - 1));
    HD_GRID_STRIDE(i, uint64_t(n) + 1)
    {
        uint32_t* c = cont + 9 * i;
        uint32_t mask = 0, nk = 0;
        uint64_t total = 0;
        uint32_t kids[8];
        if (i == n) { // the canonical full node of this level
            mask = 0xFF;
            for (int k = 0; k < 8; k++)
                kids[nk++] = child_full;
            total = 8 * child_full_count;
        } else {
            const uint32_t c2 = cls2[i];
            uint32_t j = coff[i];
            for (uint32_t k = 0; k < 8; k++) {
                const uint32_t cls = (c2 >> (2 * k)) & 3;
                if (cls == 1) {
                    mask |= 1u << k;
                    kids[nk++] = child_full;
                    total += child_full_count;
                } else if (cls == 2) {
                    const uint32_t u = child_uid[j++];
                    if (u != kEmptyId) {
                        mask |= 1u << k;
                        kids[nk++] = u;
                        total += child_ucount[u];
                    }
                }
            }
        }
        c[0] = mask;
        for (uint32_t k = 0; k < 8; k++)
            c[1 + k] = k < nk ? kids[k] : 0;
        count[i] = total;
        hash[i] = content_hash(c);
    }
}

__global__ void k_dedup_insert(const uint32_t* __restrict__ cont, const uint64_t* __restrict__ hash, uint64_t n,
                               uint32_t* __restrict__ slots, uint64_t cap, uint32_t* __restrict__ slot_of,
                               uint32_t* err)
{
    HD_GRID_STRIDE(i, n)
    {
        const uint32_t* ci = cont + 9 * i;
        if (ci[0] == 0) { // empty content
            slot_of[i] = kEmptyId;
            continue;
        }
        const uint64_t h = hash[i];
        uint64_t s = h & (cap - 1);
        uint32_t found = kEmptyId;
        for (uint64_t probe = 0; probe < cap; probe++) {
            uint32_t v = slots[s];
            if (v == 0) {
                v = atomicCAS(slots + s, 0u, uint32_t(i) + 1);
                if (v == 0) {
                    found = uint32_t(s);
                    break;
                }
            }
            const uint32_t j = v - 1;
            if (hash[j] == h) {
                const uint32_t* cj = cont + 9 * uint64_t(j);
                bool same = true;
                for (int k = 0; k < 9; k++)
                    same &= ci[k] == cj[k];
                if (same) {
                    found = uint32_t(s);
                    break;
                }
            }
            s = (s + 1) & (cap - 1);
        }
        if (found == kEmptyId)
            set_error(err, kErrCapacity);
        slot_of[i] = found;
    }
}

__global__ void k_rep_flags(const uint32_t* __restrict__ slots, const uint32_t* __restrict__ slot_of, uint64_t n,
                            uint32_t* __restrict__ flag)
{
    HD_GRID_STRIDE(i, n)
    {
        const uint32_t s = slot_of[i];
        flag[i] = s != kEmptyId && slots[s] == uint32_t(i) + 1;
    }
}

__global__ void k_assign_uid(const uint32_t* __restrict__ slots, const uint32_t* __restrict__ slot_of,
                             const uint32_t* __restrict__ dense, uint64_t n, const uint32_t* __restrict__ cont,
                             const uint64_t* __restrict__ count, uint32_t* __restrict__ uid,
                             uint32_t* __restrict__ ucont, uint64_t* __restrict__ ucount)
{
    HD_GRID_STRIDE(i, n)
    {
        const uint32_t s = slot_of[i];
        if (s == kEmptyId) {
            uid[i] = kEmptyId;
            continue;
        }
        const uint32_t rep = slots[s] - 1;
        const uint32_t u = dense[rep];
        uid[i] = u;
        if (rep == i) {
            for (int k = 0; k < 9; k++)
                ucont[9 * uint64_t(u) + k] = cont[9 * i + k];
            ucount[u] = count[i];
        }
    }
}

// ---- 4. ranks and emission -------------------------------------------------
__global__ void k_unique_child_keys(const uint32_t* __restrict__ order, uint32_t n, const uint32_t* __restrict__ ucont,
                                    uint32_t* __restrict__ key_child)
{
    HD_GRID_STRIDE(r, n)
    {
        const uint32_t* c = ucont + 9 * uint64_t(order[r]);
        const uint32_t mask = c[0];
        uint32_t k = 1;
        for (uint32_t slot = 0; slot < 8; slot++)
            if (mask & (1u << slot))
                atomicMin(key_child + c[k++], uint32_t(r) * 8 + slot);
    }
}

__global__ void k_scatter_keys(const uint32_t* __restrict__ key_child, uint32_t n_child, uint32_t* __restrict__ by_key)
{
    HD_GRID_STRIDE(u, n_child)
    {
        const uint32_t k = key_child[u];
        if (k != 0xFFFFFFFFu)
            by_key[k] = uint32_t(u);
    }
}

__global__ void k_flags(const uint32_t* __restrict__ by_key, uint64_t n, uint32_t* __restrict__ flag)
{
    HD_GRID_STRIDE(i, n) flag[i] = by_key[i] != 0xFFFFFFFFu;
}

__global__ void k_compact_order(const uint32_t* __restrict__ by_key, const uint32_t* __restrict__ pos, uint64_t n,
                                uint32_t* __restrict__ order, uint32_t* __restrict__ rank)
{
    HD_GRID_STRIDE(i, n)
    {
        const uint32_t u = by_key[i];
        if (u != 0xFFFFFFFFu) {
            order[pos[i]] = u;
            rank[u] = pos[i];
        }
    }
}

__global__ void k_node_sizes(const uint32_t* __restrict__ order, uint32_t n, const uint32_t* __restrict__ ucont,
                             bool leaf, uint32_t* __restrict__ size)
{
    HD_GRID_STRIDE(r, n) size[r] = leaf ? 2 : 1 + popc32(ucont[9 * uint64_t(order[r])]);
}

__global__ void k_word_of(const uint32_t* __restrict__ order, uint32_t n, const uint32_t* __restrict__ off,
                          uint64_t base, uint32_t* __restrict__ word_of)
{
    HD_GRID_STRIDE(r, n) word_of[order[r]] = uint32_t(base + off[r]);
}

__global__ void k_emit(uint32_t level, uint32_t T, bool leaf, const uint32_t* __restrict__ order, uint32_t n,
                       const uint32_t* __restrict__ ucont, const uint64_t* __restrict__ ucount,
                       const uint32_t* __restrict__ word_of, const uint32_t* __restrict__ child_word_of,
                       uint64_t enclosed_base, uint32_t* __restrict__ words, uint32_t* err)
{
    HD_GRID_STRIDE(r, n)
    {
        const uint32_t u = order[r];
        const uint32_t* c = ucont + 9 * uint64_t(u);
        uint32_t* w = words + word_of[u];
        if (leaf) {
            w[0] = c[1];
            w[1] = c[2];
            continue;
        }
        const uint64_t upper = level < T ? enclosed_base + r : ucount[u];
        if (upper >= (1u << 24))
            set_error(err, kErrCapacity);
        const uint32_t mask = c[0];
        w[0] = (uint32_t(upper) << 8) | mask;
        const uint32_t nk = popc32(mask);
        for (uint32_t k = 0; k < nk; k++)
            w[1 + k] = child_word_of[c[1 + k]];
    }
}

void generate_scene(hd_ctx* c, uint64_t seed, uint32_t flags, uint32_t** d_words_out, uint64_t* n_words_out)
{
    const bool shell = (flags & HD_SCENE_SHELL) != 0;
    cudaStream_t st = c->stream;
    Scratch& s = c->scratch;
    const uint32_t D = c->g.depth, leafl = c->g.leaf_level, T = c->g.T;
    if (D < 6 || D > 18)
        throw StatusError{HD_ERR_INVALID, "scene depth must be in [6, 18]"};
    {
        int64_t sp[256];
        scene_spheres(seed, D, sp);
        HD_CUDA(cudaMemcpyToSymbolAsync(c_spheres, sp, sizeof(sp), 0, cudaMemcpyHostToDevice, st));
    }
    // 1. height bounds per level (footprint of a level-L node: 2^(D-L) columns)
    std::vector<int32_t*> hmin(leafl + 1), hmax(leafl + 1);
    for (uint32_t L = 0; L <= leafl; L++) {
        char a[32], b[32];
        snprintf(a, 32, "scn_hmin_%u", L);
        snprintf(b, 32, "scn_hmax_%u", L);
        const uint64_t m = uint64_t(1) << L;
        hmin[L] = s.get<int32_t>(a, m * m);
        hmax[L] = s.get<int32_t>(b, m * m);
    }
    {
        const uint32_t n = 1u << leafl;
        k_height_leaf<<<grid_for(uint64_t(n) * n, 256, 152 * 64), 256, 0, st>>>(seed, D, n, shell, hmin[leafl],
                                                                                hmax[leafl]);
        HD_LAUNCH_CHECK();
        for (int32_t L = int32_t(leafl) - 1; L >= 0; L--) {
            const uint32_t m = 1u << L;
            k_height_reduce<<<grid_for(uint64_t(m) * m, 256), 256, 0, st>>>(m, hmin[L + 1], hmax[L + 1], hmin[L],
                                                                            hmax[L]);
            HD_LAUNCH_CHECK();
        }
    }
    // 2. frontier per level
    std::vector<Frontier> fr(leafl + 1);
    std::vector<uint32_t> nf(leafl + 1);
    std::vector<uint32_t*> cls2(leafl + 1), coff(leafl + 1);
    uint32_t* d_n = s.get<uint32_t>("scn_counter", 4);
    auto alloc_frontier = [&](uint32_t L, uint64_t n) {
        char nx[32], ny[32], nz[32], nl[32];
        snprintf(nx, 32, "scn_fx_%u", L);
        snprintf(ny, 32, "scn_fy_%u", L);
        snprintf(nz, 32, "scn_fz_%u", L);
        snprintf(nl, 32, "scn_fl_%u", L);
        Frontier f{s.get<uint32_t>(nx, n + 1), s.get<uint32_t>(ny, n + 1), s.get<uint32_t>(nz, n + 1),
                   s.get<uint64_t>(nl, n + 1)};
        return f;
    };
    auto drop_frontier = [&](uint32_t L) {
        const char* names[4] = {"scn_fx_%u", "scn_fy_%u", "scn_fz_%u", "scn_fl_%u"};
        for (const char* f : names) {
            char nm[32];
            snprintf(nm, 32, f, L);
            s.drop(nm);
        }
    };
    fr[0] = alloc_frontier(0, 1);
    {
        const uint32_t zero = 0;
        const uint64_t all = ~0ull;
        HD_CUDA(cudaMemcpyAsync(fr[0].x, &zero, 4, cudaMemcpyHostToDevice, st));
        HD_CUDA(cudaMemcpyAsync(fr[0].y, &zero, 4, cudaMemcpyHostToDevice, st));
        HD_CUDA(cudaMemcpyAsync(fr[0].z, &zero, 4, cudaMemcpyHostToDevice, st));
        HD_CUDA(cudaMemcpyAsync(fr[0].live, &all, 8, cudaMemcpyHostToDevice, st));
        HD_CUDA(cudaStreamSynchronize(st));
    }
    nf[0] = 1;
    for (uint32_t L = 0; L < leafl; L++) {
        const uint32_t n = nf[L];
        char a[32], b[32], d[32];
        snprintf(a, 32, "scn_cls2_%u", L);
        snprintf(b, 32, "scn_coff_%u", L);
        snprintf(d, 32, "scn_nm_%u", L);
        cls2[L] = s.get<uint32_t>(a, uint64_t(n) + 1);
        coff[L] = s.get<uint32_t>(b, uint64_t(n) + 1);
        uint32_t* nm = s.get<uint32_t>("scn_nm", uint64_t(n) + 1);
        k_classify_children<<<grid_for(n, 128), 128, 0, st>>>(shell, D, L, fr[L], n, hmin[L + 1], hmax[L + 1],
                                                              cls2[L], nm);
        HD_LAUNCH_CHECK();
        exclusive_scan<uint32_t, uint32_t>(s, nm, coff[L], n, d_n, st);
        const uint32_t nn = read_scalar(d_n, st);
        fr[L + 1] = alloc_frontier(L + 1, nn);
        nf[L + 1] = nn;
        k_expand<<<grid_for(n, 128), 128, 0, st>>>(shell, D, L, fr[L], n, cls2[L], coff[L], hmin[L + 1],
                                                   hmax[L + 1], fr[L + 1]);
        HD_LAUNCH_CHECK();
        // this level's paths are no longer needed (the dedup reads cls2 / coff)
        drop_frontier(L);
    }
    // height bounds no longer needed past this point: free them for the dedup
    // leaf masks
    uint64_t* masks = s.get<uint64_t>("scn_masks", uint64_t(nf[leafl]) + 1);
    if (shell)
        k_leaf_masks_shell<<<grid_for(nf[leafl], 128, 152 * 64), 128, 0, st>>>(seed, D, fr[leafl], nf[leafl], masks);
    else
        k_leaf_masks<<<grid_for(nf[leafl], 128, 152 * 64), 128, 0, st>>>(seed, D, fr[leafl], nf[leafl], masks);
    HD_LAUNCH_CHECK();
    drop_frontier(leafl);
    for (uint32_t L = 0; L <= leafl; L++) {
        char a[32], b[32];
        snprintf(a, 32, "scn_hmin_%u", L);
        snprintf(b, 32, "scn_hmax_%u", L);
        s.drop(a);
        s.drop(b);
    }
    // 3. bottom-up dedup
    std::vector<uint32_t*> ucont(leafl + 1);
    std::vector<uint64_t*> ucount(leafl + 1);
    std::vector<uint32_t> nu(leafl + 1), full_uid(leafl + 1);
    uint32_t* child_uid = nullptr;
    uint32_t root_uid = 0;
    for (int32_t L = int32_t(leafl); L >= 0; L--) {
        const uint64_t nc = uint64_t(nf[L]) + 1; // + canonical full
        uint32_t* cont = s.get<uint32_t>("scn_cont", nc * 9);
        uint64_t* cnt = s.get<uint64_t>("scn_cnt", nc);
        uint64_t* hash = s.get<uint64_t>("scn_hash", nc);
        if (L == int32_t(leafl)) {
            k_build_leaf_candidates<<<grid_for(nc, 256), 256, 0, st>>>(masks, nf[L], cont, cnt, hash);
        } else {
            k_build_interior_candidates<<<grid_for(nc, 256), 256, 0, st>>>(D, L, nf[L], cls2[L], coff[L], child_uid,
                                                                           ucount[L + 1], full_uid[L + 1], cont, cnt,
                                                                           hash);
        }
        HD_LAUNCH_CHECK();
        uint64_t cap = 1024;
        while (cap < 2 * nc)
            cap <<= 1;
        uint32_t* slots = s.get<uint32_t>("scn_slots", cap);
        HD_CUDA(cudaMemsetAsync(slots, 0, cap * 4, st));
        uint32_t* slot_of = s.get<uint32_t>("scn_slot_of", nc);
        k_dedup_insert<<<grid_for(nc, 256), 256, 0, st>>>(cont, hash, nc, slots, cap, slot_of, c->t.error);
        HD_LAUNCH_CHECK();
        uint32_t* flag = s.get<uint32_t>("scn_flag", nc);
        uint32_t* dense = s.get<uint32_t>("scn_dense", nc);
        k_rep_flags<<<grid_for(nc, 256), 256, 0, st>>>(slots, slot_of, nc, flag);
        HD_LAUNCH_CHECK();
        exclusive_scan<uint32_t, uint32_t>(s, flag, dense, nc, d_n, st);
        nu[L] = read_scalar(d_n, st);
        char a[32], b[32], d[32];
        snprintf(a, 32, "scn_ucont_%d", L);
        snprintf(b, 32, "scn_ucount_%d", L);
        snprintf(d, 32, "scn_uid_%d", L % 2);
        ucont[L] = s.get<uint32_t>(a, uint64_t(nu[L]) * 9 + 9);
        ucount[L] = s.get<uint64_t>(b, uint64_t(nu[L]) + 1);
        uint32_t* uid = s.get<uint32_t>(d, nc);
        k_assign_uid<<<grid_for(nc, 256), 256, 0, st>>>(slots, slot_of, dense, nc, cont, cnt, uid, ucont[L],
                                                        ucount[L]);
        HD_LAUNCH_CHECK();
        HD_CUDA(cudaMemcpyAsync(&full_uid[L], uid + nf[L], 4, cudaMemcpyDeviceToHost, st));
        if (L == 0)
            HD_CUDA(cudaMemcpyAsync(&root_uid, uid, 4, cudaMemcpyDeviceToHost, st));
        HD_CUDA(cudaStreamSynchronize(st));
        child_uid = uid;
    }
    if (check_error(c))
        throw StatusError{HD_ERR_OOM, "scene dedup table overflow"};
    if (root_uid == kEmptyId)
        throw StatusError{HD_ERR_INVALID, "empty scene"};
    // 4. ranks per level, top-down
    std::vector<uint32_t*> order(leafl + 1), rank(leafl + 1);
    std::vector<uint32_t> no(leafl + 1);
    order[0] = s.get<uint32_t>("scn_order_0", 1);
    rank[0] = s.get<uint32_t>("scn_rank_0", nu[0] + 1);
    HD_CUDA(cudaMemcpyAsync(order[0], &root_uid, 4, cudaMemcpyHostToDevice, st));
    no[0] = 1;
    for (uint32_t L = 0; L < leafl; L++) {
        uint32_t* key = s.get<uint32_t>("scn_key", uint64_t(nu[L + 1]) + 1);
        fill<uint32_t>(key, 0xFFFFFFFFu, nu[L + 1], st);
        k_unique_child_keys<<<grid_for(no[L], 256), 256, 0, st>>>(order[L], no[L], ucont[L], key);
        HD_LAUNCH_CHECK();
        const uint64_t nk = uint64_t(no[L]) * 8;
        uint32_t* by_key = s.get<uint32_t>("scn_by_key", nk);
        fill<uint32_t>(by_key, 0xFFFFFFFFu, nk, st);
        k_scatter_keys<<<grid_for(nu[L + 1], 256), 256, 0, st>>>(key, nu[L + 1], by_key);
        HD_LAUNCH_CHECK();
        uint32_t* flag = s.get<uint32_t>("scn_flag", nk);
        uint32_t* pos = s.get<uint32_t>("scn_pos", nk);
        k_flags<<<grid_for(nk, 256), 256, 0, st>>>(by_key, nk, flag);
        HD_LAUNCH_CHECK();
        exclusive_scan<uint32_t, uint32_t>(s, flag, pos, nk, d_n, st);
        no[L + 1] = read_scalar(d_n, st);
        char a[32], b[32];
        snprintf(a, 32, "scn_order_%u", L + 1);
        snprintf(b, 32, "scn_rank_%u", L + 1);
        order[L + 1] = s.get<uint32_t>(a, uint64_t(no[L + 1]) + 1);
        rank[L + 1] = s.get<uint32_t>(b, uint64_t(nu[L + 1]) + 1);
        k_compact_order<<<grid_for(nk, 256), 256, 0, st>>>(by_key, pos, nk, order[L + 1], rank[L + 1]);
        HD_LAUNCH_CHECK();
    }
    // 5. word layout and emission
    std::vector<uint32_t*> word_of(leafl + 1);
    std::vector<uint64_t> base(leafl + 2);
    base[0] = 0;
    for (uint32_t L = 0; L <= leafl; L++) {
        uint32_t* size = s.get<uint32_t>("scn_size", uint64_t(no[L]) + 1);
        uint32_t* off = s.get<uint32_t>("scn_off", uint64_t(no[L]) + 1);
        k_node_sizes<<<grid_for(no[L], 256), 256, 0, st>>>(order[L], no[L], ucont[L], L == leafl, size);
        HD_LAUNCH_CHECK();
        exclusive_scan<uint32_t, uint32_t>(s, size, off, no[L], d_n, st);
        const uint32_t tot = read_scalar(d_n, st);
        char a[32];
        snprintf(a, 32, "scn_word_of_%u", L);
        word_of[L] = s.get<uint32_t>(a, uint64_t(nu[L]) + 1);
        k_word_of<<<grid_for(no[L], 256), 256, 0, st>>>(order[L], no[L], off, base[L], word_of[L]);
        HD_LAUNCH_CHECK();
        base[L + 1] = base[L] + tot;
    }
    const uint64_t n_words = base[leafl + 1];
    if (n_words >= 0xFFFFFFFFull)
        throw StatusError{HD_ERR_INVALID, "scene BasicDAG exceeds 2^32 words"};
    if (c->d_basic)
        cudaFree(c->d_basic);
    c->d_basic = nullptr;
    if (cudaMalloc(&c->d_basic, n_words * 4) != cudaSuccess) {
        cudaGetLastError();
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        throw StatusError{HD_ERR_OOM, "BasicDAG allocation of " + std::to_string(n_words) + " words failed (" +
                                          std::to_string(fr >> 20) + " MiB free, scratch " +
                                          std::to_string(c->scratch.total() >> 20) + " MiB)"};
    }
    c->n_basic = n_words;
    uint64_t enclosed = 0;
    for (uint32_t L = 0; L <= leafl; L++) {
        k_emit<<<grid_for(no[L], 256), 256, 0, st>>>(L, T, L == leafl, order[L], no[L], ucont[L], ucount[L],
                                                     word_of[L], L < leafl ? word_of[L + 1] : nullptr, enclosed,
                                                     c->d_basic, c->t.error);
        HD_LAUNCH_CHECK();
        if (L < T)
            enclosed += no[L];
    }
    if (check_error(c))
        throw StatusError{HD_ERR_INVALID, "scene header overflow (count or enclosed index >= 2^24)"};
    *d_words_out = c->d_basic;
    *n_words_out = n_words;
    c->gen_scratch_peak = s.peak();
}

} // namespace hd
