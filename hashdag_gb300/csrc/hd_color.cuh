// Colours on the device: the reference's compressed variable-weight colour
// format and its colour tree, resident in HBM.
//
// Reference: CompressedColor and the colour conversions (color_utils.h:9-75,
// variable_weight_size_colors.h:86-155), CompressedColorLeaf decoding
// (:343-551, byte-swapped weights: CFG_COLOR_SWAP_BYTE_ORDER, typedefs.h:516,
// color_utils.h:115-145), the HashDAGColors tree (hash_dag_colors.h:24-55),
// DAGUtils::get_color (dag_utils.h:423-523).
//
// Layout: colour-tree nodes are 8 consecutive uint32 entries (0 = none; an
// entry with bit 31 set is a leaf index); leaves are descriptors into three
// append-only pools (blocks: colour bits << 32 | header; macro blocks: first
// block, weight bit offset; weight words).  A descriptor with base = 0 is a
// unique leaf; base > 0 makes it a view of a shared leaf whose colour i is the
// shared leaf's colour base + i (CompressedColorLeaf::set_as_shared, :235-259:
// the scenes loaded from a compressed-colours file share one main leaf).
#pragma once

#include "hd_common.cuh"

namespace hd {

constexpr uint32_t kColorsPerMacro = 16384; // CColorsPerMacroBlock (:8)
constexpr uint32_t kLeafFlag = 0x80000000u;  // Utils::set_flag (utils.h:37-51)

struct LeafDesc {
    uint64_t blocks;  // pool offsets
    uint64_t macros;
    uint64_t weights;
    uint64_t base;    // colour index offset into a shared leaf (0: unique)
    uint32_t nb;      // blocks
    uint32_t nm;      // macro words (2 per macro block)
    uint32_t nw;      // weight words
    uint32_t pad;
};

struct ColorTable {
    uint32_t* nodes;
    LeafDesc* leaves;
    uint64_t* blocks;
    uint64_t* macros;
    uint32_t* weights;
    // device counters: [0] nodes, [1] leaves, [2] blocks, [3] macro words,
    // [4] weight words
    unsigned long long* top;
    uint64_t cap_nodes, cap_leaves, cap_blocks, cap_macros, cap_weights;
};

// hd_color packed in 64 bits: colour bits | weight << 32 | bits << 40
HD_HD uint64_t pack_color(uint32_t bits, uint32_t weight, uint32_t bpw)
{
    return uint64_t(bits) | (uint64_t(weight) << 32) | (uint64_t(bpw) << 40);
}
HD_HD uint32_t pc_bits(uint64_t c) { return uint32_t(c); }
HD_HD uint32_t pc_weight(uint64_t c) { return uint32_t(c >> 32) & 0xFF; }
HD_HD uint32_t pc_bpw(uint64_t c) { return uint32_t(c >> 40) & 0xFF; }

struct F3 {
    float x, y, z;
};

HD_HD float clampf(float f, float a, float b) { return f < a ? a : f > b ? b : f; }

// ColorUtils (color_utils.h:9-75); the library builds with -fmad=false, so
// every expression rounds operation by operation as the reference's does.
HD_HD uint32_t f3_to_rgb101210(F3 c)
{
    const float r = clampf(c.x, 0.f, 1.f), g = clampf(c.y, 0.f, 1.f), b = clampf(c.z, 0.f, 1.f);
    return (uint32_t(r * 1023.0f) << 0) | (uint32_t(g * 4095.0f) << 10) | (uint32_t(b * 1023.0f) << 22);
}
HD_HD F3 rgb101210_to_f3(uint32_t v)
{
    return F3{float((v >> 0) & 0x3FF) / 1023.0f, float((v >> 10) & 0xFFF) / 4095.0f,
              float((v >> 22) & 0x3FF) / 1023.0f};
}
HD_HD uint32_t f3_to_rgb565(F3 c)
{
    const float r = clampf(c.x, 0.f, 1.f), g = clampf(c.y, 0.f, 1.f), b = clampf(c.z, 0.f, 1.f);
    return (uint32_t(r * 31.0f) << 0) | (uint32_t(g * 63.0f) << 5) | (uint32_t(b * 31.0f) << 11);
}
HD_HD F3 rgb565_to_f3(uint32_t v)
{
    return F3{float((v >> 0) & 0x1F) / 31.0f, float((v >> 5) & 0x3F) / 63.0f, float((v >> 11) & 0x1F) / 31.0f};
}
HD_HD uint32_t f3_to_rgb888(F3 c)
{
    const float r = clampf(c.x, 0.f, 1.f), g = clampf(c.y, 0.f, 1.f), b = clampf(c.z, 0.f, 1.f);
    return (uint32_t(r * 255.0f) << 0) | (uint32_t(g * 255.0f) << 8) | (uint32_t(b * 255.0f) << 16) | 0xff000000u;
}
// CompressedColor::get_color (:144-154), lerp = a * (1 - f) + b * f
HD_HD F3 color_value(uint64_t c)
{
    if (pc_bpw(c) == 0)
        return rgb101210_to_f3(pc_bits(c));
    const F3 lo = rgb565_to_f3(pc_bits(c) & 0xFFFF), hi = rgb565_to_f3((pc_bits(c) >> 16) & 0xFFFF);
    const float w = float(pc_weight(c)) / float((1 << pc_bpw(c)) - 1);
    return F3{lo.x * (1 - w) + hi.x * w, lo.y * (1 - w) + hi.y * w, lo.z * (1 - w) + hi.z * w};
}
HD_HD uint64_t single_color(F3 c) { return pack_color(f3_to_rgb101210(c), 0, 0); }

// Scene colours: RGB8 from a seeded value-noise field sampled on an aligned
// 8^3 grid (lattice period 16 cells, trilinear with integer weights), each
// voxel stored as set_single_color(rgb / 255).
HD_HD uint32_t color_rgb8(uint64_t seed, uint32_t x, uint32_t y, uint32_t z)
{
    const uint32_t cx = x >> 3, cy = y >> 3, cz = z >> 3;
    const uint32_t i = cx >> 4, j = cy >> 4, k = cz >> 4;
    const uint32_t fx = cx & 15, fy = cy & 15, fz = cz & 15;
    uint32_t out = 0;
    for (uint32_t c = 0; c < 3; c++) {
        uint32_t acc = 0;
        for (uint32_t a = 0; a < 2; a++)
            for (uint32_t b = 0; b < 2; b++)
                for (uint32_t d = 0; d < 2; d++) {
                    const uint32_t w = (a ? fx : 16 - fx) * (b ? fy : 16 - fy) * (d ? fz : 16 - fz);
                    const uint64_t key = (uint64_t(c) << 60) ^ (uint64_t(i + a) << 40) ^ (uint64_t(j + b) << 20) ^
                                         uint64_t(k + d);
                    acc += uint32_t(mix64(seed ^ mix64(key)) >> 56) * w;
                }
        out |= ((acc + 2048) >> 12) << (8 * c);
    }
    return out;
}
HD_HD uint64_t voxel_color(uint64_t seed, uint32_t x, uint32_t y, uint32_t z)
{
    const uint32_t rgb = color_rgb8(seed, x, y, z);
    return single_color(F3{float(rgb & 0xFF) / 255.0f, float((rgb >> 8) & 0xFF) / 255.0f,
                           float((rgb >> 16) & 0xFF) / 255.0f});
}

// ---- leaf decoding --------------------------------------------------------
HD_HD uint32_t hdr_index(uint32_t h) { return h & (kColorsPerMacro - 1); }
HD_HD uint32_t hdr_weight_offset(uint32_t h) { return h >> 16; }
HD_HD uint32_t hdr_bits(uint32_t h) { return hdr_weight_offset(h) == 0xFFFF ? 0 : ((h >> 14) & 3) + 1; }
// make_block_header (:31-52)
HD_HD uint32_t make_block_header(uint32_t weight_offset, uint32_t bits, uint32_t index)
{
    if (bits == 0)
        weight_offset = 0xFFFF;
    else
        bits--;
    return (weight_offset << 16) | (bits << 14) | index;
}

// extract_bits, byte-swapped layout: two bytes at bit_ptr / 8 read big-endian
HD_D uint32_t extract_bits(uint32_t bits, const uint32_t* words, uint64_t bit_ptr)
{
    if (bits == 0)
        return 0;
    const uint8_t* bytes = reinterpret_cast<const uint8_t*>(words);
    const uint64_t byte = bit_ptr / 8;
    uint32_t dst = (uint32_t(bytes[byte]) << 8) | uint32_t(bytes[byte + 1]);
    const uint32_t shift = 16 - bits - uint32_t(bit_ptr % 8);
    return (dst >> shift) & ((1u << bits) - 1);
}

// binary_search_blocks (:414-443) + get_color_for_block (:445-480); a shared
// leaf adds its offset first (:405-410)
HD_D uint64_t leaf_color(const ColorTable& ct, const LeafDesc& l, uint64_t ci)
{
    ci += l.base;
    const uint64_t* blocks = ct.blocks + l.blocks;
    const uint64_t* macros = ct.macros + l.macros;
    const uint32_t local = uint32_t(ci % kColorsPerMacro);
    const uint64_t m = ci / kColorsPerMacro;
    uint32_t lo = uint32_t(macros[2 * m]);
    uint32_t hi = 2 * (m + 1) < l.nm ? uint32_t(macros[2 * (m + 1)]) - 1 : l.nb - 1;
    uint32_t pos = (lo + hi) / 2;
    uint32_t h = uint32_t(blocks[pos]);
    while (hdr_index(h) != local && lo <= hi) {
        if (hdr_index(h) > local)
            hi = pos - 1;
        else
            lo = pos + 1;
        pos = (lo + hi) / 2;
        h = uint32_t(blocks[pos]);
    }
    const uint64_t block = blocks[pos];
    h = uint32_t(block);
    const uint32_t bpw = hdr_bits(h);
    uint32_t weight = 0;
    if (bpw) {
        const uint64_t wi = macros[2 * m + 1] + hdr_weight_offset(h) + uint64_t(local - hdr_index(h)) * bpw;
        weight = extract_bits(bpw, ct.weights + l.weights, wi);
    }
    return pack_color(uint32_t(block >> 32), weight, bpw);
}
// is_valid_index (:255-262): 2 * (index + offset) / CColorsPerMacroBlock <
// macro words
HD_D bool leaf_valid_index(const LeafDesc& l, uint64_t ci)
{
    return l.nb && 2 * (ci + l.base) / kColorsPerMacro < l.nm;
}

// DAGUtils::get_color (dag_utils.h:423-523); 0 = CompressedColor{}.
HD_D uint64_t get_color(const Table& t, const ColorTable& ct, uint32_t root, uint32_t x, uint32_t y, uint32_t z)
{
    const uint32_t D = t.g.depth, T = t.g.T, leafl = t.g.leaf_level;
    uint64_t nof = 0;
    uint32_t cn = 0;
    const LeafDesc* leaf = nullptr;
    uint32_t index = root;
    if (index == kInvalid)
        return 0;
    for (uint32_t level = 0; level < leafl;) {
        level++;
        const uint32_t* p = t.sys(index);
        const uint32_t mask = p[0] & 0xffu;
        const uint32_t sh = D - level;
        const uint32_t child = (((x >> sh) & 1) << 2) | (((y >> sh) & 1) << 1) | ((z >> sh) & 1);
        if (!(mask & (1u << child)))
            return 0;
        if (level - 1 < T) {
            cn = ct.nodes[cn + child];
            if (level == T)
                leaf = (cn & kLeafFlag) ? ct.leaves + (cn & ~kLeafFlag) : nullptr;
            else if (!cn)
                return 0;
        }
        if (level == leafl) {
            for (uint32_t cb = 0; cb < child; cb++)
                if (mask & (1u << cb)) {
                    const uint32_t* lp = t.sys(p[child_offset(mask, cb)]);
                    nof += popc32(lp[0]) + popc32(lp[1]);
                }
            const uint32_t* lp = t.sys(p[child_offset(mask, child)]);
            const uint64_t bits = uint64_t(lp[0]) | (uint64_t(lp[1]) << 32);
            const uint32_t bi = ((x & 1) ? 4 : 0) | ((y & 1) ? 2 : 0) | ((z & 1) ? 1 : 0) | ((x & 2) ? 32 : 0) |
                                ((y & 2) ? 16 : 0) | ((z & 2) ? 8 : 0);
            nof += popc64(bits & ((1ull << bi) - 1));
            break;
        }
        if (level > T)
            for (uint32_t cb = 0; cb < child; cb++)
                if (mask & (1u << cb))
                    nof += t.sys(p[child_offset(mask, cb)])[0] >> 8;
        index = p[child_offset(mask, child)];
    }
    if (!leaf)
        return 0;
    const LeafDesc l = *leaf;
    if (!leaf_valid_index(l, nof))
        return 0;
    return leaf_color(ct, l, nof);
}

} // namespace hd
