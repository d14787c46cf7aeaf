// The buffers of the noise-sphere and flood-fill editors, made on the device
// before the edit as the reference's constructors make them on the host.
//
// Both are BufferEditors (hash_dag_editors.h:129-221): a size^3 box of
// voxels from BoxEditorBase::min, each Unknown, loaded from the table
// (get_value at get_world_path, :159-195) or set by the tool.  What the edit
// needs of a voxel is whether BufferEditor::get_new_value reads it true (set
// true, or loaded true) and, for the fill, whether the tool set it and its
// colour; that is one flag byte (kBufNew | kBufSet) and one colour per voxel.
//
// SphereNoiseEditor (:712-760): FastNoise's Perlin FBM (FastNoise.cpp:
// 207-237, :760-886; the permutation from std::mt19937_64, made on the host)
// decides, per voxel, distance < radius * (1 + noise).
//
// FillEditorColors (:624-710): the reference floods depth-first from the
// box's centre through voxels that read false.  The set it reaches is the
// 6-connected component of empty voxels holding the centre (the centre
// itself is set whatever it holds), found here with a lock-free union-find.
// The voxels the flood loads true are the solid 6-neighbours of set voxels.
// Its colours walk the set voxels' bounding box in x, y, z order carrying
// the colour of the last loaded-true voxel: an inclusive max-scan of
// loaded-true indices over that box.
#include <algorithm>
#include <cmath>
#include <random>

#include "hd_color.cuh"
#include "hd_ctx.h"
#include "hd_edit.cuh"

namespace hd {

namespace {

// the 512-entry permutation tables of FastNoise::SetSeed
struct Perm {
    uint8_t perm[512];
    uint8_t perm12[512];
};

Perm fastnoise_perm(int seed)
{
    Perm p{};
    std::mt19937_64 gen(seed);
    for (int i = 0; i < 256; i++)
        p.perm[i] = uint8_t(i);
    for (int j = 0; j < 256; j++) {
        const int rng = int(gen() % uint64_t(256 - j));
        const int k = rng + j;
        const uint8_t l = p.perm[j];
        p.perm[j] = p.perm[j + 256] = p.perm[k];
        p.perm[k] = l;
        p.perm12[j] = p.perm12[j + 256] = uint8_t(p.perm[j] % 12);
    }
    return p;
}

// FastNoise::CalculateFractalBounding (:227-237), gain 0.5
float fractal_bounding(int octaves)
{
    float amp = 0.5f, amp_fractal = 1.0f;
    for (int i = 1; i < octaves; i++) {
        amp_fractal += amp;
        amp *= 0.5f;
    }
    return 1.0f / amp_fractal;
}

HD_D int fast_floor(float f) { return f >= 0 ? int(f) : int(f) - 1; }
HD_D float fn_lerp(float a, float b, float t) { return a + t * (b - a); }
HD_D float quintic(float t) { return t * t * t * (t * (t * 6 - 15) + 10); }

struct Noise {
    const uint8_t* perm;
    const uint8_t* perm12;
    float frequency, bounding;
    HD_D float grad(uint8_t offset, int x, int y, int z, float xd, float yd, float zd) const
    {
        // GRAD_X / GRAD_Y / GRAD_Z (:48-65): the 12 cube edges
        const uint32_t lut = perm12[(x & 0xff) + perm[(y & 0xff) + perm[(z & 0xff) + offset]]];
        const float gx = lut < 8 ? ((lut & 1) ? -1.f : 1.f) : 0.f;
        const float gy = lut < 4 ? ((lut & 2) ? -1.f : 1.f) : lut < 8 ? 0.f : ((lut & 1) ? -1.f : 1.f);
        const float gz = lut < 4 ? 0.f : ((lut & 2) ? -1.f : 1.f);
        return xd * gx + yd * gy + zd * gz;
    }
    HD_D float single(uint8_t offset, float x, float y, float z) const
    {
        const int x0 = fast_floor(x), y0 = fast_floor(y), z0 = fast_floor(z);
        const int x1 = x0 + 1, y1 = y0 + 1, z1 = z0 + 1;
        const float xs = quintic(x - float(x0)), ys = quintic(y - float(y0)), zs = quintic(z - float(z0));
        const float xd0 = x - float(x0), yd0 = y - float(y0), zd0 = z - float(z0);
        const float xd1 = xd0 - 1, yd1 = yd0 - 1, zd1 = zd0 - 1;
        const float xf00 = fn_lerp(grad(offset, x0, y0, z0, xd0, yd0, zd0), grad(offset, x1, y0, z0, xd1, yd0, zd0), xs);
        const float xf10 = fn_lerp(grad(offset, x0, y1, z0, xd0, yd1, zd0), grad(offset, x1, y1, z0, xd1, yd1, zd0), xs);
        const float xf01 = fn_lerp(grad(offset, x0, y0, z1, xd0, yd0, zd1), grad(offset, x1, y0, z1, xd1, yd0, zd1), xs);
        const float xf11 = fn_lerp(grad(offset, x0, y1, z1, xd0, yd1, zd1), grad(offset, x1, y1, z1, xd1, yd1, zd1), xs);
        return fn_lerp(fn_lerp(xf00, xf10, ys), fn_lerp(xf01, xf11, ys), zs);
    }
    // GetPerlinFractal with the FBM fractal, 3 octaves, lacunarity 2
    HD_D float fractal(float x, float y, float z) const
    {
        x *= frequency;
        y *= frequency;
        z *= frequency;
        float sum = single(perm[0], x, y, z), amp = 1;
        for (int i = 1; i < 3; i++) {
            x *= 2.0f;
            y *= 2.0f;
            z *= 2.0f;
            amp *= 0.5f;
            sum += single(perm[i], x, y, z) * amp;
        }
        return sum * bounding;
    }
};

// DAGUtils::get_value (dag_utils.h:138-172) on the root the edit starts from
HD_D bool dag_value(const Table& t, uint32_t root, uint32_t x, uint32_t y, uint32_t z)
{
    if (root == kInvalid)
        return false;
    const uint32_t D = t.g.depth;
    uint32_t index = root;
    for (uint32_t level = 0; level < t.g.leaf_level; level++) {
        const uint32_t* p = t.sys(index);
        const uint32_t sh = D - level - 1;
        const uint32_t c = (((x >> sh) & 1) << 2) | (((y >> sh) & 1) << 1) | ((z >> sh) & 1);
        const uint32_t mask = p[0] & 0xffu;
        if (!(mask & (1u << c)))
            return false;
        index = p[child_offset(mask, c)];
    }
    const uint32_t* lp = t.sys(index);
    const uint32_t bi = ((x & 1) ? 4 : 0) | ((y & 1) ? 2 : 0) | ((z & 1) ? 1 : 0) | ((x & 2) ? 32 : 0) |
                        ((y & 2) ? 16 : 0) | ((z & 2) ? 8 : 0);
    return ((bi < 32 ? lp[0] >> bi : lp[1] >> (bi - 32)) & 1) != 0;
}

struct Box {
    float minx, miny, minz;
    uint32_t size;
    HD_D void voxel(uint64_t i, uint32_t& x, uint32_t& y, uint32_t& z) const
    {
        x = uint32_t(i % size);
        y = uint32_t((i / size) % size);
        z = uint32_t(i / (uint64_t(size) * size));
    }
    // BufferEditor::get_world_path (:159-164)
    HD_D bool value(const Table& t, uint32_t root, uint32_t x, uint32_t y, uint32_t z) const
    {
        return dag_value(t, root, trunc_u32(minx + float(x)), trunc_u32(miny + float(y)), trunc_u32(minz + float(z)));
    }
    HD_D uint64_t index(uint32_t x, uint32_t y, uint32_t z) const
    {
        return uint64_t(x) + uint64_t(size) * y + uint64_t(size) * size * z;
    }
};

// SphereNoiseEditor: set to isAdding inside the noisy sphere, else the
// table's voxel at the world path
__global__ void k_noise(Table t, const uint32_t* __restrict__ d_root, Box box, const Perm* __restrict__ perm,
                        float frequency, float bounding, float radius, bool adding, uint8_t* __restrict__ flags)
{
    __shared__ uint8_t sp[1024];
    for (uint32_t k = threadIdx.x; k < 1024; k += blockDim.x)
        sp[k] = reinterpret_cast<const uint8_t*>(perm)[k];
    __syncthreads();
    const Noise noise{sp, sp + 512, frequency, bounding};
    const uint32_t root = *d_root;
    const uint64_t n = uint64_t(box.size) * box.size * box.size;
    const uint32_t ec = box.size / 2;
    HD_GRID_STRIDE(i, n)
    {
        uint32_t x, y, z;
        box.voxel(i, x, y, z);
        // length(editCenter - position): the uint3 difference wraps, its
        // uint32 dot product is the squared distance
        const uint32_t dx = ec - x, dy = ec - y, dz = ec - z;
        const double distance = sqrt(double(dx * dx + dy * dy + dz * dz));
        uint8_t f;
        if (distance < double(radius) * (1. + double(noise.fractal(float(x), float(y), float(z)))))
            f = adding ? uint8_t(kBufNew | kBufSet) : uint8_t(0);
        else
            f = box.value(t, root, x, y, z) ? kBufNew : 0;
        flags[i] = f;
    }
}

// ---- flood fill ---------------------------------------------------------------

constexpr uint32_t kBlocked = 0xFFFFFFFFu;
constexpr uint32_t kUnionSteps = 1u << 26;

// occupancy of the box; union-find parents: itself for passable voxels
// (empty, or the centre), kBlocked for the rest
__global__ void k_fill_init(Table t, const uint32_t* __restrict__ d_root, Box box, uint8_t* __restrict__ occ,
                            uint32_t* __restrict__ parent)
{
    const uint32_t root = *d_root;
    const uint64_t n = uint64_t(box.size) * box.size * box.size;
    const uint64_t centre = box.index(box.size / 2, box.size / 2, box.size / 2);
    HD_GRID_STRIDE(i, n)
    {
        uint32_t x, y, z;
        box.voxel(i, x, y, z);
        const bool solid = box.value(t, root, x, y, z);
        occ[i] = solid ? 1 : 0;
        parent[i] = (!solid || i == centre) ? uint32_t(i) : kBlocked;
    }
}

HD_D uint32_t uf_find(const uint32_t* parent, uint32_t x)
{
    // parents only ever point to smaller indices: the walk ends
    uint32_t p = __ldcg(parent + x);
    while (p != x) {
        x = p;
        p = __ldcg(parent + x);
    }
    return x;
}

// hook the larger root under the smaller; false if the step bound ran out
HD_D bool uf_union(uint32_t* parent, uint32_t a, uint32_t b)
{
    for (uint32_t step = 0; step < kUnionSteps; step++) {
        a = uf_find(parent, a);
        b = uf_find(parent, b);
        if (a == b)
            return true;
        if (a < b) {
            const uint32_t s = a;
            a = b;
            b = s;
        }
        const uint32_t old = atomicCAS(parent + a, a, b);
        if (old == a)
            return true;
        a = old;
    }
    return false;
}

__global__ void k_fill_union(Box box, uint32_t* __restrict__ parent, uint32_t* __restrict__ error)
{
    const uint64_t n = uint64_t(box.size) * box.size * box.size;
    HD_GRID_STRIDE(i, n)
    {
        if (__ldcg(parent + i) == kBlocked)
            continue;
        uint32_t x, y, z;
        box.voxel(i, x, y, z);
        const uint32_t nb[3] = {x + 1 < box.size ? uint32_t(box.index(x + 1, y, z)) : kBlocked,
                                y + 1 < box.size ? uint32_t(box.index(x, y + 1, z)) : kBlocked,
                                z + 1 < box.size ? uint32_t(box.index(x, y, z + 1)) : kBlocked};
        for (int k = 0; k < 3; k++)
            if (nb[k] != kBlocked && __ldcg(parent + nb[k]) != kBlocked && !uf_union(parent, uint32_t(i), nb[k]))
                atomicExch(error, 1u);
    }
}

// flags: kBufSet for the centre's component, kBufNew for set or solid;
// loaded-true voxels (solid 6-neighbours of set ones) in `loaded`; the set
// voxels' bounding box in bb[0..5] (min x, y, z, max x, y, z)
__global__ void k_fill_mark(Box box, const uint8_t* __restrict__ occ, const uint32_t* __restrict__ parent,
                            uint8_t* __restrict__ flags, uint8_t* __restrict__ loaded, uint32_t* __restrict__ bb)
{
    const uint64_t n = uint64_t(box.size) * box.size * box.size;
    const uint32_t c = box.size / 2;
    const uint32_t croot = uf_find(parent, uint32_t(box.index(c, c, c)));
    auto is_set = [&](uint64_t j) {
        const uint32_t p = __ldcg(parent + j);
        return p != kBlocked && uf_find(parent, uint32_t(j)) == croot;
    };
    HD_GRID_STRIDE(i, n)
    {
        const bool set = is_set(i);
        flags[i] = uint8_t((set ? kBufSet : 0) | ((set || occ[i]) ? kBufNew : 0));
        uint32_t x, y, z;
        box.voxel(i, x, y, z);
        bool ld = false;
        if (!set && occ[i]) {
            ld = (x > 0 && is_set(box.index(x - 1, y, z))) || (x + 1 < box.size && is_set(box.index(x + 1, y, z))) ||
                 (y > 0 && is_set(box.index(x, y - 1, z))) || (y + 1 < box.size && is_set(box.index(x, y + 1, z))) ||
                 (z > 0 && is_set(box.index(x, y, z - 1))) || (z + 1 < box.size && is_set(box.index(x, y, z + 1)));
        }
        loaded[i] = ld ? 1 : 0;
        if (set) {
            atomicMin(bb + 0, x);
            atomicMin(bb + 1, y);
            atomicMin(bb + 2, z);
            atomicMax(bb + 3, x);
            atomicMax(bb + 4, y);
            atomicMax(bb + 5, z);
        }
    }
}

// The colour carried into each set voxel: over the set voxels' box in x, y,
// z order (linear index L), key = L + 1 at loaded-true voxels; an inclusive
// max-scan gives the last loaded-true voxel at or before every L.
constexpr uint32_t kScanChunk = 1024;

struct SubBox {
    uint32_t x0, y0, z0, nx, ny, nz;
    HD_D void voxel(uint64_t l, uint32_t& x, uint32_t& y, uint32_t& z) const
    {
        z = z0 + uint32_t(l % nz);
        y = y0 + uint32_t((l / nz) % ny);
        x = x0 + uint32_t(l / (uint64_t(nz) * ny));
    }
};

HD_D uint32_t block_max_scan(uint32_t v, uint32_t* warp_tot)
{
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= uint32_t(o))
            v = max(v, u);
    }
    if (lane == 31)
        warp_tot[warp] = v;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < blockDim.x / 32 ? warp_tot[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= uint32_t(o))
                w = max(w, u);
        }
        warp_tot[lane] = w;
    }
    __syncthreads();
    const uint32_t before = warp > 0 ? warp_tot[warp - 1] : 0;
    const uint32_t r = max(v, before);
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kScanChunk) k_fill_scan_chunks(Box box, SubBox sb, const uint8_t* __restrict__ loaded,
                                                                 uint32_t* __restrict__ last,
                                                                 uint32_t* __restrict__ chunk_max)
{
    __shared__ uint32_t warp_tot[32];
    const uint64_t total = uint64_t(sb.nx) * sb.ny * sb.nz;
    const uint64_t l = uint64_t(blockIdx.x) * kScanChunk + threadIdx.x;
    uint32_t key = 0;
    if (l < total) {
        uint32_t x, y, z;
        sb.voxel(l, x, y, z);
        key = loaded[box.index(x, y, z)] ? uint32_t(l + 1) : 0u;
    }
    const uint32_t s = block_max_scan(key, warp_tot);
    if (l < total)
        last[l] = s;
    if (threadIdx.x == kScanChunk - 1)
        chunk_max[blockIdx.x] = s;
}

// one block: the exclusive running maximum of the chunk maxima (the carry
// into each chunk); thread k walks a contiguous run of chunks
__global__ void __launch_bounds__(kScanChunk) k_fill_scan_carry(uint32_t* __restrict__ chunk_max, uint32_t n_chunks)
{
    __shared__ uint32_t warp_tot[32];
    const uint32_t per = (n_chunks + kScanChunk - 1) / kScanChunk;
    const uint32_t b = threadIdx.x * per, e = min(b + per, n_chunks);
    uint32_t run = 0;
    for (uint32_t k = b; k < e; k++)
        run = max(run, chunk_max[k]);
    // inclusive scan of the runs' maxima, then the maximum before this run
    const uint32_t incl = block_max_scan(run, warp_tot);
    uint32_t carry = __shfl_up_sync(0xffffffffu, incl, 1);
    __shared__ uint32_t warp_last[32];
    if ((threadIdx.x & 31) == 31)
        warp_last[threadIdx.x >> 5] = incl;
    __syncthreads();
    if ((threadIdx.x & 31) == 0)
        carry = threadIdx.x ? warp_last[(threadIdx.x >> 5) - 1] : 0u;
    for (uint32_t k = b; k < e; k++) {
        const uint32_t v = chunk_max[k];
        chunk_max[k] = carry;
        carry = max(carry, v);
    }
}

// colours of the set voxels of the box
__global__ void k_fill_colors(Table t, ColorTable ct, const uint32_t* __restrict__ d_root, Box box, SubBox sb,
                              const uint8_t* __restrict__ flags, const uint32_t* __restrict__ last,
                              const uint32_t* __restrict__ carry, uint64_t* __restrict__ colors)
{
    const uint32_t root = *d_root;
    const uint64_t total = uint64_t(sb.nx) * sb.ny * sb.nz;
    HD_GRID_STRIDE(l, total)
    {
        uint32_t x, y, z;
        sb.voxel(l, x, y, z);
        const uint64_t i = box.index(x, y, z);
        if (!(flags[i] & kBufSet))
            continue;
        const uint32_t src = max(last[l], carry[l / kScanChunk]);
        uint64_t col = 0; // CompressedColor{} before any loaded-true voxel
        if (src) {
            uint32_t sx, sy, sz;
            sb.voxel(src - 1, sx, sy, sz);
            col = get_color(t, ct, root, trunc_u32(box.minx + float(sx)), trunc_u32(box.miny + float(sy)),
                            trunc_u32(box.minz + float(sz)));
        }
        colors[i] = col;
    }
}

} // namespace

// The noise or fill buffer of an edit (its flags in ed.values, the fill's
// colours in ed.colors) and, for the fill, the bounds of the voxels it set.
void tool_buffers(hd_ctx* c, Editor& ed)
{
    cudaStream_t st = c->stream;
    Scratch& s = c->scratch;
    const uint64_t n = uint64_t(ed.size) * ed.size * ed.size;
    if (n == 0 || n >= (1ull << 31))
        throw StatusError{HD_ERR_INVALID, "tool region too large (" + std::to_string(ed.size) + "^3 voxels)"};
    const Box box{ed.minx, ed.miny, ed.minz, ed.size};
    uint8_t* flags = s.get<uint8_t>("tool_flags", n + 1);
    const uint32_t grid = grid_for(n, 256);
    if (ed.tool == HD_TOOL_NOISE_ADD || ed.tool == HD_TOOL_NOISE_REMOVE) {
        // noise.SetSeed(abs(1923 + int32(center.x) + 23 * int32(center.y) +
        // 2938 * int32(center.z))), SetFrequency(1 / radius),
        // SetFractalOctaves(3)
        const int seed = std::abs(1923 + int32_t(ed.cx) + 23 * int32_t(ed.cy) + 2938 * int32_t(ed.cz));
        const Perm h = fastnoise_perm(seed);
        Perm* d = s.get<Perm>("tool_perm", 1);
        HD_CUDA(cudaMemcpyAsync(d, &h, sizeof(Perm), cudaMemcpyHostToDevice, st));
        k_noise<<<grid, 256, 0, st>>>(c->t, c->d_root, box, d, 1 / ed.r, fractal_bounding(3), ed.r,
                                      ed.tool == HD_TOOL_NOISE_ADD, flags);
        HD_LAUNCH_CHECK();
        ed.values = flags;
        return;
    }
    // flood fill
    uint8_t* occ = s.get<uint8_t>("tool_occ", n + 1);
    uint8_t* loaded = s.get<uint8_t>("tool_loaded", n + 1);
    uint32_t* parent = s.get<uint32_t>("tool_parent", n + 1);
    uint32_t* bb = s.get<uint32_t>("tool_bb", 8);
    const uint32_t init_bb[8] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0, 0, 0, 0, 0}; // [6]: union error
    HD_CUDA(cudaMemcpyAsync(bb, init_bb, sizeof(init_bb), cudaMemcpyHostToDevice, st));
    k_fill_init<<<grid, 256, 0, st>>>(c->t, c->d_root, box, occ, parent);
    HD_LAUNCH_CHECK();
    k_fill_union<<<grid, 256, 0, st>>>(box, parent, bb + 6);
    HD_LAUNCH_CHECK();
    k_fill_mark<<<grid, 256, 0, st>>>(box, occ, parent, flags, loaded, bb);
    HD_LAUNCH_CHECK();
    uint32_t h_bb[8];
    HD_CUDA(cudaMemcpyAsync(h_bb, bb, sizeof(h_bb), cudaMemcpyDeviceToHost, st));
    HD_CUDA(cudaStreamSynchronize(st));
    if (h_bb[6])
        throw StatusError{HD_ERR_TIMEOUT, "flood fill: a union-find step bound ran out"};
    // boundsMin / boundsMax = min + the set voxels' box (:664-667); the
    // centre is always set
    ed.bminx = ed.minx + float(h_bb[0]);
    ed.bminy = ed.miny + float(h_bb[1]);
    ed.bminz = ed.minz + float(h_bb[2]);
    ed.bmaxx = ed.minx + float(h_bb[3]);
    ed.bmaxy = ed.miny + float(h_bb[4]);
    ed.bmaxz = ed.minz + float(h_bb[5]);
    ed.values = flags;
    ed.colors = nullptr;
    if (!c->colors)
        return;
    const SubBox sb{h_bb[0], h_bb[1], h_bb[2], h_bb[3] - h_bb[0] + 1, h_bb[4] - h_bb[1] + 1, h_bb[5] - h_bb[2] + 1};
    const uint64_t total = uint64_t(sb.nx) * sb.ny * sb.nz;
    const uint32_t chunks = uint32_t((total + kScanChunk - 1) / kScanChunk);
    uint32_t* last = s.get<uint32_t>("tool_last", total + 1);
    uint32_t* chunk_max = s.get<uint32_t>("tool_chunks", uint64_t(chunks) + 1);
    uint64_t* colors = s.get<uint64_t>("tool_colors", n + 1);
    k_fill_scan_chunks<<<chunks, kScanChunk, 0, st>>>(box, sb, loaded, last, chunk_max);
    HD_LAUNCH_CHECK();
    k_fill_scan_carry<<<1, kScanChunk, 0, st>>>(chunk_max, chunks);
    HD_LAUNCH_CHECK();
    k_fill_colors<<<grid_for(total, 256), 256, 0, st>>>(c->t, c->ct, c->d_root, box, sb, flags, last, chunk_max,
                                                        colors);
    HD_LAUNCH_CHECK();
    ed.colors = colors;
}

} // namespace hd
