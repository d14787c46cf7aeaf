// Primary and shadow ray traversal over the device-resident hash DAG, and
// point queries.
//
// Reference: Tracer::trace_paths (tracer.cu:145-252) with
// compute_intersection_mask (:19-136) and next_child (:7-17);
// intersect_ray_node_out_of_order (:453-543) and trace_shadows (:589-697)
// with ray_box_intersection (:574-587); DAGUtils::get_value
// (dag_utils.h:138-172).  Camera rays as get_trace_params builds them
// (dag_tracer.cu:71-113).
//
// Arithmetic: this file is compiled with -fmad=false, so every float/double
// expression is rounded operation by operation in source order; FMA = 1
// places explicit fused multiply-adds where the reference's default nvcc
// build contracts a product into the following add.
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include <algorithm>

#include "hd_ctx.h"

namespace hd {

HD_D float fmax_r(float a, float b) { return a > b ? a : b; } // constexpr_max (cuda_math.h:13)
HD_D float fmin_r(float a, float b) { return a < b ? a : b; }

// The camera read where it is used, with loads the compiler may neither
// merge with other reads of it nor move: the camera is then dead during a
// walk instead of held (and spilled) across it.  Generic addressing (the
// camera may be a kernel parameter's copy or global memory), default
// caching.
HD_D double reload_f64(const double* p)
{
    double r;
    asm volatile("ld.f64 %0, [%1];" : "=d"(r) : "l"(p));
    return r;
}
HD_D hd_camera reload_camera(const hd_camera* c)
{
    hd_camera r;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        r.position[a] = reload_f64(c->position + a);
        r.ray_min[a] = reload_f64(c->ray_min + a);
        r.ray_ddx[a] = reload_f64(c->ray_ddx + a);
        r.ray_ddy[a] = reload_f64(c->ray_ddy + a);
    }
    return r;
}

// ray_min + px * ddx + py * ddy - position and its squared length, double
template <int FMA>
HD_D double camera_vec(const hd_camera& cam, double px, double py, double v[3])
{
#pragma unroll
    for (int a = 0; a < 3; a++) {
        double t;
        if (FMA) {
            t = __fma_rn(px, cam.ray_ddx[a], cam.ray_min[a]);
            t = __fma_rn(py, cam.ray_ddy[a], t);
        } else {
            t = cam.ray_min[a] + px * cam.ray_ddx[a];
            t = t + py * cam.ray_ddy[a];
        }
        v[a] = t - cam.position[a];
    }
    return FMA ? __fma_rn(v[2], v[2], __fma_rn(v[1], v[1], v[0] * v[0])) : (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
}

// normalize(ray_min + px * ddx + py * ddy - position), double
template <int FMA>
HD_D void camera_dir(const hd_camera& cam, double px, double py, double out[3])
{
    double v[3];
    const double dot = camera_vec<FMA>(cam, px, py, v);
    const double inv = 1.0 / sqrt(dot);
    out[0] = inv * v[0];
    out[1] = inv * v[1];
    out[2] = inv * v[2];
}

// Exact double of a 32-bit unsigned integer, built from its bits.
HD_D double u32_to_double(uint32_t u)
{
    if (u == 0)
        return 0.0;
    const uint32_t e = 31 - __clz(u);
    const uint64_t frac = (uint64_t(u) << (52 - e)) & ((1ull << 52) - 1);
    return __longlong_as_double((long long)((uint64_t(1023 + e) << 52) | frac));
}

// v rounded to the nearest float (ties to even excepted), from its bits.
// False when v lies within `margin` double ulps of a point halfway between
// two floats (margin 0: exactly on it) or outside [2^-125, 2^126].
HD_D bool round_to_float(double v, uint32_t margin, float& out)
{
    const uint64_t b = (uint64_t)__double_as_longlong(v);
    const uint32_t sign = uint32_t(b >> 32) & 0x80000000u;
    const uint64_t mag = b & 0x7FFFFFFFFFFFFFFFull;
    if (mag == 0) {
        out = __uint_as_float(sign);
        return true;
    }
    const int32_t e = int32_t(mag >> 52) - 1023 + 127;
    if (e < 2 || e > 253)
        return false;
    const uint32_t rem = uint32_t(mag) & ((1u << 29) - 1), mid = 1u << 28;
    if ((rem > mid ? rem - mid : mid - rem) <= margin)
        return false;
    out = __uint_as_float(sign | ((uint32_t(e) << 23) + (uint32_t(mag >> 29) & 0x7FFFFFu) + (rem > mid ? 1u : 0u)));
    return true;
}

// A positive normal float as a double, from its bits.
HD_D double float_to_double_bits(uint32_t fb)
{
    return __longlong_as_double(
        (long long)((uint64_t(((fb >> 23) & 0xFF) - 127 + 1023) << 52) | (uint64_t(fb & 0x7FFFFFu) << 29)));
}

// 1 / sqrt(dot) for dot in [2^-100, 2^100]: an rsqrtf seed (its argument
// dot rounded to float by its bits; the carry of the rounding bit reaches
// the exponent when it must) and one Newton-Raphson step in double,
// y1 = y0 + y0 (1 - dot y0^2) / 2: relative error below 2^-43.
HD_D double rsqrt_newton(double dot)
{
    const uint64_t db = (uint64_t)__double_as_longlong(dot);
    const uint32_t fb = ((uint32_t(db >> 52) - 1023 + 127) << 23) + ((uint32_t(db >> 29) & 0x7FFFFFu)) +
                        uint32_t((db >> 28) & 1);
    const double y0 = float_to_double_bits(__float_as_uint(rsqrtf(__uint_as_float(fb))));
    const double h = dot * y0;
    const double e = __fma_rn(-h, y0, 1.0);
    return __fma_rn(y0 * e, 0.5, y0);
}

// ---- float(normalize(v)) on the FP32 pipe ------------------------------------
// The reference normalises the camera ray in double: dot = |v|^2, 1 / sqrt(dot)
// and the products, each rounded (relative error below 2^-50.8 against the
// exact v / |v| of its own double v), then rounds each component to float.
// The GB300 runs double operations at 2 per SM cycle against 128 for float,
// and every primary ray pays for this normalisation, so it is done here in
// float-float arithmetic (pairs hi + lo of floats) from the same double v:
//  * v = hi + lo: hi keeps v's 24 leading significant bits, lo the other 29
//    rounded to float (2^-47 |v|);
//  * |v|^2 = S + Slo: the squares of the hi parts summed exactly (TwoSum),
//    their fused-multiply-add remainders and the 2 hi lo terms added in float
//    (2^-45 |v|^2);
//  * y = 1 / |v| = r0 + corr: an rsqrtf seed refined by one float
//    Newton-Raphson step (2^-22.9 even for a seed 64 ulps off), then one
//    Newton-Raphson step in float-float, r0 + r0 (1 - |v|^2 r0^2) / 2, whose
//    residual is formed with fused multiply-adds (1.5 e^2 plus roundings,
//    below 2^-44.5);
//  * each component y v = P + L, P = r0 hi and its exact remainder, plus the
//    small cross terms (2^-45.5).
// The sum P + L lies within 2^-44 (measured on 10^8 vectors: 2^-44.3) of the
// exact component, and so within 2^-43.9 of the reference's double; when
// P + L is more than 2^-40 |P + L| from every float rounding midpoint both
// round to the same float.  False (about one ray in ten thousand, and for
// components outside [2^-40, 2^40) or results below 2^-63) sends the ray to
// the exact double path.

// v = hi + lo within 2^-47 |v|; false for a nonzero |v| outside [2^-40, 2^40).
HD_D bool split_f64(double v, float& hi, float& lo)
{
    const uint64_t b = (uint64_t)__double_as_longlong(v);
    const uint32_t sign = uint32_t(b >> 32) & 0x80000000u;
    const uint64_t mag = b & 0x7FFFFFFFFFFFFFFFull;
    if (mag == 0) {
        hi = __uint_as_float(sign);
        lo = 0.0f;
        return true;
    }
    const int32_t e = int32_t(mag >> 52) - 1023;
    if (e < -40 || e >= 40)
        return false;
    hi = __uint_as_float(sign | (uint32_t(e + 127) << 23) | (uint32_t(mag >> 29) & 0x7FFFFFu));
    const float scale = __uint_as_float(sign | (uint32_t(e - 52 + 127) << 23)); // exact power of two
    lo = __fmul_rn(__uint2float_rn(uint32_t(mag) & ((1u << 29) - 1u)), scale);
    return true;
}

// s + t = a + b exactly (Knuth's TwoSum)
HD_D void two_sum(float a, float b, float& s, float& t)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    t = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// The float nearest to P + L (|L| well below |P|), when that sum lies more
// than 2^-40 |P + L| from the rounding midpoints either side of it (and the
// result's magnitude is in [2^-63, 2^64)).
HD_D bool round_pair(float P, float L, float& out)
{
    const float R = __fadd_rn(P, L);
    const float r = __fsub_rn(L, __fsub_rn(R, P)); // P + L - R exactly (Fast2Sum, |P| >= |L|)
    const uint32_t rb = __float_as_uint(R);
    const uint32_t ex = (rb >> 23) & 0xFFu;
    if (ex < 64 || ex > 190)
        return false;
    const float half_up = __uint_as_float((ex - 24) << 23);                            // ulp(R) / 2
    const float half_down = (rb & 0x7FFFFFu) ? half_up : __uint_as_float((ex - 25) << 23); // below a power of two
    const float margin = __uint_as_float((ex - 39) << 23);                              // >= 2^-40 |R|
    const float s = (rb >> 31) ? -r : r; // the remainder, positive away from zero
    if (!(__fsub_rn(half_up, s) > margin && __fadd_rn(half_down, s) > margin))
        return false;
    out = R;
    return true;
}

HD_D bool dir_from_vec(const double v[3], F3& d)
{
    float h[3], l[3];
    if (!(split_f64(v[0], h[0], l[0]) && split_f64(v[1], h[1], l[1]) && split_f64(v[2], h[2], l[2])))
        return false;
    const float p0 = __fmul_rn(h[0], h[0]), p1 = __fmul_rn(h[1], h[1]), p2 = __fmul_rn(h[2], h[2]);
    const float e = __fadd_rn(__fadd_rn(__fmaf_rn(h[0], h[0], -p0), __fmaf_rn(h[1], h[1], -p1)),
                              __fmaf_rn(h[2], h[2], -p2));
    const float c = __fadd_rn(__fadd_rn(__fmul_rn(__fadd_rn(h[0], h[0]), l[0]), __fmul_rn(__fadd_rn(h[1], h[1]), l[1])),
                              __fmul_rn(__fadd_rn(h[2], h[2]), l[2]));
    float s1, t1, S, t2;
    two_sum(p0, p1, s1, t1);
    two_sum(s1, p2, S, t2);
    const float Slo = __fadd_rn(__fadd_rn(__fadd_rn(t1, t2), e), c);
    if (!(S >= 0x1p-80f))
        return false;
    // the seed, refined once in float
    const float x0 = __fadd_rn(S, Slo);
    const float q0 = rsqrtf(x0);
    const float xq = __fmul_rn(x0, q0);
    const float r0 = __fmaf_rn(__fmul_rn(q0, __fmaf_rn(-xq, q0, 1.0f)), 0.5f, q0);
    // float-float step: hh = 1 - (S + Slo) r0^2, with S r0 = A + Al exactly
    const float A = __fmul_rn(S, r0);
    const float Al = __fmaf_rn(S, r0, -A);
    const float hh = __fsub_rn(__fmaf_rn(-A, r0, 1.0f), __fmaf_rn(Al, r0, __fmul_rn(__fmul_rn(Slo, r0), r0)));
    const float corr = __fmul_rn(__fmul_rn(r0, hh), 0.5f);
    float out[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        if (h[a] == 0.0f) { // a zero component keeps its sign, as inv * v does
            out[a] = h[a];
            continue;
        }
        const float P = __fmul_rn(r0, h[a]);
        const float Pl = __fmaf_rn(r0, h[a], -P);
        const float L =
            __fadd_rn(Pl, __fadd_rn(__fmul_rn(r0, l[a]), __fadd_rn(__fmul_rn(corr, h[a]), __fmul_rn(corr, l[a]))));
        if (!round_pair(P, L, out[a]))
            return false;
    }
    d = F3{out[0], out[1], out[2]};
    return true;
}

// float(normalize(...)) of camera_dir without double-precision arithmetic
// past the ray's vector (dir_from_vec).
template <int FMA>
HD_D bool camera_dir_float(const hd_camera& cam, uint32_t x, uint32_t y, F3& d)
{
    double v[3];
    camera_vec<FMA>(reload_camera(&cam), u32_to_double(x), u32_to_double(y), v);
    return dir_from_vec(v, d);
}

// ---- per-view camera tables -------------------------------------------------
// Of ray_min + px * ddx + py * ddy - position, the part that depends on the
// column alone, ray_min + px * ddx (rounded as camera_vec rounds it), is the
// same for every row, and with every operation rounded on its own (FMA = 0)
// py * ddy is the same for every column: tables of both per view leave a
// pixel two additions (or one fused multiply-add and a subtraction) per axis
// instead of four or five operations on the GB300's narrow FP64 pipe.  Per
// view: W column entries, then H row entries, 3 doubles each
// (camera_table_words).

template <int FMA>
__global__ void k_camera_tables(const hd_camera* __restrict__ cams, uint32_t n_views, uint32_t W, uint32_t H,
                                double* __restrict__ tables)
{
    const uint64_t per = uint64_t(W) + H;
    HD_GRID_STRIDE(i, per * n_views)
    {
        const uint32_t v = uint32_t(i / per), k = uint32_t(i % per);
        const hd_camera& cam = cams[v];
        double* out = tables + camera_table_words(W, H) * v + 3ull * k;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            if (k < W) {
                const double px = u32_to_double(k);
                out[a] = FMA ? __fma_rn(px, cam.ray_ddx[a], cam.ray_min[a]) : cam.ray_min[a] + px * cam.ray_ddx[a];
            } else {
                out[a] = u32_to_double(k - W) * cam.ray_ddy[a];
            }
        }
    }
}

// camera_vec of pixel (x, y) from its view's tables: the same doubles.
template <int FMA>
HD_D double camera_vec_tab(const hd_camera* cam, const double* __restrict__ tab, uint32_t W, uint32_t x, uint32_t y,
                           double v[3])
{
    const double* col = tab + 3ull * x;
    const double* row = tab + 3ull * (uint64_t(W) + y);
    const double py = u32_to_double(y);
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const double t = FMA ? __fma_rn(py, reload_f64(cam->ray_ddy + a), col[a]) : col[a] + row[a];
        v[a] = t - reload_f64(cam->position + a);
    }
    return FMA ? __fma_rn(v[2], v[2], __fma_rn(v[1], v[1], v[0] * v[0])) : (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
}

// The exact path of camera_dir_float, out of line: it runs for about one ray
// in ten thousand, and inlined its double-precision temporaries would
// raise the register pressure of every ray.
template <int FMA>
__device__ __noinline__ F3 camera_dir_exact(const hd_camera* cam, uint32_t x, uint32_t y)
{
    double dd[3];
    camera_dir<FMA>(*cam, double(x), double(y), dd);
    return {float(dd[0]), float(dd[1]), float(dd[2])};
}

// compute_intersection_mask: children of node `path` at `level` crossed by
// the ray, as an 8-bit mask.
template <int FMA>
HD_D uint32_t intersection_mask(uint32_t D, bool is_root, uint32_t level, uint32_t px, uint32_t py, uint32_t pz,
                                const F3& o, const F3& d, const F3& inv)
{
    const uint32_t shift = D - level;
    const float radius = float(1u << (shift - 1));
    const F3 crr = {(radius + float(px << shift)) - o.x, (radius + float(py << shift)) - o.y,
                    (radius + float(pz << shift)) - o.z};
    const F3 tmid = {crr.x * inv.x, crr.y * inv.y, crr.z * inv.z};
    const F3 slab = {radius * fabsf(inv.x), radius * fabsf(inv.y), radius * fabsf(inv.z)};
    F3 pmin, pmax;
    if (FMA) {
        pmin = {__fmaf_rn(crr.x, inv.x, -slab.x), __fmaf_rn(crr.y, inv.y, -slab.y), __fmaf_rn(crr.z, inv.z, -slab.z)};
        pmax = {__fmaf_rn(crr.x, inv.x, slab.x), __fmaf_rn(crr.y, inv.y, slab.y), __fmaf_rn(crr.z, inv.z, slab.z)};
    } else {
        pmin = {tmid.x - slab.x, tmid.y - slab.y, tmid.z - slab.z};
        pmax = {tmid.x + slab.x, tmid.y + slab.y, tmid.z + slab.z};
    }
    const float tmin = fmax_r(fmax_r(pmin.x, fmax_r(pmin.y, pmin.z)), 0.0f);
    const float tmax = fmin_r(pmax.x, fmin_r(pmax.y, pmax.z));
    if (is_root && tmin >= tmax)
        return 0;
    uint32_t result;
    {
        const float s = 0.5f * (tmin + tmax);
        const uint32_t first = ((s * d.x) >= crr.x ? 4u : 0u) + ((s * d.y) >= crr.y ? 2u : 0u) +
                               ((s * d.z) >= crr.z ? 1u : 0u);
        result = 1u << first;
    }
    const float eps = 1e-4f;
    if (tmin <= tmid.x && tmid.x <= tmax) {
        const float py_ = tmid.x * d.y, pz_ = tmid.x * d.z;
        uint32_t A = 0, B = 0;
        if (py_ >= crr.y - eps) A |= 0xCC;
        if (py_ <= crr.y + eps) A |= 0x33;
        if (pz_ >= crr.z - eps) B |= 0xAA;
        if (pz_ <= crr.z + eps) B |= 0x55;
        result |= A & B;
    }
    if (tmin <= tmid.y && tmid.y <= tmax) {
        const float px_ = tmid.y * d.x, pz_ = tmid.y * d.z;
        uint32_t C = 0, E = 0;
        if (px_ >= crr.x - eps) C |= 0xF0;
        if (px_ <= crr.x + eps) C |= 0x0F;
        if (pz_ >= crr.z - eps) E |= 0xAA;
        if (pz_ <= crr.z + eps) E |= 0x55;
        result |= C & E;
    }
    if (tmin <= tmid.z && tmid.z <= tmax) {
        const float px_ = tmid.z * d.x, py_ = tmid.z * d.y;
        uint32_t G = 0, H = 0;
        if (px_ >= crr.x - eps) G |= 0xF0;
        if (px_ <= crr.x + eps) G |= 0x0F;
        if (py_ >= crr.y - eps) H |= 0xCC;
        if (py_ <= crr.y + eps) H |= 0x33;
        result |= G & H;
    }
    return result & 0xffu;
}

HD_D uint32_t first_child_mask(uint32_t low, uint32_t high) // Leaf::get_first_child_mask (base_dag.h:16-52)
{
    const uint32_t a = __vcmpne4(low, 0u) & 0x08040201u;
    const uint32_t b = __vcmpne4(high, 0u) & 0x08040201u;
    return ((a * 0x01010101u) >> 24) | (((b * 0x01010101u) >> 24) << 4);
}

HD_D uint32_t next_child(uint32_t order, uint32_t mask) // next_child (tracer.cu:7-17)
{
    // first set bit of mask in the order child ^ order, child = 0..7: bit k
    // of the permuted mask is bit k ^ order of mask, an XOR by order built
    // from swaps of adjacent bits, bit pairs and nibbles
    uint32_t m = mask;
    if (order & 1)
        m = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
    if (order & 2)
        m = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
    if (order & 4)
        m = ((m & 0x0Fu) << 4) | ((m >> 4) & 0x0Fu);
    return (__ffs(m) - 1) ^ order;
}

// The walk's stack: per level the node (its physical pool offset) and its
// child mask | visit mask << 8.
struct LocalStack {
    struct {
        uint32_t index, masks;
    } e[HD_MAX_DEPTH];
    HD_D void set(uint32_t l, uint32_t index, uint32_t masks) { e[l] = {index, masks}; }
    HD_D uint32_t index(uint32_t l) const { return e[l].index; }
    HD_D uint32_t masks(uint32_t l) const { return e[l].masks; }
};
// The same stack in the kernel's dynamic shared memory: level l of thread k
// at [l * blockDim.x + k], node indices and 16-bit masks in two arrays (6
// bytes a level).  Addresses come from the thread index and the array
// itself, so a walk holds no pointer registers for its stack.
extern __shared__ uint32_t hd_walk_stack[];
struct SharedStack {
    uint32_t msk_words; // start of the mask array: blockDim.x * depth words
    HD_D void set(uint32_t l, uint32_t index, uint32_t masks) const
    {
        const uint32_t k = l * blockDim.x + threadIdx.x;
        hd_walk_stack[k] = index;
        reinterpret_cast<uint16_t*>(hd_walk_stack + msk_words)[k] = uint16_t(masks);
    }
    HD_D uint32_t index(uint32_t l) const { return hd_walk_stack[l * blockDim.x + threadIdx.x]; }
    HD_D uint32_t masks(uint32_t l) const
    {
        return reinterpret_cast<const uint16_t*>(hd_walk_stack + msk_words)[l * blockDim.x + threadIdx.x];
    }
};
// Shared bytes of a SharedStack for `threads` threads and depth D.
HD_HD uint32_t shared_stack_bytes(uint32_t threads, uint32_t D) { return threads * D * 6; }
HD_D SharedStack shared_stack(uint32_t D) { return SharedStack{blockDim.x * D}; }

// The stack walk shared by the primary ray (nearest hit, children in the
// ray's octant order) and the shadow ray (any hit).  The reference's shadow
// walk takes children highest first; whether a ray hits anything does not
// depend on the order (the walk visits every crossed child until a voxel is
// reached), so OCTANT shadow walks take the ray's front-to-back order as
// primary rays do and meet the nearest occluders first.
template <int FMA, bool ANY_HIT, bool OCTANT = !ANY_HIT, typename Stack = LocalStack>
HD_D bool walk(const Table& t, uint32_t root, const F3& o, const F3& d, const F3& inv, uint32_t order, uint32_t* hit,
               uint32_t& descents, uint32_t& leaves, Stack stack = Stack{})
{
    const uint32_t D = t.g.depth, leafl = t.g.leaf_level;
    uint32_t level = 0, px = 0, py = 0, pz = 0;
    // the current node by its physical pool offset: its child pointers are
    // read with one load, and only the pointer read from it is translated
    uint32_t index = t.phys(root);
    uint32_t child_mask = t.pool[index] & 0xffu;
    uint32_t visit = child_mask & intersection_mask<FMA>(D, true, 0, 0, 0, 0, o, d, inv);
    uint32_t leaf_lo = 0, leaf_hi = 0;
    for (;;) {
        uint32_t nl = level;
        while (nl > 0 && !visit) {
            nl--;
            index = stack.index(nl);
            const uint32_t m = stack.masks(nl);
            child_mask = m & 0xffu;
            visit = m >> 8;
        }
        if (nl == 0 && !visit) {
            hit[0] = hit[1] = hit[2] = 0;
            return false;
        }
        const uint32_t up = level - nl;
        px >>= up;
        py >>= up;
        pz >>= up;
        level = nl;
        const uint32_t nc = OCTANT ? next_child(order, visit) : 31u - __clz(visit);
        visit &= ~(1u << nc);
        px = (px << 1) | ((nc >> 2) & 1);
        py = (py << 1) | ((nc >> 1) & 1);
        pz = (pz << 1) | (nc & 1);
        stack.set(level, index, child_mask | (visit << 8));
        level++;
        if (level == D) {
            hit[0] = px;
            hit[1] = py;
            hit[2] = pz;
            return true;
        }
        if (level < leafl) {
            index = t.phys(t.pool[index + child_offset(child_mask, nc)]);
            child_mask = t.pool[index] & 0xffu;
            descents++;
        } else if (level == leafl) {
            const uint32_t addr = t.phys(t.pool[index + child_offset(child_mask, nc)]);
            const uint2 lf = *(reinterpret_cast<const uint2*>(t.pool + addr));
            leaf_lo = lf.x;
            leaf_hi = lf.y;
            child_mask = first_child_mask(leaf_lo, leaf_hi);
            leaves++;
        } else {
            child_mask = ((nc & 4) ? leaf_hi : leaf_lo) >> ((nc & 3) * 8) & 0xffu;
        }
        visit = child_mask & intersection_mask<FMA>(D, false, level, px, py, pz, o, d, inv);
    }
}

// The child order of a ray: children visited as child ^ octant, 0..7, run
// front to back along d (rayChildOrder, tracer.cu:161-164).
HD_D uint32_t octant(const F3& d) { return (d.x < 0.f ? 4u : 0u) + (d.y < 0.f ? 2u : 0u) + (d.z < 0.f ? 1u : 0u); }

// walk() as a resumable state machine, for kernels whose lanes take a new
// ray as soon as theirs ends: start() enters the root, each step() runs one
// iteration of walk()'s loop and returns 0 (going on), 1 (reached a voxel)
// or 2 (left the root).  Same visit order, same result as walk().
template <int FMA, bool OCTANT>
struct Walker {
    uint32_t level, px, py, pz, index, child_mask, visit, leaf_lo, leaf_hi;
    F3 o;

    HD_D void start(const Table& t, uint32_t root, const F3& origin, const F3& d, const F3& inv)
    {
        o = origin;
        level = px = py = pz = 0;
        leaf_lo = leaf_hi = 0;
        index = t.phys(root);
        child_mask = t.pool[index] & 0xffu;
        visit = child_mask & intersection_mask<FMA>(t.g.depth, true, 0, 0, 0, 0, o, d, inv);
    }

    template <typename Stack>
    HD_D uint32_t step(const Table& t, const F3& d, const F3& inv, uint32_t order, const Stack& stack,
                       uint32_t& descents, uint32_t& leaves)
    {
        const uint32_t D = t.g.depth, leafl = t.g.leaf_level;
        uint32_t nl = level;
        while (nl > 0 && !visit) {
            nl--;
            index = stack.index(nl);
            const uint32_t m = stack.masks(nl);
            child_mask = m & 0xffu;
            visit = m >> 8;
        }
        if (nl == 0 && !visit)
            return 2;
        const uint32_t up = level - nl;
        px >>= up;
        py >>= up;
        pz >>= up;
        level = nl;
        const uint32_t nc = OCTANT ? next_child(order, visit) : 31u - __clz(visit);
        visit &= ~(1u << nc);
        px = (px << 1) | ((nc >> 2) & 1);
        py = (py << 1) | ((nc >> 1) & 1);
        pz = (pz << 1) | (nc & 1);
        stack.set(level, index, child_mask | (visit << 8));
        level++;
        if (level == D)
            return 1;
        if (level < leafl) {
            index = t.phys(t.pool[index + child_offset(child_mask, nc)]);
            child_mask = t.pool[index] & 0xffu;
            descents++;
        } else if (level == leafl) {
            const uint32_t addr = t.phys(t.pool[index + child_offset(child_mask, nc)]);
            const uint2 lf = *(reinterpret_cast<const uint2*>(t.pool + addr));
            leaf_lo = lf.x;
            leaf_hi = lf.y;
            child_mask = first_child_mask(leaf_lo, leaf_hi);
            leaves++;
        } else {
            child_mask = ((nc & 4) ? leaf_hi : leaf_lo) >> ((nc & 3) * 8) & 0xffu;
        }
        visit = child_mask & intersection_mask<FMA>(D, false, level, px, py, pz, o, d, inv);
        return 0;
    }
};


// The reference takes float(1.0 / double(x)) (tracer.cu:160): the double
// quotient rounded again to float.  Rounding a quotient first to a p'-bit
// and then to a p-bit significand equals rounding it once to p bits when
// p' >= 2p + 2 (S. Figueroa, "When is double rounding innocuous?", SIGNUM
// Newsletter 30(3), 1995); double (53) and float (24) qualify.  So the
// correctly rounded float reciprocal (__frcp_rn) gives the same bits with no
// double-precision work, which the GB300's small FP64 pipe would otherwise
// spend on every ray.
HD_D F3 inverse_dir(const F3& d) { return {__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z)}; }

// 8x8 pixel tiles per 64-thread block; a warp covers 8x4 pixels.
// Traversal work counters (COUNT instances only): rays, interior descents,
// leaf fetches.
HD_D void add_counts(unsigned long long* counters, uint32_t rays, uint32_t descents, uint32_t leaves)
{
    atomicAdd(counters + 0, rays);
    atomicAdd(counters + 1, descents);
    atomicAdd(counters + 2, leaves);
}

// tab (TAB): the view's camera tables (k_camera_tables)
template <int FMA, bool COUNT, typename Stack = LocalStack, bool TAB = false>
HD_D uint4 primary_ray(const Table& t, uint32_t root, const hd_camera& cam, uint32_t W, uint32_t H, uint32_t x,
                       uint32_t y, uint4* __restrict__ out, unsigned long long* counters, Stack stack = Stack{},
                       const double* __restrict__ tab = nullptr)
{
    F3 d;
    bool fast;
    if (TAB) {
        double v[3];
        camera_vec_tab<FMA>(&cam, tab, W, x, y, v);
        fast = dir_from_vec(v, d);
    } else {
        fast = camera_dir_float<FMA>(cam, x, y, d);
    }
    if (!fast)
        d = camera_dir_exact<FMA>(&cam, x, y);
    const F3 inv = inverse_dir(d);
    F3 o;
    if (!(round_to_float(cam.position[0], 0, o.x) && round_to_float(cam.position[1], 0, o.y) &&
          round_to_float(cam.position[2], 0, o.z)))
        o = {float(cam.position[0]), float(cam.position[1]), float(cam.position[2])};
    const uint32_t order = octant(d);
    uint32_t hit[3], descents = 0, leaves = 0;
    walk<FMA, false, true, Stack>(t, root, o, d, inv, order, hit, descents, leaves, stack);
    const uint4 path = make_uint4(hit[0], hit[1], hit[2], 0);
    out[uint64_t(H - 1 - y) * W + x] = path;
    if (COUNT)
        add_counts(counters, 1, descents, leaves);
    return path;
}

template <int FMA, bool COUNT>
__global__ void __launch_bounds__(64) k_trace_primary(Table t, const uint32_t* __restrict__ d_root, hd_camera cam,
                                                      uint32_t W, uint32_t H, uint4* __restrict__ out,
                                                      unsigned long long* counters)
{
    const uint32_t x = blockIdx.x * 8 + (threadIdx.x & 7);
    const uint32_t y = blockIdx.y * 8 + (threadIdx.x >> 3);
    if (x >= W || y >= H)
        return;
    primary_ray<FMA, COUNT>(t, *d_root, cam, W, H, x, y, out, counters);
}

// A shadow ray of the compacted list: the output pixel (view * W * H +
// pixel) and its origin.
struct ShadowRay {
    uint32_t idx;
    float ox, oy, oz;
};

// sun_direction(): the light normalised in float (tracer.cu:546-549)
template <int FMA>
HD_D F3 light_dir(F3 light)
{
    const float dot = FMA ? __fmaf_rn(light.z, light.z, __fmaf_rn(light.y, light.y, light.x * light.x))
                          : (light.x * light.x + light.y * light.y) + light.z * light.z;
    const float il = 1.0f / sqrtf(dot);
    return F3{il * light.x, il * light.y, il * light.z};
}

// Origin of the shadow ray of output pixel (x, row r) whose primary ray hit
// voxel p (tracer.cu:589-697 reduced to the hit test): the exact hit point on
// the hit voxel's box (ray_box_intersection, :574-587, in double) plus
// bias * light.
// Out of line: its double-precision temporaries stay out of the register
// allocation of the walk that precedes it.
template <int FMA>
__device__ __noinline__ F3 shadow_origin(const hd_camera& cam, uint32_t H, uint32_t x, uint32_t r, uint4 p, F3 dir,
                                      float bias)
{
    double cd[3];
    camera_dir<FMA>(cam, double(x), double(H - 1 - r), cd);
    const double bmin[3] = {double(float(p.x)), double(float(p.y)), double(float(p.z))};
    double real_min[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        // min(t0, t1) with t0 = (bmin - pos) / cd, t1 = (bmin + 1 - pos) / cd:
        // the numerators are ordered (bmin + 1 is exact, rounding is
        // monotonic), so for cd > 0 the minimum is t0 and for cd < 0 it is t1
        // (equal quotients give the same value either way); only cd = 0 needs
        // both.
        const double n0 = bmin[a] - cam.position[a];
        const double n1 = (bmin[a] + 1.0) - cam.position[a];
        if (cd[a] > 0.0) {
            real_min[a] = n0 / cd[a];
        } else if (cd[a] < 0.0) {
            real_min[a] = n1 / cd[a];
        } else {
            const double t0 = n0 / cd[a], t1 = n1 / cd[a];
            real_min[a] = t0 < t1 ? t0 : t1;
        }
    }
    const double maxmin = fmax(fmax(real_min[0], real_min[1]), real_min[2]);
    F3 start, o;
    if (FMA) {
        start = {float(__fma_rn(cd[0], maxmin, cam.position[0])), float(__fma_rn(cd[1], maxmin, cam.position[1])),
                 float(__fma_rn(cd[2], maxmin, cam.position[2]))};
        o = {__fmaf_rn(bias, dir.x, start.x), __fmaf_rn(bias, dir.y, start.y), __fmaf_rn(bias, dir.z, start.z)};
    } else {
        start = {float(cam.position[0] + cd[0] * maxmin), float(cam.position[1] + cd[1] * maxmin),
                 float(cam.position[2] + cd[2] * maxmin)};
        o = {start.x + bias * dir.x, start.y + bias * dir.y, start.z + bias * dir.z};
    }
    return o;
}

// shadow_origin of pixel (x, y) without its double square root and
// divisions, for the many-view kernel (the GB300's FP64 pipe is narrow):
//  * the camera direction cd = y1 * v, y1 from rsqrt_newton: less than
//    2^-42.9 relative from the reference's double (y1 within 2^-43, the
//    product's rounding and the reference's own below 2^-50.8);
//  * each 1 / cd from a float reciprocal seed (2^-22.4 from a truncated
//    argument) and one Newton step in double, below 2^-44.5, so that each
//    candidate t = numerator / cd (the numerators are the reference's
//    doubles) lies within 2^-42.4 of the reference's quotient, and so does
//    their maximum, maxmin;
//  * x = cd * maxmin then lies within 2^-41.6 of the reference's product,
//    and hp = position + x within |x| 2^-41.6 + 1 ulp(hp) of the
//    reference's sum: at most (|x| / |hp|) 2^11.4 + 1 double ulps of hp.
// Each float(hp) is taken from hp's bits when hp lies more than
// 2^(12 + k) + 16 double ulps from a float rounding midpoint, with
// |x| / |hp| < 2^k from the exponents; there the reference's double rounds
// to the same float.  Otherwise (or for a zero or tiny direction component)
// false: the caller takes the exact path.
template <int FMA>
__device__ __noinline__ bool shadow_origin_fast(const hd_camera* cam, const double* __restrict__ tab, uint32_t W,
                                                uint32_t x, uint32_t y, uint4 p, F3 dir, float bias, F3* out)
{
    double v[3];
    const double dot = camera_vec_tab<FMA>(cam, tab, W, x, y, v);
    if (!(dot >= 0x1p-100 && dot <= 0x1p100))
        return false;
    const double y1 = rsqrt_newton(dot);
    const uint32_t pv[3] = {p.x, p.y, p.z};
    double cd[3], pos[3], maxmin = 0.0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        cd[a] = y1 * v[a];
        pos[a] = reload_f64(cam->position + a);
        const uint64_t cb = (uint64_t)__double_as_longlong(cd[a]);
        const int32_t ce = int32_t((cb >> 52) & 0x7FF) - 1023;
        if (ce < -60 || ce > 60)
            return false; // zero or tiny (the exact path handles cd = 0)
        // a float seed of |cd| from its bits (truncated), its reciprocal, one
        // Newton step, the sign put back (negation is exact)
        const uint32_t sb = (uint32_t(ce + 127) << 23) | (uint32_t(cb >> 29) & 0x7FFFFFu);
        const double r0 = float_to_double_bits(__float_as_uint(__frcp_rn(__uint_as_float(sb))));
        const double mag = fabs(cd[a]);
        const double ra = __fma_rn(r0, __fma_rn(-mag, r0, 1.0), r0);
        const double r1 = cd[a] < 0.0 ? -ra : ra;
        // the voxel's box: min(t0, t1) is t0 for cd > 0, t1 for cd < 0 (the
        // numerators are ordered)
        const double bmin = double(float(pv[a]));
        const double num = cd[a] > 0.0 ? bmin - pos[a] : (bmin + 1.0) - pos[a];
        const double t = num * r1;
        maxmin = a == 0 ? t : fmax(maxmin, t);
    }
    float start[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const double xa = cd[a] * maxmin;
        const double hp = FMA ? __fma_rn(cd[a], maxmin, pos[a]) : pos[a] + xa;
        const int32_t ex = int32_t((uint64_t(__double_as_longlong(xa)) >> 52) & 0x7FF);
        const int32_t eh = int32_t((uint64_t(__double_as_longlong(hp)) >> 52) & 0x7FF);
        if (eh == 0)
            return false;
        const int32_t k = ex - eh + 1; // |x| / |hp| < 2^k
        if (k > 14)
            return false;
        const uint32_t margin = k < -12 ? 17u : (1u << (12 + k)) + 16u;
        if (!round_to_float(hp, margin, start[a]))
            return false;
    }
    if (FMA)
        *out = {__fmaf_rn(bias, dir.x, start[0]), __fmaf_rn(bias, dir.y, start[1]), __fmaf_rn(bias, dir.z, start[2])};
    else
        *out = {start[0] + bias * dir.x, start[1] + bias * dir.y, start[2] + bias * dir.z};
    return true;
}

// Where view v's paths go when a launch splits its output (out_copied set):
// the views view_copied names (the last 8 - kCopiedFrom of every 8) to
// out_copied, packed in view order, the others to out.  The host-buffer
// entry point writes the first kind straight into host memory during the
// primary launch and copies the second during the shadow launch, so that
// both parts of the step move paths over the host link.
HD_D uint4* view_paths(uint4* out, uint4* out_copied, uint32_t v, uint64_t frame)
{
    if (out_copied && (v & 7) >= kCopiedFrom)
        return out_copied + (uint64_t(v >> 3) * (8 - kCopiedFrom) + (v & 7) - kCopiedFrom) * frame;
    return out + uint64_t(v) * frame;
}

// Several views in one launch, as persistent warps: each warp takes 8x4
// pixel tiles from a counter (view-major, then tile rows), so warps whose
// rays end early take more tiles and every resident warp stays busy to the
// end of the launch; the next tile is fetched before the current one is
// traced.  View v writes its paths at out + v * W * H (the single-view
// layout), or, with out_copied, the views view_paths sets aside there.  The
// shadow pass's set-up is fused in: a pixel whose primary ray
// hit appends its shadow ray (origin on the hit voxel, as shadow_origin) to
// the list, warp by warp; a miss gets mask 2 at once.
template <int FMA>
__global__ void __launch_bounds__(128, 16)
    k_trace_views(Table t, const uint32_t* __restrict__ d_root, const hd_camera* __restrict__ cams, uint32_t W,
                  uint32_t H, uint32_t n_views, uint4* __restrict__ out, F3 light, float bias,
                  uint8_t* __restrict__ mask, ShadowRay* __restrict__ list, uint32_t* __restrict__ head,
                  const double* __restrict__ tables, uint4* __restrict__ out_copied)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t tx = (W + 7) / 8, ty = (H + 3) / 4;
    const uint32_t per_view = tx * ty, n_tiles = per_view * n_views;
    const SharedStack stack = shared_stack(t.g.depth);
    const uint32_t root = *d_root;
    uint32_t* next_tile = head + 1;
    uint32_t tile = __shfl_sync(0xffffffffu, lane == 0 ? atomicAdd(next_tile, 1u) : 0u, 0);
    while (tile < n_tiles) {
        const uint32_t next = lane == 0 ? atomicAdd(next_tile, 1u) : 0u;
        const uint32_t v = tile / per_view, k = tile - v * per_view;
        const uint32_t x = (k % tx) * 8 + (lane & 7), y = (k / tx) * 4 + (lane >> 3);
        const uint64_t i = uint64_t(v) * W * H + uint64_t(H - 1 - y) * W + x;
        bool hit = false;
        uint4 p = make_uint4(0, 0, 0, 0);
        if (x < W && y < H) {
            p = primary_ray<FMA, false, SharedStack, true>(t, root, cams[v], W, H, x, y,
                                                           view_paths(out, out_copied, v, uint64_t(W) * H), nullptr,
                                                           stack, tables + camera_table_words(W, H) * v);
            hit = (p.x | p.y | p.z) != 0;
            if (!hit)
                mask[i] = 2;
        }
        const uint32_t b = __ballot_sync(0xffffffffu, hit);
        if (b) {
            const uint32_t base =
                __shfl_sync(0xffffffffu, lane == 0 ? atomicAdd(head, uint32_t(__popc(b))) : 0u, 0);
            if (hit) {
                const F3 ld = light_dir<FMA>(light);
                F3 o;
                if (!shadow_origin_fast<FMA>(cams + v, tables + camera_table_words(W, H) * v, W, x, y, p, ld, bias,
                                             &o))
                    o = shadow_origin<FMA>(cams[v], H, x, H - 1 - y, p, ld, bias);
                list[base + __popc(b & ((1u << lane) - 1u))] = ShadowRay{uint32_t(i), o.x, o.y, o.z};
            }
        }
        tile = __shfl_sync(0xffffffffu, next, 0);
    }
}

// Shadow rays start only at hit pixels (a path of (0, 0, 0) is a miss,
// tracer.cu:644-648).  The hit pixels of each 8x8 tile are appended to the
// list, tile by tile, with their ray origins, so that
// the traversal kernel runs full warps of rays from neighbouring pixels and
// carries none of the double-precision set-up; misses get mask 2 here.  Rows
// are output rows (the layout of the paths image).
template <int FMA>
__global__ void __launch_bounds__(64) k_shadow_list(hd_camera cam, uint32_t W, uint32_t H,
                                                    const uint4* __restrict__ paths, F3 light, float bias,
                                                    uint8_t* __restrict__ mask, ShadowRay* __restrict__ list,
                                                    uint32_t* __restrict__ count)
{
    __shared__ uint32_t warp_base[2];
    const uint32_t x = blockIdx.x * 8 + (threadIdx.x & 7);
    const uint32_t r = blockIdx.y * 8 + (threadIdx.x >> 3);
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool in = x < W && r < H;
    const uint64_t i = uint64_t(r) * W + x;
    bool hit = false;
    uint4 p = make_uint4(0, 0, 0, 0);
    if (in) {
        p = paths[i];
        hit = (p.x | p.y | p.z) != 0;
        if (!hit)
            mask[i] = 2;
    }
    const uint32_t b = __ballot_sync(0xffffffffu, hit);
    if (lane == 0)
        warp_base[warp] = __popc(b);
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t n0 = warp_base[0], n1 = warp_base[1];
        const uint32_t base = (n0 + n1) ? atomicAdd(count, n0 + n1) : 0u;
        warp_base[0] = base;
        warp_base[1] = base + n0;
    }
    __syncthreads();
    if (hit) {
        const F3 o = shadow_origin<FMA>(cam, H, x, r, p, light_dir<FMA>(light), bias);
        list[warp_base[warp] + __popc(b & ((1u << lane) - 1u))] = ShadowRay{uint32_t(i), o.x, o.y, o.z};
    }
}

// The any-hit walk of every ray of the list toward the light
// (intersect_ray_node_out_of_order, tracer.cu:453-543) as persistent warps
// whose lanes refill independently: a lane whose ray has ended takes the next
// ray of the list as soon as kShadowRefill lanes of its warp are idle, so the
// warp does not wait for its longest walk (the walks differ by orders of
// magnitude).  Each ray's result depends on that ray only.
constexpr uint32_t kShadowRefill = 8;  // idle lanes that trigger a fetch
constexpr uint32_t kShadowSteps = 16; // walk steps between fetches
template <int FMA, bool COUNT>
__global__ void __launch_bounds__(128) k_trace_shadow(Table t, const uint32_t* __restrict__ d_root, F3 light,
                                                      uint8_t* __restrict__ mask, const ShadowRay* __restrict__ list,
                                                      uint32_t* __restrict__ head, unsigned long long* counters)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t n = head[0];
    const uint32_t root = *d_root;
    const F3 dir = light_dir<FMA>(light);
    const F3 inv = inverse_dir(dir);
    const uint32_t order = octant(dir);
    const SharedStack stack = shared_stack(t.g.depth);
    Walker<FMA, true> w;
    uint32_t idx = 0, descents = 0, leaves = 0;
    bool active = false, more = true;
    for (;;) {
        const uint32_t idle = __ballot_sync(0xffffffffu, !active);
        if (more && __popc(idle) >= kShadowRefill) {
            const uint32_t k = __popc(idle);
            const uint32_t base = __shfl_sync(0xffffffffu, lane == 0 ? atomicAdd(head + 2, k) : 0u, 0);
            more = base + k < n;
            if (!active) {
                const uint32_t j = base + __popc(idle & ((1u << lane) - 1u));
                if (j < n) {
                    const ShadowRay ray = list[j];
                    idx = ray.idx;
                    w.start(t, root, F3{ray.ox, ray.oy, ray.oz}, dir, inv);
                    active = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) {
            if (more)
                continue; // every lane idle: the next pass fetches
            break;
        }
        for (uint32_t s = 0; s < kShadowSteps && active; s++) {
            const uint32_t r = w.step(t, dir, inv, order, stack, descents, leaves);
            if (r) {
                mask[idx] = r == 1 ? 1 : 0;
                active = false;
                if (COUNT) {
                    add_counts(counters, 1, descents, leaves);
                    descents = leaves = 0;
                }
            }
        }
    }
}

// Blocks of a persistent launch of `kernel` with `threads` threads: as many
// as stay resident on every SM with smem_bytes of dynamic shared memory
// (queried once per kernel and size).
static uint32_t resident_blocks(const void* kernel, int threads, uint32_t smem_bytes)
{
    static std::mutex mu;
    static std::map<std::tuple<const void*, int, uint32_t>, uint32_t> known;
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_tuple(kernel, threads, smem_bytes);
    auto it = known.find(key);
    if (it != known.end())
        return it->second;
    int dev = 0, sms = 0, per_sm = 0;
    HD_CUDA(cudaGetDevice(&dev));
    HD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    HD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem_bytes));
    const uint32_t n = uint32_t(std::max(1, sms * std::max(1, per_sm)));
    known[key] = n;
    return n;
}

void trace_primary(hd_ctx* c, const hd_camera& cam, uint32_t w, uint32_t h, uint32_t* d_paths,
                   unsigned long long* d_counters, cudaStream_t stream, const uint32_t* d_root)
{
    cudaStream_t st = stream ? stream : c->stream;
    const uint32_t* rt = d_root ? d_root : c->d_root;
    if ((h + 7) / 8 > kMaxGridRows)
        throw StatusError{HD_ERR_INVALID, "image height " + std::to_string(h) + " exceeds " +
                                              std::to_string(8 * kMaxGridRows) + " rows"};
    dim3 grid((w + 7) / 8, (h + 7) / 8);
    uint4* out = reinterpret_cast<uint4*>(d_paths);
    if (d_counters) {
        if (c->fp_mode)
            k_trace_primary<1, true><<<grid, 64, 0, st>>>(c->t, rt, cam, w, h, out, d_counters);
        else
            k_trace_primary<0, true><<<grid, 64, 0, st>>>(c->t, rt, cam, w, h, out, d_counters);
    } else {
        if (c->fp_mode)
            k_trace_primary<1, false><<<grid, 64, 0, st>>>(c->t, rt, cam, w, h, out, nullptr);
        else
            k_trace_primary<0, false><<<grid, 64, 0, st>>>(c->t, rt, cam, w, h, out, nullptr);
    }
    HD_LAUNCH_CHECK();
}

// The any-hit walks of a shadow-ray list (head: ray count, two work
// counters) over px pixels.
static void shadow_walks(hd_ctx* c, uint64_t px, const float light[3], uint8_t* d_mask,
                         unsigned long long* d_counters, cudaStream_t st, const uint32_t* rt, const ShadowRay* list,
                         uint32_t* head)
{
    const F3 l = {light[0], light[1], light[2]};
    auto launch = [&](auto kernel, unsigned long long* counters) {
        const uint32_t smem = shared_stack_bytes(128, c->t.g.depth);
        const uint32_t blocks = uint32_t(
            std::min<uint64_t>((px + 127) / 128, resident_blocks(reinterpret_cast<const void*>(kernel), 128, smem)));
        kernel<<<blocks, 128, smem, st>>>(c->t, rt, l, d_mask, list, head, counters);
    };
    if (d_counters) {
        if (c->fp_mode)
            launch(k_trace_shadow<1, true>, d_counters);
        else
            launch(k_trace_shadow<0, true>, d_counters);
    } else {
        if (c->fp_mode)
            launch(k_trace_shadow<1, false>, nullptr);
        else
            launch(k_trace_shadow<0, false>, nullptr);
    }
    HD_LAUNCH_CHECK();
}

// Shadow pass of one frame from its paths: the hit list with origins, then
// the any-hit walks.
static void shadow_pass(hd_ctx* c, const hd_camera& cam, uint32_t w, uint32_t h, const uint32_t* d_paths,
                        const float light[3], float bias, uint8_t* d_mask, unsigned long long* d_counters,
                        cudaStream_t st, const uint32_t* rt, uint32_t* d_list)
{
    const uint64_t px = uint64_t(w) * h;
    if ((h + 7) / 8 > kMaxGridRows)
        throw StatusError{HD_ERR_INVALID, "image height " + std::to_string(h) + " exceeds " +
                                              std::to_string(8 * kMaxGridRows) + " rows"};
    uint32_t* buf = d_list ? d_list : c->scratch.get<uint32_t>("shadow_list", shadow_list_words(px));
    ShadowRay* list = reinterpret_cast<ShadowRay*>(buf);
    uint32_t* head = buf + 4 * px;
    HD_CUDA(cudaMemsetAsync(head, 0, 16, st));
    dim3 tiles((w + 7) / 8, (h + 7) / 8);
    const uint4* p = reinterpret_cast<const uint4*>(d_paths);
    const F3 l = {light[0], light[1], light[2]};
    if (c->fp_mode)
        k_shadow_list<1><<<tiles, 64, 0, st>>>(cam, w, h, p, l, bias, d_mask, list, head);
    else
        k_shadow_list<0><<<tiles, 64, 0, st>>>(cam, w, h, p, l, bias, d_mask, list, head);
    HD_LAUNCH_CHECK();
    shadow_walks(c, px, light, d_mask, d_counters, st, rt, list, head);
}

void trace_shadow(hd_ctx* c, const hd_camera& cam, uint32_t w, uint32_t h, const uint32_t* d_paths,
                  const float light[3], float bias, uint8_t* d_mask, unsigned long long* d_counters,
                  cudaStream_t stream, const uint32_t* d_root, uint32_t* d_list)
{
    shadow_pass(c, cam, w, h, d_paths, light, bias, d_mask, d_counters, stream ? stream : c->stream,
                d_root ? d_root : c->d_root, d_list);
}

// n_views frames in three launches: the views' camera tables, primary rays
// of every view with the shadow-ray list, then the shadow rays of every hit
// pixel of every view.
void trace_views(hd_ctx* c, const hd_camera* d_cams, uint32_t n_views, uint32_t w, uint32_t h, uint32_t* d_paths,
                 const float light[3], float bias, uint8_t* d_mask, cudaStream_t stream, uint32_t* d_list,
                 cudaEvent_t mid, const uint32_t* d_root, double* d_tables, uint32_t* d_paths_copied)
{
    cudaStream_t st = stream ? stream : c->stream;
    const uint32_t* rt = d_root ? d_root : c->d_root;
    const uint64_t px = uint64_t(w) * h * n_views;
    if (px >= 0xFFFFFFFFull)
        throw StatusError{HD_ERR_INVALID, "views x width x height must stay below 2^32 pixels"};
    uint32_t* buf = d_list ? d_list : c->scratch.get<uint32_t>("shadow_list", shadow_list_words(px));
    ShadowRay* list = reinterpret_cast<ShadowRay*>(buf);
    uint32_t* head = buf + 4 * px;
    HD_CUDA(cudaMemsetAsync(head, 0, 16, st));
    uint4* out = reinterpret_cast<uint4*>(d_paths);
    const uint64_t tiles = uint64_t((w + 7) / 8) * ((h + 3) / 4);
    const F3 l = {light[0], light[1], light[2]};
    const uint64_t tab_words = camera_table_words(w, h) * n_views;
    double* tables = d_tables ? d_tables : c->scratch.get<double>("cam_tables", tab_words);
    const uint32_t tab_blocks = grid_for(uint64_t(w + h) * n_views, 256);
    auto launch = [&](auto tab_kernel, auto kernel) {
        tab_kernel<<<tab_blocks, 256, 0, st>>>(d_cams, n_views, w, h, tables);
        HD_LAUNCH_CHECK();
        const uint32_t smem = shared_stack_bytes(128, c->t.g.depth);
        const uint32_t blocks = uint32_t(std::min<uint64_t>(
            (tiles * n_views + 3) / 4, resident_blocks(reinterpret_cast<const void*>(kernel), 128, smem)));
        kernel<<<blocks, 128, smem, st>>>(c->t, rt, d_cams, w, h, n_views, out, l, bias, d_mask, list, head, tables,
                                          reinterpret_cast<uint4*>(d_paths_copied));
    };
    if (c->fp_mode)
        launch(k_camera_tables<1>, k_trace_views<1>);
    else
        launch(k_camera_tables<0>, k_trace_views<0>);
    HD_LAUNCH_CHECK();
    if (mid)
        HD_CUDA(cudaEventRecord(mid, st));
    shadow_walks(c, px, light, d_mask, nullptr, st, rt, list, head);
}

// DAGUtils::get_value
__global__ void k_get_values(Table t, const uint32_t* __restrict__ d_root, const uint32_t* __restrict__ xyz,
                             uint64_t n, uint8_t* __restrict__ out)
{
    const uint32_t root = *d_root;
    HD_GRID_STRIDE(i, n)
    {
        const uint32_t x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
        uint32_t index = root;
        uint8_t v = 0;
        for (uint32_t level = 0; level < t.g.depth; level++) {
            if (level < t.g.leaf_level) {
                // one translation per node: its child pointers follow the
                // header in the same page
                const uint32_t* p = t.sys(index);
                const uint32_t mask = __ldg(p) & 0xffu;
                const uint32_t s = t.g.depth - (level + 1);
                const uint32_t child = (((x >> s) & 1) << 2) | (((y >> s) & 1) << 1) | ((z >> s) & 1);
                if (!(mask & (1u << child)))
                    break;
                index = __ldg(p + child_offset(mask, child));
            } else {
                const uint32_t* p = t.sys(index);
                const uint64_t leaf = uint64_t(__ldg(p)) | (uint64_t(__ldg(p + 1)) << 32);
                v = uint8_t((leaf >> leaf_bit(x, y, z)) & 1);
                break;
            }
        }
        out[i] = v;
    }
}

void get_values(hd_ctx* c, const uint32_t* d_xyz, uint64_t n, uint8_t* d_out)
{
    if (!n)
        return;
    k_get_values<<<grid_for(n, 256), 256, 0, c->stream>>>(c->t, c->d_root, d_xyz, n, d_out);
    HD_LAUNCH_CHECK();
}

} // namespace hd

// ---------------------------------------------------------------------------
// Traversal counters without any device allocation.
//
// Some callers cannot call cudaMalloc at the time they trace: an embedding
// application (a game engine, a plugin host) that reserves the device
// memory budget at start-up and forbids allocations afterwards, or a
// real-time loop in which cudaMalloc / cudaFree, which may synchronise the
// whole device, would stall the other streams' work.  This variant of
// hd_trace_counters keeps its scratch (one partial sum per 8x8-pixel block
// and the six totals) in a file-scope device array instead of the context's
// scratch buffers.  The array holds kNoAllocMaxBlocks blocks, i.e. images of
// up to 16,777,216 pixels (4096 x 4096); larger images, and images taller
// than 65535 rows of blocks (524,280 pixels), are rejected.  The
// array lives on every GPU that loads the library until the process exits.
// All calls share it: each call writes every slot it later reads, so
// nothing needs clearing, but calls that overlap on the GPU (other streams,
// other threads) race on it.
// ---------------------------------------------------------------------------
namespace hd {

constexpr uint32_t kNoAllocMaxBlocks = 262144;
__device__ __align__(256) unsigned long long g_noalloc_scratch[3 * kNoAllocMaxBlocks + 8];

HD_D void block_sum3(uint32_t a, uint32_t b, uint32_t c, unsigned long long* dst)
{
    __shared__ unsigned long long part[2][3];
    unsigned long long v[3] = {a, b, c};
    for (int k = 0; k < 3; k++)
        for (int o = 16; o; o >>= 1)
            v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 3; k++)
            part[threadIdx.x >> 5][k] = v[k];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < 3; k++)
            dst[k] = part[0][k] + part[1][k];
}

template <int FMA>
__global__ void __launch_bounds__(64) k_trace_primary_partials(Table t, const uint32_t* __restrict__ d_root,
                                                               hd_camera cam, uint32_t W, uint32_t H,
                                                               uint4* __restrict__ out,
                                                               unsigned long long* __restrict__ partial)
{
    const uint32_t x = blockIdx.x * 8 + (threadIdx.x & 7);
    const uint32_t y = blockIdx.y * 8 + (threadIdx.x >> 3);
    uint32_t rays = 0, descents = 0, leaves = 0;
    if (x < W && y < H) {
        double dd[3];
        camera_dir<FMA>(cam, double(x), double(y), dd);
        const F3 d = {float(dd[0]), float(dd[1]), float(dd[2])};
        const F3 o = {float(cam.position[0]), float(cam.position[1]), float(cam.position[2])};
        const uint32_t order = octant(d);
        uint32_t hit[3];
        walk<FMA, false>(t, *d_root, o, d, inverse_dir(d), order, hit, descents, leaves);
        out[uint64_t(H - 1 - y) * W + x] = make_uint4(hit[0], hit[1], hit[2], 0);
        rays = 1;
    }
    block_sum3(rays, descents, leaves, partial + 3 * (uint64_t(blockIdx.y) * gridDim.x + blockIdx.x));
}

template <int FMA>
__global__ void __launch_bounds__(64) k_trace_shadow_partials(Table t, const uint32_t* __restrict__ d_root,
                                                              hd_camera cam, uint32_t W, uint32_t H,
                                                              const uint4* __restrict__ paths, F3 light, float bias,
                                                              uint8_t* __restrict__ mask,
                                                              unsigned long long* __restrict__ partial)
{
    const uint32_t x = blockIdx.x * 8 + (threadIdx.x & 7);
    const uint32_t r = blockIdx.y * 8 + (threadIdx.x >> 3);
    uint32_t rays = 0, descents = 0, leaves = 0;
    if (x < W && r < H) {
        const uint64_t i = uint64_t(r) * W + x;
        const uint4 p = paths[i];
        if (p.x == 0 && p.y == 0 && p.z == 0) {
            mask[i] = 2;
        } else {
            // the same origin and front-to-back order as the shadow pass
            const F3 dir = light_dir<FMA>(light);
            const F3 o = shadow_origin<FMA>(cam, H, x, r, p, dir, bias);
            const uint32_t order = octant(dir);
            uint32_t hit[3];
            mask[i] = walk<FMA, true, true>(t, *d_root, o, dir, inverse_dir(dir), order, hit, descents, leaves) ? 1
                                                                                                                : 0;
            rays = 1;
        }
    }
    block_sum3(rays, descents, leaves, partial + 3 * (uint64_t(blockIdx.y) * gridDim.x + blockIdx.x));
}

// One block: column sums of the partials into totals[0..2].
__global__ void k_sum_partials(const unsigned long long* __restrict__ partial, uint32_t nblocks,
                               unsigned long long* __restrict__ totals)
{
    __shared__ unsigned long long acc[3][256];
    for (int k = 0; k < 3; k++) {
        unsigned long long s = 0;
        for (uint32_t b = threadIdx.x; b < nblocks; b += blockDim.x)
            s += partial[3 * uint64_t(b) + k];
        acc[k][threadIdx.x] = s;
    }
    __syncthreads();
    for (uint32_t w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int k = 0; k < 3; k++)
                acc[k][threadIdx.x] += acc[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 3)
        totals[threadIdx.x] = acc[threadIdx.x][0];
}

} // namespace hd

namespace {
// Device address of g_noalloc_scratch per device, resolved on the first
// call made with that device current.
std::mutex g_noalloc_mutex;
unsigned long long* g_noalloc_ptr[256] = {};

unsigned long long* noalloc_scratch()
{
    int dev = 0;
    HD_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256)
        throw hd::StatusError{HD_ERR_INVALID, "device ordinal out of range"};
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        HD_CUDA(cudaGetSymbolAddress(&p, hd::g_noalloc_scratch));
        g_noalloc_ptr[dev] = static_cast<unsigned long long*>(p);
    }
    return g_noalloc_ptr[dev];
}
} // namespace

extern "C" hd_status hd_trace_counters_noalloc(hd_ctx* c, const hd_camera* cam, uint32_t w, uint32_t h,
                                               const float light[3], float bias, uint32_t* d_paths, uint8_t* d_mask,
                                               uint64_t out[6])
{
    using namespace hd;
    if (!c || !cam || !d_paths || !d_mask || !light || !out || !w || !h)
        return HD_ERR_INVALID;
    const uint64_t bx = (w + 7) / 8, by = (h + 7) / 8;
    if (bx * by > kNoAllocMaxBlocks) {
        c->err = "hd_trace_counters_noalloc: image of " + std::to_string(uint64_t(w) * h) +
                 " pixels exceeds the fixed scratch (at most 262144 blocks of 8x8 pixels, 16777216 pixels)";
        return HD_ERR_INVALID;
    }
    if (by > kMaxGridRows) {
        c->err = "hd_trace_counters_noalloc: image height " + std::to_string(h) + " exceeds " +
                 std::to_string(8 * kMaxGridRows) + " rows";
        return HD_ERR_INVALID;
    }
    try {
        unsigned long long* scratch = noalloc_scratch();
        unsigned long long* partial = scratch;
        unsigned long long* totals = scratch + 3 * uint64_t(kNoAllocMaxBlocks);
        const dim3 grid{uint32_t(bx), uint32_t(by), 1u};
        const uint32_t nb = uint32_t(bx * by);
        const F3 l = {light[0], light[1], light[2]};
        uint4* paths = reinterpret_cast<uint4*>(d_paths);
        if (c->fp_mode)
            k_trace_primary_partials<1><<<grid, 64, 0, c->stream>>>(c->t, c->d_root, *cam, w, h, paths, partial);
        else
            k_trace_primary_partials<0><<<grid, 64, 0, c->stream>>>(c->t, c->d_root, *cam, w, h, paths, partial);
        HD_LAUNCH_CHECK();
        k_sum_partials<<<1, 256, 0, c->stream>>>(partial, nb, totals);
        HD_LAUNCH_CHECK();
        if (c->fp_mode)
            k_trace_shadow_partials<1><<<grid, 64, 0, c->stream>>>(c->t, c->d_root, *cam, w, h, paths, l, bias,
                                                                   d_mask, partial);
        else
            k_trace_shadow_partials<0><<<grid, 64, 0, c->stream>>>(c->t, c->d_root, *cam, w, h, paths, l, bias,
                                                                   d_mask, partial);
        HD_LAUNCH_CHECK();
        k_sum_partials<<<1, 256, 0, c->stream>>>(partial, nb, totals + 3);
        HD_LAUNCH_CHECK();
        HD_CUDA(cudaMemcpyAsync(out, totals, 6 * sizeof(uint64_t), cudaMemcpyDeviceToHost, c->stream));
        HD_CUDA(cudaStreamSynchronize(c->stream));
        return HD_OK;
    } catch (const StatusError& e) {
        c->err = e.msg;
        return e.status;
    } catch (const CudaError& e) {
        c->err = std::string("CUDA error ") + cudaGetErrorString(e.code) + " in " + e.where;
        return HD_ERR_CUDA;
    }
}
