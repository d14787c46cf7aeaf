// ORACLE — test infrastructure only.
//
// The reference's own traversal and shading code (tracer.cu:
// Tracer::trace_paths, intersect_ray_node_out_of_order, ray_box_intersection,
// Tracer::trace_colors), compiled for the host from its unmodified sources
// on top of the host harness (ref_host.cpp), so that the golden traversal
// and colour-view fixtures come from the reference itself rather than from a
// restatement.  Built by oracle/build_ref.py (tracer=True, with colors=True
// for trace_colors) into oracle/_ref; never shipped.
//
// Host stand-ins, each for a CUDA construct the kernels use:
//  * blockIdx / blockDim / threadIdx: thread-local values set per pixel;
//  * surf2Dwrite / surf2Dread: a plain 2D byte array (RefSurface);
//  * __clz: the count of leading zeros of a 32-bit word.
// Path::store / Path::load reach their surface only in device code
// (path.h:63-77), so path.h is compiled first with __CUDA_ARCH__ defined;
// nothing else in it depends on that macro.
//
// Arithmetic: compiled with -ffp-contract=off, every float and double
// operation is rounded on its own, as the library's fp_mode 0 does; the
// reference's own CUDA build contracts some of them into fused
// multiply-adds (the library's fp_mode 1), which a host compile cannot
// reproduce, so these fixtures pin fp_mode 0.

#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>
#include <cuda_runtime.h>

struct RefSurface {
    uint8_t* data;
    size_t pitch;
};
template <class T>
inline void surf2Dwrite(T v, cudaSurfaceObject_t s, int x, int y, cudaSurfaceBoundaryMode = cudaBoundaryModeTrap)
{
    RefSurface* r = reinterpret_cast<RefSurface*>(s);
    std::memcpy(r->data + size_t(y) * r->pitch + size_t(x), &v, sizeof(T));
}
template <class T>
inline T surf2Dread(cudaSurfaceObject_t s, int x, int y, cudaSurfaceBoundaryMode = cudaBoundaryModeTrap)
{
    const RefSurface* r = reinterpret_cast<const RefSurface*>(s);
    T v;
    std::memcpy(&v, r->data + size_t(y) * r->pitch + size_t(x), sizeof(T));
    return v;
}
inline int ref_clz(unsigned int x) { return x ? __builtin_clz(x) : 32; }

#include "typedefs.h"
#include "cuda_math.h"
#define __CUDA_ARCH__ 1000
#include "path.h"
#undef __CUDA_ARCH__

#include "ref_host.cpp"

static thread_local uint3 ref_block_idx, ref_thread_idx;
static thread_local dim3 ref_block_dim;
#define blockIdx ref_block_idx
#define threadIdx ref_thread_idx
#define blockDim ref_block_dim
#define __clz ref_clz
#include "tracer.cu"
#undef blockIdx
#undef threadIdx
#undef blockDim
#undef __clz

// Runs f(x, y) for every pixel of the imageWidth x imageHeight frame, rows
// split over `threads` host threads.
template <class F>
static void for_pixels(int threads, F f)
{
    std::vector<std::thread> pool;
    const uint32 n = threads > 0 ? uint32(threads) : 1u;
    for (uint32 k = 0; k < n; k++)
        pool.emplace_back([&, k] {
            for (uint32 y = k; y < imageHeight; y += n)
                for (uint32 x = 0; x < imageWidth; x++)
                    f(x, y);
        });
    for (auto& t : pool)
        t.join();
}

// Tracer::trace_paths over the whole frame; paths: imageHeight x imageWidth
// uint4 (x, y, z, 0) in output rows, as the reference's surface holds them.
// cam: position, rayMin, rayDDx, rayDDy (12 doubles, TracePathsParams).
extern "C" uint32 ref_image_width() { return imageWidth; }
extern "C" uint32 ref_image_height() { return imageHeight; }
extern "C" void ref_trace_paths(const double* cam, uint32* paths, int threads)
{
    RefSurface surface{reinterpret_cast<uint8_t*>(paths), size_t(imageWidth) * sizeof(uint4)};
    Tracer::TracePathsParams params;
    params.cameraPosition = make_double3(cam[0], cam[1], cam[2]);
    params.rayMin = make_double3(cam[3], cam[4], cam[5]);
    params.rayDDx = make_double3(cam[6], cam[7], cam[8]);
    params.rayDDy = make_double3(cam[9], cam[10], cam[11]);
    params.pathsSurface = reinterpret_cast<cudaSurfaceObject_t>(&surface);
    const HashDAG dag = g_dag;
    for_pixels(threads, [&](uint32 x, uint32 y) {
        ref_block_dim = dim3(1, 1, 1);
        ref_thread_idx = make_uint3(0, 0, 0);
        ref_block_idx = make_uint3(x, y, 0);
        Tracer::trace_paths<HashDAG>(params, dag);
    });
}

// The hit test of Tracer::trace_shadows (tracer.cu:590-648) for every pixel
// of a paths image made by ref_trace_paths: the exact hit point on the hit
// voxel's box (ray_box_intersection, EXACT_SHADOWS = 1), the shadow ray from
// it plus bias along the light, and intersect_ray_node_out_of_order — the
// reference's own functions, in the order trace_shadows calls them, with
// the light as a parameter (sun_direction() hard-codes (0.3, 1, 0.5)).
// mask: 1 shadowed, 0 lit, 2 no hit (the reference shades those as sky).
extern "C" void ref_trace_shadows(const double* cam, const uint32* paths, const float* light, float bias,
                                  uint8_t* mask, int threads)
{
    RefSurface surface{const_cast<uint8_t*>(reinterpret_cast<const uint8_t*>(paths)),
                       size_t(imageWidth) * sizeof(uint4)};
    const cudaSurfaceObject_t paths_surface = reinterpret_cast<cudaSurfaceObject_t>(&surface);
    const double3 position = make_double3(cam[0], cam[1], cam[2]);
    const double3 ray_min = make_double3(cam[3], cam[4], cam[5]);
    const double3 ddx = make_double3(cam[6], cam[7], cam[8]);
    const double3 ddy = make_double3(cam[9], cam[10], cam[11]);
    const float3 direction = normalize(make_float3(light[0], light[1], light[2]));
    const HashDAG dag = g_dag;
    for_pixels(threads, [&](uint32 x, uint32 y) {
        const float3 rayOrigin = make_float3(Path::load(x, y, paths_surface).path);
        const double3 cameraRayDirection =
            normalize(ray_min + x * ddx + (imageHeight - 1 - y) * ddy - position);
        const double3 rayOriginDouble = make_double3(rayOrigin);
        const double3 hitPosition =
            ray_box_intersection(position, cameraRayDirection, rayOriginDouble, rayOriginDouble + 1);
        const float3 shadowStart = make_float3(hitPosition);
        uint8_t m = 2;
        if (length(rayOrigin) != 0.0f)
            m = intersect_ray_node_out_of_order(dag, shadowStart + bias * direction, direction) ? 1 : 0;
        mask[size_t(y) * imageWidth + x] = m;
    });
}

#if EDITS_ENABLE_COLORS
// Tracer::trace_colors (tracer.cu:254-451) over a paths image made by
// ref_trace_paths, on the harness's colours; colors: imageHeight x
// imageWidth uint32 (rgb888).  tool: ETool, or a negative value for no
// overlay (the overlay needs TOOL_OVERLAY=1, which build_ref.py sets for the
// tracer build).  pos / src / dst: the ToolInfo paths.
extern "C" void ref_trace_colors(const uint32* paths, uint32 debug, uint32 debug_level, int tool, const uint32* pos,
                                 float radius, const uint32* src, const uint32* dst, uint32* colors, int threads)
{
    RefSurface ps{const_cast<uint8_t*>(reinterpret_cast<const uint8_t*>(paths)), size_t(imageWidth) * sizeof(uint4)};
    RefSurface cs{reinterpret_cast<uint8_t*>(colors), size_t(imageWidth) * sizeof(uint32)};
    Tracer::TraceColorsParams params;
    params.debugColors = EDebugColors(debug);
    params.debugColorsIndexLevel = debug_level;
    // no overlay: a sphere of radius 1e-30 at the null path, whose strength
    // 1 - distance / radius is negative at every voxel path
    params.toolInfo = tool < 0 ? ToolInfo(ETool::Sphere, make_uint3(0u, 0u, 0u), 1e-30f, make_uint3(0u, 0u, 0u),
                                          make_uint3(0u, 0u, 0u))
                               : ToolInfo(ETool(tool), make_uint3(pos[0], pos[1], pos[2]), radius,
                                          make_uint3(src[0], src[1], src[2]), make_uint3(dst[0], dst[1], dst[2]));
    params.pathsSurface = reinterpret_cast<cudaSurfaceObject_t>(&ps);
    params.colorsSurface = reinterpret_cast<cudaSurfaceObject_t>(&cs);
    const HashDAG dag = g_dag;
    const HashDAGColors cols = g_colors;
    for_pixels(threads, [&](uint32 x, uint32 y) {
        ref_block_dim = dim3(1, 1, 1);
        ref_thread_idx = make_uint3(0, 0, 0);
        ref_block_idx = make_uint3(x, y, 0);
        Tracer::trace_colors<HashDAG, HashDAGColors>(params, dag, cols);
    });
}
#endif
