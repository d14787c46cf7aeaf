// ORACLE — test and measurement infrastructure only.
//
// The reference's own traversal kernels, compiled from its unmodified
// tracer.cu for sm_103a into a cubin (oracle/_ref/ref_tracer_d<D>.cubin, by
// oracle/build_ref.py build_gpu_tracer), so that the GB300 can run the
// reference's GPU tracer beside the library's: Tracer::trace_paths<HashDAG>
// (tracer.cu:145-252) and Tracer::trace_shadows<HashDAG> (tracer.cu:589-697)
// as tracer.cu instantiates them (tracer.cu:699-703).  Compiled as the
// reference's CMake build compiles its CUDA code (CMakeLists.txt:21-28:
// nvcc defaults, --expt-relaxed-constexpr; fused multiply-adds contracted).
//
// Beside them, three small kernels of this harness (extern "C", so the
// loader finds them by name):
//  * ref_layout: sizeof of the kernel parameter types, so that the loader
//    (oracle/refgpu_loader.cpp, which includes no reference header) can
//    check its byte layouts;
//  * ref_make_dag: a HashDAG value over a device pool and page table (the
//    fields HashTable::create and upload_to_gpu fill on the device side);
//  * ref_shadow_hits: the hit test of Tracer::trace_shadows with the light
//    as a parameter (its sun_direction() hard-codes (0.3, 1, 0.5),
//    tracer.cu:546-549): the reference's own ray_box_intersection and
//    intersect_ray_node_out_of_order, called in the order trace_shadows
//    calls them, writing a mask (1 shadowed, 0 lit, 2 no hit) instead of a
//    shaded colour.  Launched with resolve_shadows' block shape.
//
// Configuration: HARNESS_DEPTH (scene depth; typedefs.h forces 17),
// HARNESS_CTL (C_colorTreeLevels),
// BENCHMARK=1, no Bloom filter, no colours; imageWidth x imageHeight stay
// the reference's 1920 x 1080 (typedefs.h:683-684).

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <functional>
#include <limits>
#include <memory>
#include <mutex>
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
// `constexpr uint32 C_colorTreeLevels = 10;` (hash_dag_globals.h:7) becomes
// `constexpr uint32 CTL_VALUE = HARNESS_CTL, CTL_IGNORED = 10;`
#define C_colorTreeLevels CTL_VALUE = HARNESS_CTL, CTL_IGNORED

#include "typedefs.h"
#undef SCENE_DEPTH
#define SCENE_DEPTH HARNESS_DEPTH
#include "dags/hash_dag/hash_dag_globals.h"
#undef C_colorTreeLevels
#define C_colorTreeLevels CTL_VALUE

#include "camera_view.h"
#include "tracer.cu"

extern "C" __global__ void ref_layout(uint32_t* out)
{
    out[0] = uint32_t(sizeof(HashDAG));
    out[1] = uint32_t(sizeof(Tracer::TracePathsParams));
    out[2] = uint32_t(sizeof(Tracer::TraceShadowsParams));
    out[3] = uint32_t(imageWidth);
    out[4] = uint32_t(imageHeight);
    out[5] = uint32_t(MAX_LEVELS);
}

extern "C" __global__ void ref_make_dag(HashDAG* out, uint32_t* pool, uint32_t* page_table, uint32_t page_table_size,
                                        uint32_t pool_top, uint32_t root)
{
    HashDAG dag;
    dag.data.gpuPool = pool;
    dag.data.gpuPageTable = page_table;
    dag.data.pageTableSize = page_table_size;
    dag.data.poolTop = pool_top;
    dag.firstNodeIndex = root;
    *out = dag;
}

extern "C" __global__ void ref_shadow_hits(const double* __restrict__ cam, cudaSurfaceObject_t paths,
                                           const HashDAG dag, float lx, float ly, float lz, float bias,
                                           uint8_t* __restrict__ mask)
{
    const uint2 pixel = make_uint2(blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y);
    if (pixel.x >= imageWidth || pixel.y >= imageHeight)
        return;
    const double3 position = make_double3(cam[0], cam[1], cam[2]);
    const double3 ray_min = make_double3(cam[3], cam[4], cam[5]);
    const double3 ddx = make_double3(cam[6], cam[7], cam[8]);
    const double3 ddy = make_double3(cam[9], cam[10], cam[11]);
    const float3 rayOrigin = make_float3(Path::load(pixel.x, pixel.y, paths).path);
    const double3 cameraRayDirection =
        normalize(ray_min + pixel.x * ddx + (imageHeight - 1 - pixel.y) * ddy - position);
    const double3 rayOriginDouble = make_double3(rayOrigin);
    const double3 hitPosition =
        ray_box_intersection(position, cameraRayDirection, rayOriginDouble, rayOriginDouble + 1);
    const float3 shadowStart = make_float3(hitPosition);
    uint8_t m = 2;
    if (length(rayOrigin) != 0.0f) {
        const float3 direction = normalize(make_float3(lx, ly, lz));
        m = intersect_ray_node_out_of_order(dag, shadowStart + bias * direction, direction) ? 1 : 0;
    }
    mask[size_t(pixel.y) * imageWidth + pixel.x] = m;
}
