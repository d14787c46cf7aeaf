// ORACLE — test and measurement infrastructure only.
//
// Loads the cubin of the reference's own GPU tracer (made from the
// reference's unmodified tracer.cu by oracle/build_ref.py build_gpu_tracer,
// see oracle/refharness/ref_tracer_gpu.cu) and runs it the way the
// reference's headless DAGTracer does (dag_tracer.cu:9-24, :116-219): a
// 1920 x 1080 uint4 cudaArray surface for the paths, one launch per view
// with block (4, 64) and grid (W / 4 + 1, H / 64 + 1), cudaEvents around
// each launch.  The shadow pass is the harness's ref_shadow_hits kernel (the
// reference's hit test with the light as a parameter), launched with
// resolve_shadows' block shape.  Includes no reference header: the kernel
// parameter layouts are checked against the sizes the cubin reports.
//
// Built on any machine from this file alone (g++, CUDA runtime) into
// oracle/_build/libhdrefgpu.so by oracle/build_ref.py build_loader; never
// linked by the library.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace {

// Tracer::TracePathsParams (tracer.h:81-91)
struct PathsParams {
    double position[3], ray_min[3], ray_ddx[3], ray_ddy[3];
    unsigned long long paths_surface;
};
// Tracer::TraceShadowsParams (tracer.h:114-127)
struct ShadowsParams {
    double position[3], ray_min[3], ray_ddx[3], ray_ddy[3];
    float shadow_bias, fog_density;
    unsigned long long paths_surface, colors_surface;
};

struct State {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t trace_paths = nullptr, trace_shadows = nullptr, layout = nullptr, make_dag = nullptr,
                 shadow_hits = nullptr;
    uint32_t sizes[6] = {0, 0, 0, 0, 0, 0};
    std::vector<unsigned char> dag;  // HashDAG bytes, as the kernels take them
    uint32_t *pool = nullptr, *page_table = nullptr;
    cudaArray_t paths_array = nullptr, colors_array = nullptr;
    cudaSurfaceObject_t paths_surface = 0, colors_surface = 0;
    uint8_t* mask = nullptr;
    double* cam = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    std::string err;
} g;

void fail(const char* what, cudaError_t e) { g.err = std::string(what) + ": " + cudaGetErrorString(e); }
// returns 1 from the calling function, with the message, when a call fails
#define CK(call)                   \
    do {                           \
        cudaError_t e_ = (call);   \
        if (e_ != cudaSuccess) {   \
            fail(#call, e_);       \
            return 1;              \
        }                          \
    } while (0)

// The kernel whose name contains every one of `parts` (the mangled names of
// the reference's template kernels).
bool find_kernel(cudaKernel_t* out, const std::vector<std::string>& parts)
{
    unsigned int n = 0;
    if (cudaLibraryGetKernelCount(&n, g.lib) != cudaSuccess)
        return false;
    std::vector<cudaKernel_t> ks(n);
    if (cudaLibraryEnumerateKernels(ks.data(), n, g.lib) != cudaSuccess)
        return false;
    for (cudaKernel_t k : ks) {
        const char* name = nullptr;
        if (cudaFuncGetName(&name, reinterpret_cast<const void*>(k)) != cudaSuccess || !name)
            continue;
        bool all = true;
        for (const auto& p : parts)
            all &= std::strstr(name, p.c_str()) != nullptr;
        if (all) {
            *out = k;
            return true;
        }
    }
    return false;
}

} // namespace

extern "C" {

const char* refgpu_error() { return g.err.c_str(); }

// Loads the cubin; layout (optional, 6 words): sizeof(HashDAG),
// sizeof(TracePathsParams), sizeof(TraceShadowsParams), imageWidth,
// imageHeight, MAX_LEVELS.  Returns 0 on success.
int refgpu_open(const char* cubin, uint32_t* layout)
{
    CK(cudaLibraryLoadFromFile(&g.lib, cubin, nullptr, nullptr, 0, nullptr, nullptr, 0));
    CK(cudaLibraryGetKernel(&g.layout, g.lib, "ref_layout"));
    CK(cudaLibraryGetKernel(&g.make_dag, g.lib, "ref_make_dag"));
    CK(cudaLibraryGetKernel(&g.shadow_hits, g.lib, "ref_shadow_hits"));
    if (!find_kernel(&g.trace_paths, {"trace_paths", "7HashDAG"}) ||
        !find_kernel(&g.trace_shadows, {"trace_shadows", "7HashDAG"})) {
        g.err = "the reference's trace_paths / trace_shadows kernels are not in " + std::string(cubin);
        return 1;
    }
    uint32_t* d = nullptr;
    CK(cudaMalloc(&d, sizeof(g.sizes)));
    void* args[] = {&d};
    CK(cudaLaunchKernel(reinterpret_cast<const void*>(g.layout), dim3(1), dim3(1), args, 0, nullptr));
    CK(cudaMemcpy(g.sizes, d, sizeof(g.sizes), cudaMemcpyDeviceToHost));
    cudaFree(d);
    if (g.sizes[1] != sizeof(PathsParams) || g.sizes[2] != sizeof(ShadowsParams)) {
        g.err = "kernel parameter layout differs from the loader's";
        return 1;
    }
    const cudaChannelFormatDesc pd = cudaCreateChannelDesc(32, 32, 32, 32, cudaChannelFormatKindUnsigned);
    CK(cudaMallocArray(&g.paths_array, &pd, g.sizes[3], g.sizes[4], cudaArraySurfaceLoadStore));
    const cudaChannelFormatDesc cd = cudaCreateChannelDesc(8, 8, 8, 8, cudaChannelFormatKindUnsigned);
    CK(cudaMallocArray(&g.colors_array, &cd, g.sizes[3], g.sizes[4], cudaArraySurfaceLoadStore));
    cudaResourceDesc rd{};
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = g.paths_array;
    CK(cudaCreateSurfaceObject(&g.paths_surface, &rd));
    rd.res.array.array = g.colors_array;
    CK(cudaCreateSurfaceObject(&g.colors_surface, &rd));
    CK(cudaMalloc(&g.mask, size_t(g.sizes[3]) * g.sizes[4]));
    CK(cudaMalloc(&g.cam, 12 * sizeof(double)));
    for (auto& e : g.ev)
        CK(cudaEventCreate(&e));
    if (layout)
        std::memcpy(layout, g.sizes, sizeof(g.sizes));
    return 0;
}

// Uploads a table (the reference's HashTable device arrays: pool pages and
// page table) and builds the HashDAG value the kernels take.
int refgpu_set_dag(const uint32_t* pool, uint64_t pool_words, const uint32_t* page_table, uint32_t pt_entries,
                   uint32_t pool_top, uint32_t root)
{
    cudaFree(g.pool);
    cudaFree(g.page_table);
    g.pool = g.page_table = nullptr;
    CK(cudaMalloc(&g.pool, pool_words * 4 + 256));
    CK(cudaMalloc(&g.page_table, size_t(pt_entries) * 4));
    CK(cudaMemcpy(g.pool, pool, pool_words * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(g.page_table, page_table, size_t(pt_entries) * 4, cudaMemcpyHostToDevice));
    void* d = nullptr;
    CK(cudaMalloc(&d, g.sizes[0]));
    void* args[] = {&d, &g.pool, &g.page_table, &pt_entries, &pool_top, &root};
    CK(cudaLaunchKernel(reinterpret_cast<const void*>(g.make_dag), dim3(1), dim3(1), args, 0, nullptr));
    g.dag.resize(g.sizes[0]);
    CK(cudaMemcpy(g.dag.data(), d, g.sizes[0], cudaMemcpyDeviceToHost));
    cudaFree(d);
    return 0;
}

// One view: trace_paths, then the shadow hits (the reference's own
// trace_shadows as well when own_shadows is set, which shades the colour
// surface with its hard-coded sun).  cam: the 12 doubles of
// TracePathsParams.  paths (optional): W * H uint4 read back from the
// surface; mask (optional): W * H bytes.  ms[0..2]: event time of
// trace_paths, of the shadow hits, of trace_shadows.
int refgpu_trace_view(const double* cam, const float* light, float bias, int own_shadows, uint32_t* paths,
                      uint8_t* mask, float* ms)
{
    const uint32_t W = g.sizes[3], H = g.sizes[4];
    PathsParams pp{};
    std::memcpy(pp.position, cam, 12 * sizeof(double));
    pp.paths_surface = g.paths_surface;
    const dim3 block(4, 64), grid(W / block.x + 1, H / block.y + 1);
    void* a_paths[] = {&pp, g.dag.data()};
    CK(cudaMemcpyAsync(g.cam, cam, 12 * sizeof(double), cudaMemcpyHostToDevice, nullptr));
    CK(cudaEventRecord(g.ev[0], nullptr));
    CK(cudaLaunchKernel(reinterpret_cast<const void*>(g.trace_paths), grid, block, a_paths, 0, nullptr));
    CK(cudaEventRecord(g.ev[1], nullptr));
    float lx = light[0], ly = light[1], lz = light[2];
    void* a_hits[] = {&g.cam, &g.paths_surface, g.dag.data(), &lx, &ly, &lz, &bias, &g.mask};
    CK(cudaLaunchKernel(reinterpret_cast<const void*>(g.shadow_hits), grid, block, a_hits, 0, nullptr));
    CK(cudaEventRecord(g.ev[2], nullptr));
    if (own_shadows) {
        ShadowsParams sp{};
        std::memcpy(sp.position, cam, 12 * sizeof(double));
        sp.shadow_bias = bias;
        sp.fog_density = 0.0f;
        sp.paths_surface = g.paths_surface;
        sp.colors_surface = g.colors_surface;
        void* a_sh[] = {&sp, g.dag.data()};
        CK(cudaLaunchKernel(reinterpret_cast<const void*>(g.trace_shadows), grid, block, a_sh, 0, nullptr));
    }
    CK(cudaEventRecord(g.ev[3], nullptr));
    CK(cudaEventSynchronize(g.ev[3]));
    if (ms) {
        CK(cudaEventElapsedTime(&ms[0], g.ev[0], g.ev[1]));
        CK(cudaEventElapsedTime(&ms[1], g.ev[1], g.ev[2]));
        ms[2] = 0.0f;
        if (own_shadows)
            CK(cudaEventElapsedTime(&ms[2], g.ev[2], g.ev[3]));
    }
    if (paths)
        CK(cudaMemcpy2DFromArray(paths, size_t(W) * 16, g.paths_array, 0, 0, size_t(W) * 16, H,
                                 cudaMemcpyDeviceToHost));
    if (mask)
        CK(cudaMemcpy(mask, g.mask, size_t(W) * H, cudaMemcpyDeviceToHost));
    return 0;
}

void refgpu_close()
{
    if (g.paths_surface)
        cudaDestroySurfaceObject(g.paths_surface);
    if (g.colors_surface)
        cudaDestroySurfaceObject(g.colors_surface);
    if (g.paths_array)
        cudaFreeArray(g.paths_array);
    if (g.colors_array)
        cudaFreeArray(g.colors_array);
    cudaFree(g.pool);
    cudaFree(g.page_table);
    cudaFree(g.mask);
    cudaFree(g.cam);
    for (auto& e : g.ev)
        if (e)
            cudaEventDestroy(e);
    if (g.lib)
        cudaLibraryUnload(g.lib);
    g = State{};
}

} // extern "C"
