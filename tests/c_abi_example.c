/* A plain C program on the C ABI, as a caller of the reference's hot path
 * would use it: create a context, generate the seeded scene, trace one
 * primary + shadow frame, carve a sphere, trace again, report, destroy.
 * tests/test_c_abi_example.py compiles and links it with gcc (no GPU
 * needed for that) and runs it when a GPU is present.
 *
 *   gcc -std=c99 -I include tests/c_abi_example.c \
 *       -L hashdag_gb300 -lhashdag_gb300 -o c_abi_example
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "hashdag_gb300.h"

#define CHECK(call)                                                                  \
    do {                                                                             \
        hd_status s_ = (call);                                                       \
        if (s_ != HD_OK) {                                                           \
            fprintf(stderr, "%s failed (%d): %s\n", #call, (int)s_, hd_last_error(ctx)); \
            return 1;                                                                \
        }                                                                            \
    } while (0)

/* get_trace_params (dag_tracer.cu:71-113) for a camera at p looking along
 * -z with a 90 degree field of view */
static void camera(hd_camera* cam, double px, double py, double pz, uint32_t w, uint32_t h)
{
    const double aspect = (double)w / (double)h, s = 0.70710678118654752, c = 0.70710678118654752;
    memset(cam, 0, sizeof(*cam));
    cam->position[0] = px;
    cam->position[1] = py;
    cam->position[2] = pz;
    /* forward (0, 0, -1), right (1, 0, 0), up (0, 1, 0) */
    cam->ray_min[0] = px - s * aspect;
    cam->ray_min[1] = py - s;
    cam->ray_min[2] = pz - c;
    cam->ray_ddx[0] = 2.0 * s * aspect / w;
    cam->ray_ddy[1] = 2.0 * s / h;
}

static uint64_t hits(const uint32_t* paths, uint64_t n)
{
    uint64_t k = 0;
    for (uint64_t i = 0; i < n; i++)
        k += (paths[4 * i] | paths[4 * i + 1] | paths[4 * i + 2]) != 0;
    return k;
}

int main(void)
{
    const uint32_t depth = 10, w = 320, h = 180;
    const uint64_t px = (uint64_t)w * h;
    hd_ctx* ctx = NULL;
    hd_config cfg;
    hd_camera cam;
    hd_edit_stats st;
    hd_edit edit;
    const float light[3] = {0.3f, 1.0f, 0.2f};
    float ms_primary = 0.0f, ms_shadow = 0.0f;
    uint32_t *d_paths = NULL, *h_paths = NULL;
    uint8_t* d_mask = NULL;
    uint32_t root0 = 0, root1 = 0;
    uint64_t before, after;

    if (hd_abi_version() != HD_ABI_VERSION) {
        fprintf(stderr, "ABI %u, header %u\n", hd_abi_version(), (unsigned)HD_ABI_VERSION);
        return 1;
    }
    hd_default_config(depth, &cfg);
    if (hd_create(&cfg, &ctx) != HD_OK) {
        fprintf(stderr, "hd_create failed\n");
        return 1;
    }
    CHECK(hd_generate_scene(ctx, 1));
    CHECK(hd_get_root(ctx, &root0));
    if (cudaMalloc((void**)&d_paths, px * 16) != cudaSuccess || cudaMalloc((void**)&d_mask, px) != cudaSuccess)
        return 1;
    h_paths = (uint32_t*)malloc(px * 16);
    camera(&cam, 512.0, 900.0, 1700.0, w, h);
    CHECK(hd_trace_frame(ctx, &cam, w, h, light, 1.0f, d_paths, d_mask, &ms_primary, &ms_shadow));
    cudaMemcpy(h_paths, d_paths, px * 16, cudaMemcpyDeviceToHost);
    before = hits(h_paths, px);

    memset(&edit, 0, sizeof(edit));
    edit.tool = HD_TOOL_SPHERE_REMOVE;
    edit.center[0] = 512.0f;
    edit.center[1] = 640.0f;
    edit.center[2] = 512.0f;
    edit.radius = 200.0f;
    CHECK(hd_edit_apply(ctx, &edit, &st));
    CHECK(hd_get_root(ctx, &root1));
    CHECK(hd_trace_frame(ctx, &cam, w, h, light, 1.0f, d_paths, d_mask, &ms_primary, &ms_shadow));
    cudaMemcpy(h_paths, d_paths, px * 16, cudaMemcpyDeviceToHost);
    after = hits(h_paths, px);

    printf("root %u -> %u, edited voxels %llu, find_or_add %llu, hits %llu -> %llu\n", root0, root1,
           (unsigned long long)st.num_voxels, (unsigned long long)st.find_or_add_calls,
           (unsigned long long)before, (unsigned long long)after);
    free(h_paths);
    cudaFree(d_paths);
    cudaFree(d_mask);
    CHECK(hd_destroy(ctx));
    return (root0 != root1 && st.num_voxels > 0 && before > 0) ? 0 : 2;
}
