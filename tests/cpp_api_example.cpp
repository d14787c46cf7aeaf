// A C++ caller written against include/hashdag_gb300.hpp the way the
// reference's engine calls its own classes (Engine::edit, engine.h:77-103;
// DAGTracer in Engine::tick, engine.cpp:575-720; undo / redo and GC,
// engine.cpp:178-185): load a BasicDAG through HashDAGFactory, render with
// a CameraView, edit with SphereEditor / BoxEditor through edit_threads,
// undo / redo, collect, paint a coloured scene and draw its colours.
// tests/test_cpp_api_example.py compiles it with g++ (no GPU needed) and runs
// it on a GPU.
#include <cstdio>
#include <vector>

#include "hashdag_gb300.hpp"

using namespace hashdag_gb300;

static uint64_t hits(const DAGTracer& tr)
{
    std::vector<uint32_t> p(size_t(tr.imageWidth) * tr.imageHeight * 4);
    check_cuda(cudaMemcpy(p.data(), tr.paths(), p.size() * 4, cudaMemcpyDeviceToHost), "paths");
    uint64_t n = 0;
    for (size_t i = 0; i < p.size(); i += 4)
        n += (p[i] | p[i + 1] | p[i + 2]) != 0;
    return n;
}

static int run()
{
    const uint32 depth = 10;
    // a BasicDAG to load: the seeded scene's words
    std::vector<uint32_t> words;
    {
        HashDAG gen(depth);
        check(gen.context(), hd_generate_scene(gen.context(), 1), "hd_generate_scene");
        uint64_t n = 0;
        check(gen.context(), hd_export_basic_dag(gen.context(), nullptr, 0, &n), "size");
        words.resize(n);
        check(gen.context(), hd_export_basic_dag(gen.context(), words.data(), n, &n), "hd_export_basic_dag");
    }
    HashDAG dag;
    HashDAGFactory::load_from_DAG(dag, words, depth);
    HashDAGColors colors;
    HashDAGUndoRedo undoRedo;
    StatsRecorder stats;

    // a camera outside the volume looking at its centre (scene box 0..1024)
    CameraView view;
    view.position = {512.f, 900.f, 1900.f};
    // rows: -right, up, forward (camera_view.h:13-27); forward toward -z
    view.rotation = Matrix3x3{-1, 0, 0, 0, 1, 0, 0, 0, -1};
    DAGInfo info;
    info.boundsAABBMin = {0.f, 0.f, 0.f};
    info.boundsAABBMax = {1024.f, 1024.f, 1024.f};

    DAGTracer tracer(true, 640, 360);
    const float ms = tracer.resolve_paths(view, info, dag);
    tracer.resolve_shadows(view, info, dag, 1.0f, 0.0f);
    const uint64_t before = hits(tracer);
    if (!(ms > 0.f) || before == 0) {
        std::printf("no hits before the edit\n");
        return 1;
    }
    const uint32 root0 = dag.firstNodeIndex;

    dag.edit_threads(SphereEditor<false>(make_float3(512.f, 512.f, 512.f), 96.f), colors, undoRedo, stats);
    const uint32 root1 = dag.firstNodeIndex;
    const double voxels = stats.get("num voxels");
    stats.next_frame();
    dag.edit_threads(BoxEditor<true>(make_float3(300.f, 700.f, 300.f), 40.f), colors, undoRedo, stats);
    const uint32 root2 = dag.firstNodeIndex;
    if (root1 == root0 || root2 == root1 || !(voxels > 0)) {
        std::printf("edits did not change the scene\n");
        return 1;
    }
    undoRedo.undo(dag, colors);
    undoRedo.undo(dag, colors);
    if (dag.firstNodeIndex != root0) {
        std::printf("undo did not restore the root\n");
        return 1;
    }
    undoRedo.redo(dag, colors);
    if (dag.firstNodeIndex != root1) {
        std::printf("redo did not restore the first edit\n");
        return 1;
    }
    tracer.resolve_paths(view, info, dag);
    const uint64_t edited = hits(tracer);
    const uint3 centre = tracer.get_path(320, 180);
    dag.remove_stale_nodes(depth - 2);
    tracer.resolve_paths(view, info, dag);
    if (hits(tracer) != edited) {
        std::printf("GC changed the frame\n");
        return 1;
    }
    const hd_level_stats ls = dag.level_stats();

    // colours: the shell scene, a blue paint, the colour view
    HashDAG shell(depth);
    check(shell.context(), hd_generate_scene_ex(shell.context(), 1, HD_SCENE_SHELL), "hd_generate_scene_ex");
    shell.refresh();
    HashDAGColors shellColors;
    shellColors.colors_from_scene(shell, 2);
    shell.edit_threads(SpherePaintEditor(make_float3(512.f, 512.f, 512.f), 200.f), shellColors, undoRedo, stats);
    tracer.resolve_paths(view, info, shell);
    const float cms = tracer.resolve_colors(shell, shellColors, EDebugColors::None, 0, ToolInfo());

    std::printf("hits %llu -> %llu, centre (%u %u %u), edited voxels %.0f, pages %llu, colours %.3f ms\n",
                (unsigned long long)before, (unsigned long long)edited, centre.x, centre.y, centre.z, voxels,
                (unsigned long long)ls.pages_used, cms);

    // errors are exceptions with the C status
    try {
        dag.edit_threads(SphereEditor<false>(make_float3(0.f, 0.f, 0.f), -1.f), colors, undoRedo, stats);
        std::printf("a negative radius was accepted\n");
        return 1;
    } catch (const Error& e) {
        if (e.status != HD_ERR_INVALID)
            return 1;
    }
    std::printf("cpp api ok\n");
    return 0;
}

int main()
{
    try {
        return run();
    } catch (const Error& e) {
        std::printf("error %d: %s\n", int(e.status), e.what());
        return 1;
    }
}
