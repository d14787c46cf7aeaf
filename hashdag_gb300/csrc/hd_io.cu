// Files: the reference's on-disk formats and the snapshot.
//
// The reference writes raw little-endian values with FileWriter and reads
// them back with FileReader (serializer.h:11-121); an array is its uint64
// element count followed by its elements, a DAGInfo six doubles (AABB min,
// then max).
//   BasicDAG file (BasicDAGFactory::save_dag_to_file / load_dag_from_file,
//     basic_dag.cpp:94-117): DAGInfo, uint32 levels, the node words array.
//   Compressed colours (save/load_compressed_colors_to_file,
//     basic_dag.cpp:34-92): uint32 topLevels, enclosedLeaves (uint64 each,
//     or uint32 in old files, which the reference then zeroes), the main
//     leaf's weights (uint32 words in file order; byte-swapped on load),
//     blocks and macro blocks (uint64).
//   Hash-DAG file (HashDAGFactory::save_dag_to_file / load_dag_from_file,
//     hash_dag_factory.cpp:199-246): DAGInfo, uint32 levels, firstNodeIndex,
//     poolMaxSize, pageTableSize, poolTop, then poolTop pages of the pool and
//     the page table.  It has no bucket sizes, so a table read from it can
//     be traced but not edited until a GC has rebuilt its buckets.
//   Snapshot: a hash-DAG file followed by an extension the reference's
//     reader never reaches: "HDGB-SNP", uint32 version, uint32 flags (1:
//     colours), the hd_config, the bucket sizes array, the full-node indices
//     (depth words), the stored node count of every level (HD_MAX_DEPTH
//     uint64) and, with colours, the five colour-table counters and
//     the colour nodes, leaf descriptors, blocks, macro blocks and weights.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "hd_ctx.h"

namespace hd {
namespace {

const char kSnapshotMagic[8] = {'H', 'D', 'G', 'B', '-', 'S', 'N', 'P'};
constexpr uint32_t kSnapshotVersion = 1;

struct InFile {
    FILE* f = nullptr;
    std::string path;
    uint64_t size = 0;
    explicit InFile(const char* p) : path(p)
    {
        f = std::fopen(p, "rb");
        if (!f)
            throw StatusError{HD_ERR_IO, "cannot open " + path};
        std::fseek(f, 0, SEEK_END);
        size = uint64_t(std::ftell(f));
        std::fseek(f, 0, SEEK_SET);
    }
    ~InFile()
    {
        if (f)
            std::fclose(f);
    }
    uint64_t left() const { return size - uint64_t(std::ftell(f)); }
    void read(void* d, uint64_t n)
    {
        if (n && std::fread(d, 1, n, f) != n)
            throw StatusError{HD_ERR_IO, "short read in " + path};
    }
    template <typename T>
    T value()
    {
        T v{};
        read(&v, sizeof(T));
        return v;
    }
    // FileReader::read(StaticArray&): the count, then the elements
    template <typename T>
    std::vector<T> array()
    {
        const uint64_t n = value<uint64_t>();
        if (n > left() / sizeof(T))
            throw StatusError{HD_ERR_IO, "array of " + std::to_string(n) + " elements runs past the end of " + path};
        std::vector<T> v(n);
        read(v.data(), n * sizeof(T));
        return v;
    }
};

struct OutFile {
    FILE* f = nullptr;
    std::string path;
    explicit OutFile(const char* p) : path(p)
    {
        f = std::fopen(p, "wb");
        if (!f)
            throw StatusError{HD_ERR_IO, "cannot create " + path};
    }
    ~OutFile()
    {
        if (f)
            std::fclose(f);
    }
    void write(const void* d, uint64_t n)
    {
        if (n && std::fwrite(d, 1, n, f) != n)
            throw StatusError{HD_ERR_IO, "write failed on " + path};
    }
    template <typename T>
    void value(const T& v)
    {
        write(&v, sizeof(T));
    }
    template <typename T>
    void array(const T* d, uint64_t n)
    {
        value<uint64_t>(n);
        write(d, n * sizeof(T));
    }
    void close()
    {
        const bool ok = std::fflush(f) == 0 && !std::ferror(f);
        std::fclose(f);
        f = nullptr;
        if (!ok)
            throw StatusError{HD_ERR_IO, "write failed on " + path};
    }
};

void read_info(InFile& in, hd_dag_info* info)
{
    hd_dag_info i{};
    in.read(i.aabb_min, 24);
    in.read(i.aabb_max, 24);
    if (info)
        *info = i;
}

void write_info(OutFile& out, const hd_dag_info* info)
{
    const hd_dag_info i = info ? *info : hd_dag_info{};
    out.write(i.aabb_min, 24);
    out.write(i.aabb_max, 24);
}

void check_levels(hd_ctx* c, uint32_t levels, const std::string& path)
{
    if (levels != c->cfg.depth)
        throw StatusError{HD_ERR_INVALID, path + " holds a scene of " + std::to_string(levels) +
                                              " levels; the context has " + std::to_string(c->cfg.depth)};
}

void clear_history(hd_ctx* c)
{
    c->undo.clear();
    c->redo.clear();
}

} // namespace

// The context keeps the BasicDAG it imported (for hd_export_basic_dag and
// hd_save_basic_dag_file).
void keep_basic(hd_ctx* c, const uint32_t* h_words, uint64_t n)
{
    if (c->d_basic)
        cudaFree(c->d_basic);
    c->d_basic = nullptr;
    c->n_basic = 0;
    if (cudaMalloc(&c->d_basic, n * 4) != cudaSuccess) {
        cudaGetLastError();
        c->d_basic = nullptr;
        throw StatusError{HD_ERR_OOM, "BasicDAG copy allocation failed"};
    }
    HD_CUDA(cudaMemcpyAsync(c->d_basic, h_words, n * 4, cudaMemcpyDefault, c->stream));
    c->n_basic = n;
}

} // namespace hd

using namespace hd;

extern "C" {

hd_status hd_load_basic_dag_file(hd_ctx* c, const char* path, hd_dag_info* info)
{
    if (!c || !path)
        return HD_ERR_INVALID;
    return guarded(c, [&] {
        InFile in(path);
        read_info(in, info);
        check_levels(c, in.value<uint32_t>(), in.path);
        const std::vector<uint32_t> words = in.array<uint32_t>();
        if (words.size() < 2)
            throw StatusError{HD_ERR_INVALID, in.path + " holds no nodes"};
        keep_basic(c, words.data(), words.size());
        table_reset(c);
        import_basic_dag(c, c->d_basic, words.size());
        color_release(c);
        clear_history(c);
        c->needs_gc = false;
    });
}

hd_status hd_save_basic_dag_file(hd_ctx* c, const char* path, const hd_dag_info* info)
{
    if (!c || !path)
        return HD_ERR_INVALID;
    if (!c->d_basic)
        return HD_ERR_STATE;
    return guarded(c, [&] {
        std::vector<uint32_t> words(c->n_basic);
        HD_CUDA(cudaMemcpyAsync(words.data(), c->d_basic, c->n_basic * 4, cudaMemcpyDeviceToHost, c->stream));
        HD_CUDA(cudaStreamSynchronize(c->stream));
        OutFile out(path);
        write_info(out, info);
        out.value<uint32_t>(c->cfg.depth);
        out.array(words.data(), words.size());
        out.close();
    });
}

hd_status hd_load_colors_file(hd_ctx* c, const char* path, uint32_t flags)
{
    if (!c || !path || (flags & ~uint32_t(HD_COLORS_ENCLOSED_32)))
        return HD_ERR_INVALID;
    return guarded(c, [&] {
        InFile in(path);
        const uint32_t top_levels = in.value<uint32_t>();
        std::vector<uint64_t> enclosed;
        if (flags & HD_COLORS_ENCLOSED_32)
            enclosed.assign(in.array<uint32_t>().size(), 0); // load_compressed_colors_from_file, :64-75
        else
            enclosed = in.array<uint64_t>();
        std::vector<uint32_t> weights = in.array<uint32_t>();
        for (uint32_t& w : weights) // ColorUtils::swap_byte_order (color_utils.h:85-105)
            w = (w >> 24) | ((w >> 8) & 0xFF00u) | ((w << 8) & 0xFF0000u) | (w << 24);
        const std::vector<uint64_t> blocks = in.array<uint64_t>();
        const std::vector<uint64_t> macros = in.array<uint64_t>();
        colors_from_main_leaf(c, top_levels, enclosed, weights, blocks, macros);
        clear_history(c);
    });
}

hd_status hd_save_snapshot(hd_ctx* c, const char* path, const hd_dag_info* info)
{
    if (!c || !path)
        return HD_ERR_INVALID;
    return guarded(c, [&] {
        cudaStream_t st = c->stream;
        const Geom& g = c->g;
        uint32_t pool_top = 0;
        HD_CUDA(cudaMemcpyAsync(&pool_top, c->t.pool_top, 4, cudaMemcpyDeviceToHost, st));
        HD_CUDA(cudaStreamSynchronize(st));
        std::vector<uint32_t> pool(uint64_t(pool_top) * kPage), pt(g.total_vpages), bs(g.total_buckets),
            full(c->cfg.depth);
        std::vector<uint64_t> level_nodes(HD_MAX_DEPTH);
        HD_CUDA(cudaMemcpyAsync(level_nodes.data(), c->t.level_nodes, HD_MAX_DEPTH * 8, cudaMemcpyDeviceToHost, st));
        HD_CUDA(cudaMemcpyAsync(pool.data(), c->t.pool, pool.size() * 4, cudaMemcpyDeviceToHost, st));
        HD_CUDA(cudaMemcpyAsync(pt.data(), c->t.page_table, pt.size() * 4, cudaMemcpyDeviceToHost, st));
        HD_CUDA(cudaMemcpyAsync(bs.data(), c->t.bucket_sizes, bs.size() * 4, cudaMemcpyDeviceToHost, st));
        HD_CUDA(cudaMemcpyAsync(full.data(), c->t.full_nodes, full.size() * 4, cudaMemcpyDeviceToHost, st));
        const uint64_t* tops = c->ctop;
        std::vector<uint32_t> nodes, weights;
        std::vector<LeafDesc> leaves;
        std::vector<uint64_t> blocks, macros;
        if (c->colors) {
            nodes.resize(tops[0]);
            leaves.resize(tops[1]);
            blocks.resize(tops[2]);
            macros.resize(tops[3]);
            weights.resize(tops[4]);
            if (tops[0])
                HD_CUDA(cudaMemcpyAsync(nodes.data(), c->ct.nodes, tops[0] * 4, cudaMemcpyDeviceToHost, st));
            if (tops[1])
                HD_CUDA(cudaMemcpyAsync(leaves.data(), c->ct.leaves, tops[1] * sizeof(LeafDesc),
                                        cudaMemcpyDeviceToHost, st));
            if (tops[2])
                HD_CUDA(cudaMemcpyAsync(blocks.data(), c->ct.blocks, tops[2] * 8, cudaMemcpyDeviceToHost, st));
            if (tops[3])
                HD_CUDA(cudaMemcpyAsync(macros.data(), c->ct.macros, tops[3] * 8, cudaMemcpyDeviceToHost, st));
            if (tops[4])
                HD_CUDA(cudaMemcpyAsync(weights.data(), c->ct.weights, tops[4] * 4, cudaMemcpyDeviceToHost, st));
        }
        HD_CUDA(cudaStreamSynchronize(st));
        OutFile out(path);
        // the reference's hash-DAG file
        write_info(out, info);
        out.value<uint32_t>(c->cfg.depth);
        out.value<uint32_t>(c->root);
        out.value<uint32_t>(c->cfg.pool_pages);
        out.value<uint32_t>(uint32_t(g.total_vpages));
        out.value<uint32_t>(pool_top);
        out.write(pool.data(), pool.size() * 4);
        out.write(pt.data(), pt.size() * 4);
        // the extension
        out.write(kSnapshotMagic, 8);
        out.value<uint32_t>(kSnapshotVersion);
        out.value<uint32_t>(c->colors ? 1u : 0u);
        out.value(c->cfg);
        out.array(bs.data(), bs.size());
        out.write(full.data(), full.size() * 4);
        out.write(level_nodes.data(), HD_MAX_DEPTH * 8);
        if (c->colors) {
            out.write(tops, 5 * 8);
            out.write(nodes.data(), nodes.size() * 4);
            out.write(leaves.data(), leaves.size() * sizeof(LeafDesc));
            out.write(blocks.data(), blocks.size() * 8);
            out.write(macros.data(), macros.size() * 8);
            out.write(weights.data(), weights.size() * 4);
        }
        out.close();
    });
}

hd_status hd_load_snapshot(hd_ctx* c, const char* path, hd_dag_info* info)
{
    if (!c || !path)
        return HD_ERR_INVALID;
    return guarded(c, [&] {
        cudaStream_t st = c->stream;
        const Geom& g = c->g;
        InFile in(path);
        read_info(in, info);
        check_levels(c, in.value<uint32_t>(), in.path);
        const uint32_t root = in.value<uint32_t>();
        in.value<uint32_t>(); // poolMaxSize: the writer's pool capacity
        const uint32_t pt_size = in.value<uint32_t>();
        const uint32_t pool_top = in.value<uint32_t>();
        if (pt_size != g.total_vpages)
            throw StatusError{HD_ERR_INVALID, in.path + " has a page table of " + std::to_string(pt_size) +
                                                  " pages; the context's geometry has " +
                                                  std::to_string(g.total_vpages)};
        if (pool_top < 1 || pool_top > g.pool_pages)
            throw StatusError{HD_ERR_INVALID, in.path + " uses " + std::to_string(pool_top) +
                                                  " pool pages; the context holds " + std::to_string(g.pool_pages)};
        if (uint64_t(pool_top) * kPage * 4 + uint64_t(pt_size) * 4 > in.left())
            throw StatusError{HD_ERR_IO, "short file " + in.path};
        std::vector<uint32_t> pool(uint64_t(pool_top) * kPage), pt(pt_size);
        in.read(pool.data(), pool.size() * 4);
        in.read(pt.data(), pt.size() * 4);
        std::vector<uint32_t> bs(g.total_buckets, 0), full(c->cfg.depth, 0);
        std::vector<uint64_t> level_nodes(HD_MAX_DEPTH, 0);
        bool extension = false, colors = false;
        uint64_t tops[5] = {0, 0, 0, 0, 0};
        std::vector<uint32_t> nodes, weights;
        std::vector<LeafDesc> leaves;
        std::vector<uint64_t> blocks, macros;
        if (in.left() > 0) {
            char magic[8];
            in.read(magic, 8);
            if (std::memcmp(magic, kSnapshotMagic, 8) != 0)
                throw StatusError{HD_ERR_INVALID, in.path + ": unknown data after the page table"};
            if (in.value<uint32_t>() != kSnapshotVersion)
                throw StatusError{HD_ERR_INVALID, in.path + ": unsupported snapshot version"};
            colors = (in.value<uint32_t>() & 1u) != 0;
            const hd_config cfg = in.value<hd_config>();
            if (cfg.depth != c->cfg.depth || cfg.color_tree_levels != c->cfg.color_tree_levels ||
                cfg.top_levels != c->cfg.top_levels || cfg.top_bucket_bits != c->cfg.top_bucket_bits ||
                cfg.low_bucket_bits != c->cfg.low_bucket_bits || cfg.top_bucket_size != c->cfg.top_bucket_size ||
                cfg.low_bucket_size != c->cfg.low_bucket_size)
                throw StatusError{HD_ERR_INVALID, in.path + " was written with another table geometry"};
            bs = in.array<uint32_t>();
            if (bs.size() != g.total_buckets)
                throw StatusError{HD_ERR_INVALID, in.path + ": bucket count differs"};
            in.read(full.data(), full.size() * 4);
            in.read(level_nodes.data(), HD_MAX_DEPTH * 8);
            if (colors) {
                in.read(tops, sizeof(tops));
                if (tops[0] * 4 + tops[1] * sizeof(LeafDesc) + tops[2] * 8 + tops[3] * 8 + tops[4] * 4 > in.left())
                    throw StatusError{HD_ERR_IO, "short file " + in.path};
                nodes.resize(tops[0]);
                leaves.resize(tops[1]);
                blocks.resize(tops[2]);
                macros.resize(tops[3]);
                weights.resize(tops[4]);
                in.read(nodes.data(), tops[0] * 4);
                in.read(leaves.data(), tops[1] * sizeof(LeafDesc));
                in.read(blocks.data(), tops[2] * 8);
                in.read(macros.data(), tops[3] * 8);
                in.read(weights.data(), tops[4] * 4);
            }
            extension = true;
        }
        check_table(g, pt.data(), extension ? bs.data() : nullptr, pool_top, root, in.path);
        table_reset(c);
        HD_CUDA(cudaMemcpyAsync(c->t.pool, pool.data(), pool.size() * 4, cudaMemcpyHostToDevice, st));
        HD_CUDA(cudaMemcpyAsync(c->t.page_table, pt.data(), pt.size() * 4, cudaMemcpyHostToDevice, st));
        HD_CUDA(cudaMemcpyAsync(c->t.bucket_sizes, bs.data(), bs.size() * 4, cudaMemcpyHostToDevice, st));
        HD_CUDA(cudaMemcpyAsync(c->t.full_nodes, full.data(), full.size() * 4, cudaMemcpyHostToDevice, st));
        HD_CUDA(cudaMemcpyAsync(c->t.level_nodes, level_nodes.data(), HD_MAX_DEPTH * 8, cudaMemcpyHostToDevice, st));
        const uint32_t top[2] = {pool_top, 0};
        HD_CUDA(cudaMemcpyAsync(c->t.pool_top, top, 8, cudaMemcpyHostToDevice, st));
        HD_CUDA(cudaMemcpyAsync(c->d_root, &root, 4, cudaMemcpyHostToDevice, st));
        bloom_rebuild(c);
        color_release(c);
        if (colors) {
            const uint64_t add[5] = {tops[0], tops[1], tops[2], tops[3], tops[4]};
            color_reserve(c, add);
            if (tops[0])
                HD_CUDA(cudaMemcpyAsync(c->ct.nodes, nodes.data(), tops[0] * 4, cudaMemcpyHostToDevice, st));
            if (tops[1])
                HD_CUDA(cudaMemcpyAsync(c->ct.leaves, leaves.data(), tops[1] * sizeof(LeafDesc),
                                        cudaMemcpyHostToDevice, st));
            if (tops[2])
                HD_CUDA(cudaMemcpyAsync(c->ct.blocks, blocks.data(), tops[2] * 8, cudaMemcpyHostToDevice, st));
            if (tops[3])
                HD_CUDA(cudaMemcpyAsync(c->ct.macros, macros.data(), tops[3] * 8, cudaMemcpyHostToDevice, st));
            if (tops[4])
                HD_CUDA(cudaMemcpyAsync(c->ct.weights, weights.data(), tops[4] * 4, cudaMemcpyHostToDevice, st));
            HD_CUDA(cudaMemcpyAsync(c->ct.top, tops, sizeof(tops), cudaMemcpyHostToDevice, st));
            for (int k = 0; k < 5; k++)
                c->ctop[k] = tops[k];
            c->colors = true;
        }
        HD_CUDA(cudaStreamSynchronize(st));
        c->root = root;
        c->needs_gc = !extension;
        clear_history(c);
    });
}

} // extern "C"
