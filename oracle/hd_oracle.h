/*
 * ORACLE — test infrastructure only.  A plain-C restatement of the
 * reference's (Phyronnaz/HashDAG) hashed-DAG hot path, used by tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline leg as the checker.
 * The product (hashdag_gb300/) never links or calls it.
 *
 * Parity pin: tests/golden/ holds outputs of the reference's own code built
 * from its sources (oracle/refharness, oracle/_ref) on the same seeded
 * scenes; tests/test_oracle_golden.py checks this restatement against them.
 * Floating point follows IEEE single/double with every operation rounded on
 * its own (build with -ffp-contract=off), except where fp_mode = 1 asks for
 * the explicit fused multiply-adds listed at each site.
 */
#ifndef HD_ORACLE_H
#define HD_ORACLE_H

#include <stdint.h>
#include "../include/hashdag_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_table or_table;

/* ---- geometry / hashes (hash_table.h:19-89, utils.h:355-396) ---------- */
uint32_t or_make_ptr(const hd_config* cfg, uint32_t level, uint32_t bucket, uint32_t pos);
uint32_t or_hash_leaf(uint64_t leaf);
uint32_t or_hash_interior(uint32_t n, const uint32_t* node);
uint32_t or_murmurhash32(uint32_t h);
uint64_t or_murmurhash64(uint64_t h);
uint64_t or_total_buckets(const hd_config* cfg);
uint64_t or_total_virtual_pages(const hd_config* cfg);

/* ---- table (hash_table.h / hash_table.cpp) ----------------------------- */
or_table* or_table_create(const hd_config* cfg);
void or_table_destroy(or_table* t);
int or_table_error(const or_table* t);          /* hd_status of the first failure */
uint32_t or_table_root(const or_table* t);
void or_table_set_root(or_table* t, uint32_t root);
const uint32_t* or_table_full_nodes(const or_table* t);
uint32_t or_table_pool_top(const or_table* t);  /* poolTop: pages used + 1 */
void or_table_export(const or_table* t, uint32_t* bucket_sizes, uint32_t* page_table,
                     uint32_t* pool, uint64_t pool_words_capacity, uint32_t* full_nodes);
int or_table_import(or_table* t, const uint32_t* bucket_sizes, const uint32_t* page_table,
                    const uint32_t* pool, uint64_t pool_words, const uint32_t* full_nodes,
                    uint32_t root);
void or_level_stats(const or_table* t, hd_level_stats* out);
uint32_t or_find_or_add_leaf(or_table* t, uint64_t leaf);
uint32_t or_find_or_add_interior(or_table* t, uint32_t level, uint32_t n, const uint32_t* node);
uint32_t or_read_word(const or_table* t, uint32_t vptr);

/* ---- scene generator (own seeded format) ------------------------------ */
int32_t or_scene_height(uint64_t seed, uint32_t depth, uint32_t x, uint32_t z);
void or_scene_spheres(uint64_t seed, uint32_t depth, int64_t* out /* 64 x 4: cx cy cz r */);
int or_scene_solid(uint64_t seed, uint32_t depth, uint32_t x, uint32_t y, uint32_t z);
/* shell scene: solid voxels with an empty face neighbour (outside = empty) */
int or_scene_shell(uint64_t seed, uint32_t depth, uint32_t x, uint32_t y, uint32_t z);
/* Builds the BasicDAG words of the scene; returns malloc'd words. */
uint32_t* or_generate_basic_dag(uint64_t seed, uint32_t depth, uint32_t color_tree_levels,
                                uint64_t* n_words);
/* flags: HD_SCENE_SHELL keeps only the surface shell of the solid scene */
uint32_t* or_generate_basic_dag_ex(uint64_t seed, uint32_t depth, uint32_t color_tree_levels, uint32_t flags,
                                   uint64_t* n_words);
/* the same words, built by `threads` threads (0: every online core) */
uint32_t* or_generate_basic_dag_mt(uint64_t seed, uint32_t depth, uint32_t color_tree_levels, uint32_t flags,
                                   uint32_t threads, uint64_t* n_words);
void or_free(void* p);

/* ---- ingest: HashDAGFactory::load_from_DAG ---------------------------- */
int or_load_basic_dag(or_table* t, const uint32_t* words, uint64_t n_words);

/* ---- queries ----------------------------------------------------------- */
int or_get_value(const or_table* t, uint32_t x, uint32_t y, uint32_t z);
/* Pointer-independent fingerprint of the volume under the root: every node
 * hashed from its child mask (and leaf words) and its children's
 * fingerprints, headers' count bits ignored. */
uint64_t or_occupancy_fingerprint(const or_table* t, uint32_t root);
/* Distinct node addresses reachable from root, per level. */
void or_reachable_counts(const or_table* t, uint32_t root, uint64_t* out);
void or_reachable_words(const or_table* t, uint32_t root, uint64_t* out, uint64_t* words);

/* ---- traversal (tracer.cu) -------------------------------------------- */
void or_trace_primary(const or_table* t, const hd_camera* cam, uint32_t width, uint32_t height,
                      uint32_t fp_mode, uint32_t* paths, uint32_t row0, uint32_t row1,
                      uint64_t* node_visits);
void or_trace_shadow(const or_table* t, const hd_camera* cam, uint32_t width, uint32_t height,
                     uint32_t fp_mode, const uint32_t* paths, const float light[3], float bias,
                     uint8_t* mask, uint32_t row0, uint32_t row1, uint64_t* node_visits);
/* Multi-threaded frame (primary then shadow) with n_threads POSIX threads. */
void or_trace_frame_mt(const or_table* t, const hd_camera* cam, uint32_t width, uint32_t height,
                       uint32_t fp_mode, const float light[3], float bias, uint32_t* paths,
                       uint8_t* mask, uint32_t n_threads, uint32_t row0, uint32_t row1);

/* ---- edits (hash_dag_edits.h) and GC (hash_dag.h:407-547) ------------- */
int or_edit(or_table* t, const hd_edit* edit, hd_edit_stats* stats);
/* edit_threads with THREADED_EDITS: level-T tasks on `threads` threads (0:
   every core); same voxels as or_edit, node order may differ */
int or_edit_mt(or_table* t, const hd_edit* edit, hd_edit_stats* stats, uint32_t threads);
int or_gc(or_table* t, uint32_t* extra_roots, uint32_t n_extra);
/* ---- colours (variable_weight_size_colors.h, hash_dag_colors.h) ------- */
typedef struct or_colors or_colors;
or_colors* or_colors_create(void);
void or_colors_destroy(or_colors* c);
/* colour tree + one leaf per level-T slot from the scene's colour field */
int or_colors_from_scene(or_colors* c, const or_table* t, uint64_t color_seed);
/* the same colours, leaves built by `threads` threads (0: every core) */
int or_colors_from_scene_mt(or_colors* col, const or_table* t, uint64_t color_seed, uint32_t threads);
hd_color or_get_color(const or_table* t, const or_colors* c, uint32_t x, uint32_t y, uint32_t z);
/* every tool incl. paint and copy; records an undo frame */
int or_edit_colored(or_table* t, or_colors* c, const hd_edit* e, hd_edit_stats* stats);
int or_undo(or_table* t, or_colors* c); /* 1 if a frame was applied */
int or_redo(or_table* t, or_colors* c);
void or_colors_stats(const or_colors* c, uint64_t* out);
/* Tracer::trace_colors of a paths image (uint4 per pixel) */
void or_trace_colors(const or_table* t, const or_colors* c, const uint32_t* paths, uint64_t n,
                     const hd_trace_colors_params* params, uint32_t* rgba);
/* FastNoise's GetPerlinFractal (FBM, quintic, lacunarity 2, gain 0.5) */
float or_perlin_fractal(int seed, float frequency, int octaves, float x, float y, float z);
/* The BasicDAGCompressedColors shipped beside a BasicDAG (enclosedLeaves and
 * one main leaf for the colour field of `seed`); arrays malloc'd, or_free. */
int or_main_leaf(const uint32_t* words, uint64_t n_words, uint32_t depth, uint32_t top_levels, uint64_t seed,
                 uint64_t** enclosed, uint64_t* n_enclosed, uint64_t** blocks, uint64_t* nb, uint64_t** macros,
                 uint64_t* nm, uint32_t** weights, uint64_t* nw);
uint32_t or_color_rgb8(uint64_t seed, uint32_t x, uint32_t y, uint32_t z);
hd_color or_voxel_color(uint64_t seed, uint32_t x, uint32_t y, uint32_t z);
uint32_t or_color_rgb888(hd_color k);
uint32_t or_f3_to_rgb888(float x, float y, float z);

/* Debugging aid: log every find_or_add call (level, content, result). */
void or_set_foa_log(const char* path);

#ifdef __cplusplus
}
#endif
#endif
