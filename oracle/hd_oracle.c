/*
 * ORACLE — test infrastructure only (see hd_oracle.h).  Plain-C restatement
 * of the reference's hashed-DAG hot path; every function cites the
 * reference file:line it follows.  Build: oracle/build_oracle.py
 * (gcc -O2 -ffp-contract=off -fno-fast-math).
 */
#include "hd_oracle.h"

#include <math.h>
#include <stdio.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define PAGE HD_PAGE_SIZE
#define NOT_FOUND 0xFFFFFFFFu
#define INVALID HD_INVALID_NODE

/* ======================================================================
 * Geometry (hash_table.h:19-77, hash_dag_globals.h:10-30)
 * ====================================================================== */

static uint32_t bucket_count(const hd_config* c, uint32_t level)
{
    return level < c->top_levels ? (1u << c->top_bucket_bits) : (1u << c->low_bucket_bits);
}
static uint32_t bucket_capacity(const hd_config* c, uint32_t level)
{
    return level < c->top_levels ? c->top_bucket_size : c->low_bucket_size;
}
static uint32_t n_top(const hd_config* c)
{
    return c->top_levels < c->depth ? c->top_levels : c->depth;
}
/* get_bucket_global_index (hash_table.h:19-36) */
static uint32_t bucket_global(const hd_config* c, uint32_t level, uint32_t bucket)
{
    if (level < c->top_levels)
        return level * (1u << c->top_bucket_bits) + bucket;
    return n_top(c) * (1u << c->top_bucket_bits) + (level - c->top_levels) * (1u << c->low_bucket_bits) + bucket;
}
/* make_ptr (hash_table.h:45-63) */
uint32_t or_make_ptr(const hd_config* c, uint32_t level, uint32_t bucket, uint32_t pos)
{
    uint64_t index;
    if (level < c->top_levels)
        index = ((uint64_t)level * (1u << c->top_bucket_bits) + bucket) * c->top_bucket_size;
    else
        index = (uint64_t)n_top(c) * (1u << c->top_bucket_bits) * c->top_bucket_size +
                ((uint64_t)(level - c->top_levels) * (1u << c->low_bucket_bits) + bucket) * c->low_bucket_size;
    return (uint32_t)(index + pos);
}
uint64_t or_total_buckets(const hd_config* c)
{
    uint64_t low = c->depth > c->top_levels ? c->depth - c->top_levels : 0;
    return (uint64_t)n_top(c) * (1u << c->top_bucket_bits) + low * (1u << c->low_bucket_bits);
}
uint64_t or_total_virtual_pages(const hd_config* c)
{
    uint64_t low = c->depth > c->top_levels ? c->depth - c->top_levels : 0;
    return ((uint64_t)n_top(c) * (1u << c->top_bucket_bits) * c->top_bucket_size +
            low * (1u << c->low_bucket_bits) * c->low_bucket_size) / PAGE;
}

/* ======================================================================
 * Hashes (utils.h:355-396, hash_table.h:80-89)
 * ====================================================================== */

uint32_t or_murmurhash32(uint32_t h)
{
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}
uint64_t or_murmurhash64(uint64_t h)
{
    h ^= h >> 33;
    h *= 0xff51afd7ed558ccdull;
    h ^= h >> 33;
    h *= 0xc4ceb9fe1a85ec53ull;
    h ^= h >> 33;
    return h;
}
/* murmurhash32xN with seed 0 (utils.h:375-396, USE_ALTERNATE_HASH) */
static uint32_t murmurhash32xN(const uint32_t* ph, uint32_t n)
{
    uint32_t h = 0;
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t k = ph[i];
        k *= 0xcc9e2d51u;
        k = (k << 15) | (k >> 17);
        k *= 0x1b873593u;
        h ^= k;
        h = (h << 13) | (h >> 19);
        h = h * 5u + 0xe6546b64u;
    }
    h ^= n;
    return or_murmurhash32(h);
}
uint32_t or_hash_leaf(uint64_t leaf) { return (uint32_t)or_murmurhash64(leaf); }
uint32_t or_hash_interior(uint32_t n, const uint32_t* node) { return murmurhash32xN(node, n); }

static uint32_t popc32(uint32_t v) { return (uint32_t)__builtin_popcount(v); }
static uint32_t popc64(uint64_t v) { return (uint32_t)__builtin_popcountll(v); }
/* Utils::total_size / child_offset (utils.h:343-354) */
static uint32_t total_size(uint32_t header) { return popc32(header & 0xffu) + 1; }
static uint32_t child_offset(uint32_t mask, uint32_t child) { return popc32(mask & ((1u << child) - 1u)) + 1; }

/* ======================================================================
 * Paged hash table (hash_table.h:137-898, hash_table.cpp)
 * ====================================================================== */

struct or_table {
    hd_config cfg;
    uint32_t leaf_level;
    uint32_t* pool;        /* pool_pages * PAGE words (physical)            */
    uint32_t* page_table;  /* virtual page -> physical page (0 = unmapped)  */
    uint32_t* bucket_sizes;
    uint64_t n_buckets, n_vpages;
    uint32_t pool_top;     /* poolTop (hash_table.h:818): starts at 1       */
    uint32_t full[HD_MAX_DEPTH];
    uint64_t level_nodes[HD_MAX_DEPTH];
    uint32_t root;
    int error;
    /* find-or-add counters of the current edit */
    uint64_t foa_calls, nodes_added, words_scanned;
    /* or_edit_mt: one lock byte per bucket while edit tasks run on several
       threads (NULL otherwise) */
    uint8_t* locks;
};

/* Counters and poolTop are shared by the threads of or_edit_mt: relaxed
   atomic adds (uncontended on one thread). */
static void cnt_add(uint64_t* p, uint64_t v) { __atomic_fetch_add(p, v, __ATOMIC_RELAXED); }

static uint64_t unique_sorted(uint32_t* v, uint64_t n);

static void set_error(or_table* t, int e)
{
    int none = 0;
    __atomic_compare_exchange_n(&t->error, &none, e, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED);
}

or_table* or_table_create(const hd_config* cfg)
{
    if (!cfg || cfg->depth < 4 || cfg->depth > HD_MAX_DEPTH || cfg->color_tree_levels > cfg->depth - 2)
        return NULL;
    or_table* t = (or_table*)calloc(1, sizeof(or_table));
    t->cfg = *cfg;
    t->leaf_level = cfg->depth - 2;
    t->n_buckets = or_total_buckets(cfg);
    t->n_vpages = or_total_virtual_pages(cfg);
    t->pool = (uint32_t*)calloc((size_t)cfg->pool_pages * PAGE, sizeof(uint32_t));
    t->page_table = (uint32_t*)calloc(t->n_vpages, sizeof(uint32_t));
    t->bucket_sizes = (uint32_t*)calloc(t->n_buckets, sizeof(uint32_t));
    t->pool_top = 1;
    if (!t->pool || !t->page_table || !t->bucket_sizes) {
        or_table_destroy(t);
        return NULL;
    }
    return t;
}
void or_table_destroy(or_table* t)
{
    if (!t)
        return;
    free(t->pool);
    free(t->page_table);
    free(t->bucket_sizes);
    free(t);
}
int or_table_error(const or_table* t) { return t->error; }
uint32_t or_table_root(const or_table* t) { return t->root; }
void or_table_set_root(or_table* t, uint32_t root) { t->root = root; }
const uint32_t* or_table_full_nodes(const or_table* t) { return t->full; }
uint32_t or_table_pool_top(const or_table* t) { return t->pool_top; }

/* get_sys_ptr (hash_table.h:155-173) */
static uint32_t* sys_ptr(const or_table* t, uint32_t vptr)
{
    uint32_t phys = t->page_table[vptr / PAGE];
    return t->pool + (uint64_t)phys * PAGE + (vptr % PAGE);
}
uint32_t or_read_word(const or_table* t, uint32_t vptr) { return *sys_ptr(t, vptr); }

/* allocate_page (hash_table.h:794-809) */
static void allocate_page(or_table* t, uint32_t page)
{
    const uint32_t p = __atomic_fetch_add(&t->pool_top, 1u, __ATOMIC_RELAXED);
    if (p >= t->cfg.pool_pages) {
        __atomic_fetch_sub(&t->pool_top, 1u, __ATOMIC_RELAXED);
        set_error(t, HD_ERR_POOL_FULL);
        return;
    }
    t->page_table[page] = p;
}

/* find_leaf_node_in_bucket (hash_table.h:196-274), Bloom filter off */
static uint32_t find_leaf(or_table* t, uint32_t bucket_size, uint32_t bucket, uint64_t leaf)
{
    const uint32_t level = t->leaf_level;
    const uint32_t base = or_make_ptr(&t->cfg, level, bucket, 0);
    for (uint32_t pindex = 0; pindex < bucket_size; pindex += PAGE) {
        const uint32_t* p = sys_ptr(t, base + pindex);
        uint32_t end = bucket_size < pindex + PAGE ? bucket_size : pindex + PAGE;
        for (uint32_t index = pindex; index < end; index += 2, p += 2) {
            uint64_t bits = (uint64_t)p[0] | ((uint64_t)p[1] << 32);
            if (bits == leaf) {
                cnt_add(&t->words_scanned, index + 2);
                return base + index;
            }
        }
    }
    cnt_add(&t->words_scanned, bucket_size);
    return NOT_FOUND;
}

/* find_interior_node_in_bucket (hash_table.h:276-357).  Note the two
 * boundary rules kept as written: the scan returns "not found" as soon as a
 * page holds no more than n used words, and a node is only compared while
 * index < pageEnd - n, so a node flush with the bucket tail or the page end
 * is never found by a query of its own size. */
static uint32_t find_interior(or_table* t, uint32_t bucket_size, uint32_t level, uint32_t bucket,
                              uint32_t n, const uint32_t* node)
{
    const uint32_t base = or_make_ptr(&t->cfg, level, bucket, 0);
    for (uint32_t pindex = 0; pindex < bucket_size; pindex += PAGE) {
        const uint32_t* page = sys_ptr(t, base + pindex);
        uint32_t page_end = bucket_size < pindex + PAGE ? bucket_size : pindex + PAGE;
        if (pindex + n >= page_end) {
            cnt_add(&t->words_scanned, bucket_size);
            return NOT_FOUND;
        }
        page_end -= n;
        for (uint32_t index = pindex; index < page_end;) {
            const uint32_t* p = page + (index - pindex);
            if (memcmp(node, p, n * sizeof(uint32_t)) == 0) {
                cnt_add(&t->words_scanned, index + n);
                return base + index;
            }
            index += total_size(*p);
        }
    }
    cnt_add(&t->words_scanned, bucket_size);
    return NOT_FOUND;
}

/* add_leaf_node (hash_table.h:359-400) */
static uint32_t add_leaf(or_table* t, uint64_t leaf, uint32_t hash)
{
    const uint32_t level = t->leaf_level;
    const uint32_t bucket = hash & (bucket_count(&t->cfg, level) - 1);
    uint32_t* size_ptr = &t->bucket_sizes[bucket_global(&t->cfg, level, bucket)];
    const uint32_t size = *size_ptr;
    if (size + 2 > bucket_capacity(&t->cfg, level)) {
        set_error(t, HD_ERR_BUCKET_FULL);
        return INVALID;
    }
    const uint32_t ptr = or_make_ptr(&t->cfg, level, bucket, size);
    const uint32_t page = ptr / PAGE;
    if (size % PAGE == 0 && t->page_table[page] == 0)
        allocate_page(t, page);
    if (t->error)
        return INVALID;
    uint32_t* p = sys_ptr(t, ptr);
    p[0] = (uint32_t)leaf;
    p[1] = (uint32_t)(leaf >> 32);
    *size_ptr = size + 2;
    cnt_add(&t->level_nodes[level], 1);
    cnt_add(&t->nodes_added, 1);
    return ptr;
}

/* add_interior_node (hash_table.h:401-468): a node never straddles a page;
 * the rest of the page is skipped as padding. */
static uint32_t add_interior(or_table* t, uint32_t level, uint32_t n, const uint32_t* node, uint32_t hash)
{
    const uint32_t bucket = hash & (bucket_count(&t->cfg, level) - 1);
    uint32_t* size_ptr = &t->bucket_sizes[bucket_global(&t->cfg, level, bucket)];
    uint32_t size = *size_ptr;
    const uint32_t left = PAGE - (size % PAGE);
    uint32_t ptr;
    if (left == PAGE || left < n) {
        if (left != PAGE)
            size += left;
        if (size + n > bucket_capacity(&t->cfg, level)) {
            set_error(t, HD_ERR_BUCKET_FULL);
            return INVALID;
        }
        ptr = or_make_ptr(&t->cfg, level, bucket, size);
        if (t->page_table[ptr / PAGE] == 0)
            allocate_page(t, ptr / PAGE);
    } else {
        if (size + n > bucket_capacity(&t->cfg, level)) {
            set_error(t, HD_ERR_BUCKET_FULL);
            return INVALID;
        }
        ptr = or_make_ptr(&t->cfg, level, bucket, size);
    }
    if (t->error)
        return INVALID;
    uint32_t* p = sys_ptr(t, ptr);
    for (uint32_t i = 0; i < n; i++)
        p[i] = node[i];
    *size_ptr = size + n;
    cnt_add(&t->level_nodes[level], 1);
    cnt_add(&t->nodes_added, 1);
    return ptr;
}

/* Optional call log of find_or_add (level, 9 content words, result), for
 * debugging comparisons. */
static FILE* g_foa_log = NULL;
void or_set_foa_log(const char* path)
{
    if (g_foa_log)
        fclose(g_foa_log);
    g_foa_log = path ? fopen(path, "wb") : NULL;
}
static void log_foa(uint32_t level, uint32_t n, const uint32_t* node, uint32_t result)
{
    if (!g_foa_log)
        return;
    uint32_t rec[11] = {level};
    for (uint32_t i = 0; i < n && i < 9; i++)
        rec[1 + i] = node[i];
    rec[10] = result;
    fwrite(rec, 4, 11, g_foa_log);
}

/* find_or_add_leaf_node (hash_table.h:470-514), single writer */
static void bucket_lock(or_table* t, uint64_t gb)
{
    if (t->locks)
        while (__atomic_test_and_set(t->locks + gb, __ATOMIC_ACQUIRE))
            ;
}
static void bucket_unlock(or_table* t, uint64_t gb)
{
    if (t->locks)
        __atomic_clear(t->locks + gb, __ATOMIC_RELEASE);
}

uint32_t or_find_or_add_leaf(or_table* t, uint64_t leaf)
{
    const uint32_t level = t->leaf_level;
    const uint32_t hash = or_hash_leaf(leaf);
    const uint32_t bucket = hash & (bucket_count(&t->cfg, level) - 1);
    const uint64_t gb = bucket_global(&t->cfg, level, bucket);
    bucket_lock(t, gb);
    const uint32_t size = t->bucket_sizes[gb];
    cnt_add(&t->foa_calls, 1);
    uint32_t r = find_leaf(t, size, bucket, leaf);
    if (r == NOT_FOUND)
        r = add_leaf(t, leaf, hash);
    bucket_unlock(t, gb);
    const uint32_t words[2] = {(uint32_t)leaf, (uint32_t)(leaf >> 32)};
    log_foa(level, 2, words, r);
    return r;
}
/* find_or_add_interior_node (hash_table.h:515-560), single writer */
uint32_t or_find_or_add_interior(or_table* t, uint32_t level, uint32_t n, const uint32_t* node)
{
    const uint32_t hash = or_hash_interior(n, node);
    const uint32_t bucket = hash & (bucket_count(&t->cfg, level) - 1);
    const uint64_t gb = bucket_global(&t->cfg, level, bucket);
    bucket_lock(t, gb);
    const uint32_t size = t->bucket_sizes[gb];
    cnt_add(&t->foa_calls, 1);
    uint32_t r = find_interior(t, size, level, bucket, n, node);
    if (r == NOT_FOUND)
        r = add_interior(t, level, n, node, hash);
    bucket_unlock(t, gb);
    log_foa(level, n, node, r);
    return r;
}

/* add_full_node (hash_table.h:749-789) */
static void add_full_node(or_table* t, uint32_t level)
{
    if (level == t->leaf_level) {
        const uint64_t leaf = ~0ull;
        t->full[level] = add_leaf(t, leaf, or_hash_leaf(leaf));
    } else {
        const uint32_t depth = t->cfg.depth - level;
        const uint32_t voxels = level < t->cfg.color_tree_levels ? 0u : (1u << (3 * depth));
        uint32_t node[9];
        node[0] = (voxels << 8) | 0xffu;
        for (uint32_t c = 0; c < 8; c++)
            node[1 + c] = t->full[level + 1];
        t->full[level] = add_interior(t, level, 9, node, or_hash_interior(9, node));
    }
}

void or_table_export(const or_table* t, uint32_t* bucket_sizes, uint32_t* page_table, uint32_t* pool,
                     uint64_t pool_words_capacity, uint32_t* full_nodes)
{
    if (bucket_sizes)
        memcpy(bucket_sizes, t->bucket_sizes, t->n_buckets * sizeof(uint32_t));
    if (page_table)
        memcpy(page_table, t->page_table, t->n_vpages * sizeof(uint32_t));
    if (pool) {
        uint64_t words = (uint64_t)t->pool_top * PAGE;
        if (words > pool_words_capacity)
            words = pool_words_capacity;
        memcpy(pool, t->pool, words * sizeof(uint32_t));
    }
    if (full_nodes)
        memcpy(full_nodes, t->full, t->cfg.depth * sizeof(uint32_t));
}

int or_table_import(or_table* t, const uint32_t* bucket_sizes, const uint32_t* page_table, const uint32_t* pool,
                    uint64_t pool_words, const uint32_t* full_nodes, uint32_t root)
{
    if (pool_words > (uint64_t)t->cfg.pool_pages * PAGE || pool_words % PAGE)
        return HD_ERR_INVALID;
    memcpy(t->bucket_sizes, bucket_sizes, t->n_buckets * sizeof(uint32_t));
    memcpy(t->page_table, page_table, t->n_vpages * sizeof(uint32_t));
    memset(t->pool, 0, (size_t)t->cfg.pool_pages * PAGE * sizeof(uint32_t));
    memcpy(t->pool, pool, pool_words * sizeof(uint32_t));
    memcpy(t->full, full_nodes, t->cfg.depth * sizeof(uint32_t));
    t->pool_top = (uint32_t)(pool_words / PAGE);
    t->root = root;
    /* node counts are not part of the reference's table: recount by walks */
    for (uint32_t level = 0; level < t->cfg.depth - 1; level++) {
        uint64_t count = 0;
        for (uint32_t b = 0; b < bucket_count(&t->cfg, level); b++) {
            uint32_t size = t->bucket_sizes[bucket_global(&t->cfg, level, b)];
            if (level == t->leaf_level) {
                count += size / 2;
                continue;
            }
            uint32_t base = or_make_ptr(&t->cfg, level, b, 0);
            for (uint32_t pindex = 0; pindex < size; pindex += PAGE) {
                uint32_t end = size < pindex + PAGE ? size : pindex + PAGE;
                uint32_t i = pindex;
                while (i < end) {
                    uint32_t h = *sys_ptr(t, base + i);
                    if ((h & 0xffu) == 0)
                        break; /* zero padding to the page end */
                    i += total_size(h);
                    count++;
                }
            }
        }
        t->level_nodes[level] = count;
    }
    return HD_OK;
}

void or_level_stats(const or_table* t, hd_level_stats* out)
{
    memset(out, 0, sizeof(*out));
    for (uint32_t level = 0; level < t->cfg.depth - 1; level++) {
        uint64_t words = 0;
        for (uint32_t b = 0; b < bucket_count(&t->cfg, level); b++)
            words += t->bucket_sizes[bucket_global(&t->cfg, level, b)];
        out->words[level] = words;
        out->nodes[level] = t->level_nodes[level];
    }
    out->pages_used = t->pool_top - 1;
    out->root = t->root;
    out->levels = t->cfg.depth;
}

/* ======================================================================
 * Seeded scene generator (own format; identical integer arithmetic on the
 * device in hashdag_gb300/csrc/hd_scene.cu).
 *   height(x, z) = E/2 + floor(E/4 * fbm(x, z) / 1.9375), fbm = 5 octaves of
 *   value noise (lattice period E/4 >> o, amplitude 2^-o, smoothstep
 *   interpolation), all in Q16 fixed point;  solid = {y <= height} united
 *   with 64 spheres (centres uniform in [0, E)^3, radius uniform in [8, 64]).
 * ====================================================================== */

static uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static int64_t lattice(uint64_t seed, uint32_t octave, uint32_t i, uint32_t j)
{
    uint64_t k = mix64(seed ^ mix64(((uint64_t)octave << 58) ^ ((uint64_t)i << 29) ^ (uint64_t)j));
    return (int64_t)(k >> 47) - 65536;
}
static int64_t smooth_q16(int64_t t) { return (t * t * (3 * 65536 - 2 * t)) >> 32; }
static int64_t floor_div(int64_t a, int64_t b)
{
    int64_t q = a / b;
    if ((a % b) != 0 && a < 0)
        q -= 1;
    return q;
}
int32_t or_scene_height(uint64_t seed, uint32_t depth, uint32_t x, uint32_t z)
{
    int64_t total = 0;
    for (uint32_t o = 0; o < 5; o++) {
        const uint32_t lp = depth - 2 - o; /* log2 of the lattice period */
        const uint32_t i = x >> lp, j = z >> lp;
        const uint32_t fx = x & ((1u << lp) - 1), fz = z & ((1u << lp) - 1);
        const int64_t sx = smooth_q16((int64_t)(((uint64_t)fx << 16) >> lp));
        const int64_t sz = smooth_q16((int64_t)(((uint64_t)fz << 16) >> lp));
        const int64_t v00 = lattice(seed, o, i, j), v10 = lattice(seed, o, i + 1, j);
        const int64_t v01 = lattice(seed, o, i, j + 1), v11 = lattice(seed, o, i + 1, j + 1);
        const int64_t a = v00 + (((v10 - v00) * sx) >> 16);
        const int64_t b = v01 + (((v11 - v01) * sx) >> 16);
        const int64_t n = a + (((b - a) * sz) >> 16);
        total += n >> o;
    }
    const int64_t e = (int64_t)1 << depth;
    return (int32_t)((e >> 1) + floor_div(total * e, 31 * 16384));
}
void or_scene_spheres(uint64_t seed, uint32_t depth, int64_t* out)
{
    uint64_t state = seed ^ 0x5EED5EED12345678ull;
    const uint64_t mask = ((uint64_t)1 << depth) - 1;
    for (int s = 0; s < 64; s++) {
        state += 0x9E3779B97F4A7C15ull;
        out[4 * s + 0] = (int64_t)(mix64(state) & mask);
        state += 0x9E3779B97F4A7C15ull;
        out[4 * s + 1] = (int64_t)(mix64(state) & mask);
        state += 0x9E3779B97F4A7C15ull;
        out[4 * s + 2] = (int64_t)(mix64(state) & mask);
        state += 0x9E3779B97F4A7C15ull;
        out[4 * s + 3] = 8 + (int64_t)(mix64(state) % 57);
    }
}
static int in_sphere(const int64_t* s, int64_t x, int64_t y, int64_t z)
{
    int64_t dx = x - s[0], dy = y - s[1], dz = z - s[2];
    return dx * dx + dy * dy + dz * dz <= s[3] * s[3];
}
int or_scene_solid(uint64_t seed, uint32_t depth, uint32_t x, uint32_t y, uint32_t z)
{
    if ((int64_t)y <= or_scene_height(seed, depth, x, z))
        return 1;
    int64_t sp[256];
    or_scene_spheres(seed, depth, sp);
    for (int s = 0; s < 64; s++)
        if (in_sphere(sp + 4 * s, x, y, z))
            return 1;
    return 0;
}

/* --- BasicDAG construction: top-down classification, bottom-up dedup --- */

typedef struct {
    uint64_t* keys;   /* per entry: content hash                      */
    uint32_t* ids;    /* entry -> node id + 1 (0 = empty slot)        */
    uint64_t cap;
} dedup_map;

typedef struct {
    /* per node: mask, count, first child slot in `kids` (interior) or the
     * 64-bit leaf mask */
    uint64_t n, cap;
    uint8_t* mask;
    uint64_t* count;
    uint64_t* leaf;
    uint32_t* kid0;
    uint32_t* kids;
    uint64_t nkids, capkids;
    dedup_map map;
} gen_level;

typedef struct {
    uint64_t seed;
    uint32_t depth, leaf_level, T;
    int shell; /* keep only solid voxels with an empty face neighbour */
    int32_t* hmin[HD_MAX_DEPTH]; /* min/max of the height over each node footprint, per level */
    int32_t* hmax[HD_MAX_DEPTH];
    int64_t spheres[256];
    gen_level lv[HD_MAX_DEPTH];
    uint32_t full_id[HD_MAX_DEPTH];
    /* threaded builds: the level whose nodes come from finished subtree
     * tasks (-1: none), their node ids and counts in visit order */
    int32_t task_level;
    const uint32_t* task_id;
    const uint64_t* task_count;
    uint64_t task_next;
} gen_ctx;

#define GEN_EMPTY 0xFFFFFFFFu

static void map_grow(dedup_map* m, gen_level* L, int is_leaf);

static uint64_t node_key(const gen_level* L, uint32_t id, int is_leaf)
{
    if (is_leaf)
        return mix64(L->leaf[id] ^ 0x1EAF1EAF1EAF1EAFull);
    uint64_t h = mix64(L->mask[id]);
    uint32_t nk = popc32(L->mask[id]);
    for (uint32_t k = 0; k < nk; k++)
        h = mix64(h ^ L->kids[L->kid0[id] + k]);
    return h;
}

static uint32_t level_insert(gen_level* L, int is_leaf, uint8_t mask, uint64_t count, uint64_t leaf,
                             const uint32_t* kids)
{
    /* tentatively append, then dedup */
    if (L->n == L->cap) {
        L->cap = L->cap ? 2 * L->cap : 1024;
        L->mask = (uint8_t*)realloc(L->mask, L->cap);
        L->count = (uint64_t*)realloc(L->count, L->cap * 8);
        L->leaf = (uint64_t*)realloc(L->leaf, L->cap * 8);
        L->kid0 = (uint32_t*)realloc(L->kid0, L->cap * 4);
    }
    uint32_t nk = is_leaf ? 0 : popc32(mask);
    if (L->nkids + nk > L->capkids) {
        L->capkids = L->capkids ? 2 * L->capkids + nk : 4096;
        L->kids = (uint32_t*)realloc(L->kids, L->capkids * 4);
    }
    uint32_t id = (uint32_t)L->n;
    L->mask[id] = mask;
    L->count[id] = count;
    L->leaf[id] = leaf;
    L->kid0[id] = (uint32_t)L->nkids;
    for (uint32_t k = 0; k < nk; k++)
        L->kids[L->nkids + k] = kids[k];
    if (2 * (L->n + 1) > L->map.cap)
        map_grow(&L->map, L, is_leaf);
    uint64_t key = node_key(L, id, is_leaf);
    uint64_t slot = key & (L->map.cap - 1);
    for (;;) {
        uint32_t e = L->map.ids[slot];
        if (e == 0)
            break;
        uint32_t other = e - 1;
        if (L->map.keys[slot] == key) {
            int same;
            if (is_leaf)
                same = L->leaf[other] == leaf;
            else
                same = L->mask[other] == mask &&
                       memcmp(L->kids + L->kid0[other], kids, nk * sizeof(uint32_t)) == 0;
            if (same)
                return other;
        }
        slot = (slot + 1) & (L->map.cap - 1);
    }
    L->map.ids[slot] = id + 1;
    L->map.keys[slot] = key;
    L->n++;
    L->nkids += nk;
    return id;
}

static void map_grow(dedup_map* m, gen_level* L, int is_leaf)
{
    uint64_t ncap = m->cap ? 2 * m->cap : 4096;
    uint64_t* keys = (uint64_t*)calloc(ncap, 8);
    uint32_t* ids = (uint32_t*)calloc(ncap, 4);
    for (uint64_t id = 0; id < L->n; id++) {
        uint64_t key = node_key(L, (uint32_t)id, is_leaf);
        uint64_t slot = key & (ncap - 1);
        while (ids[slot])
            slot = (slot + 1) & (ncap - 1);
        ids[slot] = (uint32_t)id + 1;
        keys[slot] = key;
    }
    free(m->keys);
    free(m->ids);
    m->keys = keys;
    m->ids = ids;
    m->cap = ncap;
}

static uint32_t gen_full(gen_ctx* g, uint32_t level)
{
    if (g->full_id[level] != GEN_EMPTY)
        return g->full_id[level];
    uint32_t id;
    if (level == g->leaf_level) {
        id = level_insert(&g->lv[level], 1, 0xff, 64, ~0ull, NULL);
    } else {
        uint32_t child = gen_full(g, level + 1);
        uint32_t kids[8];
        for (int c = 0; c < 8; c++)
            kids[c] = child;
        uint64_t count = (uint64_t)1 << (3 * (g->depth - level));
        id = level_insert(&g->lv[level], 0, 0xff, count, 0, kids);
    }
    g->full_id[level] = id;
    return id;
}

/* Shell scenes: a node holds no shell voxel when it holds no solid voxel, or
 * when the node grown by one voxel on every side is solid throughout (every
 * voxel then has six solid neighbours).  Only single-source fullness is
 * detected (the height field alone or one sphere alone), which is
 * conservative.  live_out = spheres touching the grown node. */
static int classify_shell(const gen_ctx* g, uint32_t level, uint32_t x0, uint32_t y0, uint32_t z0,
                          const uint8_t* live, uint8_t* live_out)
{
    const uint32_t shift = g->depth - level;
    const int64_t s = (int64_t)1 << shift, E = (int64_t)1 << g->depth;
    const uint32_t m = 1u << level;
    const uint32_t cx = x0 >> shift, cz = z0 >> shift;
    int touched = (int64_t)y0 <= g->hmax[level][(uint64_t)cx * m + cz];
    const int inside = x0 > 0 && z0 > 0 && y0 > 0 && (int64_t)x0 + s < E && (int64_t)z0 + s < E &&
                       (int64_t)y0 + s < E;
    int full = 0;
    if (inside) {
        int64_t lo = INT64_MAX;
        for (int a = -1; a <= 1; a++)
            for (int b = -1; b <= 1; b++) {
                const int64_t v = g->hmin[level][(uint64_t)(cx + a) * m + (cz + b)];
                lo = v < lo ? v : lo;
            }
        full = (int64_t)y0 + s <= lo;
    }
    for (int k = 0; k < 64; k++) {
        live_out[k] = 0;
        if (!live[k])
            continue;
        const int64_t* sp = g->spheres + 4 * k;
        const int64_t lo3[3] = {x0, y0, z0};
        int64_t d2in = 0, d2near = 0, d2far = 0;
        for (int a = 0; a < 3; a++) {
            const int64_t c = sp[a], l = lo3[a], h = lo3[a] + s - 1;
            const int64_t din = c < l ? l - c : (c > h ? c - h : 0);
            const int64_t dn = c < l - 1 ? l - 1 - c : (c > h + 1 ? c - h - 1 : 0);
            const int64_t df = (c - l + 1) > (h + 1 - c) ? (c - l + 1) : (h + 1 - c);
            d2in += din * din;
            d2near += dn * dn;
            d2far += df * df;
        }
        const int64_t r2 = sp[3] * sp[3];
        if (d2near <= r2)
            live_out[k] = 1;
        if (d2in <= r2)
            touched = 1;
        if (inside && d2far <= r2)
            full = 1;
    }
    if (!touched || full)
        return 0;
    return 2;
}

/* solid voxel test inside a leaf's neighbourhood: heights of the 6x6
 * footprint around the leaf (h[(x - x0 + 1) * 6 + (z - z0 + 1)]) and the
 * live spheres; outside the volume is empty */
static int shell_solid(const gen_ctx* g, const int64_t* h, const uint8_t* live, uint32_t x0, uint32_t z0, int64_t x,
                       int64_t y, int64_t z)
{
    const int64_t E = (int64_t)1 << g->depth;
    if (x < 0 || y < 0 || z < 0 || x >= E || y >= E || z >= E)
        return 0;
    if (y <= h[(x - x0 + 1) * 6 + (z - z0 + 1)])
        return 1;
    for (int k = 0; k < 64; k++)
        if (live[k] && in_sphere(g->spheres + 4 * k, x, y, z))
            return 1;
    return 0;
}

static uint64_t shell_leaf(const gen_ctx* g, uint32_t x0, uint32_t y0, uint32_t z0, const uint8_t* live)
{
    const int64_t E = (int64_t)1 << g->depth;
    int64_t h[36];
    for (int a = 0; a < 6; a++)
        for (int b = 0; b < 6; b++) {
            const int64_t x = (int64_t)x0 + a - 1, z = (int64_t)z0 + b - 1;
            h[a * 6 + b] = (x < 0 || z < 0 || x >= E || z >= E) ? -1
                                                                 : or_scene_height(g->seed, g->depth, (uint32_t)x,
                                                                                   (uint32_t)z);
        }
    uint64_t leaf = 0;
    for (uint32_t lx = 0; lx < 4; lx++)
        for (uint32_t ly = 0; ly < 4; ly++)
            for (uint32_t lz = 0; lz < 4; lz++) {
                const int64_t x = x0 + lx, y = y0 + ly, z = z0 + lz;
                if (!shell_solid(g, h, live, x0, z0, x, y, z))
                    continue;
                if (shell_solid(g, h, live, x0, z0, x + 1, y, z) && shell_solid(g, h, live, x0, z0, x - 1, y, z) &&
                    shell_solid(g, h, live, x0, z0, x, y + 1, z) && shell_solid(g, h, live, x0, z0, x, y - 1, z) &&
                    shell_solid(g, h, live, x0, z0, x, y, z + 1) && shell_solid(g, h, live, x0, z0, x, y, z - 1))
                    continue;
                const uint32_t c1 = ((lx >> 1) << 2) | ((ly >> 1) << 1) | (lz >> 1);
                const uint32_t c2 = ((lx & 1) << 2) | ((ly & 1) << 1) | (lz & 1);
                leaf |= 1ull << (c1 * 8 + c2);
            }
    return leaf;
}

int or_scene_shell(uint64_t seed, uint32_t depth, uint32_t x, uint32_t y, uint32_t z)
{
    const int64_t E = (int64_t)1 << depth;
    const int64_t d[7][3] = {{0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
    int s[7];
    for (int k = 0; k < 7; k++) {
        const int64_t a = (int64_t)x + d[k][0], b = (int64_t)y + d[k][1], c = (int64_t)z + d[k][2];
        s[k] = (a < 0 || b < 0 || c < 0 || a >= E || b >= E || c >= E)
                   ? 0
                   : or_scene_solid(seed, depth, (uint32_t)a, (uint32_t)b, (uint32_t)c);
    }
    return s[0] && !(s[1] && s[2] && s[3] && s[4] && s[5] && s[6]);
}

/* 0 = empty, 1 = full, 2 = maybe mixed */
static int classify(const gen_ctx* g, uint32_t level, uint32_t x0, uint32_t y0, uint32_t z0,
                    const uint8_t* live, uint8_t* live_out)
{
    if (g->shell)
        return classify_shell(g, level, x0, y0, z0, live, live_out);
    const uint32_t shift = g->depth - level;
    const int64_t s = (int64_t)1 << shift;
    const uint64_t cell = ((uint64_t)(x0 >> shift) << level) | (z0 >> shift);
    const int64_t hmin = g->hmin[level][cell], hmax = g->hmax[level][cell];
    int full = (int64_t)y0 + s - 1 <= hmin;
    int touched = (int64_t)y0 <= hmax;
    for (int k = 0; k < 64; k++) {
        live_out[k] = 0;
        if (!live[k])
            continue;
        const int64_t* sp = g->spheres + 4 * k;
        int64_t lo[3] = {x0, y0, z0};
        int64_t d2near = 0, d2far = 0;
        for (int a = 0; a < 3; a++) {
            int64_t c = sp[a], l = lo[a], h = lo[a] + s - 1;
            int64_t dn = c < l ? l - c : (c > h ? c - h : 0);
            int64_t df = (c - l) > (h - c) ? (c - l) : (h - c);
            d2near += dn * dn;
            d2far += df * df;
        }
        if (d2near <= sp[3] * sp[3]) {
            live_out[k] = 1;
            touched = 1;
            if (d2far <= sp[3] * sp[3])
                full = 1;
        }
    }
    if (full)
        return 1;
    if (!touched)
        return 0;
    return 2;
}

/* returns node id at `level` or GEN_EMPTY; *count = voxels */
static uint32_t gen_build(gen_ctx* g, uint32_t level, uint32_t x0, uint32_t y0, uint32_t z0,
                          const uint8_t* live, uint64_t* count)
{
    uint8_t live2[64];
    if ((int32_t)level == g->task_level) {
        const uint64_t i = g->task_next++;
        *count = g->task_count[i];
        return g->task_id[i];
    }
    int cls = classify(g, level, x0, y0, z0, live, live2);
    if (cls == 0) {
        *count = 0;
        return GEN_EMPTY;
    }
    if (cls == 1) {
        *count = (uint64_t)1 << (3 * (g->depth - level));
        return gen_full(g, level);
    }
    if (level == g->leaf_level && g->shell) {
        const uint64_t leaf = shell_leaf(g, x0, y0, z0, live2);
        *count = popc64(leaf);
        if (!leaf)
            return GEN_EMPTY;
        return level_insert(&g->lv[level], 1, 0, *count, leaf, NULL);
    }
    if (level == g->leaf_level) {
        uint64_t leaf = 0;
        for (uint32_t lx = 0; lx < 4; lx++)
            for (uint32_t lz = 0; lz < 4; lz++) {
                const uint32_t x = x0 + lx, z = z0 + lz;
                const int64_t h = or_scene_height(g->seed, g->depth, x, z);
                for (uint32_t ly = 0; ly < 4; ly++) {
                    const uint32_t y = y0 + ly;
                    int solid = (int64_t)y <= h;
                    for (int k = 0; k < 64 && !solid; k++)
                        if (live2[k] && in_sphere(g->spheres + 4 * k, x, y, z))
                            solid = 1;
                    if (solid) {
                        uint32_t c1 = ((lx >> 1) << 2) | ((ly >> 1) << 1) | (lz >> 1);
                        uint32_t c2 = ((lx & 1) << 2) | ((ly & 1) << 1) | (lz & 1);
                        leaf |= 1ull << (c1 * 8 + c2);
                    }
                }
            }
        *count = popc64(leaf);
        if (!leaf)
            return GEN_EMPTY;
        return level_insert(&g->lv[level], 1, 0, *count, leaf, NULL);
    }
    const uint32_t half = 1u << (g->depth - level - 1);
    uint32_t kids[8];
    uint8_t mask = 0;
    uint32_t nk = 0;
    uint64_t total = 0;
    for (uint32_t c = 0; c < 8; c++) {
        uint64_t cc;
        uint32_t id = gen_build(g, level + 1, x0 + ((c >> 2) & 1) * half, y0 + ((c >> 1) & 1) * half,
                                z0 + (c & 1) * half, live2, &cc);
        if (id != GEN_EMPTY) {
            mask |= (uint8_t)(1u << c);
            kids[nk++] = id;
            total += cc;
        }
    }
    *count = total;
    if (!mask)
        return GEN_EMPTY;
    return level_insert(&g->lv[level], 0, mask, total, 0, kids);
}

uint32_t* or_generate_basic_dag(uint64_t seed, uint32_t depth, uint32_t T, uint64_t* n_words)
{
    return or_generate_basic_dag_ex(seed, depth, T, 0, n_words);
}

/* Rows [x0, x1) of the height field, or leaf-level cells [x0, x1) of the
 * min / max pyramid, on one thread. */
typedef struct {
    gen_ctx* g;
    int32_t* h;
    uint32_t x0, x1, pass;
} pyr_job;

static void* pyramid_worker(void* arg)
{
    pyr_job* j = (pyr_job*)arg;
    gen_ctx* g = j->g;
    const uint32_t E = 1u << g->depth, n = 1u << g->leaf_level;
    for (uint32_t x = j->x0; x < j->x1; x++) {
        if (j->pass == 0) {
            for (uint32_t z = 0; z < E; z++)
                j->h[(size_t)x * E + z] = or_scene_height(g->seed, g->depth, x, z);
            continue;
        }
        for (uint32_t cz = 0; cz < n; cz++) {
            int32_t lo = 0x7fffffff, hi = -0x7fffffff;
            for (uint32_t a = 0; a < 4; a++)
                for (uint32_t b = 0; b < 4; b++) {
                    int32_t v = j->h[(size_t)(4 * x + a) * E + 4 * cz + b];
                    lo = v < lo ? v : lo;
                    hi = v > hi ? v : hi;
                }
            g->hmin[g->leaf_level][(size_t)x * n + cz] = lo;
            g->hmax[g->leaf_level][(size_t)x * n + cz] = hi;
        }
    }
    return NULL;
}

/* The height min / max pyramid over node footprints, levels leaf..0. */
static void gen_pyramid(gen_ctx* g, uint32_t threads)
{
    const uint32_t E = 1u << g->depth;
    int32_t* h = (int32_t*)malloc((size_t)E * E * 4);
    const uint32_t n = 1u << g->leaf_level; /* 4x4 footprints */
    g->hmin[g->leaf_level] = (int32_t*)malloc((size_t)n * n * 4);
    g->hmax[g->leaf_level] = (int32_t*)malloc((size_t)n * n * 4);
    if (threads < 1)
        threads = 1;
    if (threads > 256)
        threads = 256;
    pthread_t th[256];
    pyr_job jobs[256];
    for (uint32_t pass = 0; pass < 2; pass++) {
        const uint32_t rows = pass == 0 ? E : n;
        for (uint32_t i = 0; i < threads; i++) {
            jobs[i] = (pyr_job){g, h, (uint32_t)((uint64_t)rows * i / threads),
                                (uint32_t)((uint64_t)rows * (i + 1) / threads), pass};
            if (threads == 1)
                pyramid_worker(&jobs[i]);
            else
                pthread_create(&th[i], NULL, pyramid_worker, &jobs[i]);
        }
        if (threads > 1)
            for (uint32_t i = 0; i < threads; i++)
                pthread_join(th[i], NULL);
    }
    free(h);
    for (int32_t l = (int32_t)g->leaf_level - 1; l >= 0; l--) {
        const uint32_t m = 1u << l, m2 = 2 * m;
        g->hmin[l] = (int32_t*)malloc((size_t)m * m * 4);
        g->hmax[l] = (int32_t*)malloc((size_t)m * m * 4);
        for (uint32_t cx = 0; cx < m; cx++)
            for (uint32_t cz = 0; cz < m; cz++) {
                int32_t lo = 0x7fffffff, hi = -0x7fffffff;
                for (uint32_t a = 0; a < 2; a++)
                    for (uint32_t b = 0; b < 2; b++) {
                        size_t i = (size_t)(2 * cx + a) * m2 + 2 * cz + b;
                        lo = g->hmin[l + 1][i] < lo ? g->hmin[l + 1][i] : lo;
                        hi = g->hmax[l + 1][i] > hi ? g->hmax[l + 1][i] : hi;
                    }
                g->hmin[l][(size_t)cx * m + cz] = lo;
                g->hmax[l][(size_t)cx * m + cz] = hi;
            }
    }
}

static void gen_levels_free(gen_ctx* g)
{
    for (uint32_t l = 0; l <= g->leaf_level; l++) {
        gen_level* L = &g->lv[l];
        free(L->mask); free(L->count); free(L->leaf); free(L->kid0); free(L->kids);
        free(L->map.keys); free(L->map.ids);
        memset(L, 0, sizeof(*L));
    }
}

/* ---- threaded build ----------------------------------------------------
 * The subtrees below the nodes of one level (kTaskLevel) are independent:
 * each worker builds its share of them into levels of its own, deduplicated
 * within the worker; the workers' nodes are then merged level by level,
 * leaves first, into the shared levels (content-deduplicated, so the merged
 * DAG is the one a single-threaded build makes), and the levels above are
 * built with the subtrees' results in the same visit order.  The BasicDAG
 * words depend only on the DAG (depth-first ranks), not on node ids, so the
 * output is identical to the single-threaded build's. */
#define GEN_TASK_LEVEL 4

typedef struct {
    uint32_t x, y, z;
    uint8_t live[64];
} gen_task;

typedef struct {
    gen_task* v;
    uint64_t n, cap;
} gen_tasks;

static void tasks_push(gen_tasks* t, uint32_t x, uint32_t y, uint32_t z, const uint8_t* live)
{
    if (t->n == t->cap) {
        t->cap = t->cap ? 2 * t->cap : 1024;
        t->v = (gen_task*)realloc(t->v, t->cap * sizeof(gen_task));
    }
    gen_task* k = &t->v[t->n++];
    k->x = x;
    k->y = y;
    k->z = z;
    memcpy(k->live, live, 64);
}

/* The subtree roots at level P in the order gen_build visits them: every
 * child of a level-(P-1) node that gen_build descends into. */
static void gen_enumerate(const gen_ctx* g, uint32_t level, uint32_t P, uint32_t x0, uint32_t y0, uint32_t z0,
                          const uint8_t* live, gen_tasks* out)
{
    uint8_t live2[64];
    if (classify(g, level, x0, y0, z0, live, live2) != 2)
        return;
    const uint32_t half = 1u << (g->depth - level - 1);
    for (uint32_t c = 0; c < 8; c++) {
        const uint32_t x = x0 + ((c >> 2) & 1) * half, y = y0 + ((c >> 1) & 1) * half, z = z0 + (c & 1) * half;
        if (level + 1 == P)
            tasks_push(out, x, y, z, live2);
        else
            gen_enumerate(g, level + 1, P, x, y, z, live2, out);
    }
}

typedef struct {
    gen_ctx local;
    const gen_tasks* tasks;
    uint64_t* next; /* shared task counter */
    uint32_t* owner;
    uint32_t* id;
    uint64_t* count;
    uint32_t index;
} gen_worker;

static void* build_worker(void* arg)
{
    gen_worker* w = (gen_worker*)arg;
    for (;;) {
        const uint64_t i = __atomic_fetch_add(w->next, 1, __ATOMIC_RELAXED);
        if (i >= w->tasks->n)
            break;
        const gen_task* k = &w->tasks->v[i];
        uint64_t cnt;
        w->id[i] = gen_build(&w->local, GEN_TASK_LEVEL, k->x, k->y, k->z, k->live, &cnt);
        w->count[i] = cnt;
        w->owner[i] = w->index;
    }
    return NULL;
}

/* Inserts a worker's nodes of levels P..leaf into the shared levels;
 * map[l][local id] = shared id. */
static void merge_worker(gen_ctx* g, gen_ctx* w, uint32_t P, uint32_t** map)
{
    for (int32_t l = (int32_t)g->leaf_level; l >= (int32_t)P; l--) {
        gen_level* L = &w->lv[l];
        map[l] = (uint32_t*)malloc((L->n + 1) * 4);
        const int is_leaf = (uint32_t)l == g->leaf_level;
        for (uint64_t id = 0; id < L->n; id++) {
            uint32_t kids[8];
            const uint32_t nk = is_leaf ? 0 : popc32(L->mask[id]);
            for (uint32_t k = 0; k < nk; k++)
                kids[k] = map[l + 1][L->kids[L->kid0[id] + k]];
            map[l][id] = level_insert(&g->lv[l], is_leaf, L->mask[id], L->count[id], L->leaf[id], kids);
        }
    }
}

static uint32_t gen_build_threaded(gen_ctx* g, uint32_t threads, uint64_t* total)
{
    const uint32_t P = GEN_TASK_LEVEL;
    uint8_t live[64];
    memset(live, 1, 64);
    gen_tasks tasks = {0};
    gen_enumerate(g, 0, P, 0, 0, 0, live, &tasks);
    uint32_t* owner = (uint32_t*)calloc(tasks.n + 1, 4);
    uint32_t* id = (uint32_t*)calloc(tasks.n + 1, 4);
    uint64_t* count = (uint64_t*)calloc(tasks.n + 1, 8);
    if (threads > 256)
        threads = 256;
    gen_worker* w = (gen_worker*)calloc(threads, sizeof(gen_worker));
    pthread_t th[256];
    uint64_t next = 0;
    for (uint32_t i = 0; i < threads; i++) {
        w[i].local = *g;
        memset(w[i].local.lv, 0, sizeof(w[i].local.lv));
        for (uint32_t l = 0; l < HD_MAX_DEPTH; l++)
            w[i].local.full_id[l] = GEN_EMPTY;
        w[i].local.task_level = -1;
        w[i].tasks = &tasks;
        w[i].next = &next;
        w[i].owner = owner;
        w[i].id = id;
        w[i].count = count;
        w[i].index = i;
        pthread_create(&th[i], NULL, build_worker, &w[i]);
    }
    for (uint32_t i = 0; i < threads; i++)
        pthread_join(th[i], NULL);
    /* merge, worker by worker; task ids become shared ids */
    uint32_t* shared = (uint32_t*)malloc((tasks.n + 1) * 4);
    for (uint32_t i = 0; i < threads; i++) {
        uint32_t* map[HD_MAX_DEPTH + 1] = {0};
        merge_worker(g, &w[i].local, P, map);
        for (uint64_t k = 0; k < tasks.n; k++)
            if (owner[k] == i)
                shared[k] = id[k] == GEN_EMPTY ? GEN_EMPTY : map[P][id[k]];
        for (uint32_t l = 0; l <= HD_MAX_DEPTH; l++)
            free(map[l]);
        gen_levels_free(&w[i].local);
    }
    /* the levels above, taking the subtrees' results in visit order */
    g->task_level = (int32_t)P;
    g->task_id = shared;
    g->task_count = count;
    g->task_next = 0;
    const uint32_t root = gen_build(g, 0, 0, 0, 0, live, total);
    g->task_level = -1;
    free(shared);
    free(owner);
    free(id);
    free(count);
    free(tasks.v);
    free(w);
    return root;
}

uint32_t* or_generate_basic_dag_ex(uint64_t seed, uint32_t depth, uint32_t T, uint32_t flags, uint64_t* n_words)
{
    return or_generate_basic_dag_mt(seed, depth, T, flags, 1, n_words);
}

uint32_t* or_generate_basic_dag_mt(uint64_t seed, uint32_t depth, uint32_t T, uint32_t flags, uint32_t threads,
                                   uint64_t* n_words)
{
    if (depth < 6 || depth > 16 || T > depth - 2)
        return NULL;
    if (threads == 0) {
        const long n = sysconf(_SC_NPROCESSORS_ONLN);
        threads = n > 0 ? (uint32_t)n : 1;
    }
    gen_ctx* g = (gen_ctx*)calloc(1, sizeof(gen_ctx));
    g->seed = seed;
    g->shell = (flags & HD_SCENE_SHELL) != 0;
    g->depth = depth;
    g->leaf_level = depth - 2;
    g->T = T;
    g->task_level = -1;
    for (uint32_t l = 0; l < HD_MAX_DEPTH; l++)
        g->full_id[l] = GEN_EMPTY;
    or_scene_spheres(seed, depth, g->spheres);
    gen_pyramid(g, threads);
    uint8_t live[64];
    memset(live, 1, 64);
    uint64_t total;
    uint32_t root = threads > 1 && GEN_TASK_LEVEL <= g->leaf_level ? gen_build_threaded(g, threads, &total)
                                                                   : gen_build(g, 0, 0, 0, 0, live, &total);
    uint32_t* words = NULL;
    if (root != GEN_EMPTY) {
        /* depth-first first-visit rank per level (create_hash_dag order) */
        uint32_t* rank[HD_MAX_DEPTH];
        uint64_t nrank[HD_MAX_DEPTH] = {0};
        for (uint32_t l = 0; l <= g->leaf_level; l++) {
            rank[l] = (uint32_t*)malloc((g->lv[l].n + 1) * 4);
            memset(rank[l], 0xff, (g->lv[l].n + 1) * 4);
        }
        struct frame { uint32_t level, id, next; } stack[HD_MAX_DEPTH + 1];
        int sp = 0;
        rank[0][root] = (uint32_t)nrank[0]++;
        stack[sp++] = (struct frame){0, root, 0};
        while (sp) {
            struct frame* f = &stack[sp - 1];
            if (f->level == g->leaf_level || f->next == popc32(g->lv[f->level].mask[f->id])) {
                sp--;
                continue;
            }
            uint32_t child = g->lv[f->level].kids[g->lv[f->level].kid0[f->id] + f->next++];
            uint32_t cl = f->level + 1;
            if (rank[cl][child] == 0xFFFFFFFFu) {
                rank[cl][child] = (uint32_t)nrank[cl]++;
                stack[sp++] = (struct frame){cl, child, 0};
            }
        }
        /* word offsets per level in rank order */
        uint64_t level_base[HD_MAX_DEPTH + 1];
        uint32_t* order[HD_MAX_DEPTH];
        uint64_t off = 0;
        for (uint32_t l = 0; l <= g->leaf_level; l++) {
            level_base[l] = off;
            order[l] = (uint32_t*)malloc((nrank[l] + 1) * 4);
            for (uint64_t id = 0; id < g->lv[l].n; id++)
                if (rank[l][id] != 0xFFFFFFFFu)
                    order[l][rank[l][id]] = (uint32_t)id;
            for (uint64_t r = 0; r < nrank[l]; r++)
                off += l == g->leaf_level ? 2 : 1 + popc32(g->lv[l].mask[order[l][r]]);
        }
        /* word index of each node */
        uint64_t* where[HD_MAX_DEPTH];
        for (uint32_t l = 0; l <= g->leaf_level; l++) {
            where[l] = (uint64_t*)malloc((g->lv[l].n + 1) * 8);
            uint64_t o = level_base[l];
            for (uint64_t r = 0; r < nrank[l]; r++) {
                uint32_t id = order[l][r];
                where[l][id] = o;
                o += l == g->leaf_level ? 2 : 1 + popc32(g->lv[l].mask[id]);
            }
        }
        words = (uint32_t*)malloc(off * 4);
        uint64_t enclosed = 0;
        int bad = 0;
        for (uint32_t l = 0; l <= g->leaf_level; l++) {
            for (uint64_t r = 0; r < nrank[l]; r++) {
                uint32_t id = order[l][r];
                uint64_t w = where[l][id];
                if (l == g->leaf_level) {
                    words[w] = (uint32_t)g->lv[l].leaf[id];
                    words[w + 1] = (uint32_t)(g->lv[l].leaf[id] >> 32);
                    continue;
                }
                uint32_t upper;
                if (l < T)
                    upper = (uint32_t)(enclosed + r);
                else
                    upper = (uint32_t)g->lv[l].count[id];
                if ((l < T ? enclosed + r : g->lv[l].count[id]) >= (1u << 24))
                    bad = 1;
                words[w] = (upper << 8) | g->lv[l].mask[id];
                uint32_t nk = popc32(g->lv[l].mask[id]);
                for (uint32_t k = 0; k < nk; k++)
                    words[w + 1 + k] = (uint32_t)where[l + 1][g->lv[l].kids[g->lv[l].kid0[id] + k]];
            }
            if (l < T)
                enclosed += nrank[l];
        }
        *n_words = off;
        for (uint32_t l = 0; l <= g->leaf_level; l++) {
            free(rank[l]);
            free(order[l]);
            free(where[l]);
        }
        if (bad) {
            free(words);
            words = NULL;
        }
    }
    gen_levels_free(g);
    for (uint32_t l = 0; l <= g->leaf_level; l++) {
        free(g->hmin[l]);
        free(g->hmax[l]);
    }
    free(g);
    return words;
}
void or_free(void* p) { free(p); }

/* ======================================================================
 * Ingest: HashDAGFactory::load_from_DAG (hash_dag_factory.cpp:152-184) and
 * create_hash_dag (:5-99)
 * ====================================================================== */

static uint32_t create_hash_dag(or_table* t, const uint32_t* words, uint32_t* map, uint32_t level, uint32_t index)
{
    if (level == t->leaf_level) {
        uint64_t leaf = (uint64_t)words[index] | ((uint64_t)words[index + 1] << 32);
        return add_leaf(t, leaf, or_hash_leaf(leaf));
    }
    const uint32_t node = words[index];
    const uint32_t mask = node & 0xffu;
    uint32_t buf[9];
    uint32_t n = 0;
    buf[n++] = node;
    for (uint32_t c = 0; c < 8; c++) {
        if (!(mask & (1u << c)))
            continue;
        const uint32_t child = words[index + child_offset(mask, c)];
        uint32_t id = map[child];
        if (id == 0) {
            id = create_hash_dag(t, words, map, level + 1, child);
            map[child] = id + 1;
        } else {
            id--;
        }
        buf[n++] = id;
        if (t->error)
            return INVALID;
    }
    return add_interior(t, level, n, buf, or_hash_interior(n, buf));
}

int or_load_basic_dag(or_table* t, const uint32_t* words, uint64_t n_words)
{
    for (uint32_t level = t->leaf_level; level > 0; level--)
        add_full_node(t, level);
    uint32_t* map = (uint32_t*)calloc(n_words + 1, 4);
    t->root = create_hash_dag(t, words, map, 0, 0);
    free(map);
    return t->error;
}

/* ======================================================================
 * Queries (dag_utils.h:138-172)
 * ====================================================================== */

static uint32_t leaf_bit(uint32_t x, uint32_t y, uint32_t z)
{
    return ((x & 1) ? 4 : 0) | ((y & 1) ? 2 : 0) | ((z & 1) ? 1 : 0) | ((x & 2) ? 32 : 0) |
           ((y & 2) ? 16 : 0) | ((z & 2) ? 8 : 0);
}

int or_get_value(const or_table* t, uint32_t x, uint32_t y, uint32_t z)
{
    const uint32_t D = t->cfg.depth;
    uint32_t index = t->root;
    for (uint32_t level = 0; level < D; level++) {
        if (level < t->leaf_level) {
            const uint32_t mask = *sys_ptr(t, index) & 0xffu;
            const uint32_t s = D - (level + 1);
            const uint32_t child = (((x >> s) & 1) << 2) | (((y >> s) & 1) << 1) | ((z >> s) & 1);
            if (!(mask & (1u << child)))
                return 0;
            index = *sys_ptr(t, index + child_offset(mask, child));
        } else {
            const uint32_t* p = sys_ptr(t, index);
            uint64_t leaf = (uint64_t)p[0] | ((uint64_t)p[1] << 32);
            return (int)((leaf >> leaf_bit(x, y, z)) & 1);
        }
    }
    return 1;
}

typedef struct {
    uint32_t* keys;
    uint64_t* vals;
    uint64_t cap, n;
} fp_map;

static uint64_t fp_node(const or_table* t, fp_map* maps, uint32_t level, uint32_t index)
{
    fp_map* m = &maps[level];
    if (2 * (m->n + 1) > m->cap) {
        uint64_t ncap = m->cap ? 2 * m->cap : 1024;
        uint32_t* k = (uint32_t*)malloc(ncap * 4);
        uint64_t* v = (uint64_t*)malloc(ncap * 8);
        memset(k, 0xff, ncap * 4);
        for (uint64_t i = 0; i < m->cap; i++)
            if (m->keys[i] != 0xFFFFFFFFu) {
                uint64_t s = or_murmurhash64(m->keys[i]) & (ncap - 1);
                while (k[s] != 0xFFFFFFFFu)
                    s = (s + 1) & (ncap - 1);
                k[s] = m->keys[i];
                v[s] = m->vals[i];
            }
        free(m->keys);
        free(m->vals);
        m->keys = k;
        m->vals = v;
        m->cap = ncap;
    }
    uint64_t s = or_murmurhash64(index) & (m->cap - 1);
    while (m->keys[s] != 0xFFFFFFFFu) {
        if (m->keys[s] == index)
            return m->vals[s];
        s = (s + 1) & (m->cap - 1);
    }
    uint64_t h;
    const uint32_t* p = sys_ptr(t, index);
    if (level == t->leaf_level) {
        h = mix64(((uint64_t)p[0] | ((uint64_t)p[1] << 32)) ^ 0x1EAF1EAF1EAF1EAFull);
    } else {
        const uint32_t mask = p[0] & 0xffu;
        uint32_t kids[8];
        for (uint32_t k = 0; k < popc32(mask); k++)
            kids[k] = p[1 + k];
        h = mix64(mask);
        for (uint32_t k = 0; k < popc32(mask); k++)
            h = mix64(h ^ fp_node(t, maps, level + 1, kids[k]));
    }
    /* re-probe: the recursion may have grown the map */
    s = or_murmurhash64(index) & (m->cap - 1);
    while (m->keys[s] != 0xFFFFFFFFu)
        s = (s + 1) & (m->cap - 1);
    m->keys[s] = index;
    m->vals[s] = h;
    m->n++;
    return h;
}

/* Nodes reachable from root per level (out) and, when words is given, the
   words they occupy (a leaf 2, an interior node total_size): what the
   reference's GC re-appends per level besides the full node and the
   padding at page ends (hash_dag.h:407-547). */
void or_reachable_words(const or_table* t, uint32_t root, uint64_t* out, uint64_t* words)
{
    uint32_t* cur = (uint32_t*)malloc(4);
    uint64_t n = 1;
    cur[0] = root;
    for (uint32_t level = 0; level <= t->leaf_level; level++) {
        out[level] = n;
        if (words) {
            uint64_t w = 0;
            for (uint64_t i = 0; i < n; i++)
                w += level == t->leaf_level ? 2 : total_size(*sys_ptr(t, cur[i]));
            words[level] = w;
        }
        if (level == t->leaf_level)
            break;
        uint64_t cap = 0;
        for (uint64_t i = 0; i < n; i++)
            cap += total_size(*sys_ptr(t, cur[i])) - 1;
        uint32_t* nxt = (uint32_t*)malloc((cap + 1) * 4);
        uint64_t k = 0;
        for (uint64_t i = 0; i < n; i++) {
            const uint32_t* p = sys_ptr(t, cur[i]);
            for (uint32_t o = 1; o < total_size(p[0]); o++)
                nxt[k++] = p[o];
        }
        free(cur);
        cur = nxt;
        n = unique_sorted(cur, k);
    }
    free(cur);
}

void or_reachable_counts(const or_table* t, uint32_t root, uint64_t* out) { or_reachable_words(t, root, out, NULL); }

uint64_t or_occupancy_fingerprint(const or_table* t, uint32_t root)
{
    fp_map maps[HD_MAX_DEPTH];
    memset(maps, 0, sizeof(maps));
    uint64_t h = fp_node(t, maps, 0, root);
    for (uint32_t l = 0; l < HD_MAX_DEPTH; l++) {
        free(maps[l].keys);
        free(maps[l].vals);
    }
    return h;
}

/* ======================================================================
 * Traversal (tracer.cu).  fp_mode 1 places fused multiply-adds where the
 * reference's default nvcc build contracts a product into a following add.
 * ====================================================================== */

typedef struct { float x, y, z; } f3;
typedef struct { double x, y, z; } d3;

static float fmaxr(float a, float b) { return a > b ? a : b; } /* constexpr_max (cuda_math.h:13) */
static float fminr(float a, float b) { return a < b ? a : b; }

/* normalize(rayMin + x * ddx + y * ddy - position) in double
 * (tracer.cu:157, cuda_math.h:55-56) */
static d3 camera_dir(const hd_camera* cam, double px, double py, uint32_t mode)
{
    double v[3];
    for (int a = 0; a < 3; a++) {
        double t;
        if (mode) {
            t = fma(px, cam->ray_ddx[a], cam->ray_min[a]);
            t = fma(py, cam->ray_ddy[a], t);
        } else {
            t = cam->ray_min[a] + px * cam->ray_ddx[a];
            t = t + py * cam->ray_ddy[a];
        }
        v[a] = t - cam->position[a];
    }
    double dot = mode ? fma(v[2], v[2], fma(v[1], v[1], v[0] * v[0])) : (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
    double inv = 1.0 / sqrt(dot);
    d3 r = {inv * v[0], inv * v[1], inv * v[2]};
    return r;
}

/* compute_intersection_mask (tracer.cu:19-136) */
static uint32_t intersection_mask(uint32_t D, int is_root, uint32_t level, const uint32_t path[3], f3 o, f3 d,
                                  f3 inv, uint32_t mode)
{
    const uint32_t shift = D - level;
    const float radius = (float)(1u << (shift - 1));
    const float cx = radius + (float)(path[0] << shift);
    const float cy = radius + (float)(path[1] << shift);
    const float cz = radius + (float)(path[2] << shift);
    const f3 crr = {cx - o.x, cy - o.y, cz - o.z};
    const f3 tmid = {crr.x * inv.x, crr.y * inv.y, crr.z * inv.z};
    const f3 slab = {radius * fabsf(inv.x), radius * fabsf(inv.y), radius * fabsf(inv.z)};
    f3 pmin, pmax;
    if (mode) {
        pmin = (f3){fmaf(crr.x, inv.x, -slab.x), fmaf(crr.y, inv.y, -slab.y), fmaf(crr.z, inv.z, -slab.z)};
        pmax = (f3){fmaf(crr.x, inv.x, slab.x), fmaf(crr.y, inv.y, slab.y), fmaf(crr.z, inv.z, slab.z)};
    } else {
        pmin = (f3){tmid.x - slab.x, tmid.y - slab.y, tmid.z - slab.z};
        pmax = (f3){tmid.x + slab.x, tmid.y + slab.y, tmid.z + slab.z};
    }
    const float tmin = fmaxr(fmaxr(pmin.x, fmaxr(pmin.y, pmin.z)), 0.0f);
    const float tmax = fminr(pmax.x, fminr(pmax.y, pmax.z));
    if (is_root && tmin >= tmax)
        return 0;
    uint32_t result = 0;
    {
        const float s = 0.5f * (tmin + tmax);
        const f3 p = {s * d.x, s * d.y, s * d.z};
        const uint32_t first = (p.x >= crr.x ? 4u : 0u) + (p.y >= crr.y ? 2u : 0u) + (p.z >= crr.z ? 1u : 0u);
        result |= 1u << first;
    }
    const float eps = 1e-4f;
    if (tmin <= tmid.x && tmid.x <= tmax) {
        const f3 p = {tmid.x * d.x, tmid.x * d.y, tmid.x * d.z};
        uint32_t A = 0, B = 0;
        if (p.y >= crr.y - eps) A |= 0xCC;
        if (p.y <= crr.y + eps) A |= 0x33;
        if (p.z >= crr.z - eps) B |= 0xAA;
        if (p.z <= crr.z + eps) B |= 0x55;
        result |= A & B;
    }
    if (tmin <= tmid.y && tmid.y <= tmax) {
        const f3 p = {tmid.y * d.x, tmid.y * d.y, tmid.y * d.z};
        uint32_t C = 0, Dm = 0;
        if (p.x >= crr.x - eps) C |= 0xF0;
        if (p.x <= crr.x + eps) C |= 0x0F;
        if (p.z >= crr.z - eps) Dm |= 0xAA;
        if (p.z <= crr.z + eps) Dm |= 0x55;
        result |= C & Dm;
    }
    if (tmin <= tmid.z && tmid.z <= tmax) {
        const f3 p = {tmid.z * d.x, tmid.z * d.y, tmid.z * d.z};
        uint32_t E = 0, F = 0;
        if (p.x >= crr.x - eps) E |= 0xF0;
        if (p.x <= crr.x + eps) E |= 0x0F;
        if (p.y >= crr.y - eps) F |= 0xCC;
        if (p.y <= crr.y + eps) F |= 0x33;
        result |= E & F;
    }
    return result & 0xffu;
}

/* next_child (tracer.cu:7-17) */
static uint32_t next_child(uint32_t order, uint32_t mask)
{
    for (uint32_t c = 0; c < 8; c++) {
        uint32_t ci = c ^ order;
        if (mask & (1u << ci))
            return ci;
    }
    return 0;
}
static uint32_t first_child_mask(uint64_t leaf) /* Leaf::get_first_child_mask (base_dag.h:16-52) */
{
    uint32_t m = 0;
    for (uint32_t b = 0; b < 8; b++)
        if ((leaf >> (8 * b)) & 0xffu)
            m |= 1u << b;
    return m;
}
static uint32_t second_child_mask(uint64_t leaf, uint32_t c) /* base_dag.h:53-59 */
{
    return (uint32_t)(leaf >> (8 * c)) & 0xffu;
}

typedef struct {
    uint32_t index, child_mask, visit_mask;
} stack_entry;

/* The shared stack walk of trace_paths (tracer.cu:168-249) and
 * intersect_ray_node_out_of_order (:453-543).  any_hit selects the shadow
 * variant (children highest bit first, return on the first voxel). */
static int walk(const or_table* t, f3 o, f3 d, f3 inv, uint32_t order, int any_hit, uint32_t mode,
                uint32_t out_path[3], uint64_t* visits)
{
    const uint32_t D = t->cfg.depth, leafl = t->leaf_level;
    uint32_t level = 0;
    uint32_t path[3] = {0, 0, 0};
    stack_entry stack[HD_MAX_DEPTH];
    stack_entry cache;
    uint64_t cached_leaf = 0;
    cache.index = t->root;
    cache.child_mask = *sys_ptr(t, cache.index) & 0xffu;
    cache.visit_mask = cache.child_mask & intersection_mask(D, 1, 0, path, o, d, inv, mode);
    uint64_t v = 1;
    for (;;) {
        uint32_t nl = level;
        while (nl > 0 && !cache.visit_mask) {
            nl--;
            cache = stack[nl];
        }
        if (nl == 0 && !cache.visit_mask) {
            path[0] = path[1] = path[2] = 0;
            if (visits)
                *visits += v;
            if (out_path)
                out_path[0] = out_path[1] = out_path[2] = 0;
            return 0;
        }
        for (int a = 0; a < 3; a++)
            path[a] >>= (level - nl);
        level = nl;
        const uint32_t nc = any_hit ? 31u - (uint32_t)__builtin_clz(cache.visit_mask) : next_child(order, cache.visit_mask);
        cache.visit_mask &= ~(1u << nc);
        path[0] = (path[0] << 1) | ((nc >> 2) & 1);
        path[1] = (path[1] << 1) | ((nc >> 1) & 1);
        path[2] = (path[2] << 1) | (nc & 1);
        stack[level] = cache;
        level++;
        if (level == D) {
            if (visits)
                *visits += v;
            if (out_path) {
                out_path[0] = path[0];
                out_path[1] = path[1];
                out_path[2] = path[2];
            }
            return 1;
        }
        if (level < leafl) {
            cache.index = *sys_ptr(t, cache.index + child_offset(cache.child_mask, nc));
            cache.child_mask = *sys_ptr(t, cache.index) & 0xffu;
            cache.visit_mask = cache.child_mask & intersection_mask(D, 0, level, path, o, d, inv, mode);
            v++;
        } else {
            uint32_t cm;
            if (level == leafl) {
                const uint32_t addr = *sys_ptr(t, cache.index + child_offset(cache.child_mask, nc));
                const uint32_t* p = sys_ptr(t, addr);
                cached_leaf = (uint64_t)p[0] | ((uint64_t)p[1] << 32);
                cm = first_child_mask(cached_leaf);
                v++;
            } else {
                cm = second_child_mask(cached_leaf, nc);
            }
            cache.child_mask = cm;
            cache.visit_mask = cm & intersection_mask(D, 0, level, path, o, d, inv, mode);
        }
    }
}

static f3 to_f3(d3 v)
{
    f3 r = {(float)v.x, (float)v.y, (float)v.z};
    return r;
}
static f3 inverse_dir(f3 d) /* make_float3(make_double3(1. / d.x, ...)) (tracer.cu:160) */
{
    f3 r = {(float)(1.0 / (double)d.x), (float)(1.0 / (double)d.y), (float)(1.0 / (double)d.z)};
    return r;
}

void or_trace_primary(const or_table* t, const hd_camera* cam, uint32_t W, uint32_t H, uint32_t mode,
                      uint32_t* paths, uint32_t row0, uint32_t row1, uint64_t* visits)
{
    const f3 o = {(float)cam->position[0], (float)cam->position[1], (float)cam->position[2]};
    for (uint32_t y = row0; y < row1 && y < H; y++)
        for (uint32_t x = 0; x < W; x++) {
            const f3 d = to_f3(camera_dir(cam, (double)x, (double)y, mode));
            const f3 inv = inverse_dir(d);
            const uint32_t order = (d.x < 0.f ? 4u : 0u) + (d.y < 0.f ? 2u : 0u) + (d.z < 0.f ? 1u : 0u);
            uint32_t p[3];
            walk(t, o, d, inv, order, 0, mode, p, visits);
            uint32_t* out = paths + 4 * ((uint64_t)(H - 1 - y) * W + x);
            out[0] = p[0];
            out[1] = p[1];
            out[2] = p[2];
            out[3] = 0;
        }
}

/* trace_shadows (tracer.cu:589-697) reduced to its hit test; rows are
 * output rows (the layout of the paths image). */
void or_trace_shadow(const or_table* t, const hd_camera* cam, uint32_t W, uint32_t H, uint32_t mode,
                     const uint32_t* paths, const float light[3], float bias, uint8_t* mask,
                     uint32_t row0, uint32_t row1, uint64_t* visits)
{
    /* sun_direction(): normalize(float3) in float (tracer.cu:546-549) */
    const f3 L = {light[0], light[1], light[2]};
    const float dot = mode ? fmaf(L.z, L.z, fmaf(L.y, L.y, L.x * L.x)) : (L.x * L.x + L.y * L.y) + L.z * L.z;
    const float il = 1.0f / sqrtf(dot);
    const f3 dir = {il * L.x, il * L.y, il * L.z};
    const f3 inv = inverse_dir(dir);
    for (uint32_t r = row0; r < row1 && r < H; r++)
        for (uint32_t x = 0; x < W; x++) {
            const uint32_t* p = paths + 4 * ((uint64_t)r * W + x);
            uint8_t* out = mask + (uint64_t)r * W + x;
            if (p[0] == 0 && p[1] == 0 && p[2] == 0) {
                *out = 2;
                continue;
            }
            const d3 cd = camera_dir(cam, (double)x, (double)(H - 1 - r), mode);
            /* ray_box_intersection (tracer.cu:574-587) */
            const double bmin[3] = {(double)(float)p[0], (double)(float)p[1], (double)(float)p[2]};
            const double dd[3] = {cd.x, cd.y, cd.z};
            double real_min[3];
            for (int a = 0; a < 3; a++) {
                const double t0 = (bmin[a] - cam->position[a]) / dd[a];
                const double t1 = ((bmin[a] + 1.0) - cam->position[a]) / dd[a];
                real_min[a] = t0 < t1 ? t0 : t1;
            }
            const double maxmin = fmax(fmax(real_min[0], real_min[1]), real_min[2]);
            f3 start;
            if (mode)
                start = (f3){(float)fma(dd[0], maxmin, cam->position[0]), (float)fma(dd[1], maxmin, cam->position[1]),
                             (float)fma(dd[2], maxmin, cam->position[2])};
            else
                start = (f3){(float)(cam->position[0] + dd[0] * maxmin), (float)(cam->position[1] + dd[1] * maxmin),
                             (float)(cam->position[2] + dd[2] * maxmin)};
            f3 o;
            if (mode)
                o = (f3){fmaf(bias, dir.x, start.x), fmaf(bias, dir.y, start.y), fmaf(bias, dir.z, start.z)};
            else
                o = (f3){start.x + bias * dir.x, start.y + bias * dir.y, start.z + bias * dir.z};
            *out = (uint8_t)walk(t, o, dir, inv, 0, 1, mode, NULL, visits);
        }
}

typedef struct {
    const or_table* t;
    const hd_camera* cam;
    uint32_t W, H, mode;
    const float* light;
    float bias;
    uint32_t* paths;
    uint8_t* mask;
    uint32_t r0, r1;
} frame_job;

static void* frame_worker(void* arg)
{
    frame_job* j = (frame_job*)arg;
    /* primary rows [r0, r1) of pixel space land in output rows H-1-y */
    or_trace_primary(j->t, j->cam, j->W, j->H, j->mode, j->paths, j->r0, j->r1, NULL);
    return NULL;
}
static void* shadow_worker(void* arg)
{
    frame_job* j = (frame_job*)arg;
    or_trace_shadow(j->t, j->cam, j->W, j->H, j->mode, j->paths, j->light, j->bias, j->mask, j->r0, j->r1, NULL);
    return NULL;
}

void or_trace_frame_mt(const or_table* t, const hd_camera* cam, uint32_t W, uint32_t H, uint32_t mode,
                       const float light[3], float bias, uint32_t* paths, uint8_t* mask, uint32_t n_threads,
                       uint32_t row0, uint32_t row1)
{
    if (n_threads < 1)
        n_threads = 1;
    if (n_threads > 256)
        n_threads = 256;
    if (row1 > H)
        row1 = H;
    pthread_t th[256];
    frame_job jobs[256];
    const uint32_t rows = row1 > row0 ? row1 - row0 : 0;
    for (int pass = 0; pass < 2; pass++) {
        for (uint32_t i = 0; i < n_threads; i++) {
            jobs[i] = (frame_job){t, cam, W, H, mode, light, bias, paths, mask,
                                  row0 + (uint32_t)((uint64_t)rows * i / n_threads),
                                  row0 + (uint32_t)((uint64_t)rows * (i + 1) / n_threads)};
            if (pass == 1) {
                /* the shadow pass reads output rows; primary pixel row y was
                 * written to output row H-1-y */
                uint32_t a = H - jobs[i].r1, b = H - jobs[i].r0;
                jobs[i].r0 = a;
                jobs[i].r1 = b;
            }
            pthread_create(&th[i], NULL, pass == 0 ? frame_worker : shadow_worker, &jobs[i]);
        }
        for (uint32_t i = 0; i < n_threads; i++)
            pthread_join(th[i], NULL);
    }
}

/* ======================================================================
 * Colours: CompressedColor and the colour conversions (color_utils.h,
 * variable_weight_size_colors.h:86-155), ColorLeafBuilder (:557-689),
 * CompressedColorLeaf decoding (:343-551) with CFG_COLOR_SWAP_BYTE_ORDER=1
 * (typedefs.h:516), the HashDAGColors tree (hash_dag_colors.h:24-55).
 * ====================================================================== */

#define CPM 16384u /* CColorsPerMacroBlock (variable_weight_size_colors.h:8) */
#define LEAF_FLAG 0x80000000u /* Utils::set_flag (utils.h:37-51) */

static float clampf(float f, float a, float b) { return f < a ? a : f > b ? b : f; }

/* ColorUtils (color_utils.h:9-75) */
static uint16_t f3_to_rgb565(f3 c)
{
    const float r = clampf(c.x, 0.f, 1.f), g = clampf(c.y, 0.f, 1.f), b = clampf(c.z, 0.f, 1.f);
    return (uint16_t)(((uint16_t)(r * 31.0f) << 0) | ((uint16_t)(g * 63.0f) << 5) | ((uint16_t)(b * 31.0f) << 11));
}
static f3 rgb565_to_f3(uint16_t v)
{
    return (f3){(float)((v >> 0) & 0x1F) / 31.0f, (float)((v >> 5) & 0x3F) / 63.0f, (float)((v >> 11) & 0x1F) / 31.0f};
}
static uint32_t f3_to_rgb101210(f3 c)
{
    const float r = clampf(c.x, 0.f, 1.f), g = clampf(c.y, 0.f, 1.f), b = clampf(c.z, 0.f, 1.f);
    return ((uint32_t)(r * 1023.0f) << 0) | ((uint32_t)(g * 4095.0f) << 10) | ((uint32_t)(b * 1023.0f) << 22);
}
static f3 rgb101210_to_f3(uint32_t v)
{
    return (f3){(float)((v >> 0) & 0x3FF) / 1023.0f, (float)((v >> 10) & 0xFFF) / 4095.0f,
                (float)((v >> 22) & 0x3FF) / 1023.0f};
}
uint32_t or_f3_to_rgb888(float x, float y, float z)
{
    const float r = clampf(x, 0.f, 1.f), g = clampf(y, 0.f, 1.f), b = clampf(z, 0.f, 1.f);
    return ((uint32_t)(r * 255.0f) << 0) | ((uint32_t)(g * 255.0f) << 8) | ((uint32_t)(b * 255.0f) << 16) |
           0xff000000u;
}
/* CompressedColor::set_single_color / get_color (:127-154); lerp is
 * a * (1 - f) + b * f (cuda_math.h:22) */
static hd_color single_color(f3 c)
{
    hd_color k;
    memset(&k, 0, sizeof(k));
    k.color_bits = f3_to_rgb101210(c);
    return k;
}
static f3 color_value(hd_color k)
{
    if (k.bits_per_weight == 0)
        return rgb101210_to_f3(k.color_bits);
    const f3 lo = rgb565_to_f3((uint16_t)(k.color_bits & 0xFFFF));
    const f3 hi = rgb565_to_f3((uint16_t)((k.color_bits >> 16) & 0xFFFF));
    const float w = (float)k.weight / (float)((1 << k.bits_per_weight) - 1);
    return (f3){lo.x * (1 - w) + hi.x * w, lo.y * (1 - w) + hi.y * w, lo.z * (1 - w) + hi.z * w};
}
uint32_t or_color_rgb888(hd_color k)
{
    const f3 c = color_value(k);
    return or_f3_to_rgb888(c.x, c.y, c.z);
}

/* Scene colours: RGB8 from a seeded value-noise field sampled on an aligned
 * 8^3 grid (lattice period 16 cells, trilinear with integer weights), each
 * voxel stored as set_single_color(rgb / 255). */
static uint32_t color_lattice(uint64_t seed, uint32_t c, uint32_t i, uint32_t j, uint32_t k)
{
    return (uint32_t)(mix64(seed ^ mix64(((uint64_t)c << 60) ^ ((uint64_t)i << 40) ^ ((uint64_t)j << 20) ^ k)) >> 56);
}
uint32_t or_color_rgb8(uint64_t seed, uint32_t x, uint32_t y, uint32_t z)
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
                    acc += color_lattice(seed, c, i + a, j + b, k + d) * w;
                }
        out |= ((acc + 2048) >> 12) << (8 * c);
    }
    return out;
}
hd_color or_voxel_color(uint64_t seed, uint32_t x, uint32_t y, uint32_t z)
{
    const uint32_t rgb = or_color_rgb8(seed, x, y, z);
    return single_color((f3){(float)(rgb & 0xFF) / 255.0f, (float)((rgb >> 8) & 0xFF) / 255.0f,
                             (float)((rgb >> 16) & 0xFF) / 255.0f});
}

/* CompressedColorLeaf, always unique here: blocks (colour bits << 32 |
 * header), byte-swapped weight words, macro blocks (first block, weight
 * offset) */
typedef struct {
    uint64_t* blocks;
    uint64_t nb;
    uint32_t* weights; /* + one padding word: extract_bits reads two bytes */
    uint64_t nw;
    uint64_t* macros; /* 2 words per macro block */
    uint64_t nm;      /* words */
} or_leaf;

/* ColorLeafBuilder (:557-689) */
typedef struct {
    uint32_t bits, color_bits, weight_offset, index;
} bblock;
typedef struct {
    uint32_t start_weight, start_block;
} bmacro;
typedef struct {
    bblock* blocks;
    uint64_t nb, cb;
    uint32_t* weights;
    uint64_t nw, cw;
    bmacro* macros;
    uint64_t nm, cm;
    uint32_t num_weights, target_bit_pos, color_index, last_bits, last_color_bits, last_macro_color,
        last_macro_weight;
} or_builder;

#define GROW(ptr, n, cap, T)                                                \
    do {                                                                    \
        if ((n) == (cap)) {                                                 \
            (cap) = (cap) ? 2 * (cap) : 16;                                 \
            (ptr) = (T*)realloc((ptr), (size_t)(cap) * sizeof(T));          \
        }                                                                   \
    } while (0)

static void builder_free(or_builder* b)
{
    free(b->blocks);
    free(b->weights);
    free(b->macros);
    memset(b, 0, sizeof(*b));
}
static void add_weight(or_builder* b, uint32_t weight, uint32_t bits)
{
    const uint32_t target = (b->target_bit_pos + 32 - bits) % 64;
    const uint64_t ww = (uint64_t)weight << target;
    if (target > (uint32_t)(32 - bits)) {
        b->weights[b->nw - 1] |= (uint32_t)(ww >> 32);
        b->target_bit_pos -= bits;
    }
    if (target < 32) {
        GROW(b->weights, b->nw, b->cw, uint32_t);
        b->weights[b->nw++] = (uint32_t)(ww & 0xFFFFFFFFu);
        b->target_bit_pos = target;
    }
    b->num_weights += bits;
}
static void builder_add(or_builder* b, hd_color k)
{
    if (b->color_index % CPM == 0) {
        b->last_macro_color = b->color_index;
        b->last_macro_weight = b->num_weights;
        GROW(b->macros, b->nm, b->cm, bmacro);
        b->macros[b->nm++] = (bmacro){b->num_weights, (uint32_t)b->nb};
    }
    if (b->color_index % CPM == 0 || b->last_color_bits != k.color_bits || b->last_bits != k.bits_per_weight) {
        b->last_color_bits = k.color_bits;
        b->last_bits = k.bits_per_weight;
        GROW(b->blocks, b->nb, b->cb, bblock);
        b->blocks[b->nb++] = (bblock){k.bits_per_weight, k.color_bits, b->num_weights - b->last_macro_weight,
                                      b->color_index - b->last_macro_color};
    }
    if (k.bits_per_weight > 0)
        add_weight(b, k.weight, k.bits_per_weight);
    b->color_index++;
}
/* add_large_single_color (:626-656) */
static void builder_add_large(or_builder* b, f3 c, uint32_t n)
{
    const hd_color k = single_color(c);
    uint32_t left = n;
    while (left > 0) {
        const uint32_t in_macro = CPM - (b->color_index % CPM);
        const uint32_t add = in_macro < left ? in_macro : left;
        left -= add;
        builder_add(b, k);
        b->color_index += add - 1;
    }
}
static uint32_t swap32(uint32_t v)
{
    return ((v & 0xffu) << 24) | ((v & 0xff00u) << 8) | ((v & 0xff0000u) >> 8) | ((v & 0xff000000u) >> 24);
}
/* VariableColorsUtils::make_block_header (:31-52) */
static uint32_t make_block_header(uint32_t weight_offset, uint32_t bits, uint32_t index)
{
    if (bits == 0)
        weight_offset = 0xFFFF;
    else
        bits--;
    return (weight_offset << 16) | (bits << 14) | index;
}
/* ColorLeafBuilder::build (:658-689) */
static void builder_build(const or_builder* b, or_leaf* leaf)
{
    leaf->nb = b->nb;
    leaf->blocks = (uint64_t*)malloc((b->nb + 1) * 8);
    for (uint64_t i = 0; i < b->nb; i++)
        leaf->blocks[i] = ((uint64_t)b->blocks[i].color_bits << 32) |
                          make_block_header(b->blocks[i].weight_offset, b->blocks[i].bits, b->blocks[i].index);
    leaf->nw = b->nw;
    leaf->weights = (uint32_t*)calloc(b->nw + 1, 4);
    for (uint64_t i = 0; i < b->nw; i++)
        leaf->weights[i] = swap32(b->weights[i]);
    leaf->nm = 2 * b->nm;
    leaf->macros = (uint64_t*)malloc((leaf->nm + 1) * 8);
    for (uint64_t i = 0; i < b->nm; i++) {
        leaf->macros[2 * i + 0] = b->macros[i].start_block;
        leaf->macros[2 * i + 1] = b->macros[i].start_weight;
    }
}

/* VariableColorsUtils header fields (:10-30) */
static uint32_t hdr_index(uint32_t h) { return h & (CPM - 1); }
static uint32_t hdr_weight_offset(uint32_t h) { return h >> 16; }
static uint32_t hdr_bits(uint32_t h) { return hdr_weight_offset(h) == 0xFFFF ? 0 : ((h >> 14) & 3) + 1; }

/* ColorUtils::extract_bits, byte-swapped layout (color_utils.h:115-145) */
static uint32_t extract_bits(uint32_t bits, const uint32_t* words, uint64_t bit_ptr)
{
    if (bits == 0)
        return 0;
    const uint8_t* bytes = (const uint8_t*)words;
    const uint64_t byte = bit_ptr / 8;
    uint16_t dst = (uint16_t)(bytes[byte] | ((uint16_t)bytes[byte + 1] << 8));
    dst = (uint16_t)((dst << 8) | (dst >> 8));
    const uint32_t shift = 16 - bits - (uint32_t)(bit_ptr % 8);
    return (uint32_t)((dst >> shift) & ((1u << bits) - 1));
}
/* binary_search_blocks (:414-443) */
static uint32_t leaf_search(const or_leaf* l, uint64_t ci)
{
    const uint32_t local = (uint32_t)(ci % CPM);
    const uint64_t m = ci / CPM;
    uint32_t lo = (uint32_t)l->macros[2 * m];
    uint32_t hi = 2 * (m + 1) < l->nm ? (uint32_t)l->macros[2 * (m + 1)] - 1 : (uint32_t)(l->nb - 1);
    uint32_t pos = (lo + hi) / 2;
    uint32_t h = (uint32_t)l->blocks[pos];
    while (hdr_index(h) != local && lo <= hi) {
        if (hdr_index(h) > local)
            hi = pos - 1;
        else
            lo = pos + 1;
        pos = (lo + hi) / 2;
        h = (uint32_t)l->blocks[pos];
    }
    return pos;
}
/* get_color_for_block / get_color (:445-486) */
static hd_color leaf_color(const or_leaf* l, uint64_t ci)
{
    const uint32_t pos = leaf_search(l, ci);
    const uint64_t block = l->blocks[pos];
    const uint32_t h = (uint32_t)block;
    hd_color k;
    memset(&k, 0, sizeof(k));
    k.color_bits = (uint32_t)(block >> 32);
    k.bits_per_weight = (uint8_t)hdr_bits(h);
    if (k.bits_per_weight) {
        const uint64_t local = ci % CPM, m = ci / CPM;
        const uint64_t wi = l->macros[2 * m + 1] + hdr_weight_offset(h) + (local - hdr_index(h)) * k.bits_per_weight;
        k.weight = (uint8_t)extract_bits(k.bits_per_weight, l->weights, wi);
    }
    return k;
}
static int leaf_valid_index(const or_leaf* l, uint64_t ci) { return l && l->blocks && 2 * ci / CPM < l->nm; }

/* HashDAGColors: interior colour nodes of 8 entries; an entry with
 * LEAF_FLAG is a leaf index.  Every leaf here is unique (the reference's
 * import shares one main leaf through offsets; decoded colours are the
 * same). */
struct or_colors {
    uint32_t* nodes;
    uint64_t n_nodes, cap_nodes;
    or_leaf* leaves;
    uint64_t n_leaves, cap_leaves;
    /* HashDAGUndoRedo (hash_dag.h:20-212) */
    struct frame {
        uint32_t root;
        uint32_t n;
        uint32_t* index;
        or_leaf* prev;
        or_leaf* next;
    } *undo, *redo;
    uint64_t n_undo, cap_undo, n_redo, cap_redo;
};

static uint32_t colors_alloc_node(or_colors* c)
{
    for (int k = 0; k < 8; k++) {
        GROW(c->nodes, c->n_nodes, c->cap_nodes, uint32_t);
        c->nodes[c->n_nodes++] = 0;
    }
    return (uint32_t)(c->n_nodes - 8);
}
static uint32_t colors_alloc_leaf(or_colors* c)
{
    GROW(c->leaves, c->n_leaves, c->cap_leaves, or_leaf);
    memset(&c->leaves[c->n_leaves], 0, sizeof(or_leaf));
    return (uint32_t)(c->n_leaves++) | LEAF_FLAG;
}

/* ======================================================================
 * Editors (hash_dag_editors.h) and the edit recursion (hash_dag_edits.h)
 * ====================================================================== */

typedef struct {
    uint32_t tool;
    f3 c;        /* sphere centre */
    float r, r2; /* radius, radius * radius (SphereEditorBase, :99-110) */
    f3 bmin, bmax; /* box bounds (BoxEditorBase, :57-75) */
    f3 paint;    /* SpherePaintEditor's target colour (the reference: blue) */
    /* CopyEditorWithDecompression (:437-609): source / dest, the source
     * region's lower corner (copyMin) and its occupancy and colours read
     * before the edit (values / colors, size^3, x fastest) */
    f3 src, dst, copy_min;
    uint32_t size;
    uint8_t* values;
    hd_color* colors;
    /* BufferEditor (:129-221) tools (noise, fill): the buffer's lower corner
     * (BoxEditorBase::min), its radius (BoxEditorBase::radius: 1.5 r for the
     * noise tool), the EValues of the size^3 buffer (x fastest), the table
     * it reads (get_value at get_world_path) and, for the fill, the colour of
     * each set voxel */
    f3 buf_min;
    float buf_r;
    uint8_t* state;
    const or_table* dag;
} editor;

static int make_buffers(editor* e, const or_table* t, const or_colors* col);

static editor make_editor(const hd_edit* e)
{
    editor ed;
    memset(&ed, 0, sizeof(ed));
    ed.tool = e->tool;
    ed.c = (f3){e->center[0], e->center[1], e->center[2]};
    ed.r = e->radius;
    ed.r2 = e->radius * e->radius;
    f3 bc = ed.c;
    if (e->tool == HD_TOOL_COPY) {
        /* BoxEditorBase(center - source + dest, radius) */
        ed.src = (f3){e->source[0], e->source[1], e->source[2]};
        ed.dst = (f3){e->dest[0], e->dest[1], e->dest[2]};
        bc = (f3){ed.c.x - ed.src.x + ed.dst.x, ed.c.y - ed.src.y + ed.dst.y, ed.c.z - ed.src.z + ed.dst.z};
        ed.copy_min = (f3){ed.c.x - ed.r, ed.c.y - ed.r, ed.c.z - ed.r};
        ed.size = 2 * (uint32_t)ceilf(ed.r);
    }
    float br = e->radius;
    if (e->tool == HD_TOOL_NOISE_ADD || e->tool == HD_TOOL_NOISE_REMOVE)
        br = 1.5f * e->radius; /* BufferEditor(dag, center, 1.5f * radius) (:716) */
    if (e->tool >= HD_TOOL_NOISE_REMOVE) {
        ed.buf_r = br;
        ed.buf_min = (f3){bc.x - br, bc.y - br, bc.z - br};
        ed.size = 2 * (uint32_t)ceilf(br);
    }
    ed.bmin = (f3){bc.x - br, bc.y - br, bc.z - br};
    ed.bmax = (f3){bc.x + br, bc.y + br, bc.z + br};
    ed.paint = (f3){(float)(e->rgb & 0xFF) / 255.0f, (float)((e->rgb >> 8) & 0xFF) / 255.0f,
                    (float)((e->rgb >> 16) & 0xFF) / 255.0f};
    return ed;
}
static int is_sphere(const editor* e)
{
    return e->tool == HD_TOOL_SPHERE_ADD || e->tool == HD_TOOL_SPHERE_REMOVE || e->tool == HD_TOOL_SPHERE_PAINT;
}
static int is_adding(const editor* e) { return e->tool == HD_TOOL_SPHERE_ADD || e->tool == HD_TOOL_BOX_ADD; }
/* is_full / is_empty exist for the sphere and box editors only (the base
 * Editor returns false, :30-37) */
static int has_shortcuts(const editor* e) { return e->tool <= HD_TOOL_BOX_ADD; }
/* get_single_color (:256-259, :297-300) */
static f3 single_of(const editor* e) { return is_sphere(e) ? (f3){1, 0, 0} : (f3){1, 0, 1}; }
/* the copy tool's source index of a destination voxel, or -1 (:585-606) */
static int64_t copy_index(const editor* e, f3 pos)
{
    const f3 q = {((pos.x - e->dst.x) + e->src.x) - e->copy_min.x, ((pos.y - e->dst.y) + e->src.y) - e->copy_min.y,
                  ((pos.z - e->dst.z) + e->src.z) - e->copy_min.z};
    const uint32_t px = (uint32_t)(q.x < 0 ? 0 : q.x), py = (uint32_t)(q.y < 0 ? 0 : q.y),
                   pz = (uint32_t)(q.z < 0 ? 0 : q.z);
    if (px >= e->size || py >= e->size || pz >= e->size)
        return -1;
    return (int64_t)px + (int64_t)e->size * py + (int64_t)e->size * e->size * pz;
}

static float sq(float f) { return f * f; }

/* SphereEditorBase::should_edit_impl (:112-126), BoxEditorBase (:76-91) */
static int should_edit_impl(const editor* e, f3 mn, f3 mx)
{
    if (is_sphere(e)) {
        float dist = e->r2;
        if (e->c.x < mn.x) dist -= sq(e->c.x - mn.x);
        else if (e->c.x > mx.x) dist -= sq(e->c.x - mx.x);
        if (e->c.y < mn.y) dist -= sq(e->c.y - mn.y);
        else if (e->c.y > mx.y) dist -= sq(e->c.y - mx.y);
        if (e->c.z < mn.z) dist -= sq(e->c.z - mn.z);
        else if (e->c.z > mx.z) dist -= sq(e->c.z - mx.z);
        return dist > 0;
    }
    return !(e->bmin.x >= mx.x || e->bmin.y >= mx.y || e->bmin.z >= mx.z || e->bmax.x <= mn.x ||
             e->bmax.y <= mn.y || e->bmax.z <= mn.z || mn.x >= e->bmax.x || mn.y >= e->bmax.y ||
             mn.z >= e->bmax.z || mx.x <= e->bmin.x || mx.y <= e->bmin.y || mx.z <= e->bmin.z);
}
/* SphereEditor::is_full_impl/is_empty_impl (:280-295), BoxEditor (:233-252):
 * the region is inside the tool */
static int inside_tool(const editor* e, f3 mn, f3 mx)
{
    if (is_sphere(e)) {
        const float a = fmaxr(sq(mn.x - e->c.x), sq(mx.x - e->c.x));
        const float b = fmaxr(sq(mn.y - e->c.y), sq(mx.y - e->c.y));
        const float c = fmaxr(sq(mn.z - e->c.z), sq(mx.z - e->c.z));
        return (a + b) + c < e->r2;
    }
    return e->bmin.x <= mn.x && e->bmin.y <= mn.y && e->bmin.z <= mn.z && e->bmax.x >= mx.x &&
           e->bmax.y >= mx.y && e->bmax.z >= mx.z;
}

/* Editor::should_edit/is_full/is_empty on the node AABB (:12-27) */
static void node_box(const uint32_t path[3], uint32_t depth, f3* mn, f3* mx)
{
    *mn = (f3){(float)(path[0] << depth), (float)(path[1] << depth), (float)(path[2] << depth)};
    const float s = (float)(1u << depth);
    *mx = (f3){mn->x + s, mn->y + s, mn->z + s};
}

typedef struct {
    or_table* t;
    editor ed;
    uint64_t num_voxels, num_nodes;
    /* colours (NULL: off): the current task's builder, its old leaf and
     * the running oldLeavesCount (LeafEditParameters, hash_dag_edits.h:67-78) */
    or_colors* col;
    or_builder* b;
    const or_leaf* old;
    uint64_t old_count;
    /* rebuilt leaves of this edit, for the undo frame */
    uint32_t n_diff, cap_diff;
    uint32_t* diff_index;
    or_leaf* diff_prev;
    or_leaf* diff_next;
} edit_job;

static hd_color prev_color(edit_job* j, int prev)
{
    hd_color k;
    memset(&k, 0, sizeof(k));
    if (prev && j->old && leaf_valid_index(j->old, j->old_count))
        k = leaf_color(j->old, j->old_count);
    return k;
}
/* truncate(float3) (cuda_math.h:80) of a float that may be negative, as the
 * reference's x86-64 build converts it: to a 64-bit integer toward zero,
 * then its low 32 bits (so (-1, 0) gives 0 and anything below -1 a huge
 * index) */
static uint32_t trunc_u32(float f) { return (uint32_t)(int64_t)f; }

/* BufferEditor's EValues (:134-141) */
enum { EV_UNKNOWN = 0, EV_LOADED_TRUE = 1, EV_LOADED_FALSE = 2, EV_SET_TRUE = 3, EV_SET_FALSE = 4 };

static uint64_t buf_index(const editor* e, uint32_t x, uint32_t y, uint32_t z)
{
    return (uint64_t)x + (uint64_t)e->size * y + (uint64_t)e->size * e->size * z;
}
/* BufferEditor::get_world_path (:159-164) */
static void buf_world(const editor* e, uint32_t x, uint32_t y, uint32_t z, uint32_t w[3])
{
    w[0] = trunc_u32(e->buf_min.x + (float)x);
    w[1] = trunc_u32(e->buf_min.y + (float)y);
    w[2] = trunc_u32(e->buf_min.z + (float)z);
}
/* BufferEditor::get_value (:185-195): Unknown loads the table's voxel */
static int buf_get(const editor* e, uint32_t x, uint32_t y, uint32_t z)
{
    const uint64_t i = buf_index(e, x, y, z);
    if (e->state[i] == EV_UNKNOWN) {
        /* the table as it was when the editor was made: the root changes
         * only once the edit is done */
        uint32_t w[3];
        buf_world(e, x, y, z, w);
        e->state[i] = or_get_value(e->dag, w[0], w[1], w[2]) ? EV_LOADED_TRUE : EV_LOADED_FALSE;
    }
    return e->state[i] == EV_LOADED_TRUE || e->state[i] == EV_SET_TRUE;
}
/* BufferEditor::get_new_value (:211-220): `get_value(p) == EValues::Unknown`
 * compares a bool with 0, so a voxel reads true only when set or loaded
 * true, and a false one keeps its old value */
static int buf_new_value(const editor* e, f3 pos, int prev)
{
    const uint32_t p[3] = {trunc_u32(pos.x - e->buf_min.x), trunc_u32(pos.y - e->buf_min.y),
                           trunc_u32(pos.z - e->buf_min.z)};
    if (p[0] >= e->size || p[1] >= e->size || p[2] >= e->size)
        return prev;
    return buf_get(e, p[0], p[1], p[2]) ? 1 : prev;
}

static int new_value(const editor* e, f3 pos, int prev)
{
    if (e->tool >= HD_TOOL_NOISE_REMOVE)
        return buf_new_value(e, pos, prev);
    if (e->tool == HD_TOOL_SPHERE_PAINT)
        return prev;
    if (e->tool == HD_TOOL_COPY) {
        if (prev)
            return prev;
        const int64_t i = copy_index(e, pos);
        return i < 0 ? prev : e->values[i];
    }
    return is_adding(e);
}
/* get_new_color of each editor (:262-269, :302-312, :323-329, :595-608) */
static hd_color new_color(edit_job* j, f3 pos, int prev, int nv)
{
    const editor* e = &j->ed;
    if (e->tool == HD_TOOL_SPHERE_PAINT) {
        const f3 old = color_value(prev_color(j, prev));
        const f3 d = {pos.x - e->c.x, pos.y - e->c.y, pos.z - e->c.z};
        const float len = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
        const float f = clampf(1 - len / e->r, 0.f, .1f);
        return single_color((f3){old.x * (1 - f) + e->paint.x * f, old.y * (1 - f) + e->paint.y * f,
                                 old.z * (1 - f) + e->paint.z * f});
    }
    if (e->tool == HD_TOOL_COPY) {
        if (prev == nv || !nv)
            return prev_color(j, prev);
        const int64_t i = copy_index(e, pos);
        return i < 0 ? prev_color(j, prev) : e->colors[i];
    }
    if (e->tool == HD_TOOL_NOISE_ADD || e->tool == HD_TOOL_NOISE_REMOVE) {
        /* SphereNoiseEditor::get_new_color (:745-758) */
        if (prev == nv)
            return prev_color(j, prev);
        hd_color k;
        memset(&k, 0, sizeof(k));
        k.bits_per_weight = 3;
        k.color_bits = (uint32_t)f3_to_rgb565((f3){94 / 255.f, 30 / 255.f, 0 / 255.f}) |
                       ((uint32_t)f3_to_rgb565((f3){125 / 255.f, 100 / 255.f, 89 / 255.f}) << 16);
        const f3 d = {pos.x - e->c.x, pos.y - e->c.y, pos.z - e->c.z};
        const float len = (float)sqrt((double)(d.x * d.x + d.y * d.y + d.z * d.z));
        const int32_t w = (int32_t)((len / e->buf_r - 0.3f) * (float)((1 << 3) - 1));
        k.weight = (uint8_t)(w < 0 ? 0 : w > 7 ? 7 : w);
        return k;
    }
    if (e->tool == HD_TOOL_FILL) {
        /* FillEditorColors::get_new_color (:693-709) */
        if (nv && !prev) {
            const uint32_t p[3] = {trunc_u32(pos.x - e->buf_min.x), trunc_u32(pos.y - e->buf_min.y),
                                   trunc_u32(pos.z - e->buf_min.z)};
            if (p[0] < e->size && p[1] < e->size && p[2] < e->size) {
                const uint64_t i = buf_index(e, p[0], p[1], p[2]);
                if (e->state[i] == EV_SET_TRUE)
                    return e->colors[i];
            }
        }
        return prev_color(j, prev);
    }
    return single_color(single_of(e));
}

static void descend(const uint32_t in[3], uint32_t c, uint32_t out[3])
{
    out[0] = (in[0] << 1) | ((c >> 2) & 1);
    out[1] = (in[1] << 1) | ((c >> 1) & 1);
    out[2] = (in[2] << 1) | (c & 1);
}

/* HashDagEdits::edit_leaf (hash_dag_edits.h:335-643), colours off */
static uint32_t edit_leaf(edit_job* j, uint32_t level, uint32_t index, const uint32_t path[3], uint32_t* count_out)
{
    or_table* t = j->t;
    const uint32_t D = t->cfg.depth, leafl = t->leaf_level;
    j->num_nodes++;
    f3 mn, mx;
    node_box(path, D - level, &mn, &mx);
    const uint32_t full_count = 1u << (3 * (D - level));
    uint32_t old_count = 0;
    if (index != INVALID) {
        const uint32_t* p = sys_ptr(t, index);
        old_count = level < leafl ? p[0] >> 8 : popc32(p[0]) + popc32(p[1]);
    }
    if (!should_edit_impl(&j->ed, mn, mx)) {
        if (j->b && index != INVALID) { /* copy_colors (:380-392) */
            for (uint32_t k = 0; k < old_count; k++)
                builder_add(j->b, prev_color(j, 1)), j->old_count++;
        }
        *count_out = old_count;
        return index;
    }
    const int inside = has_shortcuts(&j->ed) && inside_tool(&j->ed, mn, mx);
    if (!is_adding(&j->ed) && inside) { /* is_empty */
        j->num_voxels += full_count;
        if (j->b)
            j->old_count += old_count;
        *count_out = 0;
        return INVALID;
    }
    if (is_adding(&j->ed) && inside) { /* is_full */
        j->num_voxels += full_count;
        if (j->b) {
            j->old_count += old_count;
            builder_add_large(j->b, single_of(&j->ed), full_count);
        }
        *count_out = full_count;
        return t->full[level];
    }
    if (level == leafl) {
        uint64_t leaf = 0;
        if (index != INVALID) {
            const uint32_t* p = sys_ptr(t, index);
            leaf = (uint64_t)p[0] | ((uint64_t)p[1] << 32);
        }
        const uint64_t initial = leaf;
        for (uint32_t c1 = 0; c1 < 8; c1++) {
            uint32_t p1[3];
            descend(path, c1, p1);
            for (uint32_t c2 = 0; c2 < 8; c2++) {
                uint32_t p2[3];
                descend(p1, c2, p2);
                const f3 pos = {(float)p2[0], (float)p2[1], (float)p2[2]};
                const f3 pos1 = {pos.x + 1.0f, pos.y + 1.0f, pos.z + 1.0f};
                const uint64_t bit = 1ull << (c1 * 8 + c2);
                const int se = should_edit_impl(&j->ed, pos, pos1);
                const int prev = (leaf & bit) != 0;
                const int nv = se ? new_value(&j->ed, pos, prev) : prev;
                j->num_voxels += (uint64_t)se;
                if (j->b) {
                    if (nv)
                        builder_add(j->b, se ? new_color(j, pos, prev, nv) : prev_color(j, prev));
                    j->old_count += (uint64_t)prev;
                }
                if (prev != nv) {
                    if (nv)
                        leaf |= bit;
                    else
                        leaf &= ~bit;
                }
            }
        }
        if (leaf == initial) {
            *count_out = popc64(leaf);
            return index;
        }
        if (leaf == 0) {
            *count_out = 0;
            return INVALID;
        }
        *count_out = popc64(leaf);
        return or_find_or_add_leaf(t, leaf);
    }
    uint32_t mask = 0;
    const uint32_t* p = NULL;
    if (index != INVALID) {
        p = sys_ptr(t, index);
        mask = p[0] & 0xffu;
    }
    uint32_t off = 1, kids[8], total = 0;
    int changed = 0;
    for (uint32_t c = 0; c < 8; c++) {
        uint32_t np[3];
        descend(path, c, np);
        const uint32_t old = (mask & (1u << c)) ? p[off++] : INVALID;
        uint32_t cc;
        const uint32_t nk = edit_leaf(j, level + 1, old, np, &cc);
        if (t->error)
            return INVALID;
        if (nk != INVALID)
            total += cc;
        changed |= old != nk;
        kids[c] = nk;
        if (index != INVALID)
            p = sys_ptr(t, index); /* unchanged by appends; kept explicit */
    }
    *count_out = total;
    if (!changed)
        return index;
    uint32_t node[9], n = 0;
    node[n++] = total << 8;
    for (uint32_t c = 0; c < 8; c++)
        if (kids[c] != INVALID) {
            node[n++] = kids[c];
            node[0] |= 1u << c;
        }
    if ((node[0] & 0xffu) == 0) {
        *count_out = 0;
        return INVALID;
    }
    return or_find_or_add_interior(t, level, n, node);
}

#define COLOR_IGNORE 0xFFFFFFFu /* HashDagEdits::C_IgnoreColorIndex (hash_dag_edits.h:15) */

static void push_diff(edit_job* j, uint32_t leaf_ref, const or_leaf* prev, const or_leaf* next)
{
    if (j->n_diff == j->cap_diff) {
        j->cap_diff = j->cap_diff ? 2 * j->cap_diff : 16;
        j->diff_index = (uint32_t*)realloc(j->diff_index, j->cap_diff * 4);
        j->diff_prev = (or_leaf*)realloc(j->diff_prev, j->cap_diff * sizeof(or_leaf));
        j->diff_next = (or_leaf*)realloc(j->diff_next, j->cap_diff * sizeof(or_leaf));
    }
    j->diff_index[j->n_diff] = leaf_ref;
    j->diff_prev[j->n_diff] = *prev;
    j->diff_next[j->n_diff] = *next;
    j->n_diff++;
}

/* HashDagEdits::edit_threaded (hash_dag_edits.h:106-333) with both passes
 * folded into one depth-first recursion (tasks run in depth-first order;
 * each task owns one colour leaf, so running it in place is the same as
 * running it between the passes).  cn: this node's colour node (0 = none,
 * except at the root); *cn_out: the colour index reported to the parent. */
static uint32_t edit_top(edit_job* j, uint32_t level, uint32_t index, const uint32_t path[3], uint32_t cn,
                         uint32_t* cn_out)
{
    or_table* t = j->t;
    const uint32_t D = t->cfg.depth, T = t->cfg.color_tree_levels;
    or_colors* col = j->col;
    /* the reference runs this recursion twice (queue pass, build pass) and
     * counts the node in both (hash_dag_edits.h:120, hash_dag.h:287, :358) */
    j->num_nodes += 2;
    f3 mn, mx;
    node_box(path, D - level, &mn, &mx);
    if (!should_edit_impl(&j->ed, mn, mx)) {
        *cn_out = COLOR_IGNORE;
        return index;
    }
    uint32_t mask = 0;
    const uint32_t* p = NULL;
    if (index != INVALID) {
        p = sys_ptr(t, index);
        mask = p[0] & 0xffu;
    }
    uint32_t off = 1, kids[8];
    int changed = 0;
    for (uint32_t c = 0; c < 8; c++) {
        uint32_t np[3];
        descend(path, c, np);
        const uint32_t old = (mask & (1u << c)) ? p[off++] : INVALID;
        uint32_t ccn = 0;
        if (col && (level == 0 || cn > 0))
            ccn = col->nodes[cn + c];
        uint32_t nk;
        if (level == T - 1) {
            f3 cmn, cmx;
            node_box(np, D - level - 1, &cmn, &cmx);
            if (should_edit_impl(&j->ed, cmn, cmx)) {
                uint32_t cc;
                if (col) {
                    or_builder b;
                    memset(&b, 0, sizeof(b));
                    const or_leaf* old_leaf = (ccn > 0 && (ccn & LEAF_FLAG)) ? &col->leaves[ccn & ~LEAF_FLAG] : NULL;
                    or_leaf prev;
                    memset(&prev, 0, sizeof(prev));
                    if (old_leaf)
                        prev = *old_leaf;
                    j->b = &b;
                    j->old = old_leaf ? &prev : NULL;
                    j->old_count = 0;
                    nk = edit_leaf(j, T, old, np, &cc);
                    j->b = NULL;
                    j->old = NULL;
                    if (b.color_index > 0) { /* hash_dag_edits.h:218-241 */
                        if (ccn == 0 || !(ccn & LEAF_FLAG)) {
                            if (cn == 0)
                                cn = colors_alloc_node(col);
                            ccn = colors_alloc_leaf(col);
                            col->nodes[cn + c] = ccn;
                        }
                        or_leaf next;
                        builder_build(&b, &next);
                        col->leaves[ccn & ~LEAF_FLAG] = next;
                        push_diff(j, ccn, &prev, &next);
                    }
                    builder_free(&b);
                } else {
                    nk = edit_leaf(j, T, old, np, &cc);
                }
            } else {
                nk = old;
            }
        } else {
            uint32_t child_cn;
            nk = edit_top(j, level + 1, old, np, ccn, &child_cn);
            if (col && child_cn != ccn && child_cn != COLOR_IGNORE) { /* :278-292 */
                if (level > 0 && cn == 0)
                    cn = colors_alloc_node(col);
                col->nodes[cn + c] = child_cn;
            }
        }
        if (t->error)
            return INVALID;
        changed |= old != nk;
        kids[c] = nk;
    }
    if (!changed) {
        *cn_out = cn;
        return index;
    }
    uint32_t node[9], n = 0;
    node[n++] = 0;
    for (uint32_t c = 0; c < 8; c++)
        if (kids[c] != INVALID) {
            node[n++] = kids[c];
            node[0] |= 1u << c;
        }
    if ((node[0] & 0xffu) == 0) {
        *cn_out = COLOR_IGNORE;
        return INVALID;
    }
    *cn_out = cn;
    return or_find_or_add_interior(t, level, n, node);
}

int or_edit(or_table* t, const hd_edit* e, hd_edit_stats* stats)
{
    edit_job j;
    memset(&j, 0, sizeof(j));
    j.t = t;
    j.ed = make_editor(e);
    t->foa_calls = t->nodes_added = t->words_scanned = 0;
    const uint32_t path[3] = {0, 0, 0};
    uint32_t root, cn;
    if (e->tool == HD_TOOL_SPHERE_PAINT || e->tool == HD_TOOL_COPY || e->tool > HD_TOOL_FILL)
        return HD_ERR_INVALID; /* paint and copy need colours */
    if (make_buffers(&j.ed, t, NULL))
        return HD_ERR_INVALID;
    if (t->cfg.color_tree_levels == 0) {
        uint32_t cc;
        root = edit_leaf(&j, 0, t->root, path, &cc);
    } else {
        root = edit_top(&j, 0, t->root, path, 0, &cn);
    }
    free(j.ed.state);
    free(j.ed.colors);
    if (!t->error)
        t->root = root;
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->num_voxels = j.num_voxels;
        stats->num_nodes = j.num_nodes;
        stats->find_or_add_calls = t->foa_calls;
        stats->nodes_added = t->nodes_added;
        stats->words_scanned = t->words_scanned;
    }
    return t->error;
}

/* ---- threaded edits (hash_dag.h:255-405 with THREADED_EDITS) ------------
 * The reference's edit_threads, multi-threaded: the first pass of
 * edit_threaded queues one task per level-T subtree the tool touches, a
 * pool of threads takes the tasks from an atomic counter (its NUM_THREADS
 * lambda, hash_dag.h:306-331) and runs edit_leaf on each, the hash table
 * shared under per-bucket locks (its ENABLE_THREAD_SAFE_HASHTABLE), and the
 * second pass combines the results into the top levels on one thread.
 * Which task appends first into a shared bucket depends on the threads, so
 * the table's node order (not its voxels) can differ from or_edit's; the
 * CPU timing baseline of the edit path uses it.  Geometry tools without
 * colours only. */
typedef struct {
    uint32_t old, path[3], result;
    uint64_t num_voxels, num_nodes;
} edit_task;

typedef struct {
    edit_task* v;
    uint64_t n, cap, cursor;
} edit_tasks;

static uint32_t edit_top_tasks(edit_job* j, uint32_t level, uint32_t index, const uint32_t path[3], edit_tasks* tl,
                               int build)
{
    or_table* t = j->t;
    const uint32_t D = t->cfg.depth, T = t->cfg.color_tree_levels;
    if (build)
        j->num_nodes += 2; /* both passes, as edit_top */
    f3 mn, mx;
    node_box(path, D - level, &mn, &mx);
    if (!should_edit_impl(&j->ed, mn, mx))
        return index;
    uint32_t mask = 0;
    const uint32_t* p = NULL;
    if (index != INVALID) {
        p = sys_ptr(t, index);
        mask = p[0] & 0xffu;
    }
    uint32_t off = 1, kids[8];
    int changed = 0;
    for (uint32_t c = 0; c < 8; c++) {
        uint32_t np[3];
        descend(path, c, np);
        const uint32_t old = (mask & (1u << c)) ? p[off++] : INVALID;
        uint32_t nk = old;
        if (level == T - 1) {
            f3 cmn, cmx;
            node_box(np, D - level - 1, &cmn, &cmx);
            if (should_edit_impl(&j->ed, cmn, cmx)) {
                if (!build) {
                    if (tl->n == tl->cap) {
                        tl->cap = tl->cap ? 2 * tl->cap : 64;
                        tl->v = (edit_task*)realloc(tl->v, tl->cap * sizeof(edit_task));
                    }
                    edit_task* k = &tl->v[tl->n++];
                    memset(k, 0, sizeof(*k));
                    k->old = old;
                    memcpy(k->path, np, sizeof(np));
                } else {
                    nk = tl->v[tl->cursor++].result;
                }
            }
        } else {
            nk = edit_top_tasks(j, level + 1, old, np, tl, build);
        }
        if (build && t->error)
            return INVALID;
        changed |= old != nk;
        kids[c] = nk;
    }
    if (!build || !changed)
        return index;
    uint32_t node[9], n = 0;
    node[n++] = 0;
    for (uint32_t c = 0; c < 8; c++)
        if (kids[c] != INVALID) {
            node[n++] = kids[c];
            node[0] |= 1u << c;
        }
    if ((node[0] & 0xffu) == 0)
        return INVALID;
    return or_find_or_add_interior(t, level, n, node);
}

typedef struct {
    const edit_job* proto;
    edit_tasks* tl;
    uint64_t* counter;
} edit_worker;

static void* edit_worker_run(void* arg)
{
    edit_worker* w = (edit_worker*)arg;
    const uint32_t T = w->proto->t->cfg.color_tree_levels;
    for (;;) {
        const uint64_t i = __atomic_fetch_add(w->counter, 1, __ATOMIC_RELAXED);
        if (i >= w->tl->n)
            return NULL;
        edit_task* k = &w->tl->v[i];
        edit_job j = *w->proto;
        j.num_voxels = j.num_nodes = 0;
        uint32_t cc;
        k->result = edit_leaf(&j, T, k->old, k->path, &cc);
        k->num_voxels = j.num_voxels;
        k->num_nodes = j.num_nodes;
    }
}

int or_edit_mt(or_table* t, const hd_edit* e, hd_edit_stats* stats, uint32_t threads)
{
    if (threads == 0)
        threads = (uint32_t)sysconf(_SC_NPROCESSORS_ONLN);
    if (threads <= 1 || e->tool > HD_TOOL_BOX_ADD || t->cfg.color_tree_levels == 0)
        return or_edit(t, e, stats);
    edit_job j;
    memset(&j, 0, sizeof(j));
    j.t = t;
    j.ed = make_editor(e);
    t->foa_calls = t->nodes_added = t->words_scanned = 0;
    if (make_buffers(&j.ed, t, NULL))
        return HD_ERR_INVALID;
    const uint32_t path[3] = {0, 0, 0};
    edit_tasks tl = {0};
    edit_top_tasks(&j, 0, t->root, path, &tl, 0); /* first pass: the tasks */
    t->locks = (uint8_t*)calloc(t->n_buckets, 1);
    uint64_t counter = 0;
    edit_worker w = {&j, &tl, &counter};
    pthread_t* th = (pthread_t*)malloc(threads * sizeof(pthread_t));
    uint32_t started = 0;
    for (; started < threads; started++)
        if (pthread_create(&th[started], NULL, edit_worker_run, &w))
            break;
    if (started == 0)
        edit_worker_run(&w);
    for (uint32_t i = 0; i < started; i++)
        pthread_join(th[i], NULL);
    free(th);
    free(t->locks);
    t->locks = NULL;
    for (uint64_t i = 0; i < tl.n; i++) {
        j.num_voxels += tl.v[i].num_voxels;
        j.num_nodes += tl.v[i].num_nodes;
    }
    uint32_t root = t->root;
    if (!t->error)
        root = edit_top_tasks(&j, 0, t->root, path, &tl, 1); /* second pass */
    free(tl.v);
    free(j.ed.state);
    free(j.ed.colors);
    if (!t->error)
        t->root = root;
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->num_voxels = j.num_voxels;
        stats->num_nodes = j.num_nodes;
        stats->find_or_add_calls = t->foa_calls;
        stats->nodes_added = t->nodes_added;
        stats->words_scanned = t->words_scanned;
    }
    return t->error;
}

/* ---- colour API ---------------------------------------------------- */

or_colors* or_colors_create(void) { return (or_colors*)calloc(1, sizeof(or_colors)); }

static void free_frames(struct frame* f, uint64_t n)
{
    for (uint64_t i = 0; i < n; i++) {
        free(f[i].index);
        free(f[i].prev);
        free(f[i].next);
    }
}
void or_colors_destroy(or_colors* c)
{
    if (!c)
        return;
    /* leaf arrays may be shared by undo frames and the tree; the oracle
     * keeps every leaf it ever built until the process ends */
    free_frames(c->undo, c->n_undo);
    free_frames(c->redo, c->n_redo);
    free(c->undo);
    free(c->redo);
    free(c->nodes);
    free(c->leaves);
    free(c);
}

static void leaf_voxels(const or_table* t, uint32_t level, uint32_t index, const uint32_t path[3], uint64_t seed,
                        or_builder* b)
{
    const uint32_t* p = sys_ptr(t, index);
    if (level == t->leaf_level) {
        const uint64_t leaf = (uint64_t)p[0] | ((uint64_t)p[1] << 32);
        for (uint32_t bit = 0; bit < 64; bit++) {
            if (!((leaf >> bit) & 1))
                continue;
            const uint32_t c1 = bit >> 3, c2 = bit & 7;
            const uint32_t x = (path[0] << 2) | (((c1 >> 2) & 1) << 1) | ((c2 >> 2) & 1);
            const uint32_t y = (path[1] << 2) | (((c1 >> 1) & 1) << 1) | ((c2 >> 1) & 1);
            const uint32_t z = (path[2] << 2) | ((c1 & 1) << 1) | (c2 & 1);
            builder_add(b, or_voxel_color(seed, x, y, z));
        }
        return;
    }
    const uint32_t mask = p[0] & 0xffu;
    uint32_t off = 1;
    for (uint32_t c = 0; c < 8; c++) {
        if (!(mask & (1u << c)))
            continue;
        uint32_t np[3];
        descend(path, c, np);
        leaf_voxels(t, level + 1, p[off++], np, seed, b);
    }
}
static uint32_t colors_tree(const or_table* t, or_colors* col, uint32_t level, uint32_t index, const uint32_t path[3],
                            uint64_t seed)
{
    const uint32_t T = t->cfg.color_tree_levels;
    const uint32_t cn = colors_alloc_node(col);
    const uint32_t* p = sys_ptr(t, index);
    const uint32_t mask = p[0] & 0xffu;
    uint32_t off = 1;
    for (uint32_t c = 0; c < 8; c++) {
        if (!(mask & (1u << c)))
            continue;
        const uint32_t child = sys_ptr(t, index)[off++];
        uint32_t np[3];
        descend(path, c, np);
        if (level == T - 1) {
            or_builder b;
            memset(&b, 0, sizeof(b));
            leaf_voxels(t, T, child, np, seed, &b);
            const uint32_t ref = colors_alloc_leaf(col);
            builder_build(&b, &col->leaves[ref & ~LEAF_FLAG]);
            builder_free(&b);
            col->nodes[cn + c] = ref;
        } else {
            const uint32_t sub = colors_tree(t, col, level + 1, child, np, seed);
            col->nodes[cn + c] = sub;
        }
    }
    return cn;
}
/* The colour tree of a freshly loaded scene: the tree's node layout of
 * create_hash_dag_colors (hash_dag_factory.cpp:100-147), with one unique leaf
 * per present level-T child holding its voxels' colours in depth-first
 * order (leaf voxels in bit order). */
int or_colors_from_scene(or_colors* col, const or_table* t, uint64_t color_seed)
{
    const uint32_t T = t->cfg.color_tree_levels;
    if (!col || col->n_nodes || T == 0 || T >= t->leaf_level || t->root == INVALID)
        return HD_ERR_INVALID;
    const uint32_t path[3] = {0, 0, 0};
    colors_tree(t, col, 0, t->root, path, color_seed);
    return HD_OK;
}

/* The same tree built by `threads` threads: the node and leaf slots are laid
 * out first in colors_tree's depth-first order (same indices), then the
 * leaves, independent of one another, are built in parallel. */
typedef struct {
    uint32_t slot, child, path[3];
} leaf_task;
typedef struct {
    leaf_task* v;
    uint64_t n, cap;
} leaf_tasks;

static uint32_t colors_tree_plan(const or_table* t, or_colors* col, uint32_t level, uint32_t index,
                                 const uint32_t path[3], leaf_tasks* tasks)
{
    const uint32_t T = t->cfg.color_tree_levels;
    const uint32_t cn = colors_alloc_node(col);
    const uint32_t* p = sys_ptr(t, index);
    const uint32_t mask = p[0] & 0xffu;
    uint32_t off = 1;
    for (uint32_t c = 0; c < 8; c++) {
        if (!(mask & (1u << c)))
            continue;
        const uint32_t child = sys_ptr(t, index)[off++];
        uint32_t np[3];
        descend(path, c, np);
        if (level == T - 1) {
            const uint32_t ref = colors_alloc_leaf(col);
            GROW(tasks->v, tasks->n, tasks->cap, leaf_task);
            tasks->v[tasks->n++] = (leaf_task){ref & ~LEAF_FLAG, child, {np[0], np[1], np[2]}};
            col->nodes[cn + c] = ref;
        } else {
            /* the call may grow (move) col->nodes: store after it */
            const uint32_t sub = colors_tree_plan(t, col, level + 1, child, np, tasks);
            col->nodes[cn + c] = sub;
        }
    }
    return cn;
}

typedef struct {
    const or_table* t;
    or_colors* col;
    const leaf_tasks* tasks;
    uint64_t seed;
    uint64_t* next;
} leaf_worker;

static void* leaf_worker_run(void* arg)
{
    leaf_worker* w = (leaf_worker*)arg;
    const uint32_t T = w->t->cfg.color_tree_levels;
    for (;;) {
        const uint64_t i = __atomic_fetch_add(w->next, 1, __ATOMIC_RELAXED);
        if (i >= w->tasks->n)
            break;
        const leaf_task* k = &w->tasks->v[i];
        or_builder b;
        memset(&b, 0, sizeof(b));
        leaf_voxels(w->t, T, k->child, k->path, w->seed, &b);
        builder_build(&b, &w->col->leaves[k->slot]);
        builder_free(&b);
    }
    return NULL;
}

int or_colors_from_scene_mt(or_colors* col, const or_table* t, uint64_t color_seed, uint32_t threads)
{
    const uint32_t T = t->cfg.color_tree_levels;
    if (!col || col->n_nodes || T == 0 || T >= t->leaf_level || t->root == INVALID)
        return HD_ERR_INVALID;
    if (threads == 0) {
        const long n = sysconf(_SC_NPROCESSORS_ONLN);
        threads = n > 0 ? (uint32_t)n : 1;
    }
    if (threads > 256)
        threads = 256;
    const uint32_t path[3] = {0, 0, 0};
    leaf_tasks tasks = {0};
    colors_tree_plan(t, col, 0, t->root, path, &tasks);
    uint64_t next = 0;
    pthread_t th[256];
    leaf_worker w = {t, col, &tasks, color_seed, &next};
    for (uint32_t i = 0; i < threads; i++)
        pthread_create(&th[i], NULL, leaf_worker_run, &w);
    for (uint32_t i = 0; i < threads; i++)
        pthread_join(th[i], NULL);
    free(tasks.v);
    return HD_OK;
}

/* ---- the compressed colours that ship beside a BasicDAG ------------------ */

typedef struct {
    const uint32_t* words;
    uint32_t leaf_level, top_levels;
    uint64_t* enclosed;
    uint64_t n_enclosed;
    uint64_t seed;
    or_builder* b;
} main_leaf_ctx;

/* DAGUtils::fix_enclosed_leaves_impl (dag_utils.h:525-616): the leaves under
 * a BasicDAG node; nodes above top_levels store theirs in enclosed[upper
 * header bits].  The scenes built here carry their counts at and below
 * top_levels, so the header patch of the reference's count-0 branch never
 * happens (returns 0 if it would). */
static uint64_t enclosed_count(main_leaf_ctx* m, uint32_t level, uint32_t index)
{
    const uint32_t* w = m->words;
    if (level == m->leaf_level)
        return (uint64_t)popc64((uint64_t)w[index] | ((uint64_t)w[index + 1] << 32));
    const uint32_t node = w[index], upper = node >> 8, mask = node & 0xffu;
    if (level >= m->top_levels)
        return upper;
    if (upper >= m->n_enclosed)
        return 0;
    if (m->enclosed[upper])
        return m->enclosed[upper];
    uint64_t count = 0;
    uint32_t off = 1;
    for (uint32_t c = 0; c < 8; c++)
        if (mask & (1u << c))
            count += enclosed_count(m, level + 1, w[index + off++]);
    m->enclosed[upper] = count;
    return count;
}
/* largest upper-bits index of the nodes above top_levels */
static uint32_t max_enclosed_index(const main_leaf_ctx* m, uint32_t level, uint32_t index)
{
    if (level >= m->top_levels)
        return 0;
    const uint32_t node = m->words[index], mask = node & 0xffu;
    uint32_t mx = node >> 8, off = 1;
    for (uint32_t c = 0; c < 8; c++)
        if (mask & (1u << c)) {
            const uint32_t k = max_enclosed_index(m, level + 1, m->words[index + off++]);
            mx = k > mx ? k : mx;
        }
    return mx;
}
/* every voxel's colour in depth-first order (children in order, leaf bits in
 * index order) */
static void main_leaf_voxels(main_leaf_ctx* m, uint32_t level, uint32_t index, const uint32_t path[3])
{
    const uint32_t* w = m->words;
    if (level == m->leaf_level) {
        const uint64_t leaf = (uint64_t)w[index] | ((uint64_t)w[index + 1] << 32);
        for (uint32_t bit = 0; bit < 64; bit++) {
            if (!((leaf >> bit) & 1))
                continue;
            const uint32_t c1 = bit >> 3, c2 = bit & 7;
            const uint32_t x = (path[0] << 2) | (((c1 >> 2) & 1) << 1) | ((c2 >> 2) & 1);
            const uint32_t y = (path[1] << 2) | (((c1 >> 1) & 1) << 1) | ((c2 >> 1) & 1);
            const uint32_t z = (path[2] << 2) | ((c1 & 1) << 1) | (c2 & 1);
            builder_add(m->b, or_voxel_color(m->seed, x, y, z));
        }
        return;
    }
    const uint32_t mask = w[index] & 0xffu;
    uint32_t off = 1;
    for (uint32_t c = 0; c < 8; c++) {
        if (!(mask & (1u << c)))
            continue;
        uint32_t np[3];
        descend(path, c, np);
        main_leaf_voxels(m, level + 1, w[index + off++], np);
    }
}

/* BasicDAGCompressedColors of a BasicDAG (root at word 0) and the colour
 * field of `seed`: enclosedLeaves (fix_enclosed_leaves over the nodes above
 * top_levels, sized by their largest index + 1) and the main leaf (one
 * ColorLeafBuilder fed every voxel; weights in the leaf's in-memory order).
 * Every output array is malloc'd; or_free releases it. */
int or_main_leaf(const uint32_t* words, uint64_t n_words, uint32_t depth, uint32_t top_levels, uint64_t seed,
                 uint64_t** enclosed, uint64_t* n_enclosed, uint64_t** blocks, uint64_t* nb, uint64_t** macros,
                 uint64_t* nm, uint32_t** weights, uint64_t* nw)
{
    if (!words || n_words < 2 || depth < 4 || top_levels >= depth - 2)
        return HD_ERR_INVALID;
    main_leaf_ctx m;
    memset(&m, 0, sizeof(m));
    m.words = words;
    m.leaf_level = depth - 2;
    m.top_levels = top_levels;
    m.seed = seed;
    m.n_enclosed = top_levels ? (uint64_t)max_enclosed_index(&m, 0, 0) + 1 : 0;
    m.enclosed = (uint64_t*)calloc(m.n_enclosed + 1, 8);
    if (top_levels)
        enclosed_count(&m, 0, 0);
    or_builder b;
    memset(&b, 0, sizeof(b));
    m.b = &b;
    const uint32_t path[3] = {0, 0, 0};
    main_leaf_voxels(&m, 0, 0, path);
    or_leaf leaf;
    builder_build(&b, &leaf);
    builder_free(&b);
    *enclosed = m.enclosed;
    *n_enclosed = m.n_enclosed;
    *blocks = leaf.blocks;
    *nb = leaf.nb;
    *macros = leaf.macros;
    *nm = leaf.nm;
    *weights = leaf.weights;
    *nw = leaf.nw;
    return HD_OK;
}

/* DAGUtils::get_color (dag_utils.h:423-523) */
hd_color or_get_color(const or_table* t, const or_colors* col, uint32_t x, uint32_t y, uint32_t z)
{
    hd_color none;
    memset(&none, 0, sizeof(none));
    const uint32_t D = t->cfg.depth, T = t->cfg.color_tree_levels, leafl = t->leaf_level;
    uint64_t nof = 0;
    uint32_t cn = 0;
    const or_leaf* leaf = NULL;
    uint32_t index = t->root;
    if (index == INVALID)
        return none;
    for (uint32_t level = 0; level < leafl;) {
        level++;
        const uint32_t* p = sys_ptr(t, index);
        const uint32_t mask = p[0] & 0xffu;
        const uint32_t sh = D - level;
        const uint32_t child = (((x >> sh) & 1) << 2) | (((y >> sh) & 1) << 1) | ((z >> sh) & 1);
        if (!(mask & (1u << child)))
            return none;
        if (level - 1 < T) {
            cn = col->nodes[cn + child];
            if (level == T) {
                leaf = (cn & LEAF_FLAG) ? &col->leaves[cn & ~LEAF_FLAG] : NULL;
            } else if (!cn) {
                return none;
            }
        }
        if (level == leafl) {
            for (uint32_t cb = 0; cb < child; cb++)
                if (mask & (1u << cb)) {
                    const uint32_t* lp = sys_ptr(t, p[child_offset(mask, cb)]);
                    nof += popc32(lp[0]) + popc32(lp[1]);
                }
            const uint32_t* lp = sys_ptr(t, p[child_offset(mask, child)]);
            const uint64_t bits = (uint64_t)lp[0] | ((uint64_t)lp[1] << 32);
            const uint32_t bi = ((x & 1) ? 4 : 0) | ((y & 1) ? 2 : 0) | ((z & 1) ? 1 : 0) | ((x & 2) ? 32 : 0) |
                                ((y & 2) ? 16 : 0) | ((z & 2) ? 8 : 0);
            nof += popc64(bits & ((1ull << bi) - 1));
            break;
        }
        if (level > T)
            for (uint32_t cb = 0; cb < child; cb++)
                if (mask & (1u << cb))
                    nof += sys_ptr(t, p[child_offset(mask, cb)])[0] >> 8;
        index = p[child_offset(mask, child)];
    }
    if (!leaf || !leaf_valid_index(leaf, nof))
        return none;
    return leaf_color(leaf, nof);
}

/* ToolInfo::strength (tracer.h:51-77) */
static float sphere_strength(const uint32_t pos[3], const uint32_t p[3], float radius)
{
    const float dx = (float)pos[0] - (float)p[0], dy = (float)pos[1] - (float)p[1], dz = (float)pos[2] - (float)p[2];
    return 1 - (float)sqrt((double)(dx * dx + dy * dy + dz * dz)) / radius;
}
static float cube_strength(const uint32_t pos[3], const uint32_t p[3], float radius)
{
    const float dx = fabsf((float)pos[0] - (float)p[0]), dy = fabsf((float)pos[1] - (float)p[1]),
                dz = fabsf((float)pos[2] - (float)p[2]);
    const float yz = dy > dz ? dy : dz;
    return 1 - (dx > yz ? dx : yz) / radius;
}
static float tool_strength(const hd_tool_overlay* o, const uint32_t p[3])
{
    switch (o->tool) {
    case HD_OVERLAY_SPHERE:
    case HD_OVERLAY_SPHERE_PAINT:
    case HD_OVERLAY_SPHERE_NOISE:
        return sphere_strength(o->position, p, o->radius);
    case HD_OVERLAY_CUBE:
        return cube_strength(o->position, p, o->radius);
    default: {
        const float a = sphere_strength(o->copy_source, p, 3), b = sphere_strength(o->copy_dest, p, 3);
        const float m = a > b ? a : b, c = cube_strength(o->position, p, o->radius);
        return m > c ? m : c;
    }
    }
}
static uint32_t overlay(const hd_trace_colors_params* q, float strength, uint32_t color)
{
    if (q->overlay.enabled && strength > 0) {
        const f3 a = {(float)((color >> 0) & 0xFF) / 255.0f, (float)((color >> 8) & 0xFF) / 255.0f,
                      (float)((color >> 16) & 0xFF) / 255.0f};
        const float f = clampf(100 * strength, 0.f, .5f);
        color = or_f3_to_rgb888(a.x * (1 - f) + 1 * f, a.y * (1 - f) + 0 * f, a.z * (1 - f) + 0 * f);
    }
    return color;
}
/* Tracer::trace_colors (tracer.cu:254-451) for one hit path */
static uint32_t trace_color(const or_table* t, const or_colors* col, const uint32_t p[3],
                            const hd_trace_colors_params* q)
{
    if (!(p[0] | p[1] | p[2]))
        return or_f3_to_rgb888(187 / 255.f, 242 / 255.f, 250 / 255.f);
    const float s = q->overlay.enabled ? tool_strength(&q->overlay, p) : 0.f;
    const float b = (float)((p[0] ^ p[1] ^ p[2]) & 1u);
    const uint32_t invalid = overlay(q, s, or_f3_to_rgb888(1, b, 1.f - b));
    const uint32_t D = t->cfg.depth, T = t->cfg.color_tree_levels, leafl = t->leaf_level;
    const int tree_debug = q->debug_colors == HD_DEBUG_INDEX || q->debug_colors == HD_DEBUG_POSITION ||
                           q->debug_colors == HD_DEBUG_COLOR_TREE;
    uint64_t nof = 0;
    uint32_t debug_index = 0, cn = 0;
    const or_leaf* leaf = NULL;
    uint32_t index = t->root;
    for (uint32_t level = 0; level < leafl;) {
        level++;
        const uint32_t* node = sys_ptr(t, index);
        const uint32_t mask = node[0] & 0xffu;
        const uint32_t sh = D - level;
        const uint32_t child = (((p[0] >> sh) & 1) << 2) | (((p[1] >> sh) & 1) << 1) | ((p[2] >> sh) & 1);
        if (!(mask & (1u << child)))
            return overlay(q, s, 0xFF00FFu);
        if (level - 1 < T) {
            cn = col->nodes[cn + child];
            if (level == T)
                leaf = (cn & LEAF_FLAG) ? &col->leaves[cn & ~LEAF_FLAG] : NULL;
            else if (!cn)
                return invalid;
        }
        if (tree_debug) {
            if (q->debug_colors == HD_DEBUG_INDEX && q->debug_level == level - 1)
                debug_index = index;
            if (level == leafl) {
                if (q->debug_level == leafl)
                    debug_index = node[child_offset(mask, child)];
                if (q->debug_colors == HD_DEBUG_INDEX)
                    return overlay(q, s, or_murmurhash32(debug_index));
                if (q->debug_colors == HD_DEBUG_POSITION) {
                    float c = (float)((p[0] ^ p[1] ^ p[2]) & 0x7FFu) / (float)0x7FF;
                    c = (float)(((double)c + 0.5) / 2);
                    return overlay(q, s, (index & LEAF_FLAG) ? or_f3_to_rgb888(c, 0, 0) : or_f3_to_rgb888(c, c, c));
                }
                const uint32_t off = D - T;
                const float c = (float)(((p[0] >> off) ^ (p[1] >> off) ^ (p[2] >> off)) & 1u);
                return overlay(q, s, or_f3_to_rgb888(c, c, c));
            }
            index = node[child_offset(mask, child)];
            continue;
        }
        if (level == leafl) {
            for (uint32_t cb = 0; cb < child; cb++)
                if (mask & (1u << cb)) {
                    const uint32_t* lp = sys_ptr(t, node[child_offset(mask, cb)]);
                    nof += popc32(lp[0]) + popc32(lp[1]);
                }
            const uint32_t* lp = sys_ptr(t, node[child_offset(mask, child)]);
            const uint64_t bits = (uint64_t)lp[0] | ((uint64_t)lp[1] << 32);
            const uint32_t bi = ((p[0] & 1) ? 4 : 0) | ((p[1] & 1) ? 2 : 0) | ((p[2] & 1) ? 1 : 0) |
                                ((p[0] & 2) ? 32 : 0) | ((p[1] & 2) ? 16 : 0) | ((p[2] & 2) ? 8 : 0);
            nof += popc64(bits & ((1ull << bi) - 1));
            break;
        }
        if (level > T)
            for (uint32_t cb = 0; cb < child; cb++)
                if (mask & (1u << cb))
                    nof += sys_ptr(t, node[child_offset(mask, cb)])[0] >> 8;
        index = node[child_offset(mask, child)];
    }
    if (!leaf || !leaf_valid_index(leaf, nof))
        return invalid;
    const hd_color k = leaf_color(leaf, nof);
    switch (q->debug_colors) {
    case HD_DEBUG_COLOR_BITS:
        return overlay(q, s, 0u); /* get_debug_hash without COLOR_DEBUG */
    case HD_DEBUG_MIN_COLOR: {
        const f3 c = rgb565_to_f3((uint16_t)(k.color_bits & 0xFFFF));
        return overlay(q, s, or_f3_to_rgb888(c.x, c.y, c.z));
    }
    case HD_DEBUG_MAX_COLOR: {
        const f3 c = rgb565_to_f3((uint16_t)((k.color_bits >> 16) & 0xFFFF));
        return overlay(q, s, or_f3_to_rgb888(c.x, c.y, c.z));
    }
    case HD_DEBUG_WEIGHT: {
        const float w = k.bits_per_weight ? (float)k.weight / (float)((1 << k.bits_per_weight) - 1) : 0.f;
        return overlay(q, s, or_f3_to_rgb888(w, w, w));
    }
    default:
        return overlay(q, s, or_color_rgb888(k));
    }
}
/* the colours of a paths image (uint4 per pixel) */
void or_trace_colors(const or_table* t, const or_colors* col, const uint32_t* paths, uint64_t n,
                     const hd_trace_colors_params* params, uint32_t* rgba)
{
    hd_trace_colors_params q;
    memset(&q, 0, sizeof(q));
    if (params)
        q = *params;
    for (uint64_t i = 0; i < n; i++)
        rgba[i] = trace_color(t, col, paths + 4 * i, &q);
}

static void push_frame(struct frame** stack, uint64_t* n, uint64_t* cap, struct frame f)
{
    if (*n == *cap) {
        *cap = *cap ? 2 * *cap : 16;
        *stack = (struct frame*)realloc(*stack, *cap * sizeof(struct frame));
    }
    (*stack)[(*n)++] = f;
}

/* ---- the noise and flood-fill buffers ------------------------------------ */

/* std::mt19937_64 (the standard's 64-bit Mersenne Twister: Matsumoto and
 * Nishimura's MT19937-64 parameters, seeded by the standard's recurrence) */
typedef struct {
    uint64_t mt[312];
    uint32_t i;
} mt64;
static void mt64_seed(mt64* g, uint64_t seed)
{
    g->mt[0] = seed;
    for (uint32_t i = 1; i < 312; i++)
        g->mt[i] = 6364136223846793005ull * (g->mt[i - 1] ^ (g->mt[i - 1] >> 62)) + i;
    g->i = 312;
}
static uint64_t mt64_next(mt64* g)
{
    if (g->i >= 312) {
        for (uint32_t k = 0; k < 312; k++) {
            const uint64_t x = (g->mt[k] & 0xFFFFFFFF80000000ull) | (g->mt[(k + 1) % 312] & 0x7FFFFFFFull);
            uint64_t xa = x >> 1;
            if (x & 1)
                xa ^= 0xB5026F5AA96619E9ull;
            g->mt[k] = g->mt[(k + 156) % 312] ^ xa;
        }
        g->i = 0;
    }
    uint64_t y = g->mt[g->i++];
    y ^= (y >> 29) & 0x5555555555555555ull;
    y ^= (y << 17) & 0x71D67FFFEDA60000ull;
    y ^= (y << 37) & 0xFFF7EEE000000000ull;
    y ^= y >> 43;
    return y;
}

/* FastNoise's 3D gradient Perlin noise with an FBM fractal (the reference
 * vendors FastNoise: FastNoise.cpp:207-225 SetSeed, :227-237 the fractal
 * bounding, :760-793 GetPerlinFractal / SinglePerlinFractalFBM, :841-886
 * SinglePerlin; float arithmetic, quintic interpolation, lacunarity 2, gain
 * 0.5) */
typedef struct {
    uint8_t perm[512], perm12[512];
    float frequency, bounding;
    int octaves;
} fnoise;
static const float kGradX[12] = {1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
static const float kGradY[12] = {1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
static const float kGradZ[12] = {0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
static void fn_seed(fnoise* n, int seed)
{
    mt64 g;
    mt64_seed(&g, (uint64_t)(int64_t)seed);
    for (int i = 0; i < 256; i++)
        n->perm[i] = (uint8_t)i;
    for (int j = 0; j < 256; j++) {
        const int rng = (int)(mt64_next(&g) % (uint64_t)(256 - j));
        const int k = rng + j;
        const uint8_t l = n->perm[j];
        n->perm[j] = n->perm[j + 256] = n->perm[k];
        n->perm[k] = l;
        n->perm12[j] = n->perm12[j + 256] = (uint8_t)(n->perm[j] % 12);
    }
}
static void fn_octaves(fnoise* n, int octaves)
{
    n->octaves = octaves;
    float amp = 0.5f, amp_fractal = 1.0f;
    for (int i = 1; i < octaves; i++) {
        amp_fractal += amp;
        amp *= 0.5f;
    }
    n->bounding = 1.0f / amp_fractal;
}
static int fast_floor(float f) { return f >= 0 ? (int)f : (int)f - 1; }
static float fn_lerp(float a, float b, float t) { return a + t * (b - a); }
static float quintic(float t) { return t * t * t * (t * (t * 6 - 15) + 10); }
static float grad3(const fnoise* n, uint8_t offset, int x, int y, int z, float xd, float yd, float zd)
{
    const uint8_t lut = n->perm12[(x & 0xff) + n->perm[(y & 0xff) + n->perm[(z & 0xff) + offset]]];
    return xd * kGradX[lut] + yd * kGradY[lut] + zd * kGradZ[lut];
}
static float single_perlin(const fnoise* n, uint8_t offset, float x, float y, float z)
{
    const int x0 = fast_floor(x), y0 = fast_floor(y), z0 = fast_floor(z);
    const int x1 = x0 + 1, y1 = y0 + 1, z1 = z0 + 1;
    const float xs = quintic(x - (float)x0), ys = quintic(y - (float)y0), zs = quintic(z - (float)z0);
    const float xd0 = x - (float)x0, yd0 = y - (float)y0, zd0 = z - (float)z0;
    const float xd1 = xd0 - 1, yd1 = yd0 - 1, zd1 = zd0 - 1;
    const float xf00 = fn_lerp(grad3(n, offset, x0, y0, z0, xd0, yd0, zd0), grad3(n, offset, x1, y0, z0, xd1, yd0, zd0), xs);
    const float xf10 = fn_lerp(grad3(n, offset, x0, y1, z0, xd0, yd1, zd0), grad3(n, offset, x1, y1, z0, xd1, yd1, zd0), xs);
    const float xf01 = fn_lerp(grad3(n, offset, x0, y0, z1, xd0, yd0, zd1), grad3(n, offset, x1, y0, z1, xd1, yd0, zd1), xs);
    const float xf11 = fn_lerp(grad3(n, offset, x0, y1, z1, xd0, yd1, zd1), grad3(n, offset, x1, y1, z1, xd1, yd1, zd1), xs);
    const float yf0 = fn_lerp(xf00, xf10, ys), yf1 = fn_lerp(xf01, xf11, ys);
    return fn_lerp(yf0, yf1, zs);
}
static float perlin_fractal(const fnoise* n, float x, float y, float z)
{
    x *= n->frequency;
    y *= n->frequency;
    z *= n->frequency;
    float sum = single_perlin(n, n->perm[0], x, y, z), amp = 1;
    for (int i = 1; i < n->octaves; i++) {
        x *= 2.0f;
        y *= 2.0f;
        z *= 2.0f;
        amp *= 0.5f;
        sum += single_perlin(n, n->perm[i], x, y, z) * amp;
    }
    return sum * n->bounding;
}
float or_perlin_fractal(int seed, float frequency, int octaves, float x, float y, float z)
{
    fnoise n;
    fn_seed(&n, seed);
    n.frequency = frequency;
    fn_octaves(&n, octaves);
    return perlin_fractal(&n, x, y, z);
}

/* SphereNoiseEditor's constructor (:716-744): a voxel of the buffer is set
 * to isAdding where its distance to the centre, sqrt of the uint32 dot
 * product of the (wrapping) uint3 difference, is below
 * radius * (1 + noise) in double */
static void noise_buffer(editor* e, int adding)
{
    const uint32_t n = e->size, ec = n / 2;
    fnoise fn;
    int seed = 1923 + (int32_t)e->c.x + 23 * (int32_t)e->c.y + 2938 * (int32_t)e->c.z;
    fn_seed(&fn, seed < 0 ? -seed : seed);
    fn.frequency = 1 / e->r;
    fn_octaves(&fn, 3);
    for (uint32_t x = 0; x < n; x++)
        for (uint32_t y = 0; y < n; y++)
            for (uint32_t z = 0; z < n; z++) {
                const uint32_t dx = ec - x, dy = ec - y, dz = ec - z;
                const double distance = sqrt((double)(dx * dx + dy * dy + dz * dz));
                if (distance < (double)e->r * (1. + (double)perlin_fractal(&fn, (float)x, (float)y, (float)z)))
                    e->state[buf_index(e, x, y, z)] = adding ? EV_SET_TRUE : EV_SET_FALSE;
            }
}

/* FillEditorBase's constructor (:625-668): a depth-first flood from the
 * buffer's centre through voxels that read false (get_value loads them
 * from the table), 6-neighbours in the order -x, +x, -y, +y, -z, +z; every
 * popped voxel is set; the bounds become min + the set voxels' box.  With
 * colours, FillEditorColors (:679-705) then walks that box (x, then y, then
 * z) carrying the colour of the last loaded-true voxel into every set voxel
 * after it. */
static void fill_buffer(editor* e, const or_colors* col)
{
    const uint32_t n = e->size;
    uint32_t* stack = NULL;
    uint64_t sn = 0, scap = 0;
    const uint32_t ec = n / 2;
    uint32_t mn[3] = {ec, ec, ec}, mx[3] = {ec, ec, ec};
#define FILL_PUSH(a, b, c)                                                   \
    do {                                                                     \
        if (sn + 3 > scap) {                                                 \
            scap = scap ? 2 * scap : 3 * 1024;                               \
            stack = (uint32_t*)realloc(stack, scap * 4);                     \
        }                                                                    \
        stack[sn++] = (a);                                                   \
        stack[sn++] = (b);                                                   \
        stack[sn++] = (c);                                                   \
    } while (0)
    FILL_PUSH(ec, ec, ec);
    while (sn) {
        sn -= 3;
        const uint32_t p[3] = {stack[sn], stack[sn + 1], stack[sn + 2]};
        e->state[buf_index(e, p[0], p[1], p[2])] = EV_SET_TRUE;
        for (int a = 0; a < 3; a++) {
            mn[a] = p[a] < mn[a] ? p[a] : mn[a];
            mx[a] = p[a] > mx[a] ? p[a] : mx[a];
        }
        static const int nb[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
        for (int k = 0; k < 6; k++) {
            const uint32_t q[3] = {p[0] + (uint32_t)nb[k][0], p[1] + (uint32_t)nb[k][1], p[2] + (uint32_t)nb[k][2]};
            if (q[0] < n && q[1] < n && q[2] < n && !buf_get(e, q[0], q[1], q[2]))
                FILL_PUSH(q[0], q[1], q[2]);
        }
    }
#undef FILL_PUSH
    free(stack);
    e->bmin = (f3){e->buf_min.x + (float)mn[0], e->buf_min.y + (float)mn[1], e->buf_min.z + (float)mn[2]};
    e->bmax = (f3){e->buf_min.x + (float)mx[0], e->buf_min.y + (float)mx[1], e->buf_min.z + (float)mx[2]};
    if (!col)
        return;
    hd_color color;
    memset(&color, 0, sizeof(color));
    for (uint32_t x = mn[0]; x <= mx[0]; x++)
        for (uint32_t y = mn[1]; y <= mx[1]; y++)
            for (uint32_t z = mn[2]; z <= mx[2]; z++) {
                const uint64_t i = buf_index(e, x, y, z);
                if (e->state[i] == EV_LOADED_TRUE) {
                    uint32_t w[3];
                    buf_world(e, x, y, z, w);
                    color = or_get_color(e->dag, col, w[0], w[1], w[2]);
                } else if (e->state[i] == EV_SET_TRUE) {
                    e->colors[i] = color;
                }
            }
}

/* The buffers of the noise and fill editors, made before the edit as their
 * constructors make them; 0, or HD_ERR_INVALID when the buffer would not
 * fit. */
static int make_buffers(editor* e, const or_table* t, const or_colors* col)
{
    if (e->tool < HD_TOOL_NOISE_REMOVE)
        return 0;
    const uint64_t n3 = (uint64_t)e->size * e->size * e->size;
    if (n3 > (1ull << 31))
        return HD_ERR_INVALID;
    e->dag = t;
    e->state = (uint8_t*)calloc(n3 + 1, 1);
    if (e->tool == HD_TOOL_FILL) {
        e->colors = (hd_color*)calloc(n3 + 1, sizeof(hd_color));
        fill_buffer(e, col);
    } else {
        noise_buffer(e, e->tool == HD_TOOL_NOISE_ADD);
    }
    return 0;
}

/* HashDAG::edit_threads (hash_dag.h:255-405) with colours: the edit, the
 * colour leaves rebuilt, an undo frame recorded (HashDAGUndoRedo::add_frame
 * drops the redo stack, :55-66). */
int or_edit_colored(or_table* t, or_colors* col, const hd_edit* e, hd_edit_stats* stats)
{
    if (!col || !col->n_nodes || t->cfg.color_tree_levels == 0 || e->tool > HD_TOOL_FILL)
        return HD_ERR_INVALID;
    edit_job j;
    memset(&j, 0, sizeof(j));
    j.t = t;
    j.col = col;
    j.ed = make_editor(e);
    if (make_buffers(&j.ed, t, col))
        return HD_ERR_INVALID;
    if (e->tool == HD_TOOL_COPY) {
        /* the source region read before the edit (:459-505, BENCHMARK).
         * DAGUtils::get_values' overlap test compares inclusive node bounds
         * with `boundsMax <= inMin` (dag_utils.h:264-283), so a voxel whose
         * x, y or z equals the region's start is never written and keeps
         * the memset 0. */
        const uint32_t n = j.ed.size;
        const uint32_t m0[3] = {(uint32_t)j.ed.copy_min.x, (uint32_t)j.ed.copy_min.y, (uint32_t)j.ed.copy_min.z};
        const uint64_t n3 = (uint64_t)n * n * n;
        j.ed.values = (uint8_t*)calloc(n3 + 1, 1);
        j.ed.colors = (hd_color*)calloc(n3 + 1, sizeof(hd_color));
        for (uint32_t z = 0; z < n; z++)
            for (uint32_t y = 0; y < n; y++)
                for (uint32_t x = 0; x < n; x++) {
                    const uint64_t i = x + (uint64_t)n * y + (uint64_t)n * n * z;
                    j.ed.values[i] = (x && y && z) ? (uint8_t)or_get_value(t, m0[0] + x, m0[1] + y, m0[2] + z) : 0;
                    if (j.ed.values[i])
                        j.ed.colors[i] = or_get_color(t, col, m0[0] + x, m0[1] + y, m0[2] + z);
                }
    }
    t->foa_calls = t->nodes_added = t->words_scanned = 0;
    const uint32_t path[3] = {0, 0, 0};
    uint32_t cn;
    const uint32_t before = t->root;
    const uint32_t root = edit_top(&j, 0, t->root, path, 0, &cn);
    free(j.ed.values);
    free(j.ed.colors);
    free(j.ed.state);
    if (!t->error) {
        t->root = root;
        struct frame f = {before, j.n_diff, j.diff_index, j.diff_prev, j.diff_next};
        free_frames(col->redo, col->n_redo);
        col->n_redo = 0;
        push_frame(&col->undo, &col->n_undo, &col->cap_undo, f);
    }
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->num_voxels = j.num_voxels;
        stats->num_nodes = j.num_nodes;
        stats->find_or_add_calls = t->foa_calls;
        stats->nodes_added = t->nodes_added;
        stats->words_scanned = t->words_scanned;
    }
    return t->error;
}

/* HashDAGUndoRedo::undo / redo (hash_dag.h:67-120): swap the root, put the
 * frame's leaves back, move the inverted frame to the other stack. */
static int swap_frame(or_table* t, or_colors* col, struct frame** from, uint64_t* nf, struct frame** to, uint64_t* nt,
                      uint64_t* capt)
{
    if (*nf == 0)
        return 0;
    struct frame f = (*from)[--(*nf)];
    struct frame inv = {t->root, f.n, f.index, f.next, f.prev};
    t->root = f.root;
    for (uint32_t i = 0; i < f.n; i++)
        col->leaves[f.index[i] & ~LEAF_FLAG] = f.prev[i];
    push_frame(to, nt, capt, inv);
    return 1;
}
int or_undo(or_table* t, or_colors* col)
{
    return swap_frame(t, col, &col->undo, &col->n_undo, &col->redo, &col->n_redo, &col->cap_redo);
}
int or_redo(or_table* t, or_colors* col)
{
    return swap_frame(t, col, &col->redo, &col->n_redo, &col->undo, &col->n_undo, &col->cap_undo);
}

void or_colors_stats(const or_colors* col, uint64_t* out /* nodes, leaves, blocks, weight words, macro words */)
{
    out[0] = col->n_nodes;
    out[1] = col->n_leaves;
    out[2] = out[3] = out[4] = 0;
    for (uint64_t i = 0; i < col->n_leaves; i++) {
        out[2] += col->leaves[i].nb;
        out[3] += col->leaves[i].nw;
        out[4] += col->leaves[i].nm;
    }
}

/* ======================================================================
 * GC: HashDAG::remove_stale_nodes (hash_dag.h:407-547) with a canonical
 * re-insertion order (increasing old address per level).
 * ====================================================================== */

static int cmp_u32(const void* a, const void* b)
{
    uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
    return x < y ? -1 : x > y;
}
static uint64_t unique_sorted(uint32_t* v, uint64_t n)
{
    if (!n)
        return 0;
    qsort(v, n, 4, cmp_u32);
    uint64_t m = 1;
    for (uint64_t i = 1; i < n; i++)
        if (v[i] != v[m - 1])
            v[m++] = v[i];
    return m;
}
static uint64_t find_sorted(const uint32_t* v, uint64_t n, uint32_t x)
{
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
        uint64_t mid = (lo + hi) / 2;
        if (v[mid] < x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

int or_gc(or_table* t, uint32_t* extra, uint32_t n_extra)
{
    const uint32_t maxl = t->leaf_level;
    uint32_t* live[HD_MAX_DEPTH];
    uint64_t nlive[HD_MAX_DEPTH];
    /* mark (hash_dag.h:424-438) */
    live[0] = (uint32_t*)malloc((1 + n_extra) * 4);
    live[0][0] = t->root;
    for (uint32_t i = 0; i < n_extra; i++)
        live[0][1 + i] = extra[i];
    nlive[0] = unique_sorted(live[0], 1 + n_extra);
    for (uint32_t level = 0; level < maxl; level++) {
        uint64_t cap = 0;
        for (uint64_t i = 0; i < nlive[level]; i++)
            cap += total_size(*sys_ptr(t, live[level][i])) - 1;
        live[level + 1] = (uint32_t*)malloc((cap + 1) * 4);
        uint64_t k = 0;
        for (uint64_t i = 0; i < nlive[level]; i++) {
            const uint32_t* p = sys_ptr(t, live[level][i]);
            for (uint32_t o = 1; o < total_size(p[0]); o++)
                live[level + 1][k++] = p[o];
        }
        nlive[level + 1] = unique_sorted(live[level + 1], k);
    }
    /* rebuild bottom-up (:443-538) */
    uint32_t* newidx[HD_MAX_DEPTH] = {0};
    for (int32_t level = (int32_t)maxl; level >= 0; level--) {
        const int leaf = (uint32_t)level == t->leaf_level;
        uint64_t words = 0;
        for (uint64_t i = 0; i < nlive[level]; i++)
            words += leaf ? 2 : total_size(*sys_ptr(t, live[level][i]));
        uint32_t* temp = (uint32_t*)malloc((words + 1) * 4);
        uint64_t* at = (uint64_t*)malloc((nlive[level] + 1) * 8);
        uint64_t w = 0;
        for (uint64_t i = 0; i < nlive[level]; i++) {
            const uint32_t* p = sys_ptr(t, live[level][i]);
            const uint32_t n = leaf ? 2 : total_size(p[0]);
            at[i] = w;
            temp[w] = p[0];
            for (uint32_t o = 1; o < n; o++) {
                if (!leaf && (uint32_t)level != maxl) {
                    uint64_t pos = find_sorted(live[level + 1], nlive[level + 1], p[o]);
                    temp[w + o] = newidx[level + 1][pos];
                } else {
                    temp[w + o] = p[o];
                }
            }
            w += n;
        }
        for (uint32_t b = 0; b < bucket_count(&t->cfg, (uint32_t)level); b++)
            t->bucket_sizes[bucket_global(&t->cfg, (uint32_t)level, b)] = 0;
        t->level_nodes[level] = 0;
        add_full_node(t, (uint32_t)level);
        newidx[level] = (uint32_t*)malloc((nlive[level] + 1) * 4);
        for (uint64_t i = 0; i < nlive[level]; i++) {
            const uint32_t* node = temp + at[i];
            if (leaf) {
                const uint64_t lf = (uint64_t)node[0] | ((uint64_t)node[1] << 32);
                newidx[level][i] = add_leaf(t, lf, or_hash_leaf(lf));
            } else {
                const uint32_t n = total_size(node[0]);
                newidx[level][i] = add_interior(t, (uint32_t)level, n, node, or_hash_interior(n, node));
            }
        }
        free(temp);
        free(at);
        if (level + 1 <= (int32_t)maxl) {
            free(newidx[level + 1]);
            newidx[level + 1] = NULL;
        }
    }
    t->root = newidx[0][find_sorted(live[0], nlive[0], t->root)];
    for (uint32_t i = 0; i < n_extra; i++)
        extra[i] = newidx[0][find_sorted(live[0], nlive[0], extra[i])];
    free(newidx[0]);
    for (uint32_t l = 0; l <= maxl; l++)
        free(live[l]);
    return t->error;
}
