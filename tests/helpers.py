"""Shared test helpers: pointer-independent digests of a hash table."""
import hashlib

import numpy as np

PAGE = 512


def bucket_layout(depth, top_levels=9, top_bits=10, low_bits=16, top_size=1024, low_size=4096):
    """Virtual base and capacity of every bucket in global bucket order
    (get_bucket_global_index / make_ptr, hash_table.h:19-63)."""
    bases, caps, levels = [], [], []
    ntop = min(top_levels, depth)
    for level in range(depth):
        if level < top_levels:
            nb, size = 1 << top_bits, top_size
            base0 = level * nb * size
        else:
            nb, size = 1 << low_bits, low_size
            base0 = ntop * (1 << top_bits) * top_size + (level - top_levels) * nb * size
        bases.append(base0 + np.arange(nb, dtype=np.int64) * size)
        caps.append(np.full(nb, size, np.int64))
        levels.append(np.full(nb, level, np.int64))
    return np.concatenate(bases), np.concatenate(caps), np.concatenate(levels)


def used_words(table, depth, top_bits=10):
    """Every word inside every bucket's used range, read by virtual address,
    buckets in global order."""
    bs = np.asarray(table["bucket_sizes"], np.int64)
    bases, _, _ = bucket_layout(depth, top_bits=top_bits)
    bases = bases[:bs.size]
    npages = (bs + PAGE - 1) // PAGE
    sel = np.nonzero(npages)[0]
    reps = npages[sel]
    bucket_of_page = np.repeat(sel, reps)
    first = np.cumsum(reps) - reps
    page_in_bucket = np.arange(reps.sum()) - np.repeat(first, reps)
    vpage = (bases[bucket_of_page] + page_in_bucket * PAGE) // PAGE
    used = np.minimum(PAGE, bs[bucket_of_page] - page_in_bucket * PAGE)
    phys = np.asarray(table["page_table"], np.int64)[vpage]
    pool = np.asarray(table["pool"], np.uint32).reshape(-1, PAGE)
    pages = pool[phys]  # one row per used page (no per-word index array)
    keep = np.arange(PAGE)[None, :] < used[:, None]
    return pages[keep]


def table_digest(table, depth, top_bits=10):
    """sha256 over the bucket sizes and the used words of every bucket read
    by virtual address: independent of the physical page assignment."""
    h = hashlib.sha256()
    h.update(np.asarray(table["bucket_sizes"], np.uint32).tobytes())
    h.update(used_words(table, depth, top_bits).astype(np.uint32).tobytes())
    return h.hexdigest()
