/*
 * gpma_oracle.c - CPU restatement of the reference GPMA+ (test infrastructure).
 *
 * Each function cites the reference lines it restates. The structure follows
 * the reference's CPU instantiation GPMA<CPU>: batch sort, leaf locate with
 * in-place delete/modify, grouping by leaf, the level loop of window
 * rebalances, the root resize and the bulk rebuild for >= 5M insertions.
 * Only tests/, smoke() and bench.py's CPU baseline use this file.
 */
#include "gpma_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define KEY_NONE ORACLE_KEY_NONE
#define KEY_MAX ORACLE_KEY_MAX
#define SIZE_NONE ORACLE_SIZE_NONE
#define COL_IDX_NONE ORACLE_COL_NONE

/* density thresholds, gpma.cuh:40-43 */
static const double LOWER_LEAF = 0.08;
static const double LOWER_ROOT = 0.42;
static const double UPPER_LEAF = 0.92;
static const double UPPER_ROOT = 0.84;
/* bulk-rebuild threshold on insertions, gpma.cuh:1003 */
static const uint64_t SIGNIFICANT_INSERTS = 5000000u;

static void *xmalloc(size_t n) {
    void *p = malloc(n ? n : 1);
    if (!p)
        abort();
    return p;
}

/* fls: index of the highest set bit, 1-based; 0 for 0 (gpma.cuh:111-126). */
static uint32_t fls32(uint32_t x) {
    uint32_t r = 0;
    while (x) {
        ++r;
        x >>= 1;
    }
    return r;
}

/* recalculate_density (gpma.cuh:147-168), evaluated in the same order. */
static void recalculate_density(oracle_gpma *g) {
    uint32_t h = g->tree_height;
    free(g->lower);
    free(g->upper);
    g->lower = (uint32_t *)xmalloc(sizeof(uint32_t) * (h + 1));
    g->upper = (uint32_t *)xmalloc(sizeof(uint32_t) * (h + 1));
    uint32_t level_length = g->segment_length;
    for (uint32_t i = 0; i <= h; i++) {
        double dl = LOWER_ROOT + (LOWER_LEAF - LOWER_ROOT) * (double)(h - i) / (double)h;
        double du = UPPER_ROOT + (UPPER_LEAF - UPPER_ROOT) * (double)(h - i) / (double)h;
        g->lower[i] = (uint32_t)ceil(dl * (double)level_length);
        g->upper[i] = (uint32_t)floor(du * (double)level_length);
        if (i > 0) {
            uint32_t l2 = 2 * g->lower[i - 1], u2 = 2 * g->upper[i - 1];
            if (l2 > g->lower[i])
                g->lower[i] = l2;
            if (u2 < g->upper[i])
                g->upper[i] = u2;
        }
        level_length <<= 1;
    }
}

/* ---- stable sort of (key, value) pairs: LSD radix, 8-bit digits ---------- */
static void stable_sort_kv(uint64_t *k, uint8_t *v, uint64_t n) {
    if (n < 2)
        return;
    if (n <= 32) { /* stable insertion sort */
        for (uint64_t i = 1; i < n; ++i) {
            uint64_t kk = k[i];
            uint8_t vv = v[i];
            uint64_t j = i;
            while (j > 0 && k[j - 1] > kk) {
                k[j] = k[j - 1];
                v[j] = v[j - 1];
                --j;
            }
            k[j] = kk;
            v[j] = vv;
        }
        return;
    }
    uint64_t *tk = (uint64_t *)xmalloc(n * sizeof(uint64_t));
    uint8_t *tv = (uint8_t *)xmalloc(n);
    uint64_t *sk = k, *dk = tk;
    uint8_t *sv = v, *dv = tv;
    uint64_t cnt[256];
    for (int pass = 0; pass < 8; ++pass) {
        int shift = pass * 8;
        memset(cnt, 0, sizeof(cnt));
        for (uint64_t i = 0; i < n; ++i)
            cnt[(sk[i] >> shift) & 255]++;
        int trivial = 0;
        for (int d = 0; d < 256; ++d)
            if (cnt[d] == n)
                trivial = 1;
        if (trivial)
            continue;
        uint64_t sum = 0;
        for (int d = 0; d < 256; ++d) {
            uint64_t c = cnt[d];
            cnt[d] = sum;
            sum += c;
        }
        for (uint64_t i = 0; i < n; ++i) {
            uint64_t pos = cnt[(sk[i] >> shift) & 255]++;
            dk[pos] = sk[i];
            dv[pos] = sv[i];
        }
        uint64_t *t = sk;
        sk = dk;
        dk = t;
        uint8_t *u = sv;
        sv = dv;
        dv = u;
    }
    if (sk != k) {
        memcpy(k, sk, n * sizeof(uint64_t));
        memcpy(v, sv, n);
    }
    free(tk);
    free(tv);
}

/* ---- construction ------------------------------------------------------- */

/* init_gpma_members (gpma.cuh:54-69): 4 slots, KEY_MAX at 0 and 2. */
static void init_members(oracle_gpma *g, uint32_t row_num) {
    g->row_num = row_num;
    g->row_offset = (uint32_t *)calloc((size_t)row_num + 1, sizeof(uint32_t));
    if (!g->row_offset)
        abort();
    g->size = 4;
    g->keys = (uint64_t *)xmalloc(4 * sizeof(uint64_t));
    g->values = (uint8_t *)calloc(4, 1);
    for (int i = 0; i < 4; ++i)
        g->keys[i] = KEY_NONE;
    g->segment_length = 2;
    g->tree_height = 1;
    g->keys[0] = g->keys[2] = KEY_MAX;
    g->values[0] = g->values[2] = 1;
    recalculate_density(g);
}

oracle_gpma *oracle_create(uint32_t row_num, int threads) {
    oracle_gpma *g = (oracle_gpma *)calloc(1, sizeof(oracle_gpma));
    if (!g)
        return NULL;
    g->threads = threads > 0 ? threads : 1;
    init_members(g, row_num);
    /* init_gpma_insertions (gpma.cuh:70-78): one guard (r<<32)|0xFFFFFFFF per
     * row, value 1, inserted with update_gpma. */
    uint64_t *k = (uint64_t *)xmalloc(sizeof(uint64_t) * (row_num ? row_num : 1));
    uint8_t *v = (uint8_t *)xmalloc(row_num ? row_num : 1);
    for (uint32_t r = 0; r < row_num; ++r) {
        k[r] = ((uint64_t)r << 32) + COL_IDX_NONE;
        v[r] = 1;
    }
    oracle_update(g, k, v, row_num);
    free(k);
    free(v);
    memset(&g->stats, 0, sizeof(g->stats));
    return g;
}

void oracle_destroy(oracle_gpma *g) {
    if (!g)
        return;
    free(g->keys);
    free(g->values);
    free(g->lower);
    free(g->upper);
    free(g->row_offset);
    free(g);
}

/* ---- update pipeline ----------------------------------------------------- */

/* locate_leaf_loop_body + handle_del_mod (gpma.cuh:188-220): top-down search
 * over the first slots of segments, then an equality scan of the leaf; a hit
 * stores the update's value in place (delete = 0, modify, revive) and the key
 * is no insertion; a delete that misses is dropped. */
static uint32_t locate_one(oracle_gpma *g, uint64_t key, uint8_t value) {
    uint32_t seg = g->segment_length;
    uint32_t prefix = 0;
    uint32_t bit = (seg << g->tree_height) >> 1;
    while (seg <= bit) {
        if (g->keys[prefix | bit] <= key)
            prefix |= bit;
        bit >>= 1;
    }
    uint32_t leaf = prefix;
    if (value == 0)
        leaf = SIZE_NONE;
    for (uint32_t i = 0; i < seg; ++i) {
        if (g->keys[prefix + i] == key) {
            g->values[prefix + i] = value;
            leaf = SIZE_NONE;
            break;
        }
    }
    return leaf;
}

/* Pending insertions: sorted keys with their values and current window node. */
typedef struct pending {
    uint64_t *keys;
    uint8_t *values;
    uint32_t *nodes;
    uint64_t n;
} pending;

/* compact_insertions (gpma.cuh:836-844): drop entries whose node is NONE,
 * keeping order. */
static void compact_pending(pending *p) {
    uint64_t w = 0;
    for (uint64_t i = 0; i < p->n; ++i) {
        if (p->nodes[i] == SIZE_NONE)
            continue;
        p->keys[w] = p->keys[i];
        p->values[w] = p->values[i];
        p->nodes[w] = p->nodes[i];
        ++w;
    }
    p->n = w;
}

/* group_insertion_by_node (gpma.cuh:846-873): run-length encode the nodes;
 * offsets has runs+1 entries, the last one = p->n. */
static uint64_t group_by_node(const pending *p, uint32_t *unique_nodes, uint64_t *offsets) {
    uint64_t runs = 0;
    for (uint64_t i = 0; i < p->n; ++i) {
        if (i == 0 || p->nodes[i] != p->nodes[i - 1]) {
            unique_nodes[runs] = p->nodes[i];
            offsets[runs] = i;
            ++runs;
        }
    }
    offsets[runs] = p->n;
    return runs;
}

/* redispatch_loop_body (gpma.cuh:636-654): element i of the merged window goes
 * to segment F*i/M at lane (F*i mod M)/F; a guard key records its slot in
 * row_offset[row+1]. */
static void redispatch(oracle_gpma *g, uint64_t *dst_keys, uint8_t *dst_values, const uint64_t *src_keys,
                       const uint8_t *src_values, uint32_t width, uint32_t merge_size, uint32_t node) {
    uint64_t frac = width / g->segment_length;
    uint64_t deno = merge_size;
    for (uint32_t i = 0; i < merge_size; ++i) {
        uint32_t seg_idx = (uint32_t)(frac * i / deno);
        uint32_t seg_lane = (uint32_t)(frac * i % deno / frac);
        uint32_t proj = seg_idx * g->segment_length + seg_lane;
        uint64_t key = src_keys[i];
        dst_keys[proj] = key;
        dst_values[proj] = src_values[i];
        if ((key & COL_IDX_NONE) == COL_IDX_NONE) {
            uint32_t row = (uint32_t)(key >> 32);
            g->row_offset[row + 1] = proj + node;
        }
    }
}

/* One window of rebalancing_impl_cpu (gpma.cuh:665-726): compact the live
 * entries (key != NONE and value != 0; tombstones are dropped here), accept iff
 * lower <= live + pending <= upper, then append the pending insertions, sort,
 * clear the window and redispatch evenly. Returns 1 if accepted. */
static int rebalance_window(oracle_gpma *g, uint32_t node, uint32_t level, const pending *p, uint64_t a, uint64_t b,
                            uint32_t lower, uint32_t upper, uint64_t *tmp_k, uint8_t *tmp_v) {
    uint32_t width = g->segment_length << level;
    uint64_t *wk = g->keys + node;
    uint8_t *wv = g->values + node;
    uint32_t live = 0;
    for (uint32_t i = 0; i < width; ++i) {
        if (wk[i] == KEY_NONE || wv[i] == 0)
            continue;
        tmp_k[live] = wk[i];
        tmp_v[live] = wv[i];
        ++live;
    }
    uint64_t interval = b - a;
    uint64_t merge_size = live + interval;
    if (!(lower <= merge_size && merge_size <= upper))
        return 0;
    memcpy(tmp_k + live, p->keys + a, interval * sizeof(uint64_t));
    memcpy(tmp_v + live, p->values + a, interval);
    for (uint64_t i = a; i < b; ++i)
        p->nodes[i] = SIZE_NONE;
    stable_sort_kv(tmp_k, tmp_v, merge_size);
    for (uint32_t i = 0; i < width; ++i)
        wk[i] = KEY_NONE;
    redispatch(g, wk, wv, tmp_k, tmp_v, width, (uint32_t)merge_size, node);
    return 1;
}

/* rebalance_batch (gpma.cuh:796-834) for one level over all unique nodes. */
static void rebalance_level(oracle_gpma *g, uint32_t level, pending *p, const uint32_t *unique_nodes,
                            const uint64_t *offsets, uint64_t runs, uint32_t lower, uint32_t upper) {
    uint32_t width = g->segment_length << level;
    uint64_t acc_windows = 0;
#pragma omp parallel num_threads(g->threads) reduction(+ : acc_windows)
    {
        /* per-thread window scratch, allocated on a thread's first window
         * (a root window spans the whole array); merge_size <= upper <= width */
        uint64_t *tk = NULL;
        uint8_t *tv = NULL;
#pragma omp for schedule(dynamic, 8)
        for (int64_t r = 0; r < (int64_t)runs; ++r) {
            if (!tk) {
                tk = (uint64_t *)xmalloc(sizeof(uint64_t) * ((uint64_t)width + 1));
                tv = (uint8_t *)xmalloc((uint64_t)width + 1);
            }
            acc_windows += (uint64_t)rebalance_window(g, unique_nodes[r], level, p, offsets[r], offsets[r + 1], lower,
                                                      upper, tk, tv);
        }
        free(tk);
        free(tv);
    }
    g->stats.accepted_windows += acc_windows;
    g->stats.accepted_slots += acc_windows * (uint64_t)width;
}

/* resize_gpma (gpma.cuh:906-934): stable removal of empty slots and
 * tombstones over the whole array, smallest power-of-two size >= 4 with
 * floor(0.84 * size) >= live + increase, new segment length and height,
 * thresholds recomputed. row_offset is left as it is. Returns the live count. */
static uint32_t resize_gpma(oracle_gpma *g, uint64_t increased) {
    uint32_t w = 0;
    for (uint32_t i = 0; i < g->size; ++i) {
        if (g->keys[i] == KEY_NONE || g->values[i] == 0)
            continue;
        g->keys[w] = g->keys[i];
        g->values[w] = g->values[i];
        ++w;
    }
    for (uint32_t i = w; i < g->size; ++i)
        g->keys[i] = KEY_NONE;
    uint32_t compacted = w;
    uint32_t merge_size = (uint32_t)(compacted + increased);
    uint32_t tree_size = 4;
    while (floor(UPPER_ROOT * (double)tree_size) < (double)merge_size)
        tree_size *= 2;
    g->segment_length = 1u << (fls32(fls32(tree_size)) - 1);
    g->tree_height = fls32(tree_size / g->segment_length) - 1;
    uint64_t *nk = (uint64_t *)xmalloc(sizeof(uint64_t) * tree_size);
    uint8_t *nv = (uint8_t *)calloc(tree_size, 1);
    if (!nv)
        abort();
    uint32_t keep = g->size < tree_size ? g->size : tree_size;
    memcpy(nk, g->keys, sizeof(uint64_t) * keep);
    memcpy(nv, g->values, keep);
    for (uint32_t i = keep; i < tree_size; ++i)
        nk[i] = KEY_NONE;
    free(g->keys);
    free(g->values);
    g->keys = nk;
    g->values = nv;
    g->size = tree_size;
    recalculate_density(g);
    return compacted;
}

/* significant_insert (gpma.cuh:936-966): resize, append the insertions, sort
 * everything and redispatch the whole array into fresh zero-filled arrays, so
 * gaps hold key 0 / value 0 rather than KEY_NONE. */
static void significant_insert(oracle_gpma *g, const pending *p) {
    uint32_t valid = resize_gpma(g, p->n);
    uint64_t merge_size = valid + p->n;
    memcpy(g->keys + valid, p->keys, p->n * sizeof(uint64_t));
    memcpy(g->values + valid, p->values, p->n);
    stable_sort_kv(g->keys, g->values, merge_size);
    uint64_t *nk = (uint64_t *)calloc(g->size, sizeof(uint64_t));
    uint8_t *nv = (uint8_t *)calloc(g->size, 1);
    if (!nk || !nv)
        abort();
    redispatch(g, nk, nv, g->keys, g->values, g->size, (uint32_t)merge_size, 0);
    free(g->keys);
    free(g->values);
    g->keys = nk;
    g->values = nv;
    g->stats.significant++;
    g->stats.accepted_windows++;
    g->stats.accepted_slots += g->size;
}

/* update_gpma (gpma.cuh:968-1050). */
int oracle_update(oracle_gpma *g, const uint64_t *keys, const uint8_t *values, uint64_t n) {
    g->stats.updates++;
    pending p;
    p.n = n;
    p.keys = (uint64_t *)xmalloc(sizeof(uint64_t) * (n ? n : 1));
    p.values = (uint8_t *)xmalloc(n ? n : 1);
    p.nodes = (uint32_t *)xmalloc(sizeof(uint32_t) * (n ? n : 1));
    if (n) {
        memcpy(p.keys, keys, n * sizeof(uint64_t));
        memcpy(p.values, values, n);
    }
    /* step 1: sort the batch by key (gpma.cuh:977) */
    stable_sort_kv(p.keys, p.values, n);
    /* step 2: locate leaves, applying deletes/modifies in place (gpma.cuh:984) */
#pragma omp parallel for num_threads(g->threads) schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)n; ++i)
        p.nodes[i] = locate_one(g, p.keys[i], p.values[i]);
    /* step 3: keep the insertions and group them by leaf (gpma.cuh:994-997) */
    compact_pending(&p);
    uint32_t *unique_nodes = (uint32_t *)xmalloc(sizeof(uint32_t) * (p.n + 1));
    uint64_t *offsets = (uint64_t *)xmalloc(sizeof(uint64_t) * (p.n + 2));
    uint64_t runs = group_by_node(&p, unique_nodes, offsets);
    g->stats.last_inserts = p.n;
    /* step 4: bulk rebuild for a significant insertion (gpma.cuh:1003-1007) */
    if (p.n >= SIGNIFICANT_INSERTS) {
        significant_insert(g, &p);
    } else {
        /* step 5: level loop (gpma.cuh:1012-1029) */
        for (uint32_t level = 0; level <= g->tree_height && p.n; level++) {
            g->stats.levels_visited++;
            rebalance_level(g, level, &p, unique_nodes, offsets, runs, g->lower[level], g->upper[level]);
            compact_pending(&p);
            uint32_t width = g->segment_length << level;
            for (uint64_t i = 0; i < p.n; ++i)
                p.nodes[i] &= ~width; /* up_level_kernel, gpma.cuh:881-889 */
            runs = group_by_node(&p, unique_nodes, offsets);
        }
        /* step 6: root resize + root rebalance (gpma.cuh:1034-1044); a failed
         * density check here drops the remaining insertions. */
        if (p.n > 0) {
            g->stats.root_resizes++;
            resize_gpma(g, p.n);
            uint32_t level = g->tree_height;
            uint64_t before = g->stats.accepted_windows;
            rebalance_level(g, level, &p, unique_nodes, offsets, runs, g->lower[level], g->upper[level]);
            if (g->stats.accepted_windows == before)
                g->stats.root_drops++;
        }
    }
    free(unique_nodes);
    free(offsets);
    free(p.keys);
    free(p.values);
    free(p.nodes);
    return 0;
}

/* ---- BFS ---------------------------------------------------------------- */

/* Level-synchronous semantics of gpma_bfs_multidev_single + gather/contract
 * (gpma_bfs.cuh:150-395, 446-509), computed with a FIFO queue: a slot in
 * [row_offset[v], row_offset[v+1]) is an edge unless its low 32 bits are
 * 0xFFFFFFFF (guard or empty) or its value is 0 (tombstone or bulk gap).
 * Neighbours >= row_num are ignored (the reference would write out of bounds). */
int oracle_bfs(const oracle_gpma *g, uint32_t src, uint32_t *levels, uint64_t *reached) {
    uint32_t n = g->row_num;
    if (src >= n)
        return -1;
    memset(levels, 0, sizeof(uint32_t) * n);
    uint32_t *queue = (uint32_t *)xmalloc(sizeof(uint32_t) * n);
    uint64_t head = 0, tail = 0;
    levels[src] = 1;
    queue[tail++] = src;
    while (head < tail) {
        uint32_t u = queue[head++];
        uint32_t lu = levels[u];
        uint32_t b = g->row_offset[u], e = g->row_offset[u + 1];
        for (uint32_t s = b; s < e && s < g->size; ++s) {
            uint64_t key = g->keys[s];
            uint32_t w = (uint32_t)(key & COL_IDX_NONE);
            if (w == (uint32_t)COL_IDX_NONE || g->values[s] == 0 || w >= n)
                continue;
            if (levels[w] == 0) {
                levels[w] = lu + 1;
                queue[tail++] = w;
            }
        }
    }
    free(queue);
    if (reached)
        *reached = tail;
    return 0;
}

int oracle_bfs_multi(const oracle_gpma *g, const uint32_t *srcs, uint32_t k, uint32_t *levels, uint64_t *reached) {
    int rc = 0;
#pragma omp parallel for num_threads(g->threads) schedule(dynamic, 1)
    for (int64_t i = 0; i < (int64_t)k; ++i) {
        int r = oracle_bfs(g, srcs[i], levels + (uint64_t)i * g->row_num, reached ? reached + i : NULL);
        if (r)
            rc = r;
    }
    return rc;
}

uint64_t oracle_traversed_edges(const oracle_gpma *g, const uint32_t *levels) {
    uint64_t total = 0;
    for (uint32_t v = 0; v < g->row_num; ++v) {
        if (!levels[v])
            continue;
        for (uint32_t s = g->row_offset[v]; s < g->row_offset[v + 1] && s < g->size; ++s) {
            uint32_t w = (uint32_t)(g->keys[s] & COL_IDX_NONE);
            if (w != (uint32_t)COL_IDX_NONE && g->values[s] != 0 && w < g->row_num)
                ++total;
        }
    }
    return total;
}

/* ---- views -------------------------------------------------------------- */

uint64_t oracle_compact(const oracle_gpma *g, uint64_t *out) {
    uint64_t c = 0;
    for (uint32_t i = 0; i < g->size; ++i) {
        if (g->keys[i] == KEY_NONE || g->values[i] == 0)
            continue;
        if (out)
            out[c] = g->keys[i];
        ++c;
    }
    return c;
}

void oracle_export(const oracle_gpma *g, uint64_t *keys, uint8_t *masked_values, uint32_t *row_offset) {
    if (keys)
        memcpy(keys, g->keys, sizeof(uint64_t) * g->size);
    if (masked_values)
        for (uint32_t i = 0; i < g->size; ++i)
            masked_values[i] = g->keys[i] == KEY_NONE ? 0 : g->values[i];
    if (row_offset)
        memcpy(row_offset, g->row_offset, sizeof(uint32_t) * ((uint64_t)g->row_num + 1));
}

static uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
#define DIGEST_BODY                                                                                                    \
    uint64_t acc = 0;                                                                                                  \
    for (uint64_t i = 0; i < n; ++i)                                                                                   \
        acc += mix64((uint64_t)x[i] + (i + 1) * 0x9E3779B97F4A7C15ull);                                                \
    return acc;
uint64_t oracle_digest_u64(const uint64_t *x, uint64_t n) { DIGEST_BODY }
uint64_t oracle_digest_u32(const uint32_t *x, uint64_t n) { DIGEST_BODY }
uint64_t oracle_digest_u8(const uint8_t *x, uint64_t n) { DIGEST_BODY }
