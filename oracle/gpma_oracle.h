/*
 * gpma_oracle.h - CPU restatement of the reference GPMA+ update and BFS.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker for the CUDA path:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it. The product library (gpma_bfs_gb300) never links or calls it.
 *
 * It restates, step by step, the reference's CPU instantiation GPMA<CPU>
 * (gpma.cuh) which is layout-exact with the reference GPU algorithm, plus a
 * sequential BFS with the level semantics of gpma_bfs.cuh. Parity is pinned by
 * tests/test_oracle_golden.py against vectors produced by the reference itself
 * (oracle/ref/ref_driver.cu built from the reference sources).
 */
#ifndef GPMA_ORACLE_H
#define GPMA_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORACLE_KEY_NONE 0xFFFFFFFFFFFFFFFFull /* gpma.cuh:15 */
#define ORACLE_KEY_MAX 0xFFFFFFFFFFFFFFFEull  /* gpma.cuh:16 */
#define ORACLE_SIZE_NONE 0xFFFFFFFFu          /* gpma.cuh:17 */
#define ORACLE_COL_NONE 0xFFFFFFFFull         /* gpma.cuh:19 */

typedef struct oracle_stats {
    uint64_t updates;           /* update calls */
    uint64_t accepted_windows;  /* windows redispatched (all levels, root) */
    uint64_t accepted_slots;    /* sum of window widths redispatched */
    uint64_t levels_visited;    /* level-loop iterations executed */
    uint64_t root_resizes;      /* resize_gpma calls from the root step */
    uint64_t root_drops;        /* root rebalances whose density check failed */
    uint64_t significant;       /* significant_insert rebuilds */
    uint64_t last_inserts;      /* insertions left after delete/modify in the last call */
} oracle_stats;

typedef struct oracle_gpma {
    uint64_t *keys;      /* size slots */
    uint8_t *values;     /* size slots */
    uint32_t size;
    uint32_t segment_length;
    uint32_t tree_height;
    uint32_t *lower;     /* tree_height + 1 */
    uint32_t *upper;     /* tree_height + 1 */
    uint32_t row_num;
    uint32_t *row_offset; /* row_num + 1 */
    int threads;          /* OpenMP threads for the parallel loops (>=1) */
    oracle_stats stats;
} oracle_gpma;

/* GPMA(row_num): init_gpma_members + init_gpma_insertions (gpma.cuh:54-82). */
oracle_gpma *oracle_create(uint32_t row_num, int threads);
void oracle_destroy(oracle_gpma *g);

/* update_gpma (gpma.cuh:968-1050). Inputs are copied; returns 0 on success. */
int oracle_update(oracle_gpma *g, const uint64_t *keys, const uint8_t *values, uint64_t n);

/* Sequential BFS over row_offset with the reference's level semantics
 * (gpma_bfs.cuh:446-509): levels[src] = 1, a neighbour of a level-L node gets
 * L+1, unreached nodes stay 0. Returns 0 on success, -1 if src >= row_num. */
int oracle_bfs(const oracle_gpma *g, uint32_t src, uint32_t *levels, uint64_t *reached);

/* Multi-source form: one independent BFS per source, levels laid out
 * [k][row_num]. */
int oracle_bfs_multi(const oracle_gpma *g, const uint32_t *srcs, uint32_t k, uint32_t *levels, uint64_t *reached);

/* Live out-degree sum of the nodes with levels[v] != 0 (edges traversed). */
uint64_t oracle_traversed_edges(const oracle_gpma *g, const uint32_t *levels);

/* Live keys (key != NONE and value != 0) in slot order; returns the count.
 * out may be NULL to query the count. */
uint64_t oracle_compact(const oracle_gpma *g, uint64_t *out);

/* Copy of the raw layout with values masked to 0 where the key is NONE. */
void oracle_export(const oracle_gpma *g, uint64_t *keys, uint8_t *masked_values, uint32_t *row_offset);

/* Order-sensitive digest used by the golden vectors (see ref_driver.cu). */
uint64_t oracle_digest_u64(const uint64_t *x, uint64_t n);
uint64_t oracle_digest_u32(const uint32_t *x, uint64_t n);
uint64_t oracle_digest_u8(const uint8_t *x, uint64_t n);

#ifdef __cplusplus
}
#endif
#endif
