/*
 * gpma_gb300.h - C ABI of the GB300-native GPMA+ (dynamic graph in a GPU
 * packed memory array) and its BFS.
 *
 * The reference (recolic/gpma_bfs) is a header-only C++/CUDA template library
 * with no C ABI; these entry points are what its update/BFS path would export
 * through an FFI. Types follow the reference: keys are uint64_t
 * (src << 32 | dst, utils.cuh:11,19), values are one byte (utils.cuh:20;
 * 1 = live/insert, 0 = delete/tombstone, gpma.cuh:18), slot indices and node
 * ids are uint32_t (utils.cuh:21).
 *
 * Every call returns a status and never aborts. Pointer arguments documented
 * as "host or device" may point to pageable host memory, pinned host memory
 * or device memory of the graph's GPU; the library detects which. A graph
 * handle is single-writer: concurrent calls on one handle must be serialised
 * by the caller. `stream` is a cudaStream_t (NULL = legacy default stream).
 */
#ifndef GPMA_GB300_H
#define GPMA_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define GPMA_API __attribute__((visibility("default")))
#else
#define GPMA_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gpma_status {
    GPMA_OK = 0,
    GPMA_ERR_INVALID = 1,  /* bad argument: null pointer, out-of-range node, ... */
    GPMA_ERR_CUDA = 2,     /* a CUDA runtime call failed (see gpma_last_error) */
    GPMA_ERR_NOMEM = 3,    /* device or host allocation failed */
    GPMA_ERR_CAPACITY = 4, /* the structure would exceed 2^31 slots (32-bit slot ids) */
    GPMA_ERR_TIMEOUT = 5,  /* a bounded device-side wait gave up; the context stays usable */
    GPMA_ERR_IO = 6,       /* file could not be read or written */
    GPMA_ERR_DEVICE = 7,   /* a device-side consistency check failed */
    GPMA_ERR_BUSY = 8,     /* server queue full: retry after a round has run */
    GPMA_ERR_BUDGET = 9    /* the server's HBM admission budget would be exceeded */
} gpma_status;

typedef struct gpma_graph gpma_graph;

typedef struct gpma_geometry {
    uint32_t size;           /* slots in the array (power of two), GPMA::keys.size() */
    uint32_t segment_length; /* GPMA::segment_length (gpma.cuh:37) */
    uint32_t tree_height;    /* GPMA::tree_height (gpma.cuh:38) */
    uint32_t row_num;        /* GPMA::row_num (gpma.cuh:49) */
} gpma_geometry;

typedef struct gpma_stats {
    uint64_t updates;          /* gpma_update calls */
    uint64_t submitted;        /* keys submitted over all calls */
    uint64_t last_inserts;     /* insertions left after delete/modify in the last call */
    uint64_t levels_visited;   /* level-loop iterations executed */
    uint64_t accepted_windows; /* windows redispatched */
    uint64_t accepted_slots;   /* sum of the widths of redispatched windows */
    uint64_t root_resizes;     /* root resizes (gpma.cuh:1034-1044) */
    uint64_t root_drops;       /* root rebalances that failed their density check */
    uint64_t significant;      /* bulk rebuilds for >= 5,000,000 insertions (gpma.cuh:1003) */
} gpma_stats;

/* ---- lifetime ------------------------------------------------------------
 * Replaces the reference constructor GPMA<GPU>::GPMA(SIZE_TYPE row_num)
 * (gpma.cuh:79-82): an empty structure plus one guard key (r<<32)|0xFFFFFFFF
 * per row, inserted through the update path (gpma.cuh:70-78). Uses the
 * current CUDA device. */
GPMA_API gpma_status gpma_create(uint32_t row_num, void *stream, gpma_graph **out);

/* Releases every device and host buffer of the graph (reference: ~GPMA). */
GPMA_API gpma_status gpma_destroy(gpma_graph *g);

/* ---- update --------------------------------------------------------------
 * Replaces update_gpma<GPU>(GPMA&, NATIVE_VEC_KEY&, NATIVE_VEC_VALUE&)
 * (gpma.cuh:27,968-1050). keys/values (host or device, n entries each) are a
 * batch of edge keys; value 0 deletes the key, a non-zero value inserts it or
 * overwrites the value of an existing key. Unlike the reference, the inputs
 * are not modified. Returns after the structure is updated (the stream is
 * synchronised). Keys that occur more than once in one batch with different
 * values are applied in an unspecified order, as in the reference. */
GPMA_API gpma_status gpma_update(gpma_graph *g, const uint64_t *keys, const uint8_t *values, uint64_t n, void *stream);

/* ---- BFS -----------------------------------------------------------------
 * Replaces gpma_bfs(const GPMA_multidev&, node_size, edge_size, start_node,
 * SIZE_TYPE *results) (gpma_bfs.cuh:517-533) and the single-device
 * gpma_bfs<DEV>(keys, values, row_offsets, node_size, edge_size, start_node,
 * results) (gpma_bfs.cuh:511-515). levels (host or device, row_num entries)
 * receives the BFS level of every node: 1 for src, L+1 for a neighbour of a
 * level-L node, 0 for unreached. reached (optional, host) receives the
 * number of non-zero levels. */
GPMA_API gpma_status gpma_bfs(gpma_graph *g, uint32_t src, uint32_t *levels, uint64_t *reached, void *stream);

/* Multi-source BFS: k (1..64) independent searches in one traversal, one bit
 * lane per source. levels (host or device) is [k][row_num]; reached
 * (optional, host) has k entries. Each row equals gpma_bfs from that source.
 * No reference counterpart (the reference BFS takes one source). */
GPMA_API gpma_status gpma_bfs_multi(gpma_graph *g, const uint32_t *srcs, uint32_t k, uint32_t *levels, uint64_t *reached,
                           void *stream);

/* BFS for callers that cannot allocate device memory (a host-side arena or a
 * fixed device budget owns every allocation, or allocation is forbidden
 * while serving). No counterpart in the reference. Same result as gpma_bfs,
 * but it allocates nothing: its working set (visited bitmap, two frontier
 * bitmaps, big-row chunk list, control words) is one fixed device array inside
 * the library, about 1.3 MB. A device commits it when the library's kernels are
 * first used there (CUDA loads modules lazily by default) and holds it until
 * the process exits. Rows that find the chunk list (65,536 entries) full are
 * walked in place: slower, same result.
 * Limits: row_num <= 2,097,152 (GPMA_ERR_CAPACITY beyond); levels must be
 * device memory of row_num entries (GPMA_ERR_INVALID otherwise); reached is an
 * optional host pointer. The first call on a device looks up the array's
 * device address with that device current. All calls share the one array
 * and it keeps the last call's contents, so calls whose work overlaps on the
 * GPU (other threads, other streams) race: serialise them. */
GPMA_API gpma_status gpma_bfs_noalloc(gpma_graph *g, uint32_t src, uint32_t *levels, uint64_t *reached,
                                      void *stream);

/* ---- recorded update+BFS steps ------------------------------------------------
 * One slide step of the reference's demo loop (gpma_bfs_demo.cu: update_gpma
 * of the step's batch, then gpma_bfs from a source) whose device work is
 * recorded once as a CUDA graph and replayed for every later step: table
 * upload, update kernel, BFS clears and kernels, status read-back, one host
 * synchronisation. The graph is rebuilt only when a buffer or the launch
 * shape it holds changes; batch size and source may differ per step.
 * gpma_step_run gives exactly the results of gpma_update(keys, values, n)
 * followed by gpma_bfs(src, levels, reached) (levels may be NULL: the levels
 * stay in the library; keys, values and levels may be host or device
 * memory). When the update needs host work (root resize, the bulk rebuild of
 * a large batch) the step finishes on the host and runs the BFS again.
 * Destroy a step before its graph. No reference counterpart. */
typedef struct gpma_step gpma_step;
typedef struct gpma_step_stats {
    uint64_t runs;           /* gpma_step_run calls */
    uint64_t graph_launches; /* steps replayed as one graph launch */
    uint64_t builds;         /* graph (re)builds */
    uint64_t param_updates;  /* kernel nodes whose arguments were updated in place */
    uint64_t host_runs;      /* steps whose BFS ran outside the graph (empty batch, root resize, bulk rebuild) */
    double last_ms;          /* device time of the last graph launch (CUDA events) */
    double total_ms;         /* summed over graph launches */
} gpma_step_stats;
GPMA_API gpma_status gpma_step_create(gpma_graph *g, gpma_step **out);
GPMA_API gpma_status gpma_step_destroy(gpma_step *st);
GPMA_API gpma_status gpma_step_run(gpma_step *st, const uint64_t *keys, const uint8_t *values, uint64_t n,
                                   uint32_t src, uint32_t *levels, uint64_t *reached, void *stream);
GPMA_API gpma_status gpma_step_get_stats(const gpma_step *st, gpma_step_stats *out);

/* ---- analytics on the same array --------------------------------------------
 * No reference counterpart (the reference's only analytic is the BFS). Both
 * sweep every slot of the gapped array once per iteration; an edge is a
 * slot the BFS would follow.
 *
 * PageRank with damping d over the out-edges (dangling nodes spread their
 * rank evenly): ranks start at 1/row_num; `iterations` iterations at most,
 * fewer once the L1 change of an iteration drops below tol. ranks (host or
 * device, row_num floats) receives the result; summation order is not fixed
 * (float atomics), so results vary in the last bits between runs. */
GPMA_API gpma_status gpma_pagerank(gpma_graph *g, float damping, uint32_t iterations, double tol, float *ranks,
                                   uint32_t *iterations_run, void *stream);

/* Weakly connected components: labels (host or device, row_num entries)
 * receives, for every node, the smallest node id of its component (exact and
 * deterministic); components (optional) the number of components, isolated
 * nodes included; rounds (optional) the hook-and-jump rounds run. */
GPMA_API gpma_status gpma_components(gpma_graph *g, uint32_t *labels, uint64_t *components, uint32_t *rounds,
                                     void *stream);

/* ---- many graphs per launch -------------------------------------------------
 * No reference counterpart: the reference updates one GPMA per call. A
 * gpma_batch owns the update buffers shared by the graphs of one call. All
 * graphs of a call must live on the current device and be distinct. */
typedef struct gpma_batch gpma_batch;
GPMA_API gpma_status gpma_batch_create(gpma_batch **out);
GPMA_API gpma_status gpma_batch_destroy(gpma_batch *b);

/* Applies k independent update batches, batch i (keys[i], values[i],
 * counts[i] entries, host or device) to graphs[i], in one persistent kernel
 * launch; each graph ends exactly as gpma_update(graphs[i], ...) would leave
 * it. Batches of 5,000,000 keys or more take the single-graph path. */
GPMA_API gpma_status gpma_batch_update(gpma_batch *b, gpma_graph *const *graphs, const uint64_t *const *keys,
                                       const uint8_t *const *values, const uint64_t *counts, uint32_t k,
                                       void *stream);

/* The same with all batches in one buffer: graph i's batch is
 * keys[offsets[i] .. offsets[i+1]) (and values likewise); keys/values host or
 * device, offsets a host array of k + 1 entries. One copy and one device
 * gather stage every batch, whatever the graph order. */
GPMA_API gpma_status gpma_batch_update_packed(gpma_batch *b, gpma_graph *const *graphs, const uint64_t *keys,
                                              const uint8_t *values, const uint64_t *offsets, uint32_t k,
                                              void *stream);

/* Multi-source BFS on k graphs in one persistent launch: graph i searches
 * from nsrc[i] (1..64) sources srcs[i][0..nsrc[i]), one bit lane per source.
 * levels (optional; NULL or per-graph pointers, host or device, each
 * [nsrc[i]][row_num]) receives the levels; reached (optional, host) receives
 * sum(nsrc) counts, graph by graph. Each search equals gpma_bfs from that
 * source. */
GPMA_API gpma_status gpma_batch_bfs_multi(gpma_batch *b, gpma_graph *const *graphs, const uint32_t *const *srcs,
                                          const uint32_t *nsrc, uint32_t k, uint32_t *const *levels,
                                          uint64_t *reached, void *stream);

/* The batched form's step (no reference counterpart): one packed update of
 * every graph of the step (as gpma_batch_update_packed) and one multi-source
 * BFS over all of them (as gpma_batch_bfs_multi without levels), recorded as
 * one CUDA graph. The graphs are fixed at creation (order kept); keys/values
 * are host or device memory, offsets (k + 1), srcs[i] (nsrc[i] in 1..64
 * sources) and reached (optional, sum of nsrc) are host memory. A step with
 * an empty or a bulk-sized (>= 5,000,000 keys) part, or whose update needs
 * host work, runs or finishes through the eager calls; results are always
 * those of the two calls. Destroy a step before its batch and graphs. */
typedef struct gpma_batch_step gpma_batch_step;
GPMA_API gpma_status gpma_batch_step_create(gpma_batch *b, gpma_graph *const *graphs, uint32_t k,
                                            gpma_batch_step **out);
GPMA_API gpma_status gpma_batch_step_destroy(gpma_batch_step *st);
GPMA_API gpma_status gpma_batch_step_run(gpma_batch_step *st, const uint64_t *keys, const uint8_t *values,
                                         const uint64_t *offsets, const uint32_t *const *srcs, const uint32_t *nsrc,
                                         uint64_t *reached, void *stream);
/* `steps` consecutive steps recorded in one CUDA graph and launched once: step
 * t applies keys[t]/values[t] (device memory) with offsets at offsets + t * (k
 * + 1), then searches from srcs/nsrc (the same sources every step); reached
 * (optional, host) receives steps x sum(nsrc) counts, step by step. The
 * recording is kept and replayed while the buffers and launch shapes it holds
 * stay the same (kernel arguments are refreshed in place). A step whose
 * update needs host work stops the recorded steps after it on the device;
 * that step and the later ones then finish as gpma_batch_step_run would, as
 * do all steps when one part is empty or bulk-sized or a batch is in host
 * memory. Results are always those of the per-step calls. */
GPMA_API gpma_status gpma_batch_step_run_many(gpma_batch_step *st, uint32_t steps, const uint64_t *const *keys,
                                              const uint8_t *const *values, const uint64_t *offsets,
                                              const uint32_t *const *srcs, const uint32_t *nsrc, uint64_t *reached,
                                              void *stream);
GPMA_API gpma_status gpma_batch_step_get_stats(const gpma_batch_step *st, gpma_step_stats *out);

/* ---- served form ----------------------------------------------------------
 * No reference counterpart. A gpma_server keeps many graphs resident on the
 * current device and serves update batches and BFS queries against them with
 * continuous batching: requests wait in one FIFO queue per graph; each round
 * takes, for every graph whose queue head has arrived, at most one update
 * batch and then the BFS queries queued directly behind it (packed as source
 * lanes, up to 64 per graph), and runs all of the round's updates in one
 * batched update launch followed by one multi-source BFS launch. Requests that
 * arrive while a round runs join a later round. A graph's requests therefore
 * take effect in arrival order and every result equals what the same requests
 * give applied to that graph alone. Time is the caller's: it passes the
 * current time to each round (a virtual clock, or the wall clock since some
 * start); a round's updates complete at that time plus the measured
 * wall-clock time of its update launch, its searches at that time plus the
 * whole round's; a request runs only once the time passed reaches its
 * arrival, so requests may be submitted ahead of it.
 *
 * Lanes. With lanes = k > 1 the server keeps k rounds in flight: each lane
 * has its own stream, batch buffers and pinned staging, gpma_server_run_round
 * may be called from k host threads at once (each call takes a free lane, or
 * returns an empty round when all k are busy), and a graph whose requests are
 * in one lane's round is left out of the other lanes' rounds until that round
 * completes, so a graph's requests still run in arrival order. Requests that
 * arrive while one round is on the GPU start in another lane without waiting
 * for it. The submit, poll, cancel and query calls may run concurrently with
 * rounds. With one lane (the default) rounds run one after another.
 *
 * Admission. A graph is admitted only if its estimated device bytes fit the
 * HBM budget; an update joins a round only if the graph's worst-case growth
 * (the array doubling until it holds its current capacity plus the batch's
 * insertions at the root density bound) still fits, otherwise it waits, and
 * fails with GPMA_ERR_BUDGET when it could not fit even alone. Submissions
 * beyond max_queued requests or max_queued_keys waiting update keys return
 * GPMA_ERR_BUSY. */
typedef struct gpma_server gpma_server;

#define GPMA_SERVER_PLAN_ONLY 1u /* schedule only: no device work (checks the policy on a host without a GPU) */

typedef struct gpma_server_config {
    uint64_t hbm_budget_bytes;     /* device bytes the admitted graphs may hold */
    uint64_t max_round_keys;       /* update keys per round (one larger batch may run alone) */
    uint32_t max_round_bfs_graphs; /* graphs searched per round */
    uint32_t max_queued;           /* waiting requests */
    uint64_t max_queued_keys;      /* waiting update keys (host copies) */
    uint32_t flags;                /* GPMA_SERVER_PLAN_ONLY */
    uint32_t lanes;                /* rounds in flight at once, 1..4 (0: 1) */
    uint64_t input_ring_bytes;     /* pinned host ring that queued update batches are copied into at submission
                                      (rounds upload them from there; a batch that finds it full stays in
                                      pageable memory); 0: none */
} gpma_server_config;

typedef enum gpma_request_state {
    GPMA_REQ_QUEUED = 0,
    GPMA_REQ_DONE = 1,
    GPMA_REQ_FAILED = 2,
    GPMA_REQ_CANCELLED = 3, /* withdrawn by gpma_server_cancel before a round took it */
    GPMA_REQ_RUNNING = 4    /* taken by a round that has not completed yet */
} gpma_request_state;

typedef struct gpma_request_info {
    uint64_t id;
    uint32_t graph;
    uint32_t kind;     /* 0 update, 1 BFS */
    uint32_t state;    /* gpma_request_state */
    int32_t status;    /* gpma_status of a failed request */
    double arrival;    /* virtual seconds, as submitted */
    double start;      /* start of the round that ran it */
    double done;       /* completion: start + the round's duration */
    uint64_t round;    /* 1-based round number */
    uint64_t keys;     /* update: keys in the batch */
    uint32_t nsrc;     /* BFS: sources */
    uint32_t lane;     /* BFS: first source lane of the request in its graph's search */
    uint64_t reached[64]; /* BFS: nodes reached from each source (the source included) */
} gpma_request_info;

typedef struct gpma_round_info {
    uint64_t round;
    double start, seconds;   /* virtual start; wall-clock duration of the round */
    uint32_t updates;        /* update requests run */
    uint32_t bfs_requests;   /* BFS requests run */
    uint32_t bfs_graphs;     /* graphs searched */
    uint32_t failed;         /* requests failed in this round */
    uint64_t keys;           /* update keys applied */
    uint64_t sources;        /* BFS sources searched */
    uint64_t edges;          /* edges traversed by the round's searches, all lanes */
    double update_ms, bfs_ms; /* device time of the update and BFS launches (CUDA events) */
} gpma_round_info;

/* stream: the stream every round runs on (NULL = legacy default stream). */
GPMA_API gpma_status gpma_server_create(const gpma_server_config *cfg, void *stream, gpma_server **out);
GPMA_API gpma_status gpma_server_destroy(gpma_server *s);
/* Admits a graph of row_num nodes sized for reserve_edges live edges
 * (GPMA_ERR_BUDGET when its estimate does not fit); *graph_id numbers graphs
 * from 0 in admission order. */
GPMA_API gpma_status gpma_server_add_graph(gpma_server *s, uint32_t row_num, uint64_t reserve_edges,
                                           uint32_t *graph_id);
/* The graph's handle, for loading it directly and for the views (NULL in
 * plan-only mode). Do not update it while requests for it are queued. */
GPMA_API gpma_status gpma_server_graph(gpma_server *s, uint32_t graph_id, gpma_graph **out);
/* Queues an update batch (host arrays, copied). */
GPMA_API gpma_status gpma_server_submit_update(gpma_server *s, uint32_t graph_id, const uint64_t *keys,
                                               const uint8_t *values, uint64_t n, double arrival,
                                               uint64_t *request_id);
/* Queues a BFS query from k (1..64) sources (host array, copied). levels
 * (optional, host, [k][row_num]) receives the levels when the request is done
 * and must stay valid until then. */
GPMA_API gpma_status gpma_server_submit_bfs(gpma_server *s, uint32_t graph_id, const uint32_t *sources, uint32_t k,
                                            double arrival, uint32_t *levels, uint64_t *request_id);
/* Runs one round at time `now` over the requests that arrived by then, on a
 * free lane; info (optional) describes it. A round with nothing to run (or no
 * free lane) returns GPMA_OK with info->updates == info->bfs_requests == 0. */
GPMA_API gpma_status gpma_server_run_round(gpma_server *s, double now, gpma_round_info *info);
/* A request's state and result; release != 0 forgets a finished request. */
GPMA_API gpma_status gpma_server_poll(gpma_server *s, uint64_t request_id, int release, gpma_request_info *out);
/* Withdraws a request that no round has taken yet (its client went away, or
 * it waits behind work it no longer needs): it leaves its graph's queue, its
 * keys no longer count against max_queued_keys, its level array is never
 * written, and polls report GPMA_REQ_CANCELLED. The graph's other requests
 * keep their order; a search queued behind a cancelled update sees the graph
 * without that update. GPMA_ERR_INVALID for an unknown request or one that
 * has already run. No reference counterpart. */
GPMA_API gpma_status gpma_server_cancel(gpma_server *s, uint64_t request_id);
/* Serving loop. gpma_server_start starts the server's clock at 0 and one
 * worker thread per lane; each runs rounds as soon as a queued request's
 * arrival (on that clock) has passed and a lane is free, and sleeps
 * otherwise (woken by submissions and completed rounds). Requests may be
 * submitted ahead of their arrival. gpma_server_clock reads the clock;
 * gpma_server_drain waits until no request is queued or running
 * (GPMA_ERR_TIMEOUT after timeout_seconds) and returns the first error a
 * round of the loop met; gpma_server_stop ends the loop after the rounds in
 * flight (gpma_server_destroy does too). While the loop runs, do not call
 * gpma_server_run_round. No reference counterpart. */
GPMA_API gpma_status gpma_server_start(gpma_server *s);
GPMA_API gpma_status gpma_server_clock(const gpma_server *s, double *now);
GPMA_API gpma_status gpma_server_drain(gpma_server *s, double timeout_seconds);
GPMA_API gpma_status gpma_server_stop(gpma_server *s);
/* Totals over every round run so far (by gpma_server_run_round or the loop). */
typedef struct gpma_server_stats {
    uint64_t rounds;              /* rounds that ran requests */
    uint64_t requests;            /* requests they completed or failed */
    uint64_t keys;                /* update keys applied */
    uint64_t edges;               /* edges traversed by their searches, all lanes */
    double busy_seconds;          /* sum of their wall-clock times (lanes overlap: may exceed elapsed time) */
    double update_ms;             /* device time of their update launches */
    double bfs_ms;                /* device time of their search launches */
    uint32_t max_round_requests;  /* most requests in one round */
    uint32_t max_inflight_rounds; /* most rounds in flight at once */
} gpma_server_stats;
GPMA_API gpma_status gpma_server_get_stats(const gpma_server *s, gpma_server_stats *out);
/* Ids of the requests the last round run by the calling host thread ran, in
 * execution order (updates, then searches graph by graph, lanes ascending). */
GPMA_API gpma_status gpma_server_last_round(const gpma_server *s, uint64_t *ids, uint32_t capacity, uint32_t *count);
/* Waiting requests and waiting update keys; earliest arrival among queue heads
 * (+infinity when nothing waits). */
GPMA_API gpma_status gpma_server_queued(const gpma_server *s, uint64_t *requests, uint64_t *keys,
                                        double *next_arrival);
/* Device bytes the admitted graphs are charged against the budget. */
GPMA_API gpma_status gpma_server_committed_bytes(const gpma_server *s, uint64_t *bytes);

/* ---- views ---------------------------------------------------------------
 * GPMA's public members (gpma.cuh:31-52) as read-only views. */
GPMA_API gpma_status gpma_get_geometry(const gpma_graph *g, gpma_geometry *out);

/* Density thresholds lower_element/upper_element (gpma.cuh:45-46,147-168):
 * tree_height + 1 entries each (host arrays). */
GPMA_API gpma_status gpma_get_thresholds(const gpma_graph *g, uint32_t *lower, uint32_t *upper);

/* Copies the raw layout (GPMA::keys, values and row_offset). keys has `size`
 * entries, masked_values has `size` entries (the slot's value, or 0 where the
 * key is empty), row_offset has row_num + 1 entries. Any of them may be NULL;
 * each may be host or device. */
GPMA_API gpma_status gpma_export_layout(gpma_graph *g, uint64_t *keys, uint8_t *masked_values, uint32_t *row_offset,
                               void *stream);

/* Live keys (non-empty, value != 0) in slot order, i.e. the sorted key set
 * including the row guards and the two KEY_MAX sentinels. With keys == NULL
 * only *count is written. keys (host or device) holds `capacity` entries. */
GPMA_API gpma_status gpma_export_compact(gpma_graph *g, uint64_t *keys, uint64_t capacity, uint64_t *count, void *stream);

/* Raw device pointers to the live arrays (valid until the next update). */
GPMA_API gpma_status gpma_device_arrays(gpma_graph *g, const uint64_t **keys, const uint8_t **values,
                               const uint32_t **row_offset);

GPMA_API gpma_status gpma_get_stats(const gpma_graph *g, gpma_stats *out);

/* Consistency check (no reference counterpart). The locate search compares
 * keys at segment starts, read from a dense copy that every writer of the
 * array keeps (one key per segment); *bad receives the number of segments
 * whose copy differs from the array: 0 for a consistent structure. */
GPMA_API gpma_status gpma_validate(gpma_graph *g, uint64_t *bad, void *stream);

/* ---- profiling -------------------------------------------------------------
 * With profiling on, CUDA events recorded on the caller's stream time each
 * phase; times accumulate until gpma_reset_profile. kernel_launches counts
 * every kernel the library launched on the graph's behalf (always on).
 * No reference counterpart (the reference printed wall-clock deltas,
 * rdebug.hpp:8-17). */
typedef struct gpma_profile {
    double sort_ms;          /* inside the update kernel: batch sort */
    double locate_ms;        /* inside the update kernel: leaf locate + delete/modify */
    double group_ms;         /* inside the update kernel: insertion compaction + grouping */
    double levels_ms;        /* inside the update kernel: the level loop */
    double update_kernel_ms; /* whole persistent update kernel (events on the stream) */
    double rebuild_ms;       /* root resize / bulk rebuild kernels */
    double bfs_ms;           /* BFS kernels (single- and multi-source) */
    uint64_t update_kernels; /* launches of the persistent update kernel */
    uint64_t bfs_kernels;    /* launches of BFS traversal kernels */
    uint64_t kernel_launches;
    uint64_t bfs_edges;      /* edges scanned from reached nodes by multi-source BFS, summed over sources */
    uint64_t sort_fallbacks; /* update launches whose bucket sort met a bucket of more than 1024 keys and
                                sorted by digit passes instead */
} gpma_profile;
GPMA_API gpma_status gpma_set_profiling(gpma_graph *g, int enabled);
GPMA_API gpma_status gpma_get_profile(const gpma_graph *g, gpma_profile *out);
GPMA_API gpma_status gpma_reset_profile(gpma_graph *g);
/* The same for the launches of a gpma_batch. */
GPMA_API gpma_status gpma_batch_set_profiling(gpma_batch *b, int enabled);
GPMA_API gpma_status gpma_batch_get_profile(const gpma_batch *b, gpma_profile *out);
GPMA_API gpma_status gpma_batch_reset_profile(gpma_batch *b);
/* Per level of the last gpma_bfs run with profiling on: its duration (ms, from
 * %globaltimer stamps at level starts), its frontier size (counted as the
 * previous level's claims: a node that several lanes found unvisited at once
 * counts once per lane) and whether it swept the whole array (dense). Up to `capacity` entries; *levels = levels run
 * (0 when the last BFS was not profiled). */
GPMA_API gpma_status gpma_bfs_level_profile(const gpma_graph *g, double *ms, uint32_t *frontier, uint8_t *dense,
                                            uint32_t capacity, uint32_t *levels);

/* ---- tuning -----------------------------------------------------------------
 * No reference counterpart. Launch shapes and switch points of the kernels;
 * they change speed, never results (the PMA geometry itself is fixed by the
 * reference's sizing rules). Process-wide; takes effect at the next call.
 * The settings are plain words read at each launch: change them while no
 * other host thread is inside a library call. */
typedef struct gpma_tuning {
    uint32_t bfs_dense_div;        /* single-source BFS: a level whose frontier's rows span >= size / bfs_dense_div
                                      slots sweeps the whole slot array instead of walking rows (0: never) */
    uint32_t bfs_blocks_per_sm;    /* BFS grid: CTAs per SM (capped by occupancy; 0: as many as fit) */
    uint32_t ms_dense_div;         /* multi-source BFS: the same switch on the union frontier of all lanes,
                                      against the slots of all graphs of the call */
    uint32_t ms_blocks_per_sm;     /* multi-source BFS grid */
    uint32_t update_blocks_per_sm; /* persistent update kernel: 1-2 use the 128-register build, 3 the 80-register
                                      one (more warps, some spills); 0 lets each launch choose (3 from 1M keys) */
    uint32_t update_sort;          /* batch sort inside the update kernel: 0 buckets (equal slot ranges of the
                                      array, a key placed by its row's slots) ranked, scattered and sorted in
                                      shared memory, with the digit passes taken when one bucket holds more than
                                      1024 keys; 1 digit passes always */
    uint32_t reserved[2];
} gpma_tuning;
GPMA_API gpma_status gpma_get_tuning(gpma_tuning *out);
GPMA_API gpma_status gpma_set_tuning(const gpma_tuning *t);

/* ---- test hooks ---------------------------------------------------------------
 * No reference counterpart. For tests of error paths that a correct run never
 * takes. Every device-side wait of the library (grid barriers, the sort's
 * look-back) gives up after a time limit and the call returns
 * GPMA_ERR_TIMEOUT; a stall hook makes the first grid barrier of the next
 * update (or BFS) launch wait for one arrival that never comes, with the
 * limit wait_limit_us, so that path runs without hanging the GPU. The
 * structure is unchanged by a stalled update (the barrier comes before any
 * write to the array) and the next call clears the launch state the stalled
 * one left. noalloc_chunk_cap shrinks the long-row chunk list of
 * gpma_bfs_noalloc (results do not change: rows that find the list full are
 * walked in place); noalloc_overflows reports how often the last
 * gpma_bfs_noalloc call found it full (read-only). Process-wide; set them
 * while no other host thread is inside a library call, and set all fields
 * back to zero afterwards. */
typedef struct gpma_test_hooks {
    uint32_t update_stall;      /* 1: stall the next update launches' first grid barrier */
    uint32_t bfs_stall;         /* 1: stall the next BFS launches' first grid barrier */
    uint32_t wait_limit_us;     /* limit of a stalled wait (0: the library's 2 s) */
    uint32_t noalloc_chunk_cap; /* gpma_bfs_noalloc chunk-list entries, 1..65536 (0: 65536) */
    uint32_t noalloc_overflows; /* out: full-list events of the last gpma_bfs_noalloc call */
    uint32_t reserved[3];
} gpma_test_hooks;
GPMA_API gpma_status gpma_get_test_hooks(gpma_test_hooks *out);
GPMA_API gpma_status gpma_set_test_hooks(const gpma_test_hooks *h);

/* ---- diagnostics ---------------------------------------------------------- */
GPMA_API const char *gpma_status_string(gpma_status s);
/* Detail text of the last failing call on this host thread ("" if none). */
GPMA_API const char *gpma_last_error(void);
GPMA_API const char *gpma_version(void);

/* ---- synthetic streams and the reference's text format ---------------------
 * Host-only helpers (no GPU needed). The reference's demo loads "n m" then m
 * "src dst" lines (gpma_bfs_demo.cu:6-30; dataset/prepare_dataset.sh:23-37). */

/* R-MAT with quadrant probabilities a, b, c (d = 1-a-b-c): edge_factor << scale
 * samples, then self-loops and duplicates removed and the list shuffled.
 * src/dst hold `capacity` >= edge_factor << scale entries; *m_out = edges kept. */
GPMA_API gpma_status gpma_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                          uint32_t *src, uint32_t *dst, uint64_t capacity, uint64_t *m_out);

/* Chung-Lu power-law graph with exactly m distinct non-loop edges on n nodes:
 * expected degrees ~ (i + i0)^(-1/(exponent-1)) with i0 set so the largest
 * expected degree is max_degree; node 0 is the largest out-hub; the list is
 * shuffled. */
GPMA_API gpma_status gpma_gen_chung_lu(uint32_t n, uint64_t m, double exponent, uint32_t max_degree, uint64_t seed,
                              uint32_t *src, uint32_t *dst);

/* keys[i] = (src[i] << 32) + dst[i] (gpma_bfs_demo.cu:53). */
GPMA_API gpma_status gpma_edges_to_keys(const uint32_t *src, const uint32_t *dst, uint64_t m, uint64_t *keys);

/* Text edge list in the reference's format. With src == NULL or dst == NULL
 * read only the header into *n_out and *m_out. */
GPMA_API gpma_status gpma_read_edges_text(const char *path, uint32_t *n_out, uint64_t *m_out, uint32_t *src, uint32_t *dst,
                                 uint64_t capacity);
GPMA_API gpma_status gpma_write_edges_text(const char *path, uint32_t n, const uint32_t *src, const uint32_t *dst, uint64_t m);

/* Binary edge list (no reference counterpart; the text format is slow for
 * 10^8+ edges): "GPMAEDG1", u32 n, u32 0, u64 m, m u32 sources, m u32
 * destinations, little-endian. Same header-query convention as the text
 * reader. */
GPMA_API gpma_status gpma_write_edges_bin(const char *path, uint32_t n, const uint32_t *src, const uint32_t *dst,
                                          uint64_t m);
GPMA_API gpma_status gpma_read_edges_bin(const char *path, uint32_t *n_out, uint64_t *m_out, uint32_t *src,
                                         uint32_t *dst, uint64_t capacity);

/* ---- row-range shards (host) --------------------------------------------------
 * No reference counterpart. One graph split by source-row range: shard s of
 * `shards` owns rows [gpma_shard_first_row(s), gpma_shard_first_row(s + 1)),
 * first_row(s) = floor(row_num * s / shards). An update batch reaches its
 * shards through one exchange step: gpma_partition_rows orders a host batch
 * by the shard of each key's source row, stably (input order within a shard),
 * into out_keys / out_values, with offsets[s]..offsets[s+1] the part of shard
 * s (shards + 1 entries). With rebase != 0 the source row becomes
 * shard-local (row - first_row(s)), so each shard is an ordinary graph of
 * its own rows; destinations stay global. A key whose source row is >=
 * row_num fails the call with GPMA_ERR_INVALID. */
GPMA_API uint32_t gpma_shard_first_row(uint32_t row_num, uint32_t shards, uint32_t s);
GPMA_API gpma_status gpma_partition_rows(const uint64_t *keys, const uint8_t *values, uint64_t n, uint32_t row_num,
                                         uint32_t shards, int rebase, uint64_t *out_keys, uint8_t *out_values,
                                         uint64_t *offsets);

/* ---- snapshot ----------------------------------------------------------------
 * No reference counterpart. gpma_save writes the whole structure (geometry,
 * keys, values, row_offset) with a checksum; gpma_load creates a graph on the
 * current device with exactly that layout, so updates after a resume give
 * the same layouts as updates without one. A file that is truncated,
 * corrupt, of another version or with an impossible geometry, or whose
 * layout breaks what the device code relies on (row_offset from 0,
 * non-decreasing and inside the array, each row's guard at its row_offset
 * slot, live keys ascending), is rejected with GPMA_ERR_IO before any device
 * memory is allocated. */
GPMA_API gpma_status gpma_save(gpma_graph *g, const char *path, void *stream);
GPMA_API gpma_status gpma_load(const char *path, void *stream, gpma_graph **out);

#ifdef __cplusplus
}
#endif
#endif /* GPMA_GB300_H */
