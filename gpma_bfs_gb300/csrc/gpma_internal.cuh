// gpma_internal.cuh - shared definitions of the GB300 GPMA+ library.
//
// Data layout in HBM (structure of arrays, one allocation each):
//   keys[cap]    u64  slot keys, KEY_NONE in empty slots
//   values[cap]  u8   1 = live (or any non-zero value), 0 = tombstone
//   row_offset[row_num+1] u32, row_offset[r+1] = slot of row r's guard
//   scratch keys/values [cap] for windows wider than one CTA and resizes
// plus update buffers (BatchBuffers) sized by the largest batch seen, owned
// by a graph (single-graph updates) or by a gpma_batch (many graphs at once).
#pragma once

#include "../../include/gpma_gb300.h"

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

namespace gpma {

// Reference constants (gpma.cuh:15-19, 40-43, 1003).
constexpr uint64_t KEY_NONE = 0xFFFFFFFFFFFFFFFFull;
constexpr uint64_t KEY_MAX = KEY_NONE - 1;
constexpr uint32_t SIZE_NONE = 0xFFFFFFFFu;
constexpr uint64_t COL_NONE = 0xFFFFFFFFull;
constexpr double LOWER_LEAF = 0.08, LOWER_ROOT = 0.42, UPPER_LEAF = 0.92, UPPER_ROOT = 0.84;
constexpr uint64_t SIGNIFICANT_INSERTS = 5000000ull;
constexpr uint32_t MAX_SLOTS = 1u << 31;
constexpr uint32_t MAX_LEVELS = 32;  // tree_height <= 31

// Launch shapes.
constexpr int BLOCK = 256;                 // threads of every persistent kernel
constexpr uint32_t WARP_WINDOW_MAX = 256;  // widest window handled by one warp group
constexpr uint32_t CTA_WINDOW_MAX = 2048;  // widest window handled by one CTA in shared memory
constexpr uint32_t CHUNK = 2048;           // slots per CTA step for wider windows
// Shared memory of the update kernel: three staging arrays (keys + values)
// of CTA_WINDOW_MAX slots (also holds the sort tile and the locate cache).
constexpr size_t UPDATE_SMEM = 3ull * CTA_WINDOW_MAX * 9ull + 64;

// Device error codes (DeviceStatus::err).
enum : uint32_t {
    DERR_NONE = 0,
    DERR_BARRIER_TIMEOUT = 1,
    DERR_LOOKBACK_TIMEOUT = 2,
    DERR_BOUNDS = 3,
    DERR_INVALID_KEY = 4,
};

// Bounds-checked build (-DGPMA_BOUNDS_CHECK=1): every data-dependent index
// range (a located leaf, a window, a pending-insertion range, a BFS row) is
// checked against its buffer before the access. A failing check skips the
// access and records DERR_BOUNDS | site << 8 in the launch's error word, and
// the launch stops at its next grid barrier. The product build compiles the
// checks away.
#ifndef GPMA_BOUNDS_CHECK
#define GPMA_BOUNDS_CHECK 0
#endif
enum BoundsSite : uint32_t {
    BS_LEAF = 1,      // locate: the leaf's seg slots
    BS_WINDOW = 2,    // level loop: a warp/CTA window's slots
    BS_PENDING = 3,   // level loop: a window's pending insertions
    BS_CHUNK = 4,     // level loop: a grid-wide window's chunk
    BS_REBUILD = 5,   // bulk rebuild / compacted layout: a slot
    BS_ROW = 6,       // BFS / multi-source BFS / analytics: a row's slot range
};

// Bounded waits give up after this long (ns of %globaltimer).
constexpr uint64_t WAIT_LIMIT_NS = 2000000000ull;

// Test hooks (process-wide, gpma_set_test_hooks): make one bounded wait run
// out on purpose so its error path runs on a GPU without hanging it, and
// shrink the no-allocation BFS's chunk list so its full-list branch runs.
struct TestHooks {
    uint32_t update_stall = 0;         // 1: the update kernel's first grid barrier waits for one arrival too many
    uint32_t bfs_stall = 0;            // 1: the BFS kernel's first grid barrier does the same
    uint64_t wait_limit_ns = WAIT_LIMIT_NS;  // limit of those two waits
    uint32_t noalloc_chunk_cap = 0;    // gpma_bfs_noalloc chunk-list entries (0: all it has)
    uint32_t noalloc_overflows = 0;    // full-list events of the last gpma_bfs_noalloc call (written by it)
};
extern TestHooks g_test_hooks;

struct GridBarrier {
    unsigned int count;  // tickets taken (zero at the start of every launch)
    unsigned int gen;    // generation of grid_barrier_gen
};

// Written by the update kernel, read back once per update.
struct DeviceStatus {
    uint32_t err;
    uint32_t invalid_keys;  // keys whose column is the reserved 0xFFFFFFFF
    uint32_t significant;   // single graph: >= SIGNIFICANT_INSERTS insertions (host rebuild)
    uint32_t inserts;       // insertions after delete/modify (all graphs)
    uint32_t levels;        // level iterations executed
    uint32_t sort_fallback; // a bucket of the bucket sort held more than one item: digit passes instead
    uint32_t pad[2];
    unsigned long long accepted_windows;
    unsigned long long accepted_slots;
    GridBarrier bar;
    // %globaltimer stamps taken by CTA 0 at phase boundaries: start, sorted,
    // located, grouped, level loop done
    unsigned long long stamp[5];
};

// One graph as the update kernel sees it (device table, one entry per graph).
struct GraphDesc {
    uint64_t *keys;
    uint8_t *vals;
    uint32_t *row_offset;
    uint64_t *skeys;  // scratch of `size` slots
    uint8_t *svals;
    uint64_t *heads;  // heads[s] == keys[s * seg]: the keys the locate descent compares
    uint32_t row_num, size, seg, log2seg, height;
    // bucket of a key for this launch's bucket sort: its row's slots
    // interpolated by its column (qbits: bits of the largest column), shifted
    // right by qshift, capped at qnbm1
    uint32_t qbits, qshift, qnbm1;
    uint32_t lower[MAX_LEVELS];
    uint32_t upper[MAX_LEVELS];
};

// Per-graph result of one update launch.
struct GraphStatus {
    uint32_t inserts;    // insertions of this graph after delete/modify
    uint32_t remaining;  // insertions the root rebalance still has to place
    uint32_t ins_base;   // first insertion of this graph in the compacted order
    uint32_t pad;
};

struct Geometry {
    uint32_t size = 0, seg = 0, height = 0;
    std::vector<uint32_t> lower, upper;
};

// Recomputes the density thresholds exactly as recalculate_density
// (gpma.cuh:147-168): same double expressions and evaluation order, then the
// integer clamps against the previous level.
void recalculate_density(Geometry &geo);
uint32_t fls32(uint32_t x);

// Buffers of one update launch (batch keys of all graphs, insertions, window
// lists, sort state, per-graph tables).
struct BatchBuffers {
    uint64_t cap = 0;  // keys
    uint64_t *bkeys[2] = {nullptr, nullptr};
    uint8_t *bvals[2] = {nullptr, nullptr};
    uint32_t *leaf = nullptr;
    uint64_t *ikeys[2] = {nullptr, nullptr};  // pending insertions, compacted per level (ping-pong)
    uint8_t *ivals[2] = {nullptr, nullptr};
    uint64_t *rkeys = nullptr;  // insertions left for the root rebalance
    uint8_t *rvals = nullptr;
    uint32_t *ileaf = nullptr;
    uint32_t *igraph = nullptr;
    uint32_t *wnode[2] = {nullptr, nullptr};
    uint32_t *wgraph[2] = {nullptr, nullptr};
    uint32_t *wa[2] = {nullptr, nullptr};
    uint32_t *wb[2] = {nullptr, nullptr};
    uint32_t *wflag = nullptr;  // 2 * cap: one array per level parity
    uint32_t *wlive = nullptr;
    uint64_t *top = nullptr;    // one graph: its top-of-tree heads, gathered per launch for the locate cache
    // sort state
    uint32_t *sort_tiles = nullptr;    // 8 tile counters
    uint32_t *sort_status = nullptr;   // look-back words, 8 x tiles x 256
    uint64_t sort_status_cap = 0;
    uint32_t *sort_hist = nullptr;     // [graph][8][256] digit counts
    uint32_t hist_cap = 0;             // graphs
    uint32_t *qcnt = nullptr;          // bucket sort: keys per bucket (zeroed per update)
    uint64_t *qinfo = nullptr;         // bucket sort: offset within the scan chunk | count << 32
    uint64_t q_cap = 0;                // buckets
    uint64_t *qrec = nullptr;          // bucket sort: 16-byte records (two words per key)
    uint64_t qrec_cap = 0;             // keys
    uint32_t *qbound = nullptr;        // bucket sort: first position of every item
    uint64_t qbound_cap = 0;           // items
    // per-graph tables, one upload per launch from pinned memory:
    // [GraphDesc x gcap][batch offsets x (gcap + 1)][sort tile offsets x (gcap + 1)]
    // [bucket offsets x (gcap + 1)][bucket-sort item offsets x (gcap + 1)]
    uint32_t gcap = 0;
    unsigned char *d_tab = nullptr;
    unsigned char *h_tab = nullptr;    // pinned
    GraphDesc *gd = nullptr;           // views into d_tab
    uint32_t *boff = nullptr;
    uint32_t *toff = nullptr;
    uint32_t *qoff = nullptr;
    uint32_t *qtoff = nullptr;
    // host copy of what d_tab holds after update_graphs' last upload (an
    // identical table is not uploaded again); anything else that writes
    // d_tab clears tab_shadow_valid
    std::vector<unsigned char> tab_shadow;
    bool tab_shadow_valid = false;
    // status, double-buffered: a slot is [DeviceStatus][GraphStatus x gcap]
    // (GraphStatus from STAT_GS_OFFSET); each launch zeroes the other slot and
    // the sort state it used, so steady-state launches need no memsets
    unsigned char *d_stat = nullptr;   // 2 slots
    unsigned char *h_stat = nullptr;   // 1 slot, pinned
    size_t stat_slot = 0;              // bytes per slot
    int parity = 0;
    bool dirty = true;                 // sort state / status slots need a host-side clear
    // grid-path chunk counts (sum of window widths / CHUNK)
    uint32_t *chunk_cnt = nullptr;
    uint64_t chunk_cap = 0;
    // persistent-kernel scratch
    uint32_t *cta_cnt = nullptr;       // 8 * grid: four count arrays, two window-range arrays
};
constexpr size_t STAT_GS_OFFSET = 128;
static_assert(sizeof(DeviceStatus) <= STAT_GS_OFFSET, "status slot layout");

}  // namespace gpma

// Opaque handle of the C ABI.
struct gpma_graph {
    int device = 0;
    int sms = 0;
    uint32_t row_num = 0;
    gpma::Geometry geo;
    uint32_t cap = 0;                 // allocated slots of keys/values
    uint64_t *keys = nullptr;
    uint8_t *values = nullptr;
    uint32_t *row_offset = nullptr;
    uint32_t scratch_cap = 0;
    uint64_t *skeys = nullptr;        // scratch for wide windows and resizes
    uint8_t *svals = nullptr;
    uint32_t *chunk_cnt = nullptr;    // root rebuild: compaction statuses, then merge splits
    uint64_t chunk_words = 0;         // its u32 words
    uint64_t *heads = nullptr;        // first key of every segment (size / seg entries), kept by every writer
    uint32_t heads_cap = 0;
    gpma::BatchBuffers buf;           // single-graph update buffers
    // BFS state
    uint32_t bfs_cap = 0;
    uint32_t *bfs_visited = nullptr;   // row_num/32 + 2 words
    uint32_t *bfs_front[2] = {nullptr, nullptr};  // frontier bitmaps, row_num/32 + 2 words
    uint2 *bfs_chunks = nullptr;       // big-row chunk list
    uint32_t bfs_chunk_cap = 0;        // its entries: size / 16 + 1024, more than one level can queue
    uint32_t *bfs_levels = nullptr;
    uint32_t *bfs_ctl = nullptr;       // counters + status
    uint32_t *h_bfs_ctl = nullptr;     // pinned
    int bfs_grid = 0;                  // resident BFS-kernel CTAs per SM (0: not yet known)
    gpma_batch *own_batch = nullptr;   // multi-source BFS context of this graph
    uint32_t *an_buf = nullptr;        // analytics: 4 x row_num words + control words, kept between calls
    uint32_t an_cap = 0;               // row_num it was sized for
    gpma_stats stats{};
    // profiling: events on the caller's stream around each phase
    bool profiling = false;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    gpma_profile prof{};
};

// Many graphs updated (and searched) per launch.
struct gpma_batch {
    int device = 0;
    int sms = 0;
    gpma::BatchBuffers buf;
    bool profiling = false;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    gpma_profile prof{};
    // multi-source BFS state over all graphs of a call
    uint64_t ms_cap = 0;               // nodes
    uint64_t *ms_mask[3] = {nullptr, nullptr, nullptr};
    // per-call graph table (node and slot offsets, sources, descriptors), one
    // upload from its pinned mirror
    unsigned char *ms_tab = nullptr;
    unsigned char *h_ms_tab = nullptr;
    uint32_t *ms_ctl = nullptr;
    uint32_t *h_ms_ctl = nullptr;      // pinned
    uint64_t *ms_reached = nullptr;    // graphs * 64 reached counts + the traversed-edge total
    unsigned long long *h_ms_reached = nullptr;  // pinned
    uint2 *ms_chunks = nullptr;
    uint64_t ms_chunk_cap = 0;         // entries (uint4): total slots / 32 + 1024
    uint32_t ms_gcap = 0;
    uint64_t last_traversed = 0;       // edges scanned by the last multi-source BFS, all lanes
    uint64_t *gather_tab = nullptr;    // packed-update staging table (2 * graphs + 1)
    uint64_t *h_gather_tab = nullptr;  // its pinned mirror
    uint32_t gather_cap = 0;
};

namespace gpma {

// ---- host error handling -------------------------------------------------
void set_error(const char *fmt, ...);
// Status and message for a kernel's non-zero error word (`where` names the kernel).
gpma_status device_error(const char *where, uint32_t code);
gpma_status cuda_fail(cudaError_t e, const char *what);
#define GPMA_CUDA(expr)                                                                                                \
    do {                                                                                                               \
        cudaError_t _e = (expr);                                                                                       \
        if (_e != cudaSuccess)                                                                                         \
            return ::gpma::cuda_fail(_e, #expr);                                                                       \
    } while (0)
// A named NVTX range over one C-ABI call, so timeline tools and `ncu --nvtx`
// filters see each update, BFS and round; without an attached tool a range
// costs one indirect call.
struct CallRange {
    explicit CallRange(const char *name) { nvtxRangePushA(name); }
    ~CallRange() { nvtxRangePop(); }
    CallRange(const CallRange &) = delete;
    CallRange &operator=(const CallRange &) = delete;
};

#define GPMA_TRY(expr)                                                                                                 \
    do {                                                                                                               \
        gpma_status _s = (expr);                                                                                       \
        if (_s != GPMA_OK)                                                                                             \
            return _s;                                                                                                 \
    } while (0)

// true if p is device-accessible memory of the current device
bool is_device_pointer(const void *p);
// copies between host or device pointers on a stream (kind inferred)
gpma_status copy_any(void *dst, const void *src, size_t bytes, cudaStream_t s);
template <typename T>
gpma_status dev_alloc(T **p, size_t count) {
    *p = nullptr;
    if (count == 0)
        count = 1;
    cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        set_error("cudaMalloc of %zu bytes failed: %s", count * sizeof(T), cudaGetErrorString(e));
        return GPMA_ERR_NOMEM;
    }
    return GPMA_OK;
}
template <typename T>
void dev_free(T *&p) {
    if (p)
        cudaFree((void *)p);
    p = nullptr;
}

// ---- profiling helpers -------------------------------------------------------
inline void prof_mark(bool on, cudaEvent_t *ev, int i, cudaStream_t s) {
    if (on)
        cudaEventRecord(ev[i], s);
}
// elapsed ms between two recorded events (both complete: call after a sync)
inline double prof_elapsed(bool on, cudaEvent_t *ev, int a, int b) {
    float ms = 0.f;
    if (on && cudaEventElapsedTime(&ms, ev[a], ev[b]) != cudaSuccess) {
        cudaGetLastError();
        ms = 0.f;
    }
    return ms;
}
inline void prof_mark(gpma_graph *g, int i, cudaStream_t s) { prof_mark(g->profiling, g->ev, i, s); }
inline double prof_elapsed(gpma_graph *g, int a, int b) { return prof_elapsed(g->profiling, g->ev, a, b); }

// One kernel launch whose argument is a single by-value struct, recorded so
// that it can be launched directly or added to a CUDA graph as a kernel node.
struct KernelLaunch {
    static constexpr size_t ARG_BYTES = 512;
    const void *func = nullptr;
    dim3 grid{1, 1, 1};
    dim3 block{BLOCK, 1, 1};
    size_t smem = 0;
    size_t arg_bytes = 0;
    alignas(16) unsigned char args[ARG_BYTES] = {};
    void *params[1] = {nullptr};  // points at args when handed to CUDA

    void set(const void *f, int grid_x, size_t smem_bytes, const void *a, size_t bytes) {
        func = f;
        grid = dim3((unsigned)grid_x, 1, 1);
        smem = smem_bytes;
        arg_bytes = bytes;
        memcpy(args, a, bytes);
    }
    cudaError_t launch(cudaStream_t s) {
        params[0] = args;
        return cudaLaunchKernel(func, grid, block, params, smem, s);
    }
    cudaError_t launch_cooperative(cudaStream_t s) {
        params[0] = args;
        return cudaLaunchCooperativeKernel(func, grid, block, params, smem, s);
    }
    cudaKernelNodeParams node() {
        params[0] = args;
        cudaKernelNodeParams p{};
        p.func = const_cast<void *>(func);
        p.gridDim = grid;
        p.blockDim = block;
        p.sharedMemBytes = (unsigned)smem;
        p.kernelParams = params;
        p.extra = nullptr;
        return p;
    }
    bool same(const KernelLaunch &o) const {
        return func == o.func && grid.x == o.grid.x && smem == o.smem && arg_bytes == o.arg_bytes &&
               memcmp(args, o.args, arg_bytes) == 0;
    }
};

// ---- host entry points implemented per translation unit -------------------
gpma_status ensure_buffers(BatchBuffers &b, uint64_t n, uint32_t graphs);
void free_buffers(BatchBuffers &b);
gpma_status ensure_scratch(gpma_graph *g, uint32_t slots);
// Recomputes heads[s] = keys[s * seg] over the whole array (after the array
// was written outside the level loop: creation, root rebuild, load).
gpma_status refresh_heads(gpma_graph *g, cudaStream_t s);
// Segments whose heads entry differs from the array (0 when consistent).
gpma_status count_bad_heads(gpma_graph *g, cudaStream_t s, uint64_t *bad);
// One launch updating graphs[0..k) with the batches already staged in
// buf.bkeys[0]/bvals[0] at offsets off[0..k]. Graphs must be ordered by
// segment length. check_keys=false only for the internal guard insertion.
// in_k / in_v: the batch in device memory elsewhere (read in place) instead.
gpma_status update_graphs(gpma_graph *const *graphs, const uint64_t *off, uint32_t k, BatchBuffers &buf, int sms,
                          cudaStream_t s, bool check_keys, bool profiling, cudaEvent_t *ev, gpma_profile *prof,
                          const uint64_t *in_k = nullptr, const uint8_t *in_v = nullptr);
gpma_status update_device(gpma_graph *g, uint64_t n, cudaStream_t s, bool check_keys = true,
                          const uint64_t *in_k = nullptr, const uint8_t *in_v = nullptr);
// The three host parts of update_graphs, for callers that enqueue the launch
// themselves (a CUDA graph step). update_plan sizes the buffers, fills the
// pinned tables (*tab_bytes of buf.h_tab to upload to buf.d_tab) and records
// the cooperative kernel launch; its status lands in slot buf.parity of
// buf.d_stat (update_status_bytes(k) bytes to read back). update_clear zeroes
// the sort state and status slots after a failed or first launch. update_finish
// reads the copied status, updates the graphs' stats, finishes root rebuilds
// on the host and flips the status slot. update_needs_host: the status asks
// for host work or reports an error (the array changed after the kernel).
// A non-null `abort` (a device word) makes the launch return at once while
// the word is non-zero (steps recorded after one that needs host work).
// in_k / in_v (device, optional): the batch is read from there instead of
// buf.bkeys[0] / buf.bvals[0] (which the sort then only writes).
gpma_status update_plan(gpma_graph *const *graphs, const uint64_t *off, uint32_t k, BatchBuffers &buf, int sms,
                        bool check_keys, size_t *tab_bytes, KernelLaunch *L, const uint32_t *abort = nullptr,
                        const uint64_t *in_k = nullptr, const uint8_t *in_v = nullptr);
gpma_status update_clear(BatchBuffers &buf, cudaStream_t s);
size_t update_status_bytes(uint32_t k);
gpma_status update_finish(gpma_graph *const *graphs, uint32_t k, BatchBuffers &buf, const unsigned char *stat,
                          cudaStream_t s, gpma_profile *prof, double kernel_ms);
bool update_needs_host(const unsigned char *stat, uint32_t k);
gpma_status bfs_run(gpma_graph *g, uint32_t src, cudaStream_t s, uint64_t *reached);
// The host parts of bfs_run, for callers that enqueue it themselves: the
// buffers to zero, the one-thread init kernel (its five arguments) and the
// cooperative BFS kernel; ctl_bytes of g->bfs_ctl are read back into
// g->h_bfs_ctl and checked by bfs_finish.
struct BfsPlan {
    static constexpr int CLEARS = 5;
    void *clear_ptr[CLEARS];
    size_t clear_bytes[CLEARS];
    const void *init_func;
    uint32_t *init_levels, *init_visited, *init_front0, *init_ctl;
    uint32_t init_src;
    void *init_params[5];  // point at the init_* fields when handed to CUDA
    KernelLaunch main;
    size_t ctl_bytes;
    void bind_init() {
        init_params[0] = &init_levels;
        init_params[1] = &init_visited;
        init_params[2] = &init_front0;
        init_params[3] = &init_ctl;
        init_params[4] = &init_src;
    }
};
gpma_status bfs_plan(gpma_graph *g, uint32_t src, BfsPlan *P);
gpma_status bfs_finish(gpma_graph *g, uint64_t *reached);
gpma_status bfs_noalloc_run(gpma_graph *g, uint32_t src, uint32_t *levels, uint64_t *reached, cudaStream_t s);
gpma_status batch_bfs_run(gpma_batch *b, gpma_graph *const *graphs, const uint32_t *const *srcs, const uint32_t *nsrc,
                          uint32_t k, uint32_t *const *levels, uint64_t *reached, cudaStream_t s);
// The host parts of batch_bfs_run: batch_bfs_plan sizes the buffers, fills
// the pinned table (tab_bytes of b->h_ms_tab to upload to b->ms_tab), lists
// the buffers to zero and records the cooperative kernel launch (levels go
// to stage[i] when stage is non-null); batch_bfs_enqueue_readback copies the
// control words and counts back; batch_bfs_finish checks and reports them.
struct BatchBfsPlan {
    static constexpr int CLEARS = 5;
    size_t tab_bytes;
    void *clear_ptr[CLEARS];
    size_t clear_bytes[CLEARS];
    KernelLaunch main;
    size_t ctl_bytes;
    size_t reached_bytes;
};
// Host part of a packed update of graphs[0..k) (batch i at [offsets[i],
// offsets[i+1]) of keys/values, host or device): graphs with batches of
// SIGNIFICANT_INSERTS or more are listed in `bulk` for the single-graph path;
// the others, ordered by segment length (gs, batch offsets off), get the
// gather launch that stages their batches in that order. packed_stage uploads
// a host batch into the second sort buffer and (with_table) the gather table.
struct PackedPlan {
    std::vector<uint32_t> bulk;
    uint32_t m = 0;
    std::vector<gpma_graph *> gs;
    std::vector<uint64_t> off;
    bool upload = false;
    uint64_t all_keys = 0;
    size_t gtab_bytes = 0;
    KernelLaunch gather;
};
gpma_status packed_plan(gpma_batch *b, gpma_graph *const *graphs, const uint64_t *keys, const uint8_t *values,
                        const uint64_t *offsets, uint32_t k, PackedPlan *P, const uint32_t *abort = nullptr);
gpma_status packed_stage(gpma_batch *b, const PackedPlan &P, const uint64_t *keys, const uint8_t *values,
                         const uint64_t *offsets, cudaStream_t s, bool with_table = true);
gpma_status batch_bfs_plan(gpma_batch *b, gpma_graph *const *graphs, const uint32_t *const *srcs,
                           const uint32_t *nsrc, uint32_t k, uint32_t *const *stage, BatchBfsPlan *P,
                           const uint32_t *abort = nullptr);
gpma_status batch_bfs_enqueue_readback(gpma_batch *b, const BatchBfsPlan &P, cudaStream_t s);
gpma_status batch_bfs_finish(gpma_batch *b, const uint32_t *nsrc, uint32_t k, uint64_t *reached);
void free_bfs(gpma_graph *g);
void free_batch_bfs(gpma_batch *b);
int update_grid_size(int sms, uint64_t n);

// Launch shapes and switch points: they change speed, never results
// (process-wide, set through gpma_set_tuning; defaults from measurement).
struct Tuning {
    uint32_t bfs_dense_div = 0;  // rows only: with 4 slots per lane the walk beat the sweep on every level measured
    uint32_t bfs_blocks_per_sm = 8;
    uint32_t ms_dense_div = 8;
    uint32_t ms_blocks_per_sm = 8;
    uint32_t update_blocks_per_sm = 0;  // 0: chosen per launch (3-CTA build from 1M keys)
    uint32_t update_sort = 0;           // 0: bucket sort (digit passes for crowded buckets), 1: digit passes
};
extern Tuning g_tuning;
// CTAs per SM for a kernel that fits `fit` per SM, given a tuned request (0 = fit).
inline int blocks_per_sm(int fit, uint32_t want) {
    if (fit < 1)
        return 0;
    return want == 0 ? fit : std::min<int>(fit, (int)want);
}
constexpr int MAX_BLOCKS_PER_SM = 32;

}  // namespace gpma

// ---- device helpers --------------------------------------------------------
#ifdef __CUDACC__
namespace gpma {

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t *p) { return *(const volatile uint32_t *)p; }

// True when `ok`; in the bounds-checked build a false `ok` records the site
// in *err (first error wins) and the caller skips the access.
__device__ __forceinline__ bool in_bounds(uint32_t *err, bool ok, uint32_t site) {
    if constexpr (GPMA_BOUNDS_CHECK != 0) {
        if (!ok) {
            atomicCAS(err, 0u, DERR_BOUNDS | (site << 8));
            return false;
        }
    }
    return true;
}

// Ticket barrier across the CTAs of a cooperative launch. Each CTA takes a
// ticket from one counter (it must start each launch at zero) and waits
// until the counter reaches the end of its ticket's round of gridDim.x;
// there is no separate release write, so a barrier costs one atomic per CTA
// and polling (measured 1.35 us at 304 CTAs against 2.8 us for a
// count-then-generation barrier). Every wait is bounded: after WAIT_LIMIT_NS
// the CTA records DERR_BARRIER_TIMEOUT and returns false; CTAs that see an
// error stop waiting.
// `extra` (test hooks only, 0 otherwise) adds arrivals that never come, so the
// wait runs out after `limit_ns`.
__device__ __forceinline__ bool grid_barrier(GridBarrier *bar, uint32_t *err, uint32_t extra = 0,
                                             uint64_t limit_ns = WAIT_LIMIT_NS) {
    __syncthreads();
    __shared__ uint32_t s_ok;
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned int ticket = atomicAdd(&bar->count, 1u);
        const unsigned int target = (ticket / gridDim.x + 1) * gridDim.x + extra;
        uint64_t t0 = 0;
        unsigned ns = 16;
        for (;;) {
            unsigned int c;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(c) : "l"(&bar->count) : "memory");
            if ((int)(c - target) >= 0)
                break;
            if (ld_volatile(err) != 0)
                break;
            if (t0 == 0)
                t0 = globaltimer_ns();
            __nanosleep(ns);
            if (ns < 128)
                ns <<= 1;
            if (globaltimer_ns() - t0 > limit_ns) {
                atomicCAS(err, 0u, DERR_BARRIER_TIMEOUT);
                break;
            }
        }
        // no trailing fence: the arrivals are releases (fence, then the
        // atomic) and the load that saw the last one is an acquire; the CTA
        // barrier below passes that order on to the other threads
        s_ok = ld_volatile(err) == 0;
    }
    __syncthreads();
    return s_ok != 0;
}

// Count-then-generation barrier over the same two words (the count returns
// to zero, the last arriver advances the generation the others poll). Slower
// than the ticket barrier in isolation, but measured faster inside the
// multi-source BFS, whose 900-odd CTAs poll while others still work.
__device__ __forceinline__ bool grid_barrier_gen(GridBarrier *bar, uint32_t *err) {
    __syncthreads();
    __shared__ uint32_t s_okg;
    if (threadIdx.x == 0) {
        volatile unsigned int *vgen = &bar->gen;
        unsigned int g0 = *vgen;
        __threadfence();
        unsigned int prev = atomicAdd(&bar->count, 1u);
        if (prev == gridDim.x - 1) {
            atomicExch(&bar->count, 0u);
            __threadfence();
            atomicAdd(&bar->gen, 1u);
        } else {
            uint64_t t0 = globaltimer_ns();
            unsigned ns = 32;
            while (*vgen == g0) {
                if (ld_volatile(err) != 0)
                    break;
                __nanosleep(ns);
                if (ns < 512)
                    ns <<= 1;
                if (globaltimer_ns() - t0 > WAIT_LIMIT_NS) {
                    atomicCAS(err, 0u, DERR_BARRIER_TIMEOUT);
                    break;
                }
            }
        }
        __threadfence();
        s_okg = ld_volatile(err) == 0;
    }
    __syncthreads();
    return s_okg != 0;
}

// One volatile read per CTA, broadcast through shared memory: a word that
// every warp of a persistent grid needs after a barrier costs one L2 request
// per CTA instead of one per warp. Every thread of the CTA must call it.
__device__ __forceinline__ uint32_t cta_broadcast_read(const uint32_t *p) {
    __shared__ uint32_t s_v;
    __syncthreads();  // readers of the previous value are done
    if (threadIdx.x == 0)
        s_v = ld_volatile(p);
    __syncthreads();
    return s_v;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Inclusive warp scan over `width` lanes (power of two <= 32).
__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t x, int width = 32) {
    int lane = threadIdx.x & (width - 1);
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        if (d >= width)
            break;
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, d, width);
        if (lane >= d)
            x += y;
    }
    return x;
}

// Exclusive scan over the CTA (blockDim.x == BLOCK); returns the exclusive
// prefix and writes the CTA total. `tmp` holds BLOCK/32 + 1 words.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t x, uint32_t *total, uint32_t *tmp) {
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = warp_incl_scan(x);
    if (lane == 31)
        tmp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t v = lane < BLOCK / 32 ? tmp[lane] : 0;
        uint32_t vi = warp_incl_scan(v);
        if (lane < BLOCK / 32)
            tmp[lane] = vi - v;
        if (lane == BLOCK / 32 - 1)
            tmp[BLOCK / 32] = vi;
    }
    __syncthreads();
    uint32_t res = tmp[warp] + inc - x;
    *total = tmp[BLOCK / 32];
    __syncthreads();
    return res;
}

__device__ __forceinline__ uint32_t block_sum(uint32_t x, uint32_t *tmp) {
    uint32_t total;
    block_excl_scan(x, &total, tmp);
    return total;
}

// Number of elements of sorted a[0..n) that are < key (lower) or <= key (upper).
template <typename P>
__device__ __forceinline__ uint32_t lower_bound_u64(P a, uint32_t n, uint64_t key) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (a[mid] < key)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}
template <typename P>
__device__ __forceinline__ uint32_t upper_bound_u64(P a, uint32_t n, uint64_t key) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (a[mid] <= key)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// Index of the segment of a[0..n] (increasing offsets, a[0] = 0) holding x:
// the last i with a[i] <= x.
__device__ __forceinline__ uint32_t segment_of(const uint32_t *a, uint32_t n, uint32_t x) {
    uint32_t lo = 0, hi = n;  // answer in [0, n)
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (a[mid] <= x)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// First merged index of segment s when M elements are spread over F segments
// (F a power of two, log2F its log): ceil(s*M/F). Element i of the merge
// lands in segment floor(F*i/M) at lane (F*i mod M)/F (gpma.cuh:636-654);
// inverting that, segment s holds elements [first(s), first(s+1)) packed from
// lane 0.
__device__ __forceinline__ uint64_t seg_first(uint64_t s, uint64_t M, uint32_t log2F) {
    return (s * M + ((1ull << log2F) - 1)) >> log2F;
}

__device__ __forceinline__ bool is_guard(uint64_t k) { return (k & COL_NONE) == COL_NONE && k != KEY_NONE; }

}  // namespace gpma
#endif
