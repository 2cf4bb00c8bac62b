// bfs.cu - GPU-only BFS over the gapped PMA.
//
// Replaces gpma_bfs (gpma_bfs.cuh:511-533) and its gather/contract kernels
// (:150-395), whose level loop crossed host<->device every level
// (:479,495). Semantics are the reference's: the edges of node v are the
// slots [row_offset[v], row_offset[v+1]) whose low 32 bits are not
// 0xFFFFFFFF (row guards, empty slots) and whose value is non-zero
// (tombstones, bulk-rebuild gaps); levels[src] = 1 and a node first reached
// from level L gets L+1.
//
// Single source: one persistent cooperative kernel runs every level,
// separated by bounded grid barriers. Frontiers are bitmaps (no queue, no
// queue atomics). Per level, phase 1 gives each warp one frontier word at a
// time: the short rows of its up to 32 nodes are walked as one concatenated
// slot range (warp-level load balancing, two slots per lane per step, all
// loads issued before any claim) and long rows are queued as 64-slot chunks;
// phase 2 spreads those chunks over every warp. A target is claimed with
// atomicOr on the visited bitmap (a plain load filters visited targets first)
// and enters the next frontier bitmap.
//
// Direction switch: a large frontier (>= n/64 nodes) is measured by a first
// pass that queues its long rows' chunks and sums its rows' slots. If those
// rows span >= size / dense_div slots the level instead sweeps the whole slot
// array once, coalesced (a PMA of out-edges has no in-edges to pull from; the
// sweep reads each key's source row from its high word and tests it against
// the frontier bitmap). Both give the same levels.
//
#include "gpma_internal.cuh"

#include <algorithm>
#include <mutex>

namespace gpma {
namespace {

// bfs_ctl layout (u32 words)
enum : uint32_t {
    CTL_CNT = 0,      // 3 rotating counters: nodes first reached per level
    CTL_CHUNKS = 3,   // 3 rotating counters: big-row chunks queued per level
    CTL_ERR = 6,
    CTL_LEVELS = 7,
    CTL_REACHED = 8,
    CTL_OVERFLOW = 9, // times a warp found the chunk list full and walked its long rows in place
    CTL_BAR = 10,     // GridBarrier (2 words)
    CTL_SLOTS = 12,   // 3 rotating counters: slots of the current frontier's rows (measured levels)
    CTL_WORDS = 16,
    // profiling record after the control words: u64 start stamp of each level
    // (and of the final check), then u32 per level: frontier size | dense << 31
    CTL_PROFILE_LEVELS = 64,
    CTL_PROFILE_WORDS = 3 * CTL_PROFILE_LEVELS,
};

// Rows longer than BIG_ROW slots are cut into CHUNK_SLOTS-slot chunks that
// every warp of the grid shares in a second phase of the level; shorter rows
// of one frontier word are walked together by one warp. (With node ids
// ordered by degree, one word can otherwise hold 32 heavy rows.)
// A warp walks short rows LANE_SLOTS slots per lane per step and chunks
// CHUNK_LANE_SLOTS per lane (build options), all loads of a step issued
// before any claim; a chunk is one step of a warp.
#ifndef GPMA_BFS_LANE_SLOTS
#define GPMA_BFS_LANE_SLOTS 4
#endif
#ifndef GPMA_BFS_CHUNK_LANE_SLOTS
#define GPMA_BFS_CHUNK_LANE_SLOTS 8
#endif
constexpr uint32_t LANE_SLOTS = GPMA_BFS_LANE_SLOTS;
constexpr uint32_t CHUNK_LANE_SLOTS = GPMA_BFS_CHUNK_LANE_SLOTS;
static_assert(LANE_SLOTS >= 1 && LANE_SLOTS <= 8 && CHUNK_LANE_SLOTS >= LANE_SLOTS && CHUNK_LANE_SLOTS <= 8,
              "BFS lane slots out of range");
constexpr uint32_t STEP_SLOTS = 32 * LANE_SLOTS;
constexpr uint32_t BIG_ROW = STEP_SLOTS / 2;
constexpr uint32_t CHUNK_SLOTS = 32 * CHUNK_LANE_SLOTS;
// Chunk list entries for an array of `size` slots: rows over BIG_ROW slots
// yield at most len/64 + 1 chunks each and there are at most size/33 of them,
// so one level queues fewer than size/64 + size/33 < size/16 chunks; the list
// never overflows.
inline uint32_t bfs_chunk_need(uint32_t size) { return size / 16 + 1024; }

struct BfsArgs {
    const uint64_t *keys;
    const uint8_t *vals;
    const uint32_t *ro;
    uint32_t n;
    uint32_t size;
    uint32_t *levels;
    uint32_t *visited;
    uint32_t *front0;  // frontier bitmaps (ping-pong), n/32+2 words each
    uint32_t *front1;
    uint2 *chunks;     // [slot begin, slot end) of big-row chunks
    uint32_t chunk_cap;
    uint32_t *ctl;
    uint32_t dense_div;  // a level whose frontier rows span >= size / dense_div slots sweeps every slot (0: never)
    unsigned long long *stamps;  // per-level profile (CTL_PROFILE_LEVELS stamps + info words) or null
    // test hooks: extra arrivals the first grid barrier waits for, and its limit
    uint32_t stall;
    uint64_t stall_limit_ns;
};

// N edge slots of one lane (SIZE_NONE: absent): every key, value and
// visited word is loaded before any claim, so each lane keeps several
// requests in flight. A target that was unvisited when its word was read is
// claimed without waiting for a result: every lane that saw it unvisited sets
// its visited bit, its level (next_level, the same from every claimer) and
// its next-frontier bit, all idempotent. Returns the number of such claims
// (at least the nodes this lane reached first, more when lanes raced).
template <uint32_t N>
__device__ __forceinline__ uint32_t visit_slots(const BfsArgs &A, const uint32_t (&sl)[N], uint32_t next_level,
                                                uint32_t *front_next) {
    uint32_t w[N], seen[N];
#pragma unroll
    for (uint32_t j = 0; j < N; ++j) {
        uint64_t k = KEY_NONE;
        uint8_t v = 0;
        if (sl[j] != SIZE_NONE) {
            k = A.keys[sl[j]];
            v = A.vals[sl[j]];
        }
        w[j] = (uint32_t)k;
        seen[j] = (w[j] != 0xFFFFFFFFu && v != 0 && w[j] < A.n) ? 0u : 0xFFFFFFFFu;
    }
#pragma unroll
    for (uint32_t j = 0; j < N; ++j)
        if (!seen[j])
            seen[j] = A.visited[w[j] >> 5];
    uint32_t fresh = 0;
#pragma unroll
    for (uint32_t j = 0; j < N; ++j) {
        const uint32_t bit = 1u << (w[j] & 31);
        if (!(seen[j] & bit)) {
            atomicOr(&A.visited[w[j] >> 5], bit);
            A.levels[w[j]] = next_level;
            atomicOr(&front_next[w[j] >> 5], bit);
            ++fresh;
        }
    }
    return fresh;
}

// Dense levels: 8 consecutive slots of the linear sweep. The key's high word
// is its source row, so the frontier test needs no row_offset lookup; guards,
// empty slots, tombstones and bulk-rebuild gaps fail the same tests as in the
// row walk (low word 0xFFFFFFFF or value 0; KEY_NONE's source is out of
// range). The frontier words of all 8, then their visited words, are loaded
// before any claim, so each thread keeps 8 requests in flight per stage.
__device__ __forceinline__ uint32_t dense_visit8(const BfsArgs &A, const uint64_t (&k)[8], uint2 v,
                                                 const uint32_t *front_cur, uint32_t next_level,
                                                 uint32_t *front_next) {
    uint32_t dst[8], word[8];
    bool c[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const uint32_t src = (uint32_t)(k[j] >> 32);
        const uint32_t val = ((j < 4 ? v.x : v.y) >> (8 * (j & 3))) & 0xFFu;
        dst[j] = (uint32_t)k[j];
        c[j] = dst[j] != 0xFFFFFFFFu && val != 0 && src < A.n && dst[j] < A.n;
        word[j] = c[j] ? front_cur[src >> 5] >> (src & 31) : 0u;
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        c[j] = c[j] && (word[j] & 1u);
        word[j] = c[j] ? A.visited[dst[j] >> 5] : 0xFFFFFFFFu;
    }
    // claims as in visit_slots: idempotent, none waits for a result
    uint32_t fresh = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const uint32_t bit = 1u << (dst[j] & 31);
        if (c[j] && !(word[j] & bit)) {
            atomicOr(&A.visited[dst[j] >> 5], bit);
            A.levels[dst[j]] = next_level;
            atomicOr(&front_next[dst[j] >> 5], bit);
            ++fresh;
        }
    }
    return fresh;
}

// Slot of concatenated-range position p (< total) of a warp's rows: lane r
// holds its row start b and exclusive prefix excl; finds the last r with
// excl[r] <= p. All lanes must call it together.
__device__ __forceinline__ uint32_t lb_slot(uint32_t p, uint32_t total, uint32_t b, uint32_t excl) {
    uint32_t r = 0;
#pragma unroll
    for (uint32_t step = 16; step >= 1; step >>= 1) {
        const uint32_t cand = r + step;
        const uint32_t ex_c = __shfl_sync(0xFFFFFFFFu, excl, cand & 31);
        if (cand < 32 && ex_c <= p)
            r = cand;
    }
    const uint32_t rb = __shfl_sync(0xFFFFFFFFu, b, r);
    const uint32_t rex = __shfl_sync(0xFFFFFFFFu, excl, r);
    return p < total ? rb + (p - rex) : SIZE_NONE;
}

// One pass over the frontier words, a word per warp at a time (lane l owns
// node 32*word + l); `slots` accumulates the slots of every frontier row.
//   QUEUE: rows over BIG_ROW slots are cut into CHUNK_SLOTS chunks appended
//          to `list` (the grid's list or the CTA's own; a full list leaves
//          them to this pass);
//   WALK:  the remaining rows are walked as one concatenated slot range, 64
//          slots per step (without QUEUE, rows over BIG_ROW slots are left to
//          the chunks an earlier pass queued);
//   CLEAR: each word is zeroed once read, for its reuse two levels later.
// Returns the nodes this lane claimed.
template <bool QUEUE, bool WALK, bool CLEAR>
__device__ __forceinline__ uint32_t frontier_pass(const BfsArgs &A, uint32_t *front_cur, uint32_t *front_next,
                                                  uint2 *list, uint32_t list_cap, uint32_t *chunk_cnt,
                                                  uint32_t next_level, uint32_t words, uint32_t gwarp, uint32_t nwarps,
                                                  uint32_t lane, uint32_t &slots) {
    uint32_t fresh = 0;
    // warp gwarp owns words gwarp, gwarp + nwarps, ... (hub rows spread over
    // the grid); it reads 32 of them at once, one per lane, and walks the
    // non-empty ones, so a sparse frontier costs one load round per 32 words
    for (uint32_t it = 0; gwarp + it * nwarps < words; it += 32) {
      const uint32_t wl = gwarp + (it + lane) * nwarps;
      const uint32_t mine = wl < words ? front_cur[wl] : 0u;
      uint32_t pending = __ballot_sync(0xFFFFFFFFu, mine != 0u);
      if (CLEAR && mine)
          front_cur[wl] = 0;
      // a word's row offsets are read while the previous word is walked
      uint32_t nb = 0, nr1 = 0;
      if (pending) {
          const uint32_t src = __ffs(pending) - 1;
          if (__shfl_sync(0xFFFFFFFFu, mine, src) & (1u << lane)) {
              const uint32_t u = ((gwarp + (it + src) * nwarps) << 5) + lane;
              nb = A.ro[u];
              nr1 = A.ro[u + 1];
          }
      }
      while (pending) {
        const uint32_t src = __ffs(pending) - 1;
        pending &= pending - 1;
        const uint32_t f = __shfl_sync(0xFFFFFFFFu, mine, src);
        const uint32_t rb = nb, r1 = nr1;
        nb = nr1 = 0;
        if (pending) {
            const uint32_t src2 = __ffs(pending) - 1;
            if (__shfl_sync(0xFFFFFFFFu, mine, src2) & (1u << lane)) {
                const uint32_t u2 = ((gwarp + (it + src2) * nwarps) << 5) + lane;
                nb = A.ro[u2];
                nr1 = A.ro[u2 + 1];
            }
        }
        uint32_t b = 0, e = 0, len = 0;
        if (f & (1u << lane)) {
            b = rb;
            e = min(r1, A.size);
            if (!in_bounds(A.ctl + CTL_ERR, b <= r1 && r1 <= A.size, BS_ROW))
                b = e;  // an inconsistent row_offset: the row is skipped
            len = e > b ? e - b : 0;
        }
        slots += len;
        bool overflow = false;
        if (QUEUE) {
            const uint32_t nch = len > BIG_ROW ? (len + CHUNK_SLOTS - 1) / CHUNK_SLOTS : 0;
            const uint32_t ch_incl = warp_incl_scan(nch);
            const uint32_t ch_total = __shfl_sync(0xFFFFFFFFu, ch_incl, 31);
            if (ch_total) {
                uint32_t base = 0;
                if (lane == 0)
                    base = atomicAdd(chunk_cnt, ch_total);
                base = __shfl_sync(0xFFFFFFFFu, base, 0);
                if (base + ch_total <= list_cap) {
                    const uint32_t pos = base + ch_incl - nch;
                    for (uint32_t c = 0; c < nch; ++c)
                        list[pos + c] = make_uint2(b + c * CHUNK_SLOTS, min(e, b + (c + 1) * CHUNK_SLOTS));
                } else {
                    // list full: neutralise the claimed entries, walk the rows here
                    for (uint32_t c = base + lane; c < min(base + ch_total, list_cap); c += 32)
                        list[c] = make_uint2(0, 0);
                    overflow = true;
                    if (lane == 0)
                        atomicAdd(A.ctl + CTL_OVERFLOW, 1u);
                }
            }
        }
        if (!overflow && len > BIG_ROW)
            len = 0;  // its chunks are (or were) queued
        if (!WALK && !overflow)
            len = 0;  // short rows wait for the walking pass
        const uint32_t incl = warp_incl_scan(len);
        const uint32_t excl = incl - len;
        const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
        for (uint32_t p0 = 0; p0 < total; p0 += STEP_SLOTS) {
            uint32_t sl[LANE_SLOTS];
#pragma unroll
            for (uint32_t j = 0; j < LANE_SLOTS; ++j)
                sl[j] = lb_slot(p0 + 32 * j + lane, total, b, excl);
            fresh += visit_slots<LANE_SLOTS>(A, sl, next_level, front_next);
        }
      }
    }
    return fresh;
}

// Claims of level i (the next frontier's size, or a little more when lanes
// raced for a node): one atomic per warp into the counter the next level reads.
__device__ __forceinline__ void level_count(const BfsArgs &A, uint32_t i, uint32_t fresh, uint32_t lane) {
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1)
        fresh += __shfl_xor_sync(0xFFFFFFFFu, fresh, d);
    if (lane == 0 && fresh)
        atomicAdd(A.ctl + CTL_CNT + (i + 1) % 3, fresh);
}

// A level whose frontier holds fewer than n / DENSE_GATE nodes is walked
// without measuring its rows first (it cannot span a large share of slots
// often enough to pay for the extra pass).
constexpr uint32_t DENSE_GATE = 64;

// Long-row chunks one CTA keeps in shared memory on a small level.
constexpr uint32_t LOCAL_CHUNKS = 1024;

__global__ void __launch_bounds__(BLOCK, 5) bfs_kernel(BfsArgs A) {
    __shared__ uint2 s_chunks[LOCAL_CHUNKS];
    __shared__ uint32_t s_nch;
    GridBarrier *bar = reinterpret_cast<GridBarrier *>(A.ctl + CTL_BAR);
    uint32_t *err = A.ctl + CTL_ERR;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gwarp = blockIdx.x * (BLOCK / 32) + (threadIdx.x >> 5);
    const uint32_t nwarps = gridDim.x * (BLOCK / 32);
    const uint32_t words = (A.n + 31) >> 5;
    uint32_t last_frontier = 0;
    uint32_t i = 0;
    for (;; ++i) {
        if (A.stamps && blockIdx.x == 0 && threadIdx.x == 0 && i < CTL_PROFILE_LEVELS)
            A.stamps[i] = globaltimer_ns();
        const uint32_t frontier = cta_broadcast_read(A.ctl + CTL_CNT + i % 3);
        const uint32_t stall = i == 0 ? A.stall : 0u;  // test hook: the first barrier never completes
        if (frontier == 0)
            break;
        const uint32_t prev_frontier = last_frontier;
        last_frontier = frontier;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            A.ctl[CTL_CNT + (i + 2) % 3] = 0;
            A.ctl[CTL_SLOTS + (i + 1) % 3] = 0;
            A.ctl[CTL_CHUNKS + (i + 1) % 3] = 0;
        }
        uint32_t *front_cur = (i & 1) ? A.front1 : A.front0;
        uint32_t *front_next = (i & 1) ? A.front0 : A.front1;
        uint32_t *chunk_cnt = A.ctl + CTL_CHUNKS + i % 3;
        const uint32_t next_level = i + 2;
        uint32_t fresh = 0, slots = 0;
        // A large frontier is measured first: one pass queues its long rows'
        // chunks and sums its rows' slots; then the level either sweeps every
        // slot (rows spanning >= size / dense_div slots) or walks the rest.
        const bool probe = A.dense_div && (uint64_t)frontier * DENSE_GATE >= A.n;
        bool dense = false;
        if (probe) {
            fresh += frontier_pass<true, false, false>(A, front_cur, front_next, A.chunks, A.chunk_cap, chunk_cnt,
                                                       next_level, words, gwarp, nwarps, lane, slots);
#pragma unroll
            for (int d = 16; d >= 1; d >>= 1)
                slots += __shfl_xor_sync(0xFFFFFFFFu, slots, d);
            if (lane == 0 && slots)
                atomicAdd(A.ctl + CTL_SLOTS + i % 3, slots);
            if (!grid_barrier(bar, err, stall, A.stall_limit_ns))
                return;
            dense = (uint64_t)cta_broadcast_read(A.ctl + CTL_SLOTS + i % 3) * A.dense_div >= A.size;
        }
        if (A.stamps && blockIdx.x == 0 && threadIdx.x == 0 && i < CTL_PROFILE_LEVELS)
            reinterpret_cast<uint32_t *>(A.stamps + CTL_PROFILE_LEVELS)[i] = frontier | (dense ? 1u << 31 : 0u);
        if (dense) {
            // every slot in one coalesced sweep, 8 slots per thread per step;
            // then, after a barrier, the frontier is cleared
            const uint32_t gtid = blockIdx.x * BLOCK + threadIdx.x;
            const uint32_t nthreads = gridDim.x * BLOCK;
            const ulonglong2 *kv = reinterpret_cast<const ulonglong2 *>(A.keys);
            const uint2 *vv = reinterpret_cast<const uint2 *>(A.vals);
            for (uint32_t o = gtid; o < (A.size >> 3); o += nthreads) {
                const ulonglong2 k0 = kv[4 * o], k1 = kv[4 * o + 1], k2 = kv[4 * o + 2], k3 = kv[4 * o + 3];
                const uint64_t k[8] = {k0.x, k0.y, k1.x, k1.y, k2.x, k2.y, k3.x, k3.y};
                fresh += dense_visit8(A, k, vv[o], front_cur, next_level, front_next);
            }
            // an array of 4 slots (the smallest size): one thread takes it, padded with empty slots
            if (A.size < 8 && gtid == 0) {
                const uint64_t k[8] = {A.keys[0], A.keys[1], A.keys[2], A.keys[3], KEY_NONE, KEY_NONE, KEY_NONE, KEY_NONE};
                const uint2 v = make_uint2(A.vals[0] | (A.vals[1] << 8) | (A.vals[2] << 16) | ((uint32_t)A.vals[3] << 24), 0u);
                fresh += dense_visit8(A, k, v, front_cur, next_level, front_next);
            }
            if (!grid_barrier(bar, err, stall, A.stall_limit_ns))
                return;
            for (uint32_t w = gtid; w < words; w += nthreads)
                front_cur[w] = 0;
            level_count(A, i, fresh, lane);
            if (!grid_barrier(bar, err, stall, A.stall_limit_ns))
                return;
            continue;
        }
        if (probe) {
            // the short rows now; the long rows' chunks, queued by the first pass, below
            fresh += frontier_pass<false, true, true>(A, front_cur, front_next, A.chunks, A.chunk_cap, chunk_cnt,
                                                      next_level, words, gwarp, nwarps, lane, slots);
        } else if ((uint64_t)frontier * DENSE_GATE < A.n && frontier < prev_frontier) {
            // a small, shrinking frontier (the tail of the search, past the
            // hubs): each CTA queues its long rows' chunks in shared memory
            // and its own warps take them, so the level needs one grid barrier
            // instead of two
            if (threadIdx.x == 0)
                s_nch = 0;
            __syncthreads();
            fresh += frontier_pass<true, true, true>(A, front_cur, front_next, s_chunks, LOCAL_CHUNKS, &s_nch,
                                                     next_level, words, gwarp, nwarps, lane, slots);
            __syncthreads();
            const uint32_t nloc = min(s_nch, LOCAL_CHUNKS);
            for (uint32_t c = threadIdx.x >> 5; c < nloc; c += BLOCK / 32) {
                const uint2 ch = s_chunks[c];
                for (uint32_t s0 = ch.x; s0 < ch.y; s0 += CHUNK_SLOTS) {
                    uint32_t sl[CHUNK_LANE_SLOTS];
#pragma unroll
                    for (uint32_t j = 0; j < CHUNK_LANE_SLOTS; ++j)
                        sl[j] = s0 + 32 * j + lane < ch.y ? s0 + 32 * j + lane : SIZE_NONE;
                    fresh += visit_slots<CHUNK_LANE_SLOTS>(A, sl, next_level, front_next);
                }
            }
            level_count(A, i, fresh, lane);
            if (!grid_barrier(bar, err, stall, A.stall_limit_ns))
                return;
            continue;
        } else {
            fresh += frontier_pass<true, true, true>(A, front_cur, front_next, A.chunks, A.chunk_cap, chunk_cnt,
                                                     next_level, words, gwarp, nwarps, lane, slots);
            if (!grid_barrier(bar, err, stall, A.stall_limit_ns))
                return;
        }
        // Phase 2: long-row chunks, one warp per chunk (one step).
        const uint32_t nch_all = min(cta_broadcast_read(chunk_cnt), A.chunk_cap);
        for (uint32_t c = gwarp; c < nch_all; c += nwarps) {
            const uint2 ch = A.chunks[c];
            for (uint32_t s0 = ch.x; s0 < ch.y; s0 += CHUNK_SLOTS) {
                uint32_t sl[CHUNK_LANE_SLOTS];
#pragma unroll
                for (uint32_t j = 0; j < CHUNK_LANE_SLOTS; ++j)
                    sl[j] = s0 + 32 * j + lane < ch.y ? s0 + 32 * j + lane : SIZE_NONE;
                fresh += visit_slots<CHUNK_LANE_SLOTS>(A, sl, next_level, front_next);
            }
        }
        level_count(A, i, fresh, lane);
        if (!grid_barrier(bar, err, stall, A.stall_limit_ns))
            return;
    }
    // reached nodes: the visited bits (a claim count may hold a node twice)
    uint32_t reached = 0;
    for (uint32_t w = blockIdx.x * BLOCK + threadIdx.x; w < words; w += gridDim.x * BLOCK)
        reached += __popc(A.visited[w]);
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1)
        reached += __shfl_xor_sync(0xFFFFFFFFu, reached, d);
    if (lane == 0 && reached)
        atomicAdd(A.ctl + CTL_REACHED, reached);
    if (blockIdx.x == 0 && threadIdx.x == 0)
        A.ctl[CTL_LEVELS] = i;
}

__global__ void bfs_init_kernel(uint32_t *levels, uint32_t *visited, uint32_t *front0, uint32_t *ctl, uint32_t src) {
    levels[src] = 1;
    visited[src >> 5] = 1u << (src & 31);
    front0[src >> 5] = 1u << (src & 31);
    ctl[CTL_CNT + 0] = 1;
    ctl[CTL_CNT + 1] = 0;
    ctl[CTL_CNT + 2] = 0;
    ctl[CTL_SLOTS + 0] = 0;
    ctl[CTL_SLOTS + 1] = 0;
    ctl[CTL_SLOTS + 2] = 0;
    ctl[CTL_REACHED] = 0;  // the kernel counts the visited bits at the end
}

gpma_status ensure_bfs(gpma_graph *g) {
    if (g->bfs_cap >= g->row_num && g->bfs_levels)
        return GPMA_OK;
    free_bfs(g);
    uint32_t n = std::max<uint32_t>(g->row_num, 1);
    GPMA_TRY(dev_alloc(&g->bfs_levels, n));
    GPMA_TRY(dev_alloc(&g->bfs_visited, n / 32 + 2));
    GPMA_TRY(dev_alloc(&g->bfs_front[0], n / 32 + 2));
    GPMA_TRY(dev_alloc(&g->bfs_front[1], n / 32 + 2));
    GPMA_TRY(dev_alloc(&g->bfs_ctl, CTL_WORDS + CTL_PROFILE_WORDS));
    if (!g->h_bfs_ctl) {
        cudaError_t e = cudaMallocHost((void **)&g->h_bfs_ctl, sizeof(uint32_t) * (CTL_WORDS + CTL_PROFILE_WORDS));
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaMallocHost(bfs ctl)");
    }
    g->bfs_cap = n;
    if (g->bfs_grid == 0) {
        int per_sm = 0;
        GPMA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bfs_kernel, BLOCK, 0));
        if (per_sm < 1) {
            set_error("BFS kernel cannot be resident (occupancy 0)");
            return GPMA_ERR_CUDA;
        }
        g->bfs_grid = std::min(per_sm, MAX_BLOCKS_PER_SM);  // resident CTAs per SM
    }
    return GPMA_OK;
}

}  // namespace

void free_bfs(gpma_graph *g) {
    dev_free(g->bfs_levels);
    dev_free(g->bfs_visited);
    dev_free(g->bfs_front[0]);
    dev_free(g->bfs_front[1]);
    dev_free(g->bfs_chunks);
    g->bfs_chunk_cap = 0;
    dev_free(g->bfs_ctl);
    g->bfs_cap = 0;
}

gpma_status bfs_plan(gpma_graph *g, uint32_t src, BfsPlan *P) {
    static_assert(sizeof(BfsArgs) <= KernelLaunch::ARG_BYTES, "BFS arguments exceed the launch record");
    GPMA_TRY(ensure_bfs(g));
    if (bfs_chunk_need(g->geo.size) > g->bfs_chunk_cap) {
        dev_free(g->bfs_chunks);
        g->bfs_chunk_cap = 0;
        GPMA_TRY(dev_alloc(&g->bfs_chunks, bfs_chunk_need(g->geo.size)));
        g->bfs_chunk_cap = bfs_chunk_need(g->geo.size);
    }
    const uint32_t n = g->row_num;
    const size_t bitmap = sizeof(uint32_t) * (n / 32 + 2);
    void *ptr[BfsPlan::CLEARS] = {g->bfs_levels, g->bfs_visited, g->bfs_ctl, g->bfs_front[0], g->bfs_front[1]};
    const size_t bytes[BfsPlan::CLEARS] = {sizeof(uint32_t) * n, bitmap, sizeof(uint32_t) * CTL_WORDS, bitmap, bitmap};
    for (int i = 0; i < BfsPlan::CLEARS; ++i) {
        P->clear_ptr[i] = ptr[i];
        P->clear_bytes[i] = bytes[i];
    }
    P->init_func = (const void *)bfs_init_kernel;
    P->init_levels = g->bfs_levels;
    P->init_visited = g->bfs_visited;
    P->init_front0 = g->bfs_front[0];
    P->init_ctl = g->bfs_ctl;
    P->init_src = src;
    BfsArgs A;
    memset(&A, 0, sizeof(A));  // padding too: launches are compared byte-wise
    A.keys = g->keys;
    A.vals = g->values;
    A.ro = g->row_offset;
    A.n = n;
    A.size = g->geo.size;
    A.levels = g->bfs_levels;
    A.visited = g->bfs_visited;
    A.front0 = g->bfs_front[0];
    A.front1 = g->bfs_front[1];
    A.chunks = g->bfs_chunks;
    A.chunk_cap = g->bfs_chunk_cap;
    A.ctl = g->bfs_ctl;
    A.dense_div = g_tuning.bfs_dense_div;
    A.stamps = g->profiling ? reinterpret_cast<unsigned long long *>(g->bfs_ctl + CTL_WORDS) : nullptr;
    A.stall = g_test_hooks.bfs_stall;
    A.stall_limit_ns = g_test_hooks.bfs_stall ? g_test_hooks.wait_limit_ns : WAIT_LIMIT_NS;
    P->main.set((const void *)bfs_kernel, g->sms * blocks_per_sm(g->bfs_grid, g_tuning.bfs_blocks_per_sm), 0, &A,
                sizeof(A));
    P->ctl_bytes = sizeof(uint32_t) * (CTL_WORDS + (g->profiling ? CTL_PROFILE_WORDS : 0));
    return GPMA_OK;
}

gpma_status bfs_finish(gpma_graph *g, uint64_t *reached) {
    if (g->h_bfs_ctl[CTL_ERR])
        return device_error("the BFS kernel", g->h_bfs_ctl[CTL_ERR]);
    if (reached)
        *reached = g->h_bfs_ctl[CTL_REACHED];
    return GPMA_OK;
}

// Levels land in g->bfs_levels; *reached is the count of reached nodes.
gpma_status bfs_run(gpma_graph *g, uint32_t src, cudaStream_t s, uint64_t *reached) {
    BfsPlan P;
    GPMA_TRY(bfs_plan(g, src, &P));
    for (int i = 0; i < BfsPlan::CLEARS; ++i) {
        if (i == 3)
            prof_mark(g, 0, s);
        GPMA_CUDA(cudaMemsetAsync(P.clear_ptr[i], 0, P.clear_bytes[i], s));
    }
    bfs_init_kernel<<<1, 1, 0, s>>>(P.init_levels, P.init_visited, P.init_front0, P.init_ctl, P.init_src);
    GPMA_CUDA(P.main.launch_cooperative(s));
    prof_mark(g, 1, s);
    GPMA_CUDA(cudaMemcpyAsync(g->h_bfs_ctl, g->bfs_ctl, P.ctl_bytes, cudaMemcpyDeviceToHost, s));
    GPMA_CUDA(cudaStreamSynchronize(s));
    g->prof.kernel_launches += 2;
    g->prof.bfs_kernels++;
    g->prof.bfs_ms += prof_elapsed(g, 0, 1);
    return bfs_finish(g, reached);
}

// ---- BFS without device allocation ------------------------------------------
// Some callers cannot allocate device memory on the fly: code that runs under
// a host-side memory arena or a fixed device-memory budget, plug-ins whose
// host process owns every cudaMalloc, or hosts whose pool forbids growth once
// serving starts. For them gpma_bfs_noalloc keeps the BFS working set (visited
// bitmap, two frontier bitmaps, big-row chunk list, control words) in one file-scope device array
// of a fixed size instead of buffers allocated per graph. Every GPU that loads
// this library holds the array (about 1.3 MB) until the process exits.
namespace {

constexpr uint32_t NOALLOC_MAX_ROWS = 1u << 21;  // 2,097,152 nodes
constexpr uint32_t NOALLOC_BITMAP_WORDS = NOALLOC_MAX_ROWS / 32 + 2;
constexpr uint32_t NOALLOC_CHUNK_CAP = 1u << 16;  // more big-row chunks are walked in place
constexpr size_t NOALLOC_WORDS = CTL_WORDS + 3ull * NOALLOC_BITMAP_WORDS + 2ull * NOALLOC_CHUNK_CAP;
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) uint32_t g_noalloc_scratch[NOALLOC_WORDS];

std::mutex g_noalloc_mu;
uint32_t *g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};
int g_noalloc_grid[NOALLOC_MAX_DEVICES] = {};

// Device address of the scratch array on the current device. The host-side
// symbol is only a stand-in, so the address is looked up once per device
// (with that device current) and cached.
gpma_status noalloc_scratch(uint32_t **out, int *grid, int sms) {
    int dev = 0;
    GPMA_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
        set_error("gpma_bfs_noalloc: device %d outside the supported range 0..%d", dev, NOALLOC_MAX_DEVICES - 1);
        return GPMA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        int per_sm = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bfs_kernel, BLOCK, 0);
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor(bfs_kernel)");
        if (per_sm < 1) {
            set_error("gpma_bfs_noalloc: BFS kernel cannot be resident (occupancy 0)");
            return GPMA_ERR_CUDA;
        }
        g_noalloc_grid[dev] = std::min(per_sm, MAX_BLOCKS_PER_SM);
        g_noalloc_ptr[dev] = static_cast<uint32_t *>(p);
    }
    *out = g_noalloc_ptr[dev];
    *grid = sms * blocks_per_sm(g_noalloc_grid[dev], g_tuning.bfs_blocks_per_sm);
    return GPMA_OK;
}

}  // namespace

gpma_status bfs_noalloc_run(gpma_graph *g, uint32_t src, uint32_t *levels, uint64_t *reached, cudaStream_t s) {
    const uint32_t n = g->row_num;
    if (n > NOALLOC_MAX_ROWS) {
        set_error("gpma_bfs_noalloc: graph has %u nodes; the fixed scratch holds at most %u", n, NOALLOC_MAX_ROWS);
        return GPMA_ERR_CAPACITY;
    }
    uint32_t *scratch = nullptr;
    int grid = 0;
    GPMA_TRY(noalloc_scratch(&scratch, &grid, g->sms));
    uint32_t *ctl = scratch;
    uint32_t *visited = scratch + CTL_WORDS;
    uint32_t *front0 = visited + NOALLOC_BITMAP_WORDS;
    uint32_t *front1 = front0 + NOALLOC_BITMAP_WORDS;
    uint2 *chunks = reinterpret_cast<uint2 *>(front1 + NOALLOC_BITMAP_WORDS);
    // the scratch keeps the previous call's contents: clear what must start at zero
    GPMA_CUDA(cudaMemsetAsync(levels, 0, sizeof(uint32_t) * n, s));
    GPMA_CUDA(cudaMemsetAsync(visited, 0, sizeof(uint32_t) * (n / 32 + 2), s));
    GPMA_CUDA(cudaMemsetAsync(front0, 0, sizeof(uint32_t) * (n / 32 + 2), s));
    GPMA_CUDA(cudaMemsetAsync(front1, 0, sizeof(uint32_t) * (n / 32 + 2), s));
    GPMA_CUDA(cudaMemsetAsync(ctl, 0, sizeof(uint32_t) * CTL_WORDS, s));
    bfs_init_kernel<<<1, 1, 0, s>>>(levels, visited, front0, ctl, src);
    BfsArgs A;
    memset(&A, 0, sizeof(A));
    A.keys = g->keys;
    A.vals = g->values;
    A.ro = g->row_offset;
    A.n = n;
    A.size = g->geo.size;
    A.levels = levels;
    A.visited = visited;
    A.front0 = front0;
    A.front1 = front1;
    A.chunks = chunks;
    A.chunk_cap = g_test_hooks.noalloc_chunk_cap ? std::min(g_test_hooks.noalloc_chunk_cap, NOALLOC_CHUNK_CAP)
                                                 : NOALLOC_CHUNK_CAP;
    A.ctl = ctl;
    A.dense_div = g_tuning.bfs_dense_div;
    A.stamps = nullptr;
    A.stall = g_test_hooks.bfs_stall;
    A.stall_limit_ns = g_test_hooks.bfs_stall ? g_test_hooks.wait_limit_ns : WAIT_LIMIT_NS;
    void *params[] = {&A};
    GPMA_CUDA(cudaLaunchCooperativeKernel((const void *)bfs_kernel, dim3(grid), dim3(BLOCK), params, 0, s));
    uint32_t h_ctl[CTL_WORDS];
    GPMA_CUDA(cudaMemcpyAsync(h_ctl, ctl, sizeof(h_ctl), cudaMemcpyDeviceToHost, s));
    GPMA_CUDA(cudaStreamSynchronize(s));
    g_test_hooks.noalloc_overflows = h_ctl[CTL_OVERFLOW];
    if (h_ctl[CTL_ERR])
        return device_error("the BFS kernel", h_ctl[CTL_ERR]);
    if (reached)
        *reached = h_ctl[CTL_REACHED];
    return GPMA_OK;
}

}  // namespace gpma

extern "C" gpma_status gpma_bfs_level_profile(const gpma_graph *g, double *ms, uint32_t *frontier, uint8_t *dense,
                                              uint32_t capacity, uint32_t *levels) {
    using namespace gpma;
    if (!g || !levels) {
        gpma::set_error("gpma_bfs_level_profile: null argument");
        return GPMA_ERR_INVALID;
    }
    *levels = 0;
    if (!g->profiling || !g->h_bfs_ctl)
        return GPMA_OK;
    const uint32_t L = std::min<uint32_t>(g->h_bfs_ctl[CTL_LEVELS], CTL_PROFILE_LEVELS - 1);
    const uint64_t *st = reinterpret_cast<const uint64_t *>(g->h_bfs_ctl + CTL_WORDS);
    const uint32_t *info = reinterpret_cast<const uint32_t *>(st + CTL_PROFILE_LEVELS);
    *levels = L;
    for (uint32_t i = 0; i < std::min(L, capacity); ++i) {
        if (ms)
            ms[i] = (double)(st[i + 1] - st[i]) * 1e-6;
        if (frontier)
            frontier[i] = info[i] & 0x7FFFFFFFu;
        if (dense)
            dense[i] = (uint8_t)(info[i] >> 31);
    }
    return GPMA_OK;
}
