// sort.cuh - stable sort of the update batches of one or more graphs (u64
// key, u8 value), run as phases of the persistent update kernel: a bucket
// sort (below) and, for batches that crowd one bucket, LSD radix passes.
//
// Replaces thrust::sort_by_key of the batch (gpma.cuh:977), a stable radix
// sort. The digit passes are a onesweep design, segmented by graph (graph g's
// batch occupies [boff[g], boff[g+1]) and stays there):
//   1. one pass histograms all eight 8-bit digits of every graph's batch at
//      once (and flags keys whose column is the reserved 0xFFFFFFFF);
//   2. digits constant over every batch are skipped;
//   3. per remaining digit, CTAs take tiles in the order of a global counter
//      (graph g owns tiles [toff[g], toff[g+1])), rank the tile's keys with
//      warp match/ballot (stable: input order), publish per-digit counts and
//      resolve their offsets by decoupled look-back over the earlier tiles of
//      the same graph (bounded waits), then write through shared memory so
//      each digit run leaves as a contiguous burst.
// Tiles are claimed in counter order by co-resident CTAs, so every look-back
// waits only on tiles that are already being processed.
//
// The default is a bucket sort with no look-back and four grid barriers
// (bsort_* below); the digit passes above remain for batches that crowd one
// bucket (a burst into a few rows, a bulk load with hub rows).
#pragma once

#include "gpma_internal.cuh"

namespace gpma {

// Keys per thread of a tile (build option; a tile of 2048 keys by default).
#ifndef GPMA_SORT_ITEMS
#define GPMA_SORT_ITEMS 8
#endif
constexpr int SORT_ITEMS = GPMA_SORT_ITEMS;
// Predecessor tiles a look-back step reads at once (build option).
#ifndef GPMA_SORT_LOOKBACK
#define GPMA_SORT_LOOKBACK 8
#endif
constexpr uint32_t SORT_LOOKBACK = GPMA_SORT_LOOKBACK;
constexpr uint32_t SORT_TILE = BLOCK * SORT_ITEMS;
static_assert(SORT_TILE * 9 + (BLOCK / 32 + 2) * 256 * 4 <= UPDATE_SMEM, "sort tile exceeds the update kernel's smem");
constexpr uint32_t SORT_FLAG_AGG = 1u << 30;
constexpr uint32_t SORT_FLAG_INC = 2u << 30;
constexpr uint32_t SORT_VALUE_MASK = (1u << 30) - 1;

// Histograms of all 8 digits into hist[g][8][256] for each graph g < G and
// the totals into hist[G][8][256] (zeroed by the caller); sets
// st->invalid_keys when check_keys and a reserved column occurs. Each CTA
// walks a contiguous key range graph by graph.
__device__ __forceinline__ void sort_histogram(const uint64_t *__restrict__ keys, const uint32_t *boff, uint32_t G,
                                               uint32_t *hist, DeviceStatus *st, bool check_keys, uint32_t *sh) {
    const uint32_t n = boff[G];
    const uint32_t per = (n + gridDim.x - 1) / gridDim.x;
    const uint32_t lo = min(n, blockIdx.x * per), hi = min(n, lo + per);
    uint32_t bad = 0;
    uint32_t pos = lo;
    while (__syncthreads_or(pos < hi)) {
        const uint32_t g = G == 1 ? 0 : segment_of(boff, G, pos);
        const uint32_t end = min(hi, boff[g + 1]);
        for (int i = threadIdx.x; i < 8 * 256; i += BLOCK)
            sh[i] = 0;
        __syncthreads();
        for (uint32_t i = pos + threadIdx.x; i < end; i += BLOCK) {
            uint64_t k = keys[i];
            bad |= (uint32_t)((k & COL_NONE) == COL_NONE);
#pragma unroll
            for (int p = 0; p < 8; ++p)
                atomicAdd(&sh[p * 256 + ((k >> (8 * p)) & 255)], 1u);
        }
        __syncthreads();
        for (int i = threadIdx.x; i < 8 * 256; i += BLOCK) {
            uint32_t c = sh[i];
            if (c) {
                atomicAdd(&hist[(size_t)g * 2048 + i], c);
                if (G > 1)
                    atomicAdd(&hist[(size_t)G * 2048 + i], c);
            }
        }
        pos = end;
    }
    if (__syncthreads_or(bad) && check_keys && threadIdx.x == 0)
        atomicOr(&st->invalid_keys, 1u);
}

// Bit p set when digit p is the same for every key of every graph (that
// pass is skipped); `total` is the all-graph histogram.
__device__ __forceinline__ uint32_t sort_trivial_mask(const uint32_t *total, uint32_t n) {
    // all eight loads in flight before the first CTA vote
    uint32_t c[8];
#pragma unroll
    for (int p = 0; p < 8; ++p)
        c[p] = total[p * 256 + threadIdx.x];
    uint32_t mask = 0;
#pragma unroll
    for (int p = 0; p < 8; ++p)
        if (__syncthreads_or(c[p] == n))
            mask |= 1u << p;
    return mask;
}

// One tile of digit pass `pass`: keys in_k/in_v -> out_k/out_v.
__device__ void sort_tile(int pass, uint32_t tile, const uint64_t *__restrict__ in_k, const uint8_t *__restrict__ in_v,
                          uint64_t *__restrict__ out_k, uint8_t *__restrict__ out_v, const uint32_t *boff,
                          const uint32_t *toff, uint32_t G, const uint32_t *hist, uint32_t *status_all,
                          DeviceStatus *st, unsigned char *smem, uint32_t *tmp) {
    const int shift = 8 * pass;
    const uint32_t tiles = toff[G];
    const uint32_t g = G == 1 ? 0 : segment_of(toff, G, tile);
    const uint32_t first_tile = toff[g];
    const uint32_t seg_lo = boff[g], seg_hi = boff[g + 1];
    uint32_t *status = status_all + (size_t)pass * tiles * 256;
    uint64_t *s_keys = reinterpret_cast<uint64_t *>(smem);
    uint8_t *s_vals = smem + SORT_TILE * 8;
    uint32_t *whist = reinterpret_cast<uint32_t *>(smem + SORT_TILE * 9);  // [BLOCK/32][256]
    uint32_t *s_start = whist + (BLOCK / 32) * 256;
    uint32_t *s_global = s_start + 256;

    for (int i = threadIdx.x; i < (BLOCK / 32) * 256; i += BLOCK)
        whist[i] = 0;
    __syncthreads();
    const uint32_t tile_lo = seg_lo + (tile - first_tile) * SORT_TILE;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t warp_lo = tile_lo + warp * 32 * SORT_ITEMS;
    uint32_t *wh = whist + warp * 256;

    uint64_t k[SORT_ITEMS];
    uint8_t v[SORT_ITEMS];
    uint32_t rank[SORT_ITEMS];
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; ++j) {
        uint32_t idx = warp_lo + j * 32 + lane;
        bool ok = idx < seg_hi;
        k[j] = ok ? in_k[idx] : 0;
        v[j] = ok ? in_v[idx] : 0;
    }
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; ++j) {
        uint32_t idx = warp_lo + j * 32 + lane;
        bool ok = idx < seg_hi;
        uint32_t d = ok ? (uint32_t)((k[j] >> shift) & 255) : 256u + lane;
        uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        uint32_t prior = ok ? wh[d] : 0;
        __syncwarp();
        if (ok) {
            rank[j] = prior + __popc(peers & lanemask_lt());
            if ((peers & lanemask_lt()) == 0)
                wh[d] = prior + __popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();
    // Per digit: tile total and per-warp exclusive offsets (thread d owns digit d).
    const int d = threadIdx.x;
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < BLOCK / 32; ++w) {
        uint32_t c = whist[w * 256 + d];
        whist[w * 256 + d] = run;
        run += c;
    }
    const uint32_t local = run;
    uint32_t total;
    s_start[d] = block_excl_scan(local, &total, tmp);
    const uint32_t base = seg_lo + block_excl_scan(hist[(size_t)g * 2048 + pass * 256 + d], &total, tmp);

    // Decoupled look-back for digit d over this graph's earlier tiles.
    uint32_t prefix = 0;
    if (tile == first_tile) {
        atomicExch(&status[(size_t)tile * 256 + d], SORT_FLAG_INC | local);
    } else {
        atomicExch(&status[(size_t)tile * 256 + d], SORT_FLAG_AGG | local);
        // windows of LOOKBACK predecessors are read at once and summed
        // nearest first, up to the first inclusive value or unpublished word
        int64_t t = (int64_t)tile - 1;
        uint64_t t0 = 0;
        unsigned ns = 32;
        while (t >= (int64_t)first_tile) {
            uint32_t w[SORT_LOOKBACK];
#pragma unroll
            for (uint32_t i = 0; i < SORT_LOOKBACK; ++i)
                w[i] = t - (int64_t)i >= (int64_t)first_tile ? ld_volatile(&status[(size_t)(t - i) * 256 + d])
                                                              : SORT_FLAG_INC;  // never read: the first tile is inclusive
            uint32_t take = 0;
            bool inc = false, blocked = false;
#pragma unroll
            for (uint32_t i = 0; i < SORT_LOOKBACK; ++i) {
                if (inc || blocked)
                    continue;
                const uint32_t flag = w[i] & ~SORT_VALUE_MASK;
                if (flag == 0) {
                    blocked = true;
                    continue;
                }
                prefix += w[i] & SORT_VALUE_MASK;
                ++take;
                inc = flag == SORT_FLAG_INC;
            }
            if (inc)
                break;
            t -= take;
            if (blocked) {
                if (t0 == 0)
                    t0 = globaltimer_ns();
                __nanosleep(ns);
                if (ns < 256)
                    ns <<= 1;
                if (globaltimer_ns() - t0 > WAIT_LIMIT_NS || ld_volatile(&st->err) != 0) {
                    atomicCAS(&st->err, 0u, DERR_LOOKBACK_TIMEOUT);
                    break;
                }
            }
        }
        atomicExch(&status[(size_t)tile * 256 + d], SORT_FLAG_INC | (prefix + local));
    }
    s_global[d] = base + prefix;
    __syncthreads();

    // Stage the tile in digit order, then write each digit run contiguously.
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; ++j) {
        uint32_t idx = warp_lo + j * 32 + lane;
        if (idx < seg_hi) {
            uint32_t dd = (uint32_t)((k[j] >> shift) & 255);
            uint32_t pos = s_start[dd] + wh[dd] + rank[j];
            s_keys[pos] = k[j];
            s_vals[pos] = v[j];
        }
    }
    __syncthreads();
    const uint32_t tile_n = min(SORT_TILE, seg_hi - tile_lo);
    for (uint32_t i = threadIdx.x; i < tile_n; i += BLOCK) {
        uint64_t kk = s_keys[i];
        uint32_t dd = (uint32_t)((kk >> shift) & 255);
        uint32_t pos = s_global[dd] + (i - s_start[dd]);
        out_k[pos] = kk;
        out_v[pos] = s_vals[i];
    }
    __syncthreads();
}

// ---- bucket sort ----------------------------------------------------------------
// Each graph's slot array is cut into a power of two of equal slot ranges,
// sized on the host for about BSORT_AVG keys each; a key's bucket is the range
// its row's slots fall in, interpolated linearly by its column (bucket_of).
// Rows hold slots in proportion to their degree, so power-law hub rows spread
// over several buckets as long as the batch follows the graph's own degrees
// (a sliding window does). Four phases, one grid barrier after each; every
// key costs about three scattered 32-byte sectors (its row's offsets, its
// bucket's atomic, its record), the rest is coalesced:
//   Q1 every key takes a rank in its bucket (one atomic per key); rank and
//      bucket are stored per key;
//   Q2 the bucket counts are scanned chunk by chunk (one chunk per CTA); a
//      bucket of more than BSORT_MAX_BUCKET keys sends the launch to the digit
//      passes;
//   Q3 every key's record (key, batch index, bucket, value: 16 bytes) is
//      written to its bucket's range at its rank; the key that lands on an
//      item's nominal start records the item's bound;
//   Q4 items of whole buckets (item j of a graph holds the buckets that start
//      in [j, j + 1) * BSORT_ITEM of its range, fewer than BSORT_CAP keys) are
//      staged in shared memory; a key's place in its bucket is the number of
//      keys of the bucket before it in (key, batch index) order (a bucket
//      holds a few dozen keys), or, in an item with a bucket of more than
//      BSORT_RANK_MAX keys, the item is sorted by a bitonic network.
// Equal keys end in batch order, so the result is the stable sort's whatever
// order the ranks were taken in.
constexpr uint32_t BSORT_ITEM = 1024;
constexpr uint32_t BSORT_MAX_BUCKET = 1024;
constexpr uint32_t BSORT_CAP = BSORT_ITEM + BSORT_MAX_BUCKET;
constexpr uint32_t BSORT_AVG = 32;
constexpr uint32_t BSORT_RANK_MAX = 256;
constexpr uint32_t BSORT_MAX_BUCKETS = 1u << 24;  // bucket ids share a word with the value
constexpr int BSORT_ILP = 4;
constexpr uint32_t BSORT_PER_THREAD = BSORT_CAP / BLOCK;  // item entries per thread
// Q4 stages the item (a key, a packed word and the bucket's place in the item
// per entry) in shared memory, followed by the chunk prefix (one word per
// CTA) that Q3 and Q4 read
constexpr size_t BSORT_SMEM_ITEM = (size_t)BSORT_CAP * 20;
constexpr uint32_t BSORT_MAX_GRID = (uint32_t)((UPDATE_SMEM - BSORT_SMEM_ITEM) / 4);
static_assert(BSORT_SMEM_ITEM < UPDATE_SMEM && BSORT_CAP % BLOCK == 0, "bucket sort item layout");

struct BucketSort {
    const uint32_t *qoff;   // first bucket of each graph, G + 1
    const uint32_t *qtoff;  // first item of each graph, G + 1
    uint32_t nq;            // buckets of all graphs (< BSORT_MAX_BUCKETS)
    uint32_t *qcnt;         // keys per bucket (zero at launch, zeroed again after use)
    unsigned long long *qinfo;  // per bucket: offset within its scan chunk | count << 32
    uint32_t *rank;         // per batch key: its rank in its bucket
    uint32_t *bkt;          // per batch key: its bucket
    uint4 *rec;             // per sorted position: key (x, y), batch index (z), bucket << 8 | value (w)
    uint32_t *bound;        // per item: its first position
};

// Bucket of `key` within its graph: the slot row_offset[src] + (row length x
// column) >> qbits (qbits: bits of the largest column), shifted right by
// qshift and capped at qnbm1; keys of rows past row_num go to the last bucket.
// Monotone in the key (a row's interpolated slots stay below the next row's
// first), so buckets in order hold keys in order.
__device__ __forceinline__ uint32_t bucket_of(uint64_t key, const GraphDesc &D) {
    const uint32_t src = (uint32_t)(key >> 32);
    if (src >= D.row_num)
        return D.qnbm1;
    const uint64_t a = D.row_offset[src], e = D.row_offset[src + 1];
    const uint64_t dmax = (1ull << D.qbits) - 1;
    const uint64_t dst = key & 0xFFFFFFFFull;
    const uint64_t slot = a + (((e - a) * (dst < dmax ? dst : dmax)) >> D.qbits);
    const uint64_t b = slot >> D.qshift;
    return b < D.qnbm1 ? (uint32_t)b : D.qnbm1;
}

__device__ __forceinline__ void bsort_range(uint32_t n, uint32_t &lo, uint32_t &hi) {
    const uint32_t per = (n + gridDim.x - 1) / gridDim.x;
    lo = min(n, blockIdx.x * per);
    hi = min(n, lo + per);
}

// Graph of batch position i for a thread walking upwards from graph g (a
// search only for the first position).
__device__ __forceinline__ uint32_t graph_at(const uint32_t *boff, uint32_t G, uint32_t i, uint32_t g) {
    if (G == 1)
        return 0;
    if (g == 0xFFFFFFFFu)
        return segment_of(boff, G, i);
    while (boff[g + 1] <= i)
        ++g;
    return g;
}

// Q1: ranks and buckets (and the reserved-column check of the digit histogram).
__device__ void bsort_rank(const uint64_t *keys, const uint32_t *boff, uint32_t G, const GraphDesc *gd,
                           const BucketSort &Q, DeviceStatus *st, bool check_keys) {
    uint32_t lo, hi;
    bsort_range(boff[G], lo, hi);
    uint32_t bad = 0, g = 0xFFFFFFFFu;
    for (uint32_t i0 = lo + threadIdx.x; i0 < hi; i0 += BSORT_ILP * BLOCK) {
        uint64_t k[BSORT_ILP];
        uint32_t b[BSORT_ILP], r[BSORT_ILP];
#pragma unroll
        for (int j = 0; j < BSORT_ILP; ++j) {
            const uint32_t i = i0 + j * BLOCK;
            k[j] = i < hi ? keys[i] : 0ull;
        }
#pragma unroll
        for (int j = 0; j < BSORT_ILP; ++j) {
            const uint32_t i = i0 + j * BLOCK;
            if (i < hi) {
                bad |= (uint32_t)((k[j] & COL_NONE) == COL_NONE);
                g = graph_at(boff, G, i, g);
                b[j] = Q.qoff[g] + bucket_of(k[j], gd[g]);
            }
        }
        // all atomics in flight before the first rank is stored
#pragma unroll
        for (int j = 0; j < BSORT_ILP; ++j)
            if (i0 + j * BLOCK < hi)
                r[j] = atomicAdd(Q.qcnt + b[j], 1u);
#pragma unroll
        for (int j = 0; j < BSORT_ILP; ++j) {
            const uint32_t i = i0 + j * BLOCK;
            if (i < hi) {
                Q.rank[i] = r[j];
                Q.bkt[i] = b[j];
            }
        }
    }
    if (__syncthreads_or(bad) && check_keys && threadIdx.x == 0)
        atomicOr(&st->invalid_keys, 1u);
}

// Q2: chunk-local exclusive offsets and counts of the buckets, the chunk's
// total into chunk_tot[blockIdx.x]; flags the fallback when a bucket is too large.
__device__ void bsort_scan(const BucketSort &Q, uint32_t *chunk_tot, DeviceStatus *st, uint32_t *tmp) {
    const uint32_t per = (Q.nq + gridDim.x - 1) / gridDim.x;
    const uint32_t b0 = min(Q.nq, blockIdx.x * per), b1 = min(Q.nq, b0 + per);
    uint32_t run = 0, big = 0;
    for (uint32_t x = b0; x < b1; x += BLOCK) {
        const uint32_t b = x + threadIdx.x;
        const uint32_t c = b < b1 ? __ldcg(Q.qcnt + b) : 0u;
        big |= (uint32_t)(c > BSORT_MAX_BUCKET);
        uint32_t tot;
        const uint32_t ex = block_excl_scan(c, &tot, tmp);
        if (b < b1)
            Q.qinfo[b] = (unsigned long long)(run + ex) | ((unsigned long long)c << 32);
        run += tot;
    }
    if (threadIdx.x == 0)
        chunk_tot[blockIdx.x] = run;
    if (__syncthreads_or(big) && threadIdx.x == 0)
        atomicOr(&st->sort_fallback, 1u);
}

// Exclusive prefix of the chunk totals into shared memory (gridDim.x words).
__device__ void bsort_chunk_prefix(const uint32_t *chunk_tot, uint32_t *cpre, uint32_t *tmp) {
    uint32_t run = 0;
    for (uint32_t x = 0; x < gridDim.x; x += BLOCK) {
        const uint32_t j = x + threadIdx.x;
        const uint32_t c = j < gridDim.x ? __ldcg(chunk_tot + j) : 0u;
        uint32_t tot;
        const uint32_t ex = block_excl_scan(c, &tot, tmp);
        if (j < gridDim.x)
            cpre[j] = run + ex;
        run += tot;
    }
    __syncthreads();
}

// Q3: every key's record into its bucket's range; item bounds.
__device__ void bsort_scatter(const uint64_t *keys, const uint8_t *vals, const uint32_t *boff, uint32_t G,
                              const BucketSort &Q, const uint32_t *cpre) {
    uint32_t lo, hi;
    bsort_range(boff[G], lo, hi);
    const uint32_t per = (Q.nq + gridDim.x - 1) / gridDim.x;
    uint32_t g = 0xFFFFFFFFu;
    for (uint32_t i0 = lo + threadIdx.x; i0 < hi; i0 += BSORT_ILP * BLOCK) {
        uint64_t k[BSORT_ILP];
        uint32_t r[BSORT_ILP], b[BSORT_ILP], v[BSORT_ILP];
        unsigned long long inf[BSORT_ILP];
#pragma unroll
        for (int j = 0; j < BSORT_ILP; ++j) {
            const uint32_t i = i0 + j * BLOCK;
            const bool ok = i < hi;
            k[j] = ok ? keys[i] : 0ull;
            v[j] = ok ? vals[i] : 0u;
            r[j] = ok ? Q.rank[i] : 0u;  // both written by this thread in Q1
            b[j] = ok ? Q.bkt[i] : 0u;
        }
#pragma unroll
        for (int j = 0; j < BSORT_ILP; ++j)
            inf[j] = i0 + j * BLOCK < hi ? __ldcg(Q.qinfo + b[j]) : 0ull;
#pragma unroll
        for (int j = 0; j < BSORT_ILP; ++j) {
            const uint32_t i = i0 + j * BLOCK;
            if (i < hi) {
                const uint32_t f = cpre[b[j] / per] + (uint32_t)inf[j];
                const uint32_t pos = f + r[j];
                Q.rec[pos] = make_uint4((uint32_t)k[j], (uint32_t)(k[j] >> 32), i, (b[j] << 8) | v[j]);
                g = graph_at(boff, G, i, g);
                const uint32_t rel = pos - boff[g];
                if (rel % BSORT_ITEM == 0)  // the item starts at the first bucket start at or after here
                    Q.bound[Q.qtoff[g] + rel / BSORT_ITEM] = f == pos ? pos : f + (uint32_t)(inf[j] >> 32);
            }
        }
    }
}

// Bitonic sort of s_k/s_x[0..N) (N a power of two) by (key, x); x holds the
// batch index in its high half, so equal keys order by batch index.
__device__ __forceinline__ void bsort_bitonic(uint64_t *s_k, uint64_t *s_x, uint32_t N) {
    for (uint32_t k = 2; k <= N; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < (N >> 1); i += BLOCK) {
                const uint32_t a = ((i & ~(j - 1)) << 1) | (i & (j - 1));
                const uint32_t c = a + j;
                const uint64_t ka = s_k[a], kc = s_k[c];
                const uint64_t xa = s_x[a], xc = s_x[c];
                const bool gt = ka > kc || (ka == kc && xa > xc);
                if (gt == ((a & k) == 0)) {
                    s_k[a] = kc;
                    s_k[c] = ka;
                    s_x[a] = xc;
                    s_x[c] = xa;
                }
            }
            __syncthreads();
        }
    }
}

// Q4: sort of every item into out_k / out_v. Thread t holds entries t + j *
// BLOCK of the item; every global load of a step is issued before the first
// use, and entries live in shared memory between steps.
__device__ void bsort_items(uint64_t *__restrict__ out_k, uint8_t *__restrict__ out_v, const uint32_t *boff,
                            uint32_t G, const BucketSort &Q, const uint32_t *cpre, unsigned char *smem) {
    uint64_t *s_k = reinterpret_cast<uint64_t *>(smem);
    uint64_t *s_x = reinterpret_cast<uint64_t *>(smem + (size_t)BSORT_CAP * 8);  // index << 32 | bucket << 8 | value
    uint32_t *s_b = reinterpret_cast<uint32_t *>(smem + (size_t)BSORT_CAP * 16);  // bucket: first | size << 16
    __shared__ uint32_t s_range[2];
    const uint32_t per = (Q.nq + gridDim.x - 1) / gridDim.x;
    const uint32_t items = Q.qtoff[G];
    for (uint32_t t = blockIdx.x; t < items; t += gridDim.x) {
        if (threadIdx.x < 2) {
            const uint32_t g = G == 1 ? 0u : segment_of(Q.qtoff, G, t);
            s_range[threadIdx.x] = threadIdx.x == 0 || t + 1 < Q.qtoff[g + 1] ? __ldcg(Q.bound + t + threadIdx.x)
                                                                               : boff[g + 1];
        }
        __syncthreads();
        const uint32_t p0 = s_range[0], p1 = s_range[1];
        __syncthreads();
        const uint32_t m = p1 - p0;  // < BSORT_ITEM + BSORT_MAX_BUCKET = BSORT_CAP
        if (m == 0)
            continue;
        uint32_t big = 0;
        {
            uint4 e[BSORT_PER_THREAD];
#pragma unroll
            for (uint32_t j = 0; j < BSORT_PER_THREAD; ++j) {
                const uint32_t r = threadIdx.x + j * BLOCK;
                if (r < m)
                    e[j] = __ldcg(Q.rec + p0 + r);
            }
            unsigned long long qi[BSORT_PER_THREAD];
#pragma unroll
            for (uint32_t j = 0; j < BSORT_PER_THREAD; ++j) {
                const uint32_t r = threadIdx.x + j * BLOCK;
                if (r < m) {
                    s_k[r] = ((uint64_t)e[j].y << 32) | e[j].x;
                    s_x[r] = ((uint64_t)e[j].z << 32) | e[j].w;
                    qi[j] = __ldcg(Q.qinfo + (e[j].w >> 8));
                }
            }
#pragma unroll
            for (uint32_t j = 0; j < BSORT_PER_THREAD; ++j) {
                const uint32_t r = threadIdx.x + j * BLOCK;
                if (r < m) {
                    const uint32_t size = (uint32_t)(qi[j] >> 32);
                    const uint32_t first = cpre[(e[j].w >> 8) / per] + (uint32_t)qi[j] - p0;
                    s_b[r] = first | (size << 16);  // both <= BSORT_CAP
                    big |= (uint32_t)(size > BSORT_RANK_MAX);
                }
            }
        }
        if (!__syncthreads_or(big)) {
            // place = first slot of the bucket + its keys ordered before this one
            for (uint32_t r = threadIdx.x; r < m; r += BLOCK) {
                const uint64_t k = s_k[r], x = s_x[r];
                const uint32_t fb = s_b[r];
                const uint32_t first = fb & 0xFFFFu, last = first + (fb >> 16);
                // both words loaded unconditionally, eight entries per step:
                // the loads of a step overlap instead of one latency per entry
                uint32_t before = 0, q = first;
                for (; q + 8 <= last; q += 8) {
                    uint64_t kq[8], xq[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        kq[u] = s_k[q + u];
                        xq[u] = s_x[q + u];
                    }
#pragma unroll
                    for (int u = 0; u < 8; ++u)
                        before += (uint32_t)(kq[u] < k) | ((uint32_t)(kq[u] == k) & (uint32_t)(xq[u] < x));
                }
                for (; q < last; ++q) {
                    const uint64_t kq = s_k[q], xq = s_x[q];
                    before += (uint32_t)(kq < k) | ((uint32_t)(kq == k) & (uint32_t)(xq < x));
                }
                out_k[p0 + first + before] = k;
                out_v[p0 + first + before] = (uint8_t)x;
            }
        } else {
            const uint32_t N = m <= 1 ? 1u : 1u << (32 - __clz(m - 1));
            for (uint32_t r = m + threadIdx.x; r < N; r += BLOCK) {
                s_k[r] = KEY_NONE;
                s_x[r] = ~0ull;  // pads sort after every real key
            }
            __syncthreads();
            bsort_bitonic(s_k, s_x, N);
            for (uint32_t r = threadIdx.x; r < m; r += BLOCK) {
                out_k[p0 + r] = s_k[r];
                out_v[p0 + r] = (uint8_t)s_x[r];
            }
        }
        __syncthreads();
    }
}

}  // namespace gpma
