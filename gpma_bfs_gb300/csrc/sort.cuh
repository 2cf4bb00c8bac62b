// sort.cuh - stable LSD radix sort of the update batches of one or more
// graphs (u64 key, u8 value), run as phases of the persistent update kernel.
//
// Replaces thrust::sort_by_key of the batch (gpma.cuh:977), a stable radix
// sort. Onesweep design, segmented by graph (graph g's batch occupies
// [boff[g], boff[g+1]) and stays there):
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

}  // namespace gpma
