// sort.cuh - stable LSD radix sort of an update batch (u64 key, u8 value),
// run as phases of the persistent update kernel.
//
// Replaces thrust::sort_by_key of the batch (gpma.cuh:977), a stable radix
// sort. Onesweep design:
//   1. one pass over the batch histograms all eight 8-bit digits at once (and
//      flags keys whose column is the reserved 0xFFFFFFFF);
//   2. digits that are constant over the batch are skipped;
//   3. per remaining digit, CTAs take tiles in the order of a global counter,
//      rank the tile's keys with warp match/ballot (stable: input order),
//      publish per-digit counts and resolve their global offsets by decoupled
//      look-back over earlier tiles (bounded waits), then write through shared
//      memory so each digit run leaves as a contiguous burst.
// Tiles are claimed in counter order by co-resident CTAs, so every look-back
// waits only on tiles that are already being processed.
#pragma once

#include "gpma_internal.cuh"

namespace gpma {

constexpr int SORT_ITEMS = 4;
constexpr uint32_t SORT_TILE = BLOCK * SORT_ITEMS;  // 1024 keys
constexpr uint32_t SORT_FLAG_AGG = 1u << 30;
constexpr uint32_t SORT_FLAG_INC = 2u << 30;
constexpr uint32_t SORT_VALUE_MASK = (1u << 30) - 1;
// shared memory of one tile: keys, values, per-warp digit counts, starts
constexpr size_t SORT_SMEM = SORT_TILE * 9ull + (BLOCK / 32) * 256 * 4ull + 2 * 256 * 4ull;

// Histogram of all 8 digits of keys[0..n) into hist (8 x 256, zeroed by the
// caller); sets st->invalid_keys when check_keys and a reserved column occurs.
__device__ __forceinline__ void sort_histogram(const uint64_t *__restrict__ keys, uint32_t n, uint32_t *hist,
                                               DeviceStatus *st, bool check_keys, uint32_t *sh) {
    for (int i = threadIdx.x; i < 8 * 256; i += BLOCK)
        sh[i] = 0;
    __syncthreads();
    uint32_t bad = 0;
    for (uint32_t i = blockIdx.x * BLOCK + threadIdx.x; i < n; i += gridDim.x * BLOCK) {
        uint64_t k = keys[i];
        bad |= (uint32_t)((k & COL_NONE) == COL_NONE);
#pragma unroll
        for (int p = 0; p < 8; ++p)
            atomicAdd(&sh[p * 256 + ((k >> (8 * p)) & 255)], 1u);
    }
    if (__syncthreads_or(bad) && check_keys && threadIdx.x == 0)
        atomicOr(&st->invalid_keys, 1u);
    for (int i = threadIdx.x; i < 8 * 256; i += BLOCK) {
        uint32_t c = sh[i];
        if (c)
            atomicAdd(&hist[i], c);
    }
    __syncthreads();
}

// Bit p set when digit p is the same for every key (that pass is skipped).
__device__ __forceinline__ uint32_t sort_trivial_mask(const uint32_t *hist, uint32_t n) {
    uint32_t mask = 0;
    for (int p = 0; p < 8; ++p)
        if (__syncthreads_or(hist[p * 256 + threadIdx.x] == n))
            mask |= 1u << p;
    return mask;
}

// One tile of digit pass `pass`: keys in_k/in_v -> out_k/out_v.
__device__ void sort_tile(int pass, uint32_t tile, const uint64_t *__restrict__ in_k, const uint8_t *__restrict__ in_v,
                          uint64_t *__restrict__ out_k, uint8_t *__restrict__ out_v, uint32_t n,
                          const uint32_t *hist, uint32_t *status_all, DeviceStatus *st, unsigned char *smem,
                          uint32_t *tmp) {
    const int shift = 8 * pass;
    const uint32_t tiles = (n + SORT_TILE - 1) / SORT_TILE;
    uint32_t *status = status_all + (size_t)pass * tiles * 256;
    uint64_t *s_keys = reinterpret_cast<uint64_t *>(smem);
    uint8_t *s_vals = smem + SORT_TILE * 8;
    uint32_t *whist = reinterpret_cast<uint32_t *>(smem + SORT_TILE * 9);  // [BLOCK/32][256]
    uint32_t *s_start = whist + (BLOCK / 32) * 256;
    uint32_t *s_global = s_start + 256;

    for (int i = threadIdx.x; i < (BLOCK / 32) * 256; i += BLOCK)
        whist[i] = 0;
    __syncthreads();
    const uint32_t tile_lo = tile * SORT_TILE;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t warp_lo = tile_lo + warp * 32 * SORT_ITEMS;
    uint32_t *wh = whist + warp * 256;

    uint64_t k[SORT_ITEMS];
    uint8_t v[SORT_ITEMS];
    uint32_t rank[SORT_ITEMS];
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; ++j) {
        uint32_t idx = warp_lo + j * 32 + lane;
        bool ok = idx < n;
        k[j] = ok ? in_k[idx] : 0;
        v[j] = ok ? in_v[idx] : 0;
    }
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; ++j) {
        uint32_t idx = warp_lo + j * 32 + lane;
        bool ok = idx < n;
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
    const uint32_t base = block_excl_scan(hist[pass * 256 + d], &total, tmp);

    // Decoupled look-back for digit d.
    uint32_t prefix = 0;
    if (tile == 0) {
        atomicExch(&status[d], SORT_FLAG_INC | local);
    } else {
        atomicExch(&status[(size_t)tile * 256 + d], SORT_FLAG_AGG | local);
        int64_t t = (int64_t)tile - 1;
        uint64_t t0 = 0;
        unsigned ns = 32;
        while (t >= 0) {
            uint32_t w = ld_volatile(&status[(size_t)t * 256 + d]);
            uint32_t flag = w & ~SORT_VALUE_MASK;
            if (flag == 0) {
                if (t0 == 0)
                    t0 = globaltimer_ns();
                __nanosleep(ns);
                if (ns < 256)
                    ns <<= 1;
                if (globaltimer_ns() - t0 > WAIT_LIMIT_NS || ld_volatile(&st->err) != 0) {
                    atomicCAS(&st->err, 0u, DERR_LOOKBACK_TIMEOUT);
                    break;
                }
                continue;
            }
            prefix += w & SORT_VALUE_MASK;
            if (flag == SORT_FLAG_INC)
                break;
            --t;
        }
        atomicExch(&status[(size_t)tile * 256 + d], SORT_FLAG_INC | (prefix + local));
    }
    s_global[d] = base + prefix;
    __syncthreads();

    // Stage the tile in digit order, then write each digit run contiguously.
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; ++j) {
        uint32_t idx = warp_lo + j * 32 + lane;
        if (idx < n) {
            uint32_t dd = (uint32_t)((k[j] >> shift) & 255);
            uint32_t pos = s_start[dd] + wh[dd] + rank[j];
            s_keys[pos] = k[j];
            s_vals[pos] = v[j];
        }
    }
    __syncthreads();
    const uint32_t tile_n = min(SORT_TILE, n - tile_lo);
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
