// sort.cu - stable LSD radix sort of an update batch (u64 key, u8 value).
//
// Replaces thrust::sort_by_key of the batch (gpma.cuh:977), a stable radix
// sort. Design (onesweep):
//   1. one histogram pass counts all eight 8-bit digits at once and flags
//      keys whose column is the reserved 0xFFFFFFFF;
//   2. a one-CTA plan kernel scans each digit histogram into global bin
//      bases and marks digits that are constant over the batch (skipped);
//   3. one kernel per non-trivial digit: each CTA takes the next tile id,
//      ranks its 4096 keys with warp match/ballot (stable: input order),
//      publishes its per-digit counts and resolves its global offsets by
//      decoupled look-back over earlier tiles (bounded waits), then writes
//      through shared memory so each digit run leaves as a contiguous burst.
// Which ping-pong buffer each pass reads is decided on the device, so the
// whole sort is enqueued without a host round trip.
#include "gpma_internal.cuh"

namespace gpma {
namespace {

constexpr int SORT_ITEMS = 16;
constexpr int SORT_TILE = BLOCK * SORT_ITEMS;  // 4096 keys
constexpr uint32_t FLAG_AGG = 1u << 30;
constexpr uint32_t FLAG_INC = 2u << 30;
constexpr uint32_t VALUE_MASK = (1u << 30) - 1;

__global__ void __launch_bounds__(BLOCK) hist_kernel(const uint64_t *__restrict__ keys, uint32_t n,
                                                     uint32_t *__restrict__ hist, DeviceStatus *st, bool check_keys) {
    __shared__ uint32_t sh[8][256];
    for (int i = threadIdx.x; i < 8 * 256; i += BLOCK)
        (&sh[0][0])[i] = 0;
    __syncthreads();
    uint32_t bad = 0;
    for (uint32_t i = blockIdx.x * BLOCK + threadIdx.x; i < n; i += gridDim.x * BLOCK) {
        uint64_t k = keys[i];
        bad |= (uint32_t)((k & COL_NONE) == COL_NONE);
#pragma unroll
        for (int p = 0; p < 8; ++p)
            atomicAdd(&sh[p][(k >> (8 * p)) & 255], 1u);
    }
    if (__syncthreads_or(bad) && check_keys && threadIdx.x == 0)
        atomicOr(&st->invalid_keys, 1u);
    for (int i = threadIdx.x; i < 8 * 256; i += BLOCK) {
        uint32_t c = (&sh[0][0])[i];
        if (c)
            atomicAdd(&hist[i], c);
    }
}

__global__ void __launch_bounds__(BLOCK) plan_kernel(const uint32_t *__restrict__ hist, uint32_t n,
                                                     uint32_t *__restrict__ base, SortPlan *plan) {
    __shared__ uint32_t tmp[BLOCK / 32 + 1];
    __shared__ uint32_t triv[8];
    int d = threadIdx.x;
    for (int p = 0; p < 8; ++p) {
        uint32_t c = hist[p * 256 + d];
        uint32_t total;
        uint32_t ex = block_excl_scan(c, &total, tmp);
        base[p * 256 + d] = ex;
        int t = __syncthreads_or(c == n);
        if (d == 0)
            triv[p] = (uint32_t)t;
    }
    __syncthreads();
    if (d == 0) {
        uint32_t sel = 0;
        for (int p = 0; p < 8; ++p) {
            plan->trivial[p] = triv[p];
            plan->in_sel[p] = sel;
            if (!triv[p])
                sel ^= 1u;
        }
        plan->final_sel = sel;
    }
}

__global__ void __launch_bounds__(BLOCK) onesweep_kernel(int pass, uint64_t *k0, uint8_t *v0, uint64_t *k1, uint8_t *v1,
                                                         uint32_t n, const uint32_t *__restrict__ base_all,
                                                         const SortPlan *plan, uint32_t *tile_counter,
                                                         uint32_t *status_all, DeviceStatus *st) {
    if (plan->trivial[pass])
        return;
    const uint32_t sel = plan->in_sel[pass];
    const uint64_t *in_k = sel ? k1 : k0;
    const uint8_t *in_v = sel ? v1 : v0;
    uint64_t *out_k = sel ? k0 : k1;
    uint8_t *out_v = sel ? v0 : v1;
    const int shift = 8 * pass;
    const uint32_t tiles = (n + SORT_TILE - 1) / SORT_TILE;
    uint32_t *status = status_all + (size_t)pass * tiles * 256;
    const uint32_t *base = base_all + pass * 256;

    __shared__ uint32_t s_tile;
    __shared__ uint32_t whist[BLOCK / 32][256];
    __shared__ uint32_t s_start[256];   // tile-local start of each digit
    __shared__ uint32_t s_global[256];  // global start of this tile's run of each digit
    __shared__ uint32_t tmp[BLOCK / 32 + 1];
    __shared__ uint64_t s_keys[SORT_TILE];
    __shared__ uint8_t s_vals[SORT_TILE];

    if (threadIdx.x == 0)
        s_tile = atomicAdd(&tile_counter[pass], 1u);
    for (int i = threadIdx.x; i < (BLOCK / 32) * 256; i += BLOCK)
        (&whist[0][0])[i] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t tile_lo = tile * SORT_TILE;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t warp_lo = tile_lo + warp * 32 * SORT_ITEMS;

    uint64_t k[SORT_ITEMS];
    uint8_t v[SORT_ITEMS];
    uint32_t rank[SORT_ITEMS];
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; ++j) {
        uint32_t idx = warp_lo + j * 32 + lane;
        bool ok = idx < n;
        k[j] = ok ? in_k[idx] : 0;
        v[j] = ok ? in_v[idx] : 0;
        uint32_t d = ok ? (uint32_t)((k[j] >> shift) & 255) : 256u + lane;
        uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        uint32_t prior = ok ? whist[warp][d] : 0;
        __syncwarp();
        if (ok) {
            rank[j] = prior + __popc(peers & lanemask_lt());
            if ((peers & lanemask_lt()) == 0)
                whist[warp][d] = prior + __popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();
    // Per digit: tile total and per-warp exclusive offsets (thread d owns digit d).
    const int d = threadIdx.x;
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < BLOCK / 32; ++w) {
        uint32_t c = whist[w][d];
        whist[w][d] = run;
        run += c;
    }
    const uint32_t local = run;
    uint32_t total;
    s_start[d] = block_excl_scan(local, &total, tmp);

    // Decoupled look-back for digit d.
    uint32_t prefix = 0;
    if (tile == 0) {
        atomicExch(&status[d], FLAG_INC | local);
    } else {
        atomicExch(&status[(size_t)tile * 256 + d], FLAG_AGG | local);
        int64_t t = (int64_t)tile - 1;
        uint64_t t0 = 0;
        unsigned ns = 32;
        while (t >= 0) {
            uint32_t w = ld_volatile(&status[(size_t)t * 256 + d]);
            uint32_t flag = w & ~VALUE_MASK;
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
            prefix += w & VALUE_MASK;
            if (flag == FLAG_INC)
                break;
            --t;
        }
        atomicExch(&status[(size_t)tile * 256 + d], FLAG_INC | (prefix + local));
    }
    s_global[d] = base[d] + prefix;
    __syncthreads();

    // Stage the tile in digit order, then write each digit run contiguously.
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; ++j) {
        uint32_t idx = warp_lo + j * 32 + lane;
        if (idx < n) {
            uint32_t dd = (uint32_t)((k[j] >> shift) & 255);
            uint32_t pos = s_start[dd] + whist[warp][dd] + rank[j];
            s_keys[pos] = k[j];
            s_vals[pos] = v[j];
        }
    }
    __syncthreads();
    const uint32_t tile_n = min((uint32_t)SORT_TILE, n - tile_lo);
    for (uint32_t i = threadIdx.x; i < tile_n; i += BLOCK) {
        uint64_t kk = s_keys[i];
        uint32_t dd = (uint32_t)((kk >> shift) & 255);
        uint32_t pos = s_global[dd] + (i - s_start[dd]);
        out_k[pos] = kk;
        out_v[pos] = s_vals[i];
    }
}

}  // namespace

// Sorts bkeys[0]/bvals[0] (n entries); the result lands in
// bkeys[plan.final_sel]. Also flags reserved-column keys in the status.
gpma_status sort_batch(gpma_graph *g, uint64_t n, cudaStream_t s, bool check_keys) {
    if (n == 0)
        return GPMA_OK;
    const uint32_t tiles = (uint32_t)((n + SORT_TILE - 1) / SORT_TILE);
    uint64_t need = 8ull * tiles * 256;
    if (need > g->sort_status_cap) {
        dev_free(g->sort_status);
        GPMA_TRY(dev_alloc(&g->sort_status, need));
        g->sort_status_cap = need;
    }
    GPMA_CUDA(cudaMemsetAsync(g->sort_hist, 0, 8 * 256 * sizeof(uint32_t), s));
    GPMA_CUDA(cudaMemsetAsync(g->sort_tiles, 0, 8 * sizeof(uint32_t), s));
    GPMA_CUDA(cudaMemsetAsync(g->sort_status, 0, need * sizeof(uint32_t), s));
    int hist_grid = (int)std::min<uint64_t>((n + BLOCK * 8 - 1) / (BLOCK * 8), (uint64_t)g->sms * 4);
    hist_kernel<<<hist_grid, BLOCK, 0, s>>>(g->bkeys[0], (uint32_t)n, g->sort_hist, g->status, check_keys);
    plan_kernel<<<1, BLOCK, 0, s>>>(g->sort_hist, (uint32_t)n, g->sort_base, g->sort_plan);
    for (int p = 0; p < 8; ++p)
        onesweep_kernel<<<tiles, BLOCK, 0, s>>>(p, g->bkeys[0], g->bvals[0], g->bkeys[1], g->bvals[1], (uint32_t)n,
                                                g->sort_base, g->sort_plan, g->sort_tiles, g->sort_status, g->status);
    GPMA_CUDA(cudaGetLastError());
    return GPMA_OK;
}

}  // namespace gpma
