// update.cu - GPMA+ batch update on one GB300, for one graph or many.
//
// Replaces update_gpma (gpma.cuh:968-1050). One persistent cooperative kernel
// runs every step of the update of one or more independent graphs, with
// bounded grid barriers instead of host round trips:
//   S  stable sort of each graph's batch (sort.cuh, gpma.cuh:977): a bucket
//      sort, or radix digit passes for a batch that crowds one bucket;
//   P1 locate: the reference's top-down search over segment first keys (its
//      upper levels from a shared-memory copy when one graph is updated), then
//      an equality scan of the leaf with 16-byte loads; hits store the
//      update's value in place (delete/modify/revive, gpma.cuh:188-220);
//   P2 keep the insertions in sorted order (compact_insertions, :836-844);
//   P3 group them by (graph, leaf) into level-0 windows
//      (group_insertion_by_node, :846-873). A window is (graph, node, [a, b))
//      into the current insertion buffer;
//   level loop (:1012-1029): each window of width W = seg << level counts its
//      live slots, is accepted iff lower <= live + pending <= upper (the
//      graph's thresholds), and an accepted window is rewritten as the stable
//      merge of its live entries and its insertions, redispatched evenly
//      (:636-654) in one coalesced pass. The insertions of rejected windows
//      are compacted into the other buffer (one scan over windows) and a
//      rejected right sibling joins its rejected left sibling in the parent.
//      Windows are ordered by graph and graphs by segment length, so the list
//      splits into one contiguous run per segment length and each run has one
//      window width: up to 256 slots per warp group, up to 2048 per CTA in
//      shared memory, wider ones chunk by chunk over the whole grid. For one
//      graph, a level of windows up to 2048 slots costs one grid barrier:
//      each CTA dispatches, counts and carries a contiguous range of the
//      windows and goes on with the next-level windows it wrote itself.
// The host reads the status blocks once. Only the root resize (:1034-1044)
// and the >= 5M-insertion rebuild (:936-966) run host-driven, per graph.
#include "gpma_internal.cuh"
#include "sort.cuh"

#include <algorithm>
#include <cmath>
#include <numeric>

namespace gpma {

uint32_t fls32(uint32_t x) {
    uint32_t r = 0;
    while (x) {
        ++r;
        x >>= 1;
    }
    return r;
}

void recalculate_density(Geometry &geo) {
    const uint32_t h = geo.height;
    geo.lower.assign(h + 1, 0);
    geo.upper.assign(h + 1, 0);
    uint32_t level_length = geo.seg;
    for (uint32_t i = 0; i <= h; i++) {
        // Same association as gpma.cuh:155-156: ((leaf - root) * (h - i)) / h.
        volatile double dl = LOWER_ROOT + (LOWER_LEAF - LOWER_ROOT) * (double)(h - i) / (double)h;
        volatile double du = UPPER_ROOT + (UPPER_LEAF - UPPER_ROOT) * (double)(h - i) / (double)h;
        volatile double pl = dl * (double)level_length;
        volatile double pu = du * (double)level_length;
        geo.lower[i] = (uint32_t)std::ceil((double)pl);
        geo.upper[i] = (uint32_t)std::floor((double)pu);
        if (i > 0) {
            geo.lower[i] = std::max(geo.lower[i], 2 * geo.lower[i - 1]);
            geo.upper[i] = std::min(geo.upper[i], 2 * geo.upper[i - 1]);
        }
        level_length <<= 1;
    }
}

namespace {

struct UpdateArgs {
    const GraphDesc *gd;
    GraphStatus *gs;
    uint32_t G;
    uint32_t max_height;
    uint32_t min_height;    // below it no graph has a root window
    const uint32_t *boff;   // batch offsets, G + 1
    const uint32_t *toff;   // sort tile offsets, G + 1
    uint32_t n;
    const uint64_t *in_k;   // the batch as submitted (bk[0] or the caller's device buffer; only read)
    const uint8_t *in_v;
    uint64_t *bk[2];        // batches, ping-pong buffers of the sort
    uint8_t *bv[2];
    uint32_t *sort_hist;    // [G + 1][8][256] digit counts (zeroed per update)
    uint32_t *sort_tiles;   // 8 tile counters (zeroed per update)
    uint32_t *sort_status;  // look-back words, 8 x tiles x 256 (zeroed per update)
    BucketSort q;           // bucket sort state (q.nq == 0: digit passes only)
    bool check_keys;
    uint32_t *leaf;
    uint64_t *ikeys[2];
    uint8_t *ivals[2];
    uint32_t *ileaf;
    uint32_t *igraph;
    uint64_t *rkeys;
    uint8_t *rvals;
    uint32_t *wnode[2];
    uint32_t *wgraph[2];
    uint32_t *wa[2];
    uint32_t *wb[2];
    uint32_t *wflag[2];  // window flags by level parity: a level may start before every CTA read the last
    uint32_t *wlive;
    uint32_t *chunk_cnt;
    uint32_t *cta_cnt;
    DeviceStatus *st;
    // clean-up for the next launch: the other status slot (as words) and the
    // sort state this launch used
    uint32_t *next_slot;
    uint32_t next_slot_words;
    uint32_t hist_words;
    uint32_t status_words;
    // test hooks: extra arrivals the first grid barrier waits for, and its limit
    uint32_t stall;
    uint64_t stall_limit_ns;
    uint64_t *top;  // one graph: its LOCATE_CACHE top-of-tree heads gathered contiguously
    const uint32_t *abort;  // non-zero: return at once (a recorded step after one needing host work)
};


// Current window list of a level.
struct Windows {
    const uint32_t *node, *graph, *a, *b;
    uint32_t *flag;  // per window: accepted (1) or rejected (0) at this level
};

__device__ __forceinline__ uint32_t graph_of(const UpdateArgs &A, uint32_t i) {
    return A.G == 1 ? 0u : segment_of(A.boff, A.G, i);
}

// ---- P1: locate ------------------------------------------------------------

// The top levels of the descent read segment first keys at multiples of
// `stride` slots; with one graph each CTA copies those (at most LOCATE_CACHE
// of them) into shared memory once, so a key walks the upper levels in shared
// memory and only the last log2(stride/seg) levels in HBM. The comparisons and
// their order are the reference's bit-by-bit descent (gpma.cuh:209-216).
constexpr uint32_t LOCATE_CACHE = 4096;

// The leaf's first slot equal to `key` (handle_del_mod scans all seg slots),
// or SIZE_NONE. All seg/2 16-byte loads are issued before any comparison.
__device__ __forceinline__ uint32_t leaf_find(const GraphDesc &D, uint32_t leaf, uint64_t key) {
    const ulonglong2 *p = reinterpret_cast<const ulonglong2 *>(D.keys + leaf);
    const uint32_t halves = D.seg >> 1;  // 1..16
    ulonglong2 q[16];
#pragma unroll
    for (uint32_t j = 0; j < 16; ++j)
        if (j < halves)
            q[j] = p[j];
    uint32_t hit = SIZE_NONE;
#pragma unroll
    for (int j = 15; j >= 0; --j) {
        if ((uint32_t)j < halves) {
            if (q[j].y == key)
                hit = 2 * j + 1;
            if (q[j].x == key)
                hit = 2 * j;
        }
    }
    return hit;
}

// Locates LOC_ILP updates per thread together: at each level of the descent
// every key's probe is issued before any comparison, so a thread keeps
// LOC_ILP dependent chains in flight instead of one.
constexpr int LOC_ILP = 4;
// Consecutive items per thread in the grouping passes.
constexpr uint32_t GROUP_ITEMS = 4;

// Keys i0 + j * stride (j < LOC_ILP) below `end`; returns how many of them
// are insertions (leaf set).
template <bool SCANS_FIRST>
__device__ __forceinline__ uint32_t locate_keys(const UpdateArgs &A, const uint64_t *bk, const uint8_t *bv,
                                                uint32_t i0, uint32_t stride, uint32_t end, const uint64_t *fk,
                                                uint32_t log2stride) {
    uint32_t idx[LOC_ILP], prefix[LOC_ILP], bit[LOC_ILP], g[LOC_ILP];
    uint64_t key[LOC_ILP];
#pragma unroll
    for (int j = 0; j < LOC_ILP; ++j) {
        idx[j] = i0 + j * stride;
        prefix[j] = 0;
        bit[j] = 0;
        g[j] = 0;
        key[j] = 0;
        if (idx[j] < end) {
            g[j] = graph_of(A, idx[j]);
            const GraphDesc &D = A.gd[g[j]];
            key[j] = bk[idx[j]];
            bit[j] = (D.seg << D.height) >> 1;
            if (fk) {  // one graph: the top levels from shared memory
                const uint32_t sstride = 1u << log2stride;
                while (sstride <= bit[j]) {
                    if (fk[(prefix[j] | bit[j]) >> log2stride] <= key[j])
                        prefix[j] |= bit[j];
                    bit[j] >>= 1;
                }
            }
        }
    }
    // the remaining levels of the reference's descent (gpma.cuh:209-216),
    // interleaved. Every probed slot starts a segment (prefix and bit are
    // multiples of seg), so its key is read from the dense heads array.
    for (;;) {
        uint64_t probe[LOC_ILP];
        bool any = false;
#pragma unroll
        for (int j = 0; j < LOC_ILP; ++j) {
            const GraphDesc &D = A.gd[g[j]];
            const bool live = idx[j] < end && D.seg <= bit[j];
            probe[j] = live ? D.heads[(prefix[j] | bit[j]) >> D.log2seg] : 0;
            any |= live;
        }
        if (!any)
            break;
#pragma unroll
        for (int j = 0; j < LOC_ILP; ++j) {
            if (idx[j] < end && A.gd[g[j]].seg <= bit[j]) {
                if (probe[j] <= key[j])
                    prefix[j] |= bit[j];
                bit[j] >>= 1;
            }
        }
    }
    uint32_t inserts = 0;
    if constexpr (SCANS_FIRST) {
        // every leaf scan before any store: a value store (a byte) may alias
        // the next scan's loads, which would otherwise wait for it (one graph:
        // measured 30 -> 25 us on the social step; the many-graph build, with
        // fewer registers, keeps the interleaved order)
        uint32_t hit[LOC_ILP];
        uint8_t value[LOC_ILP];
#pragma unroll
        for (int j = 0; j < LOC_ILP; ++j) {
            hit[j] = SIZE_NONE;
            value[j] = 0;
            if (idx[j] >= end)
                continue;
            const GraphDesc &D = A.gd[g[j]];
            value[j] = bv[idx[j]];
            if (!in_bounds(&A.st->err, (uint64_t)prefix[j] + D.seg <= D.size, BS_LEAF)) {
                prefix[j] = SIZE_NONE;  // the key is skipped
                continue;
            }
            hit[j] = leaf_find(D, prefix[j], key[j]);
        }
#pragma unroll
        for (int j = 0; j < LOC_ILP; ++j) {
            if (idx[j] >= end)
                continue;
            uint32_t leaf = value[j] == 0 || prefix[j] == SIZE_NONE ? SIZE_NONE : prefix[j];
            if (hit[j] != SIZE_NONE) {
                A.gd[g[j]].vals[prefix[j] + hit[j]] = value[j];  // delete / modify / revive in place
                leaf = SIZE_NONE;
            }
            A.leaf[idx[j]] = leaf;
            inserts += leaf != SIZE_NONE;
        }
    } else {
#pragma unroll
        for (int j = 0; j < LOC_ILP; ++j) {
            if (idx[j] >= end)
                continue;
            const GraphDesc &D = A.gd[g[j]];
            const uint8_t value = bv[idx[j]];
            uint32_t leaf = value == 0 ? SIZE_NONE : prefix[j];
            if (!in_bounds(&A.st->err, (uint64_t)prefix[j] + D.seg <= D.size, BS_LEAF)) {
                A.leaf[idx[j]] = SIZE_NONE;
                continue;
            }
            const uint32_t hit = leaf_find(D, prefix[j], key[j]);
            if (hit != SIZE_NONE) {
                D.vals[prefix[j] + hit] = value;  // delete / modify / revive in place
                leaf = SIZE_NONE;
            }
            A.leaf[idx[j]] = leaf;
            inserts += leaf != SIZE_NONE;
        }
    }
    return inserts;
}

// ---- grid-wide exclusive scan helpers ------------------------------------
// CTA b owns items [lo, hi) of a contiguous split of [0, N).
__device__ __forceinline__ void cta_range(uint32_t N, uint32_t &lo, uint32_t &hi) {
    uint32_t per = (N + gridDim.x - 1) / gridDim.x;
    lo = min(N, blockIdx.x * per);
    hi = min(N, lo + per);
}

// Four sums over the CTA in one shared-memory round (every thread gets them).
__device__ __forceinline__ uint4 block_sum4(uint4 x) {
    __shared__ uint4 s_red[BLOCK / 32];
    x.x = __reduce_add_sync(0xFFFFFFFFu, x.x);
    x.y = __reduce_add_sync(0xFFFFFFFFu, x.y);
    x.z = __reduce_add_sync(0xFFFFFFFFu, x.z);
    x.w = __reduce_add_sync(0xFFFFFFFFu, x.w);
    __syncthreads();  // readers of the previous sums are done
    if ((threadIdx.x & 31) == 0)
        s_red[threadIdx.x >> 5] = x;
    __syncthreads();
    uint4 r = make_uint4(0, 0, 0, 0);
#pragma unroll
    for (int w = 0; w < BLOCK / 32; ++w) {
        const uint4 q = s_red[w];
        r.x += q.x;
        r.y += q.y;
        r.z += q.z;
        r.w += q.w;
    }
    return r;
}

// Four exclusive scans over the CTA in one shared-memory round (every thread
// gets its four prefixes and the four totals).
__device__ __forceinline__ uint4 block_excl_scan4(uint4 x, uint4 &total) {
    __shared__ uint4 s_scan[BLOCK / 32 + 1];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint4 inc = make_uint4(warp_incl_scan(x.x), warp_incl_scan(x.y), warp_incl_scan(x.z), warp_incl_scan(x.w));
    if (lane == 31)
        s_scan[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const uint4 v = lane < BLOCK / 32 ? s_scan[lane] : make_uint4(0, 0, 0, 0);
        const uint4 vi =
            make_uint4(warp_incl_scan(v.x), warp_incl_scan(v.y), warp_incl_scan(v.z), warp_incl_scan(v.w));
        if (lane < BLOCK / 32)
            s_scan[lane] = make_uint4(vi.x - v.x, vi.y - v.y, vi.z - v.z, vi.w - v.w);
        if (lane == BLOCK / 32 - 1)
            s_scan[BLOCK / 32] = vi;
    }
    __syncthreads();
    const uint4 pre = s_scan[warp];
    total = s_scan[BLOCK / 32];
    __syncthreads();  // the next call may overwrite s_scan
    return make_uint4(pre.x + inc.x - x.x, pre.y + inc.y - x.y, pre.z + inc.z - x.z, pre.w + inc.w - x.w);
}

// Sum of ca[0..blockIdx.x) and of ca[0..gridDim.x), and the same of cb (or
// zeros without cb): per-CTA counts written before the last grid barrier. A
// thread's loads are all issued before the first is used.
__device__ __forceinline__ void cta_prefix2(const uint32_t *ca, const uint32_t *cb, uint32_t &base_a,
                                            uint32_t &total_a, uint32_t &base_b, uint32_t &total_b) {
    uint4 s = make_uint4(0, 0, 0, 0);
    for (uint32_t j0 = 0; j0 < gridDim.x; j0 += 4 * BLOCK) {
        uint32_t va[4], vb[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t j = j0 + u * BLOCK + threadIdx.x;
            va[u] = j < gridDim.x ? __ldcg(ca + j) : 0u;
            vb[u] = cb && j < gridDim.x ? __ldcg(cb + j) : 0u;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const bool before = j0 + u * BLOCK + threadIdx.x < blockIdx.x;
            s.x += before ? va[u] : 0u;
            s.y += va[u];
            s.z += before ? vb[u] : 0u;
            s.w += vb[u];
        }
    }
    s = block_sum4(s);
    base_a = s.x;
    total_a = s.y;
    base_b = s.z;
    total_b = s.w;
}

// ---- redispatch of a chunk of a window ------------------------------------
// Writes slots [t0, t0+len) of the window at `node` (width F << log2seg): slot
// (s, lane) gets element first(s)+lane of the stable merge of live[0..L) and
// pend[0..P) (ties: live first), or gap_key/0 if the segment holds fewer.
// len is a multiple of the segment length; mk/mv hold len entries.
__device__ void redispatch_chunk(uint64_t *keys, uint8_t *vals, uint64_t *heads, uint32_t *row_offset,
                                 uint32_t row_num, uint32_t node, uint32_t log2seg, uint32_t log2F, uint32_t t0, uint32_t len, const uint64_t *lk,
                                 const uint8_t *lv, uint32_t L, const uint64_t *pk, const uint8_t *pv, uint32_t P,
                                 uint64_t gap_key, uint64_t *mk, uint8_t *mv) {
    const uint64_t M = (uint64_t)L + P;
    const uint32_t seg = 1u << log2seg;
    const uint32_t i_lo = (uint32_t)seg_first(t0 >> log2seg, M, log2F);
    const uint64_t f_end = seg_first((t0 + len) >> log2seg, M, log2F);
    const uint32_t i_hi = (uint32_t)(f_end < M ? f_end : M);
    const uint32_t cnt = i_hi - i_lo;
    const uint32_t ipt = (cnt + BLOCK - 1) / BLOCK;
    uint32_t d = i_lo + threadIdx.x * ipt;
    if (d < i_hi) {
        // merge-path split: x live elements among the first d merged
        uint32_t lo = d > P ? d - P : 0, hi = min(d, L);
        while (lo < hi) {
            uint32_t mid = (lo + hi) >> 1;
            if (pk[d - mid - 1] < lk[mid])
                hi = mid;
            else
                lo = mid + 1;
        }
        uint32_t x = lo, y = d - lo;
        uint32_t end = min(i_hi, d + ipt);
        for (uint32_t e = d; e < end; ++e) {
            bool take_live = x < L && (y >= P || lk[x] <= pk[y]);
            if (take_live) {
                mk[e - i_lo] = lk[x];
                mv[e - i_lo] = lv[x];
                ++x;
            } else {
                mk[e - i_lo] = pk[y];
                mv[e - i_lo] = pv[y];
                ++y;
            }
        }
    }
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < len; t += BLOCK) {
        uint32_t slot = t0 + t;
        uint32_t s = slot >> log2seg, ln = slot & (seg - 1);
        uint64_t f0 = seg_first(s, M, log2F), f1 = seg_first(s + 1, M, log2F);
        uint64_t k = gap_key;
        uint8_t v = 0;
        if (ln < f1 - f0) {
            k = mk[f0 + ln - i_lo];
            v = mv[f0 + ln - i_lo];
        }
        keys[node + slot] = k;
        vals[node + slot] = v;
        if (ln == 0)
            heads[(node + slot) >> log2seg] = k;
        if (is_guard(k)) {
            uint32_t row = (uint32_t)(k >> 32);
            if (row < row_num)
                row_offset[row + 1] = node + slot;
        }
    }
    __syncthreads();
}

// ---- windows up to WARP_WINDOW_MAX slots: a group of lanes per window -------
// K contiguous slots per lane (4, or 8 at 256 slots), loaded and stored with
// 16-byte key and 4/8-byte value vectors; a W-slot window takes W/K lanes, so
// a warp holds 32K/W windows at once.

template <uint32_t K>
__device__ __forceinline__ void load_slots(const uint64_t *keys, const uint8_t *vals, uint32_t t0, uint64_t (&k)[K],
                                           uint8_t (&v)[K]) {
    if constexpr (K >= 2) {
#pragma unroll
        for (uint32_t j = 0; j < K; j += 2) {
            const ulonglong2 q = *reinterpret_cast<const ulonglong2 *>(keys + t0 + j);
            k[j] = q.x;
            k[j + 1] = q.y;
        }
    } else {
        k[0] = keys[t0];
    }
    if constexpr (K == 8) {
        const uint2 q = *reinterpret_cast<const uint2 *>(vals + t0);
#pragma unroll
        for (uint32_t j = 0; j < 4; ++j) {
            v[j] = (uint8_t)(q.x >> (8 * j));
            v[4 + j] = (uint8_t)(q.y >> (8 * j));
        }
    } else if constexpr (K == 4) {
        const uint32_t q = *reinterpret_cast<const uint32_t *>(vals + t0);
#pragma unroll
        for (uint32_t j = 0; j < 4; ++j)
            v[j] = (uint8_t)(q >> (8 * j));
    } else if constexpr (K == 2) {
        const uint16_t q = *reinterpret_cast<const uint16_t *>(vals + t0);
        v[0] = (uint8_t)q;
        v[1] = (uint8_t)(q >> 8);
    } else {
        v[0] = vals[t0];
    }
}

template <uint32_t K>
__device__ __forceinline__ void store_slots(uint64_t *keys, uint8_t *vals, uint32_t t0, const uint64_t (&k)[K],
                                            const uint8_t (&v)[K]) {
    if constexpr (K >= 2) {
#pragma unroll
        for (uint32_t j = 0; j < K; j += 2)
            *reinterpret_cast<ulonglong2 *>(keys + t0 + j) = make_ulonglong2(k[j], k[j + 1]);
    } else {
        keys[t0] = k[0];
    }
    if constexpr (K == 8) {
        uint2 q = make_uint2(0, 0);
#pragma unroll
        for (uint32_t j = 0; j < 4; ++j) {
            q.x |= (uint32_t)v[j] << (8 * j);
            q.y |= (uint32_t)v[4 + j] << (8 * j);
        }
        *reinterpret_cast<uint2 *>(vals + t0) = q;
    } else if constexpr (K == 4) {
        uint32_t q = 0;
#pragma unroll
        for (uint32_t j = 0; j < 4; ++j)
            q |= (uint32_t)v[j] << (8 * j);
        *reinterpret_cast<uint32_t *>(vals + t0) = q;
    } else if constexpr (K == 2) {
        *reinterpret_cast<uint16_t *>(vals + t0) = (uint16_t)(v[0] | ((uint32_t)v[1] << 8));
    } else {
        vals[t0] = v[0];
    }
}

template <uint32_t W>
__device__ void warp_windows(const UpdateArgs &A, Windows L, uint32_t r0, uint32_t r1, uint32_t level,
                             const uint64_t *pk, const uint8_t *pv, unsigned char *smem, unsigned long long &acc,
                             uint32_t part, uint32_t parts) {
    constexpr uint32_t G = W >= 128 ? 32 : (W >= 4 ? W / 4 : 1);  // lanes per window
    constexpr uint32_t GPW = 32 / G;                                // windows per warp
    constexpr uint32_t K = W / G;                                   // slots per lane
    constexpr uint32_t STRIDE = (27 * W + 15) & ~15u;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t gl = lane % G, grp = lane / G;
    unsigned char *base = smem + (warp * GPW + grp) * STRIDE;
    uint64_t *pend_k = reinterpret_cast<uint64_t *>(base);  // the window's pending insertions
    uint64_t *ck = pend_k + W;                               // its live entries, compacted
    uint64_t *mk = ck + W;                                   // the merge
    uint8_t *pend_v = reinterpret_cast<uint8_t *>(mk + W);
    uint8_t *cv = pend_v + W;
    uint8_t *mv = cv + W;
    // windows [r0, r1) over `parts` CTAs, this one being `part`
    const uint32_t total_warps = parts * (BLOCK / 32);
    const uint32_t g_r0 = L.graph[r0];  // stands in for groups without a window
    // the next round's window descriptor is read while this round works
    uint32_t wbase = r0 + (part * (BLOCK / 32) + warp) * GPW;
    uint32_t n_g = g_r0, n_node = 0, n_a = 0, n_b = 0;
    if (wbase + grp < r1) {
        n_g = L.graph[wbase + grp];
        n_node = L.node[wbase + grp];
        n_a = L.a[wbase + grp];
        n_b = L.b[wbase + grp];
    }
    for (; wbase < r1; wbase += total_warps * GPW) {
        const uint32_t w = wbase + grp;
        const GraphDesc &D = A.gd[n_g];
        const uint32_t node = n_node, a = n_a, b = n_b;
        const bool has =
            w < r1 && in_bounds(&A.st->err, (uint64_t)node + W <= D.size && a <= b && b <= A.n, BS_WINDOW);
        const uint32_t log2seg = D.log2seg, seg_mask = D.seg - 1;
        const uint32_t log2F = (31 - __clz(W)) - log2seg;
        const uint32_t lo = D.lower[level], hi = D.upper[level];
        const uint32_t t0 = node + gl * K;
        uint64_t k[K];
        uint8_t v[K];
        uint32_t c_l = 0;
        // the window's first pending insertions, loaded beside its slots
        uint64_t pk0 = 0;
        uint8_t pv0 = 0;
        if (has) {
            load_slots<K>(D.keys, D.vals, t0, k, v);
            if (gl < b - a) {
                pk0 = pk[a + gl];
                pv0 = pv[a + gl];
            }
        }
        {
            const uint32_t wn = w + total_warps * GPW;
            n_g = g_r0;
            n_node = n_a = n_b = 0;
            if (wn < r1) {
                n_g = L.graph[wn];
                n_node = L.node[wn];
                n_a = L.a[wn];
                n_b = L.b[wn];
            }
        }
        if (has) {
#pragma unroll
            for (uint32_t j = 0; j < K; ++j)
                c_l += (k[j] != KEY_NONE && v[j] != 0);
        }
        const uint32_t inc = warp_incl_scan(c_l, G);
        const uint32_t c = __shfl_sync(0xFFFFFFFFu, inc, grp * G + G - 1);
        const uint32_t p = b - a;
        const uint32_t M = c + p;
        const bool accept = has && lo <= M && M <= hi;
        if (accept) {
            uint32_t o = inc - c_l;
#pragma unroll
            for (uint32_t j = 0; j < K; ++j) {
                if (k[j] != KEY_NONE && v[j] != 0) {
                    ck[o] = k[j];
                    cv[o] = v[j];
                    ++o;
                }
            }
            if (gl < p) {
                pend_k[gl] = pk0;
                pend_v[gl] = pv0;
            }
            for (uint32_t j = gl + G; j < p; j += G) {
                pend_k[j] = pk[a + j];
                pend_v[j] = pv[a + j];
            }
        }
        __syncwarp();
        if (accept) {
            for (uint32_t r = gl; r < c; r += G) {
                uint32_t pos = r + lower_bound_u64(pend_k, p, ck[r]);
                mk[pos] = ck[r];
                mv[pos] = cv[r];
            }
            for (uint32_t j = gl; j < p; j += G) {
                uint32_t pos = j + upper_bound_u64(ck, c, pend_k[j]);
                mk[pos] = pend_k[j];
                mv[pos] = pend_v[j];
            }
        }
        __syncwarp();
        if (accept) {
#pragma unroll
            for (uint32_t j = 0; j < K; ++j) {
                const uint32_t t = gl * K + j;
                const uint32_t s = t >> log2seg, ln = t & seg_mask;
                const uint32_t f0 = (uint32_t)seg_first(s, M, log2F), f1 = (uint32_t)seg_first(s + 1, M, log2F);
                k[j] = KEY_NONE;
                v[j] = 0;
                if (ln < f1 - f0) {
                    k[j] = mk[f0 + ln];
                    v[j] = mv[f0 + ln];
                }
                if (ln == 0)
                    D.heads[(node >> log2seg) + s] = k[j];
                if (is_guard(k[j])) {
                    const uint32_t row = (uint32_t)(k[j] >> 32);
                    if (row < D.row_num)
                        D.row_offset[row + 1] = node + t;
                }
            }
            store_slots<K>(D.keys, D.vals, t0, k, v);
            if (gl == 0)
                ++acc;
        }
        if (has && gl == 0)
            L.flag[w] = accept ? 1u : 0u;
        __syncwarp();
    }
}

// ---- windows of 512..CTA_WINDOW_MAX slots: one CTA each ---------------------
template <uint32_t W>
__device__ void cta_windows(const UpdateArgs &A, Windows L, uint32_t r0, uint32_t r1, uint32_t level,
                            const uint64_t *pk, const uint8_t *pv, unsigned char *smem, uint32_t *tmp,
                            unsigned long long &acc, uint32_t part, uint32_t parts) {
    constexpr uint32_t K = W / BLOCK;
    uint64_t *sk = reinterpret_cast<uint64_t *>(smem);
    uint64_t *ck = sk + W;
    uint64_t *mk = ck + W;
    uint8_t *sv = reinterpret_cast<uint8_t *>(mk + W);
    uint8_t *cv = sv + W;
    uint8_t *mv = cv + W;
    const uint32_t tid = threadIdx.x;
    for (uint32_t w = r0 + part; w < r1; w += parts) {
        const GraphDesc &D = A.gd[L.graph[w]];
        const uint32_t node = L.node[w], a = L.a[w], b = L.b[w];
        // the same condition in every thread: the whole CTA skips the window
        if (!in_bounds(&A.st->err, (uint64_t)node + W <= D.size && a <= b && b <= A.n, BS_WINDOW))
            continue;
        const uint32_t log2seg = D.log2seg, seg_mask = D.seg - 1;
        const uint32_t log2F = (31 - __clz(W)) - log2seg;
        const uint32_t lo = D.lower[level], hi = D.upper[level];
#pragma unroll
        for (uint32_t j = 0; j < K; ++j) {
            uint32_t t = tid + j * BLOCK;
            sk[t] = D.keys[node + t];
            sv[t] = D.vals[node + t];
        }
        __syncthreads();
        uint32_t c_l = 0;
#pragma unroll
        for (uint32_t j = 0; j < K; ++j) {
            uint32_t t = tid * K + j;
            c_l += (sk[t] != KEY_NONE && sv[t] != 0);
        }
        uint32_t c;
        const uint32_t ex = block_excl_scan(c_l, &c, tmp);
        const uint32_t p = b - a;
        const uint32_t M = c + p;
        const bool accept = lo <= M && M <= hi;
        if (accept) {
            uint32_t o = ex;
#pragma unroll
            for (uint32_t j = 0; j < K; ++j) {
                uint32_t t = tid * K + j;
                if (sk[t] != KEY_NONE && sv[t] != 0) {
                    ck[o] = sk[t];
                    cv[o] = sv[t];
                    ++o;
                }
            }
        }
        __syncthreads();
        if (accept) {
            for (uint32_t j = tid; j < p; j += BLOCK) {
                sk[j] = pk[a + j];
                sv[j] = pv[a + j];
            }
        }
        __syncthreads();
        if (accept) {
            for (uint32_t r = tid; r < c; r += BLOCK) {
                uint32_t pos = r + lower_bound_u64(sk, p, ck[r]);
                mk[pos] = ck[r];
                mv[pos] = cv[r];
            }
            for (uint32_t j = tid; j < p; j += BLOCK) {
                uint32_t pos = j + upper_bound_u64(ck, c, sk[j]);
                mk[pos] = sk[j];
                mv[pos] = sv[j];
            }
        }
        __syncthreads();
        if (accept) {
#pragma unroll
            for (uint32_t j = 0; j < K; ++j) {
                uint32_t t = tid + j * BLOCK;
                uint32_t s = t >> log2seg, ln = t & seg_mask;
                uint32_t f0 = (uint32_t)seg_first(s, M, log2F), f1 = (uint32_t)seg_first(s + 1, M, log2F);
                uint64_t k = KEY_NONE;
                uint8_t v = 0;
                if (ln < f1 - f0) {
                    k = mk[f0 + ln];
                    v = mv[f0 + ln];
                }
                D.keys[node + t] = k;
                D.vals[node + t] = v;
                if (ln == 0)
                    D.heads[(node + t) >> log2seg] = k;
                if (is_guard(k)) {
                    uint32_t row = (uint32_t)(k >> 32);
                    if (row < D.row_num)
                        D.row_offset[row + 1] = node + t;
                }
            }
            if (tid == 0)
                ++acc;
        }
        if (tid == 0)
            L.flag[w] = accept ? 1u : 0u;
        __syncthreads();
    }
}

// ---- windows wider than one CTA: the whole grid, chunk by chunk -------------
__device__ bool grid_windows(const UpdateArgs &A, Windows L, uint32_t r0, uint32_t r1, uint32_t W, uint32_t level,
                             const uint64_t *pk, const uint8_t *pv, unsigned char *smem, uint32_t *tmp,
                             unsigned long long &acc) {
    const uint32_t cpw = W / CHUNK;
    const uint32_t total = (r1 - r0) * cpw;
    constexpr uint32_t K = CHUNK / BLOCK;
    // B1: live count of every chunk
    for (uint32_t c = blockIdx.x; c < total; c += gridDim.x) {
        const uint32_t w = r0 + c / cpw, k = c % cpw;
        const GraphDesc &D = A.gd[L.graph[w]];
        // a failed check stops the launch at the barrier after this pass,
        // before B3/B4 touch the window
        if (!in_bounds(&A.st->err, (uint64_t)L.node[w] + W <= D.size, BS_CHUNK))
            continue;
        const uint32_t base = L.node[w] + k * CHUNK + threadIdx.x * K;
        uint32_t cl = 0;
#pragma unroll
        for (uint32_t j = 0; j < K; ++j)
            cl += (D.keys[base + j] != KEY_NONE && D.vals[base + j] != 0);
        uint32_t t = block_sum(cl, tmp);
        if (threadIdx.x == 0)
            A.chunk_cnt[c] = t;
    }
    if (!grid_barrier(&A.st->bar, &A.st->err))
        return false;
    // B2: per window, chunk offsets, live total and the density decision
    for (uint32_t w = r0 + blockIdx.x; w < r1; w += gridDim.x) {
        const GraphDesc &D = A.gd[L.graph[w]];
        uint32_t *cc = A.chunk_cnt + (w - r0) * cpw;
        uint32_t run = 0;
        for (uint32_t k0 = 0; k0 < cpw; k0 += BLOCK) {
            uint32_t k = k0 + threadIdx.x;
            uint32_t v = k < cpw ? cc[k] : 0;
            uint32_t tot;
            uint32_t ex = block_excl_scan(v, &tot, tmp);
            if (k < cpw)
                cc[k] = run + ex;
            run += tot;
        }
        uint32_t M = run + (L.b[w] - L.a[w]);
        bool accept = D.lower[level] <= M && M <= D.upper[level];
        if (!in_bounds(&A.st->err, L.a[w] <= L.b[w] && L.b[w] <= A.n, BS_PENDING))
            accept = false;
        if (threadIdx.x == 0) {
            L.flag[w] = accept ? 1u : 0u;
            A.wlive[w] = run;
            if (accept)
                ++acc;
        }
    }
    if (!grid_barrier(&A.st->bar, &A.st->err))
        return false;
    // B3: stable compaction of accepted windows into the graph's scratch arrays
    for (uint32_t c = blockIdx.x; c < total; c += gridDim.x) {
        const uint32_t w = r0 + c / cpw, k = c % cpw;
        if (!L.flag[w])
            continue;
        const GraphDesc &D = A.gd[L.graph[w]];
        const uint32_t node = L.node[w];
        const uint32_t base = node + k * CHUNK + threadIdx.x * K;
        uint64_t kk[K];
        uint8_t vv[K];
        uint32_t cl = 0;
#pragma unroll
        for (uint32_t j = 0; j < K; ++j) {
            kk[j] = D.keys[base + j];
            vv[j] = D.vals[base + j];
            cl += (kk[j] != KEY_NONE && vv[j] != 0);
        }
        uint32_t tot;
        uint32_t o = node + A.chunk_cnt[c] + block_excl_scan(cl, &tot, tmp);
#pragma unroll
        for (uint32_t j = 0; j < K; ++j) {
            if (kk[j] != KEY_NONE && vv[j] != 0) {
                D.skeys[o] = kk[j];
                D.svals[o] = vv[j];
                ++o;
            }
        }
    }
    if (!grid_barrier(&A.st->bar, &A.st->err))
        return false;
    // B4: merge with the window's insertions and redispatch chunk by chunk
    uint64_t *mk = reinterpret_cast<uint64_t *>(smem);
    uint8_t *mv = reinterpret_cast<uint8_t *>(mk + CHUNK);
    for (uint32_t c = blockIdx.x; c < total; c += gridDim.x) {
        const uint32_t w = r0 + c / cpw, k = c % cpw;
        if (!L.flag[w])
            continue;
        const GraphDesc &D = A.gd[L.graph[w]];
        const uint32_t node = L.node[w], a = L.a[w];
        const uint32_t log2F = (31 - __clz(W)) - D.log2seg;
        redispatch_chunk(D.keys, D.vals, D.heads, D.row_offset, D.row_num, node, D.log2seg, log2F, k * CHUNK, CHUNK,
                         D.skeys + node, D.svals + node, A.wlive[w], pk + a, pv + a, L.b[w] - a, KEY_NONE, mk, mv);
    }
    return true;
}

template <uint32_t W>
__device__ __forceinline__ void small_dispatch(const UpdateArgs &A, Windows L, uint32_t r0, uint32_t r1,
                                               uint32_t level, const uint64_t *pk, const uint8_t *pv,
                                               unsigned char *smem, uint32_t *tmp, unsigned long long &acc,
                                               uint32_t part, uint32_t parts) {
    if constexpr (W <= WARP_WINDOW_MAX)
        warp_windows<W>(A, L, r0, r1, level, pk, pv, smem, acc, part, parts);
    else
        cta_windows<W>(A, L, r0, r1, level, pk, pv, smem, tmp, acc, part, parts);
}

// First window in [0, nw) whose graph has segment length >= s (windows are
// ordered by graph, graphs by segment length).
__device__ __forceinline__ uint32_t first_window_of_seg(const UpdateArgs &A, const uint32_t *wg, uint32_t nw,
                                                        uint32_t s) {
    uint32_t lo = 0, hi = nw;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (A.gd[wg[mid]].seg < s)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// Rejected windows of [lo, hi) that start a window of the next level (a
// rejected right sibling joins its rejected left sibling) into cnt_h, and
// their insertions into cnt_i, at blockIdx.x; root windows count in neither.
// first_is_head: window lo counts as a start whatever its left neighbour
// (whose flag may not be written yet); level_prefix removes those that
// are not.
__device__ __forceinline__ void count_rejected(const UpdateArgs &A, const Windows &L, uint32_t level, uint32_t lo,
                                               uint32_t hi, bool first_is_head, uint32_t *cnt_h, uint32_t *cnt_i) {
    uint32_t ch = 0, ci = 0;
    constexpr int CU = 2;  // windows per thread per step, their fields loaded together
    for (uint32_t w0 = lo + threadIdx.x; w0 < hi; w0 += CU * BLOCK) {
        uint32_t f0[CU], fl[CU], g[CU], gl[CU], nd[CU], ndl[CU], wa[CU], wb[CU];
#pragma unroll
        for (int u = 0; u < CU; ++u) {
            // the window's and its left neighbour's fields
            const uint32_t w = w0 + u * BLOCK;
            const bool ok = w < hi;
            const bool left = ok && w > 0 && !(first_is_head && w == lo);
            f0[u] = ok ? L.flag[w] : 1u;
            fl[u] = left ? L.flag[w - 1] : 1u;
            g[u] = ok ? L.graph[w] : 0u;
            gl[u] = left ? L.graph[w - 1] : 0u;
            nd[u] = ok ? L.node[w] : 0u;
            ndl[u] = left ? L.node[w - 1] : 0u;
            wa[u] = ok ? L.a[w] : 0u;
            wb[u] = ok ? L.b[w] : 0u;
        }
#pragma unroll
        for (int u = 0; u < CU; ++u) {
            if (f0[u])
                continue;  // accepted (or past the range)
            const GraphDesc &Dg = A.gd[g[u]];
            if (level >= Dg.height)
                continue;  // root window: to the remaining buffer
            const uint32_t W = Dg.seg << level;
            ci += wb[u] - wa[u];
            const uint32_t par = nd[u] & ~W;
            const bool merged = !fl[u] && gl[u] == g[u] && (ndl[u] & ~W) == par;  // fl = 1 without a left neighbour
            ch += merged ? 0u : 1u;
        }
    }
    const uint4 t = block_sum4(make_uint4(ch, ci, 0, 0));
    if (threadIdx.x == 0) {
        cnt_h[blockIdx.x] = t.x;
        cnt_i[blockIdx.x] = t.y;
    }
}

// The level's prefix sums over the per-CTA counts of count_rejected (written
// before the last grid barrier): this CTA's first next-level window (base_h)
// and insertion (base_i), and the totals. fused: one graph, counts taken with
// first_is_head; a CTA c >= 1 whose first window was counted as a start but
// joins its left neighbour (both rejected, one parent, not root windows) has
// that start taken off here, its fields read in the same round as the counts.
// slices: each CTA's range as (lo, hi) pairs, or null for cta_range's.
__device__ __forceinline__ void level_prefix(const UpdateArgs &A, const Windows &L, uint32_t nw, uint32_t level,
                                             bool fused, const uint32_t *slices, const uint32_t *cnt_h,
                                             const uint32_t *cnt_i, uint32_t &base_h, uint32_t &total_h,
                                             uint32_t &base_i, uint32_t &total_i) {
    const uint32_t per = (nw + gridDim.x - 1) / gridDim.x;
    const GraphDesc &D = A.gd[0];
    const uint32_t W = D.seg << level;
    const bool starts = fused && level < D.height;  // else no correction
    constexpr int CU = 2;  // CTAs per thread per step
    uint4 s = make_uint4(0, 0, 0, 0);
    for (uint32_t j0 = 0; j0 < gridDim.x; j0 += CU * BLOCK) {
        uint32_t vh[CU], vi[CU], w[CU], w_end[CU];
#pragma unroll
        for (int u = 0; u < CU; ++u) {
            const uint32_t c = j0 + u * BLOCK + threadIdx.x;
            const bool in = c < gridDim.x;
            vh[u] = in ? __ldcg(cnt_h + c) : 0u;
            vi[u] = in ? __ldcg(cnt_i + c) : 0u;
            w[u] = 0;
            w_end[u] = 0;
            if (starts && in && c >= 1) {
                w[u] = slices ? __ldcg(slices + 2 * c) : c * per;
                w_end[u] = slices ? __ldcg(slices + 2 * c + 1) : min(nw, c * per + per);
            }
        }
        uint32_t f0[CU], fl[CU], nd[CU], ndl[CU];
#pragma unroll
        for (int u = 0; u < CU; ++u) {
            const bool chk = w[u] < w_end[u] && w[u] > 0;  // a non-empty range with a window to its left
            f0[u] = chk ? L.flag[w[u]] : 1u;
            fl[u] = chk ? L.flag[w[u] - 1] : 1u;
            nd[u] = chk ? L.node[w[u]] : 0u;
            ndl[u] = chk ? L.node[w[u] - 1] : 0u;
        }
#pragma unroll
        for (int u = 0; u < CU; ++u) {
            const uint32_t c = j0 + u * BLOCK + threadIdx.x;
            const uint32_t h = vh[u] - ((!f0[u] && !fl[u] && (nd[u] & ~W) == (ndl[u] & ~W)) ? 1u : 0u);
            const bool before = c < blockIdx.x;
            s.x += before ? h : 0u;
            s.y += h;
            s.z += before ? vi[u] : 0u;
            s.w += vi[u];
        }
    }
    s = block_sum4(s);
    base_h = s.x;
    total_h = s.y;
    base_i = s.z;
    total_i = s.w;
}

// Two register budgets of the same kernel: MINB resident CTAs per SM. Two
// (128 registers, almost no spills) suits single large graphs, whose phases
// are short and barrier-bound; three (80 registers, some spills to local
// memory) suits many graphs per launch, whose phases are longer and gain from
// the extra warps. gpma_tuning.update_blocks_per_sm selects one.
template <int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) update_kernel(UpdateArgs A) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint32_t tmp[BLOCK / 32 + 1];
    if (A.abort && ld_volatile(A.abort))
        return;  // every CTA: nothing written, the status slot stays as the previous launch left it
    DeviceStatus *st = A.st;
    const bool stamper = blockIdx.x == 0 && threadIdx.x == 0;
    if (stamper)
        st->stamp[0] = globaltimer_ns();
    // One graph: the heads at every stride-th segment, which every CTA copies
    // into shared memory for the top of the descent, are gathered once into a
    // contiguous array here (before the sort's first barrier), so each CTA's
    // copy is a coalesced read instead of LOCATE_CACHE scattered ones.
    if (A.G == 1 && blockIdx.x < LOCATE_CACHE / BLOCK) {
        const GraphDesc &D = A.gd[0];
        const uint32_t segs = D.size >> D.log2seg;
        const uint32_t cached = segs < LOCATE_CACHE ? segs : LOCATE_CACHE;
        const uint32_t hstep = (31 - __clz(D.size / cached)) - D.log2seg;
        for (uint32_t j = blockIdx.x * BLOCK + threadIdx.x; j < cached; j += gridDim.x * BLOCK)
            A.top[j] = D.heads[(size_t)j << hstep];
    }

    // S: stable sort of each graph's batch (gpma.cuh:977): the bucket sort,
    // or digit passes separated by grid barriers (digits constant over all
    // batches skipped) when it is off or a bucket is crowded.
    const uint64_t *bk = A.bk[0];
    const uint8_t *bv = A.bv[1];
    bool digits = A.q.nq == 0;
    if (!digits) {
        bsort_rank(A.in_k, A.boff, A.G, A.gd, A.q, st, A.check_keys);
        if (!grid_barrier(&st->bar, &st->err, A.stall, A.stall_limit_ns))
            return;
        if (ld_volatile(&st->invalid_keys) != 0)
            return;  // reserved-column keys: reject the batch before any change
        bsort_scan(A.q, A.cta_cnt, st, tmp);
        if (!grid_barrier(&st->bar, &st->err))
            return;
        digits = cta_broadcast_read(&st->sort_fallback) != 0;
        if (!digits) {
            // records of the batch scattered into buckets, then items sorted into bk[0] / bv[1]
            uint32_t *cpre = reinterpret_cast<uint32_t *>(smem + BSORT_SMEM_ITEM);
            bsort_chunk_prefix(A.cta_cnt, cpre, tmp);
            bsort_scatter(A.in_k, A.in_v, A.boff, A.G, A.q, cpre);
            if (!grid_barrier(&st->bar, &st->err))
                return;
            bsort_items(A.bk[0], A.bv[1], A.boff, A.G, A.q, cpre, smem);
            if (!grid_barrier(&st->bar, &st->err))
                return;
        }
    }
    if (digits) {
        sort_histogram(A.in_k, A.boff, A.G, A.sort_hist, st, A.check_keys, reinterpret_cast<uint32_t *>(smem));
        if (!grid_barrier(&st->bar, &st->err, A.q.nq == 0 ? A.stall : 0u, A.stall_limit_ns))
            return;
        if (ld_volatile(&st->invalid_keys) != 0)
            return;  // reserved-column keys: reject the batch before any change
        uint32_t sel = 0;
        bool first = true;  // the first pass reads the batch as submitted
        {
            const uint32_t trivial = sort_trivial_mask(A.sort_hist + (size_t)(A.G == 1 ? 0 : A.G) * 2048, A.n);
            const uint32_t tiles = A.toff[A.G];
            for (int p = 0; p < 8; ++p) {
                if (trivial & (1u << p))
                    continue;
                const uint64_t *ink = first ? A.in_k : (sel ? A.bk[1] : A.bk[0]);
                const uint8_t *inv = first ? A.in_v : (sel ? A.bv[1] : A.bv[0]);
                uint64_t *outk = sel ? A.bk[0] : A.bk[1];
                uint8_t *outv = sel ? A.bv[0] : A.bv[1];
                first = false;
                // CTA b takes tiles b, b + G, b + 2G, ... in order: every look-back
                // waits on lower tiles only, and the lowest unfinished tile never
                // waits on anything unfinished, so the pass always progresses
                for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x)
                    sort_tile(p, tile, ink, inv, outk, outv, A.boff, A.toff, A.G, A.sort_hist, A.sort_status, st, smem,
                              tmp);
                sel ^= 1u;
                if (!grid_barrier(&st->bar, &st->err))
                    return;
            }
        }
        bk = first ? A.in_k : (sel ? A.bk[1] : A.bk[0]);  // no pass: every digit constant
        bv = first ? A.in_v : (sel ? A.bv[1] : A.bv[0]);
    }
    const uint32_t G = gridDim.x;

    uint32_t scan_id = 0;
#define CNT(id) ((id) ? A.cta_cnt + G : A.cta_cnt)
#define CNTI(id) ((id) ? A.cta_cnt + 3 * G : A.cta_cnt + 2 * G)
#define SLICES(p) (A.cta_cnt + 4 * G + 2 * (p) * G)  // per CTA (lo, hi) of its windows, by level parity
    unsigned long long acc = 0, acc_slots = 0;
    if (stamper)
        st->stamp[1] = globaltimer_ns();

    // P1: locate every update, applying deletes / modifies in place. The top
    // of the descent comes from a shared-memory copy of the first keys at
    // every `stride`-th slot (of the one graph, or of each graph in turn).
    {
        const uint64_t *fk = nullptr;
        uint32_t log2stride = 0;
        if (A.G == 1) {
            const GraphDesc &D = A.gd[0];
            const uint32_t segs = D.size >> D.log2seg;
            const uint32_t cached = segs < LOCATE_CACHE ? segs : LOCATE_CACHE;
            log2stride = 31 - __clz(D.size / cached);
            uint64_t *f = reinterpret_cast<uint64_t *>(smem);
            // the contiguous copy gathered at the start of the launch; all of
            // a thread's loads issued together
            uint64_t hv[LOCATE_CACHE / BLOCK];
#pragma unroll
            for (uint32_t r = 0; r < LOCATE_CACHE / BLOCK; ++r) {
                const uint32_t j = threadIdx.x + r * BLOCK;
                hv[r] = j < cached ? A.top[j] : 0ull;
            }
#pragma unroll
            for (uint32_t r = 0; r < LOCATE_CACHE / BLOCK; ++r) {
                const uint32_t j = threadIdx.x + r * BLOCK;
                if (j < cached)
                    f[j] = hv[r];
            }
            __syncthreads();
            fk = f;
        }
        if (A.G == 1) {
            // one graph: each CTA takes a contiguous range (neighbouring keys
            // share descent paths in L1) and counts its insertions for the
            // compaction after the barrier
            uint32_t lo, hi, mine = 0;
            cta_range(A.n, lo, hi);
            for (uint32_t i0 = lo + threadIdx.x; i0 < hi; i0 += LOC_ILP * BLOCK)
                mine += locate_keys<true>(A, bk, bv, i0, BLOCK, hi, fk, log2stride);
            const uint32_t t = block_sum(mine, tmp);
            if (threadIdx.x == 0)
                CNT(scan_id)[blockIdx.x] = t;
        } else {
            // many graphs: each CTA takes a contiguous range of the sorted
            // batches (a graph or two) and, graph by graph, copies the graph's
            // top-of-tree heads into shared memory, so its keys walk the upper
            // levels there as with one graph
            uint64_t *f = reinterpret_cast<uint64_t *>(smem);
            uint32_t lo, hi;
            cta_range(A.n, lo, hi);
            uint32_t pos = lo;
            while (__syncthreads_or(pos < hi)) {
                const uint32_t g = segment_of(A.boff, A.G, pos);
                const uint32_t end = min(hi, A.boff[g + 1]);
                const GraphDesc &D = A.gd[g];
                const uint32_t segs = D.size >> D.log2seg;
                const uint32_t cached = segs < LOCATE_CACHE ? segs : LOCATE_CACHE;
                const uint32_t l2s = 31 - __clz(D.size / cached);
                const uint32_t hstep = l2s - D.log2seg;
                uint64_t hv[LOCATE_CACHE / BLOCK];
#pragma unroll
                for (uint32_t r = 0; r < LOCATE_CACHE / BLOCK; ++r) {
                    const uint32_t j = threadIdx.x + r * BLOCK;
                    hv[r] = j < cached ? D.heads[(size_t)j << hstep] : 0ull;
                }
#pragma unroll
                for (uint32_t r = 0; r < LOCATE_CACHE / BLOCK; ++r) {
                    const uint32_t j = threadIdx.x + r * BLOCK;
                    if (j < cached)
                        f[j] = hv[r];
                }
                __syncthreads();
                for (uint32_t i0 = pos + threadIdx.x; i0 < end; i0 += LOC_ILP * BLOCK)
                    locate_keys<false>(A, bk, bv, i0, BLOCK, end, f, l2s);
                __syncthreads();  // the copy is replaced for the next graph
                pos = end;
            }
        }
    }
    if (!grid_barrier(&st->bar, &st->err))
        return;
    {
        // every CTA is past the sort (trivial-digit mask, passes): zero its
        // state and the next launch's status slot
        const uint32_t gt = blockIdx.x * BLOCK + threadIdx.x, nt = G * BLOCK;
        for (uint32_t i = gt; i < A.hist_words; i += nt)
            A.sort_hist[i] = 0;
        for (uint32_t i = gt; i < A.status_words; i += nt)
            A.sort_status[i] = 0;
        for (uint32_t i = gt; i < A.q.nq; i += nt)
            A.q.qcnt[i] = 0;
        if (gt < 8)
            A.sort_tiles[gt] = 0;
        for (uint32_t i = gt; i < A.next_slot_words; i += nt)
            A.next_slot[i] = 0;
    }
    if (stamper)
        st->stamp[2] = globaltimer_ns();

    // P2: stable compaction of the insertions (with their graph), each CTA
    // writing the insertions of its locate range; then it counts the
    // run-length heads of its own output (its first insertion counted as one).
    uint32_t lo, hi;
    cta_range(A.n, lo, hi);
    if (A.G > 1) {
        uint32_t cl = 0;
        for (uint32_t i = lo + threadIdx.x; i < hi; i += BLOCK)
            cl += A.leaf[i] != SIZE_NONE;
        const uint32_t t = block_sum(cl, tmp);
        if (threadIdx.x == 0)
            CNT(scan_id)[blockIdx.x] = t;
        if (!grid_barrier(&st->bar, &st->err))
            return;
    }
    uint32_t base, m, unused_b, unused_t;
    cta_prefix2(CNT(scan_id), nullptr, base, m, unused_b, unused_t);
    const uint32_t out_lo = base;
    // GROUP_ITEMS consecutive items per thread and one scan per round
    for (uint32_t r0 = lo; r0 < hi; r0 += GROUP_ITEMS * BLOCK) {
        const uint32_t i0 = r0 + GROUP_ITEMS * threadIdx.x;
        uint32_t lf[GROUP_ITEMS], cnt = 0;
#pragma unroll
        for (uint32_t j = 0; j < GROUP_ITEMS; ++j) {
            lf[j] = i0 + j < hi ? A.leaf[i0 + j] : SIZE_NONE;
            cnt += lf[j] != SIZE_NONE;
        }
        uint32_t tot;
        uint32_t o = base + block_excl_scan(cnt, &tot, tmp);
#pragma unroll
        for (uint32_t j = 0; j < GROUP_ITEMS; ++j) {
            if (lf[j] == SIZE_NONE)
                continue;
            const uint32_t i = i0 + j;
            A.ikeys[0][o] = bk[i];
            A.ivals[0][o] = bv[i];
            A.ileaf[o] = lf[j];
            A.igraph[o] = graph_of(A, i);
            ++o;
        }
        base += tot;
    }
    const uint32_t out_hi = base;
    __syncthreads();  // this CTA's output is visible to all its threads
    {
        uint32_t h = 0;
        for (uint32_t j = out_lo + threadIdx.x; j < out_hi; j += BLOCK)
            h += (j == out_lo || A.ileaf[j] != A.ileaf[j - 1] || A.igraph[j] != A.igraph[j - 1]);
        const uint32_t t = block_sum(h, tmp);
        if (threadIdx.x == 0)
            CNT(scan_id ^ 1)[blockIdx.x] = t;
    }
    if (!grid_barrier(&st->bar, &st->err))
        return;
    if (A.G == 1 && m >= SIGNIFICANT_INSERTS) {
        if (stamper) {
            st->significant = 1;
            st->inserts = m;
            A.gs[0].inserts = m;
            A.gs[0].ins_base = 0;
        }
        return;
    }

    // P3: run-length grouping of the insertions by (graph, leaf) -> level-0
    // windows; also each graph's first insertion and its count. A CTA whose
    // first insertion continues the run of the previous output counted one
    // head too many: the window offsets subtract those.
    uint32_t nw = 0;
    {
        const uint32_t *ins_cnt = CNT(scan_id);
        const uint32_t *head_cnt = CNT(scan_id ^ 1);
        uint32_t carry = 0, before = 0, all = 0;
        // two CTAs' counts per thread per step, each kind of load issued for
        // both before the first is used
        for (uint32_t c0 = 0; c0 < G; c0 += 2 * BLOCK) {
            uint32_t n_c[2], h_c[2], b_c[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const uint32_t c = c0 + u * BLOCK + threadIdx.x;
                n_c[u] = c < G ? __ldcg(ins_cnt + c) : 0u;
                h_c[u] = c < G ? __ldcg(head_cnt + c) : 0u;
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                uint32_t tot;
                b_c[u] = carry + block_excl_scan(n_c[u], &tot, tmp);  // first output of CTA c
                carry += tot;
            }
            uint32_t l0[2], l1[2], g0[2], g1[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const bool chk = n_c[u] && b_c[u] > 0;
                l0[u] = chk ? A.ileaf[b_c[u]] : 0u;
                l1[u] = chk ? A.ileaf[b_c[u] - 1] : 1u;
                g0[u] = chk ? A.igraph[b_c[u]] : 0u;
                g1[u] = chk ? A.igraph[b_c[u] - 1] : 0u;
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const uint32_t c = c0 + u * BLOCK + threadIdx.x;
                uint32_t h = 0;
                if (c < G && n_c[u]) {
                    h = h_c[u];
                    if (l0[u] == l1[u] && g0[u] == g1[u])  // continues the previous CTA's last run
                        --h;
                }
                all += h;
                if (c < blockIdx.x)
                    before += h;
            }
        }
        const uint4 t = block_sum4(make_uint4(all, before, 0, 0));
        nw = t.x;
        base = t.y;
    }
    for (uint32_t r0 = out_lo; r0 < out_hi; r0 += GROUP_ITEMS * BLOCK) {
        const uint32_t j0 = r0 + GROUP_ITEMS * threadIdx.x;
        // items j0 - 1 .. j0 + GROUP_ITEMS: each item's run test needs its
        // neighbours on both sides
        uint32_t lf[GROUP_ITEMS + 2], gr[GROUP_ITEMS + 2];
#pragma unroll
        for (uint32_t q = 0; q < GROUP_ITEMS + 2; ++q) {
            const uint32_t j = j0 + q - 1;  // wraps to UINT32_MAX for j0 == 0, q == 0
            const bool ok = j0 + q >= 1 && j < m;
            lf[q] = ok ? A.ileaf[j] : SIZE_NONE;
            gr[q] = ok ? A.igraph[j] : SIZE_NONE;
        }
        uint32_t heads = 0;
        uint32_t hd[GROUP_ITEMS];
#pragma unroll
        for (uint32_t q = 0; q < GROUP_ITEMS; ++q) {
            const uint32_t j = j0 + q;
            hd[q] = 0;
            if (j < out_hi) {
                const bool new_graph = j == 0 || gr[q] != gr[q + 1];
                hd[q] = (new_graph || lf[q + 1] != lf[q]) ? 1u : 0u;
                if (new_graph)
                    A.gs[gr[q + 1]].ins_base = j;
                if (j + 1 == m || gr[q + 2] != gr[q + 1])
                    A.gs[gr[q + 1]].inserts = j + 1;  // end for now; made a count by the host
            }
            heads += hd[q];
        }
        uint32_t tot;
        // a run continued from the previous CTA's output extends window base - 1
        uint32_t e = base + block_excl_scan(heads, &tot, tmp);
#pragma unroll
        for (uint32_t q = 0; q < GROUP_ITEMS; ++q) {
            const uint32_t j = j0 + q;
            if (j >= out_hi)
                continue;
            if (hd[q]) {
                A.wnode[0][e] = lf[q + 1];
                A.wgraph[0][e] = gr[q + 1];
                A.wa[0][e] = j;
                ++e;
            }
            const bool last = j + 1 == m || lf[q + 2] != lf[q + 1] || gr[q + 2] != gr[q + 1];
            if (last)
                A.wb[0][e - 1] = j + 1;
        }
        base += tot;
    }
    scan_id ^= 1;
    if (!grid_barrier(&st->bar, &st->err))
        return;
    if (stamper)
        st->stamp[3] = globaltimer_ns();

    // Level loop. Windows and their pending insertions live in ping-pong
    // buffers selected by `cur`; each window's insertions are the contiguous
    // range [wa, wb) of the current insertion buffer.
    uint32_t cur = 0, level = 0;
    // own: this level's windows [olo, ohi) of this CTA are the ones it wrote
    // in the last level's carry pass, which ended without a grid barrier
    bool own = false;
    uint32_t olo = 0, ohi = 0;
    for (; level <= A.max_height && nw > 0; ++level) {
        // one graph, windows of at most CTA_WINDOW_MAX slots: each CTA
        // dispatches a contiguous range of the windows and counts its rejected
        // ones right away, so the level needs one grid barrier fewer
        const bool fused = A.G == 1 && (A.gd[0].seg << level) <= CTA_WINDOW_MAX;
        Windows L;
        L.node = cur ? A.wnode[1] : A.wnode[0];
        L.graph = cur ? A.wgraph[1] : A.wgraph[0];
        L.a = cur ? A.wa[1] : A.wa[0];
        L.b = cur ? A.wb[1] : A.wb[0];
        L.flag = A.wflag[level & 1];
        const uint64_t *pk = cur ? A.ikeys[1] : A.ikeys[0];
        const uint8_t *pv = cur ? A.ivals[1] : A.ivals[0];
        // one run of windows per segment length (a single run for one graph)
        for (uint32_t s = 2; s <= 32; s <<= 1) {
            uint32_t r0 = 0, r1 = nw;
            if (A.G > 1) {
                r0 = first_window_of_seg(A, L.graph, nw, s);
                r1 = first_window_of_seg(A, L.graph, nw, 2 * s);
            } else if (A.gd[0].seg != s) {
                continue;
            }
            if (r0 >= r1)
                continue;
            uint32_t W = s << level;
            const unsigned long long before = acc;
            // windows over the grid; with the count fused into this phase,
            // each CTA takes the contiguous range it counts (and copies) next
            uint32_t d0 = r0, d1 = r1, part = blockIdx.x, parts = gridDim.x;
            if (fused) {
                if (own) {
                    d0 = olo;
                    d1 = ohi;
                } else {
                    cta_range(nw, d0, d1);
                }
                part = 0;
                parts = 1;
                if (d0 >= d1)
                    W = 0;  // nothing for this CTA: no dispatch
            }
            switch (W) {
            case 0: break;
            case 2: small_dispatch<2>(A, L, d0, d1, level, pk, pv, smem, tmp, acc, part, parts); break;
            case 4: small_dispatch<4>(A, L, d0, d1, level, pk, pv, smem, tmp, acc, part, parts); break;
            case 8: small_dispatch<8>(A, L, d0, d1, level, pk, pv, smem, tmp, acc, part, parts); break;
            case 16: small_dispatch<16>(A, L, d0, d1, level, pk, pv, smem, tmp, acc, part, parts); break;
            case 32: small_dispatch<32>(A, L, d0, d1, level, pk, pv, smem, tmp, acc, part, parts); break;
            case 64: small_dispatch<64>(A, L, d0, d1, level, pk, pv, smem, tmp, acc, part, parts); break;
            case 128: small_dispatch<128>(A, L, d0, d1, level, pk, pv, smem, tmp, acc, part, parts); break;
            case 256: small_dispatch<256>(A, L, d0, d1, level, pk, pv, smem, tmp, acc, part, parts); break;
            case 512: small_dispatch<512>(A, L, d0, d1, level, pk, pv, smem, tmp, acc, part, parts); break;
            case 1024: small_dispatch<1024>(A, L, d0, d1, level, pk, pv, smem, tmp, acc, part, parts); break;
            case 2048: small_dispatch<2048>(A, L, d0, d1, level, pk, pv, smem, tmp, acc, part, parts); break;
            default:
                if (!grid_windows(A, L, r0, r1, W, level, pk, pv, smem, tmp, acc))
                    return;
            }
            acc_slots += (acc - before) * (unsigned long long)W;
            // the next run lays out shared memory differently: every warp of
            // the CTA must be done with this run's staging first
            __syncthreads();
        }
        if (own) {
            lo = olo;
            hi = ohi;
        } else {
            cta_range(nw, lo, hi);
        }
        if (fused)  // the CTA's own range was dispatched (and flagged) by its own warps
            count_rejected(A, L, level, lo, hi, true, CNT(scan_id), CNTI(scan_id));
        if (!grid_barrier(&st->bar, &st->err))
            return;
        // Next level. Rejected windows keep their insertions, which are
        // compacted into the other buffer (new offsets from one scan over the
        // windows, as compact_insertions does over insertions, gpma.cuh:1022);
        // a rejected right sibling joins its rejected left sibling in the
        // parent window (up_level, gpma.cuh:881-889 + regrouping). A rejected
        // root window leaves its insertions to the root rebalance: they go to
        // the graph's area of the remaining-insertion buffer.
        const uint32_t nxt = cur ^ 1;
        uint32_t *nwn = nxt ? A.wnode[1] : A.wnode[0];
        uint32_t *nwg = nxt ? A.wgraph[1] : A.wgraph[0];
        uint32_t *nwa = nxt ? A.wa[1] : A.wa[0];
        uint32_t *nwb = nxt ? A.wb[1] : A.wb[0];
        uint64_t *nk = nxt ? A.ikeys[1] : A.ikeys[0];
        uint8_t *nv = nxt ? A.ivals[1] : A.ivals[0];
        if (!fused) {
            count_rejected(A, L, level, lo, hi, false, CNT(scan_id), CNTI(scan_id));
            if (!grid_barrier(&st->bar, &st->err))
                return;
        }
        uint32_t nw_next, base_i, total_i;
        level_prefix(A, L, nw, level, fused, own ? SLICES(level & 1) : nullptr, CNT(scan_id), CNTI(scan_id), base,
                     nw_next, base_i, total_i);
        if (nw_next == 0 && level < A.min_height) {
            // every window of this level was accepted and none can be a root
            // window: nothing to carry, no next level (counted as the loop's
            // own exit would count it)
            nw = 0;
            ++level;
            break;
        }
        // GROUP_ITEMS consecutive windows per thread per round; the rejected
        // windows' copy plan goes to a compact list in shared memory (free
        // again once the level's windows are written): source, destination
        // (the next level's buffer, or the remaining buffer for a root
        // window) and the exclusive prefix of the counts, so the whole CTA
        // copies the concatenated ranges (a window of a million insertions is
        // not left to one warp)
        // not left to one warp). A window whose left sibling ends the previous
        // CTA's range has its insertions copied by that CTA, which writes the
        // parent window: every next-level window's insertions come from the
        // CTA that writes the window.
        uint32_t *l_src = reinterpret_cast<uint32_t *>(smem);
        uint32_t *l_pre = l_src + GROUP_ITEMS * BLOCK + 1;
        uint32_t *l_to = l_pre + GROUP_ITEMS * BLOCK + 1;  // destination offset | root << 31
        const uint32_t next_lo = base;  // this CTA's first window of the next level
        for (uint32_t r0 = lo; r0 < hi; r0 += GROUP_ITEMS * BLOCK) {
            const uint32_t w0 = r0 + GROUP_ITEMS * threadIdx.x;
            // windows w0 - 1 .. w0 + GROUP_ITEMS: each needs both neighbours
            uint32_t fl[GROUP_ITEMS + 2], gg[GROUP_ITEMS + 2], nd[GROUP_ITEMS + 2], wa[GROUP_ITEMS + 2],
                wb[GROUP_ITEMS + 2];
#pragma unroll
            for (uint32_t q = 0; q < GROUP_ITEMS + 2; ++q) {
                const uint32_t j = w0 + q - 1;
                const bool ok = w0 + q >= 1 && j < nw;
                fl[q] = ok ? L.flag[j] : 1u;
                gg[q] = ok ? L.graph[j] : 0u;
                nd[q] = ok ? L.node[j] : 0u;
                wa[q] = ok ? L.a[j] : 0u;
                wb[q] = ok ? L.b[j] : 0u;
            }
            uint32_t csum = 0, hsum = 0, rsum = 0, asum = 0;
#pragma unroll
            for (uint32_t q = 0; q < GROUP_ITEMS; ++q) {
                const uint32_t j = w0 + q;
                const bool rej = j < hi && !fl[q + 1];
                if (!rej)
                    continue;
                const GraphDesc &Dg = A.gd[gg[q + 1]];
                const bool root = level >= Dg.height;
                const uint32_t W = Dg.seg << level;
                const bool merged =
                    !root && j > 0 && !fl[q] && gg[q] == gg[q + 1] && (nd[q] & ~W) == (nd[q + 1] & ~W);
                if (!(merged && j == lo)) {  // else the previous CTA copies it
                    ++rsum;
                    asum += wb[q + 1] - wa[q + 1];
                }
                if (root)
                    continue;
                csum += wb[q + 1] - wa[q + 1];
                hsum += merged ? 0u : 1u;
            }
            uint4 tot;
            const uint4 ex = block_excl_scan4(make_uint4(csum, hsum, rsum, asum), tot);
            const uint32_t tot_i = tot.x, tot_h = tot.y, tot_r = tot.z, tot_a = tot.w;
            uint32_t nb = base_i + ex.x;
            uint32_t e = base + ex.y;
            uint32_t li = ex.z;
            uint32_t pre = ex.w;
#pragma unroll
            for (uint32_t q = 0; q < GROUP_ITEMS; ++q) {
                const uint32_t j = w0 + q;
                const bool rej = j < hi && !fl[q + 1];
                if (!rej)
                    continue;
                const uint32_t g = gg[q + 1];
                const GraphDesc &Dg = A.gd[g];
                const uint32_t c = wb[q + 1] - wa[q + 1];
                const uint32_t W = Dg.seg << level;
                const uint32_t par = nd[q + 1] & ~W;
                const bool merged = level < Dg.height && j > 0 && !fl[q] && gg[q] == g && (nd[q] & ~W) == par;
                if (merged && j == lo) {
                    nb += c;  // copied by the previous CTA
                    continue;
                }
                l_src[li] = wa[q + 1];
                l_pre[li] = pre;
                pre += c;
                if (level >= Dg.height) {
                    // the root rebalance takes these: the graph's area of the
                    // remaining-insertion buffer, at its first insertion
                    A.gs[g].remaining = c;
                    l_to[li] = A.gs[g].ins_base | 0x80000000u;
                    ++li;
                    continue;
                }
                l_to[li] = nb;
                ++li;
                if (!merged) {
                    const bool right = j + 1 < nw && !fl[q + 2] && gg[q + 2] == g && (nd[q + 2] & ~W) == par;
                    nwn[e] = par;
                    nwg[e] = g;
                    nwa[e] = nb;
                    nwb[e] = nb + c + (right ? wb[q + 2] - wa[q + 2] : 0u);
                    ++e;
                }
                nb += c;
            }
            __syncthreads();
            // copy the kept insertions: position p of the round's
            // concatenation (p < tot_a) is element p - l_pre[t] of entry t,
            // the last entry with l_pre <= p
            for (uint32_t p = threadIdx.x; p < tot_a; p += BLOCK) {
                uint32_t lo2 = 0, hi2 = tot_r;  // answer in [0, tot_r)
                while (hi2 - lo2 > 1) {
                    const uint32_t mid = (lo2 + hi2) >> 1;
                    if (l_pre[mid] <= p)
                        lo2 = mid;
                    else
                        hi2 = mid;
                }
                const uint32_t k = p - l_pre[lo2], to = l_to[lo2];
                const uint32_t from = l_src[lo2] + k;
                uint64_t *dk = (to >> 31) ? A.rkeys : nk;
                uint8_t *dv = (to >> 31) ? A.rvals : nv;
                dk[(to & 0x7FFFFFFFu) + k] = pk[from];
                dv[(to & 0x7FFFFFFFu) + k] = pv[from];
            }
            __syncthreads();
            base += tot_h;
            base_i += tot_i;
        }
        if (hi > lo && hi < nw) {
            // the last window's right sibling, rejected, begins the next
            // CTA's range: its insertions follow this CTA's
            const uint32_t j = hi - 1;
            const uint32_t g = L.graph[j];
            const GraphDesc &Dg = A.gd[g];
            const uint32_t W = Dg.seg << level;
            if (level < Dg.height && !L.flag[j] && !L.flag[hi] && L.graph[hi] == g &&
                (L.node[j] & ~W) == (L.node[hi] & ~W)) {
                const uint32_t a = L.a[hi], c = L.b[hi] - a;
                for (uint32_t k = threadIdx.x; k < c; k += BLOCK) {
                    nk[base_i + k] = pk[a + k];
                    nv[base_i + k] = pv[a + k];
                }
            }
            __syncthreads();
        }
        scan_id ^= 1;
        // The next level goes on without a grid barrier when it too is fused:
        // each CTA then takes the windows it just wrote, whose insertions it
        // copied itself, and the slots they cover were last written before
        // this level's barrier. The window flags alternate by level, so a CTA
        // flagging the next level's windows does not overwrite ones a slower
        // CTA still reads here.
        own = fused && nw_next > 0 && level + 1 <= A.max_height && (A.gd[0].seg << (level + 1)) <= CTA_WINDOW_MAX;
        if (own) {
            olo = next_lo;
            ohi = base;
            if (threadIdx.x == 0) {
                SLICES((level + 1) & 1)[2 * blockIdx.x] = olo;
                SLICES((level + 1) & 1)[2 * blockIdx.x + 1] = ohi;
            }
        } else if (!grid_barrier(&st->bar, &st->err)) {
            return;
        }
        nw = nw_next;
        cur = nxt;
    }
    if (stamper)
        st->stamp[4] = globaltimer_ns();

    // one atomic per CTA for the statistics
    __shared__ unsigned long long s_acc[2];
    if (threadIdx.x == 0) {
        s_acc[0] = 0;
        s_acc[1] = 0;
    }
    __syncthreads();
    if (acc)
        atomicAdd(&s_acc[0], acc);
    if (acc_slots)
        atomicAdd(&s_acc[1], acc_slots);
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_acc[0])
            atomicAdd(&st->accepted_windows, s_acc[0]);
        if (s_acc[1])
            atomicAdd(&st->accepted_slots, s_acc[1]);
    }
    if (stamper) {
        st->levels = level;
        st->inserts = m;
    }
#undef CNT
#undef CNTI
}

// ---- whole-array kernels for the root resize and the bulk rebuild ----------

// Live elements among the first d of the stable merge of live[0..L) and
// pend[0..P) (ties: live first).
__device__ __forceinline__ uint32_t merge_split(const uint64_t *lk, uint32_t L, const uint64_t *pk, uint32_t P,
                                                uint64_t d) {
    uint32_t lo = d > P ? (uint32_t)(d - P) : 0u, hi = (uint32_t)(d < L ? d : L);
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (pk[d - mid - 1] < lk[mid])
            hi = mid;
        else
            lo = mid + 1;
    }
    return lo;
}

// First merged element of each CHUNK-slot chunk of the redispatched array
// (and of its end), split into live and pending parts: split[c] = live
// elements before chunk c. One search per chunk boundary, all in parallel.
__global__ void merge_split_kernel(const uint64_t *lk, uint32_t L, const uint64_t *pk, uint32_t P, uint32_t size,
                                   uint32_t log2seg, uint32_t log2F, uint32_t *split) {
    const uint64_t M = (uint64_t)L + P;
    const uint32_t chunks = (size + CHUNK - 1) / CHUNK;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c <= chunks; c += gridDim.x * blockDim.x) {
        const uint32_t t0 = (uint32_t)min((uint64_t)c * CHUNK, (uint64_t)size);
        const uint64_t f = seg_first(t0 >> log2seg, M, log2F);
        split[c] = merge_split(lk, L, pk, P, f < M ? f : M);
    }
}

// Redispatch of the whole array [0, size) from live[0..L) and pend[0..P):
// chunk c's merged elements come from live[split[c] .. split[c+1]) and the
// matching pending range; both are staged in shared memory (coalesced) and
// merged there, then every slot of the chunk is written once, coalesced.
__global__ void __launch_bounds__(BLOCK) rebuild_kernel(uint64_t *keys, uint8_t *vals, uint64_t *heads,
                                                        uint32_t *row_offset, uint32_t row_num, uint32_t size,
                                                        uint32_t log2seg,
                                                        uint32_t log2F, const uint64_t *lk, const uint8_t *lv,
                                                        uint32_t L, const uint64_t *pk, const uint8_t *pv, uint32_t P,
                                                        const uint32_t *split, uint64_t gap_key, uint32_t *err) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint64_t *sk = reinterpret_cast<uint64_t *>(smem);  // staged: live part, then pending part
    uint64_t *mk = sk + CHUNK;                          // merged
    uint8_t *sv = reinterpret_cast<uint8_t *>(mk + CHUNK);
    uint8_t *mv = sv + CHUNK;
    const uint64_t M = (uint64_t)L + P;
    const uint32_t seg = 1u << log2seg;
    const uint32_t chunks = (size + CHUNK - 1) / CHUNK;
    for (uint32_t c = blockIdx.x; c < chunks; c += gridDim.x) {
        const uint32_t t0 = c * CHUNK;
        const uint32_t len = min(CHUNK, size - t0);
        const uint64_t f_lo = seg_first(t0 >> log2seg, M, log2F), f_hi = seg_first((t0 + len) >> log2seg, M, log2F);
        const uint32_t i_lo = (uint32_t)(f_lo < M ? f_lo : M), i_hi = (uint32_t)(f_hi < M ? f_hi : M);
        const uint32_t x0 = split[c], x1 = split[c + 1];
        // the same condition in every thread: the whole CTA skips the chunk
        if (!in_bounds(err,
                       x0 <= x1 && x1 <= L && x0 <= i_lo && x1 <= i_hi && i_lo - x0 <= i_hi - x1 &&
                           i_hi - x1 <= P && i_hi - i_lo <= CHUNK,
                       BS_REBUILD))
            continue;
        const uint32_t y0 = i_lo - x0, y1 = i_hi - x1;
        const uint32_t nl = x1 - x0, np = y1 - y0;  // nl + np = i_hi - i_lo <= len
        for (uint32_t k = threadIdx.x; k < nl; k += BLOCK) {
            sk[k] = lk[x0 + k];
            sv[k] = lv[x0 + k];
        }
        for (uint32_t k = threadIdx.x; k < np; k += BLOCK) {
            sk[nl + k] = pk[y0 + k];
            sv[nl + k] = pv[y0 + k];
        }
        __syncthreads();
        const uint32_t cnt = nl + np;
        const uint32_t ipt = (cnt + BLOCK - 1) / BLOCK;
        const uint32_t d = threadIdx.x * ipt;
        if (d < cnt) {
            uint32_t lo = d > np ? d - np : 0, hi = min(d, nl);
            while (lo < hi) {
                const uint32_t mid = (lo + hi) >> 1;
                if (sk[nl + (d - mid - 1)] < sk[mid])
                    hi = mid;
                else
                    lo = mid + 1;
            }
            uint32_t x = lo, y = d - lo;
            const uint32_t end = min(cnt, d + ipt);
            for (uint32_t e = d; e < end; ++e) {
                const bool take_live = x < nl && (y >= np || sk[x] <= sk[nl + y]);
                if (take_live) {
                    mk[e] = sk[x];
                    mv[e] = sv[x];
                    ++x;
                } else {
                    mk[e] = sk[nl + y];
                    mv[e] = sv[nl + y];
                    ++y;
                }
            }
        }
        __syncthreads();
        for (uint32_t t = threadIdx.x; t < len; t += BLOCK) {
            const uint32_t slot = t0 + t;
            const uint32_t s = slot >> log2seg, ln = slot & (seg - 1);
            const uint64_t g0 = seg_first(s, M, log2F), g1 = seg_first(s + 1, M, log2F);
            uint64_t k = gap_key;
            uint8_t v = 0;
            if (ln < g1 - g0) {
                k = mk[g0 + ln - i_lo];
                v = mv[g0 + ln - i_lo];
            }
            keys[slot] = k;
            vals[slot] = v;
            if (ln == 0)
                heads[s] = k;
            if (is_guard(k)) {
                const uint32_t row = (uint32_t)(k >> 32);
                if (row < row_num)
                    row_offset[row + 1] = slot;
            }
        }
        __syncthreads();
    }
}

// ---- bulk copies: global memory -> this CTA's own shared memory -----------
// cp.async.bulk (TMA, no tensor map, no multicast) completing on an mbarrier
// of the CTA. Copies start and end on 16-byte boundaries.
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for phase `parity` of the barrier; false (and DERR_BARRIER_TIMEOUT in
// *err) after WAIT_LIMIT_NS.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t *err) {
    if (mbar_try_wait(bar, parity))
        return true;
    const uint64_t t0 = globaltimer_ns();
    for (;;) {
        if (mbar_try_wait(bar, parity))
            return true;
        if (globaltimer_ns() - t0 > WAIT_LIMIT_NS) {
            atomicCAS(err, 0u, DERR_BARRIER_TIMEOUT);
            return false;
        }
    }
}

// One-pass stable compaction of the live slots of [0, size) into dk/dv
// (resize_gpma, gpma.cuh:909-915): CHUNK-slot chunks, a decoupled look-back
// over the chunks' live counts for each chunk's output offset. status[c]
// (zeroed before the launch) holds chunk c's live count once it has loaded
// its slots (CST_AGG) and its inclusive prefix once its look-back is done
// (CST_INC); status[chunks] receives the total. CTAs take chunks b, b + grid,
// ... in order in a cooperative launch (all resident), so a look-back waits
// only on chunks already being processed; every wait gives up after
// WAIT_LIMIT_NS (DERR_LOOKBACK_TIMEOUT in *err). Each chunk's slots arrive by
// bulk copies into one of two stage buffers while the CTA compacts the
// previous chunk, so the look-back's latency overlaps the next chunk's loads
// (arrays under CHUNK slots are read directly). Replaces a count pass, a
// single-CTA scan and a second read of the array.
constexpr unsigned long long CST_AGG = 1ull << 62, CST_INC = 2ull << 62, CST_VAL = (1ull << 62) - 1;
constexpr uint32_t CP_STAGE_BYTES = CHUNK * 9;
constexpr size_t CP_SMEM = 2ull * CP_STAGE_BYTES + 2 * sizeof(uint64_t);

// Warp 0: decoupled look-back for chunk c with T live slots; returns the
// chunk's exclusive prefix (in every lane) and publishes its inclusive one.
// Each step reads 32 predecessors at once (lane l reads chunk t - l): the
// chunks of one wave of CTAs publish their counts together, and a look-back
// that read them a few at a time would walk a whole wave one L2 round trip
// per few chunks.
__device__ __forceinline__ unsigned long long compact_lookback(uint32_t c, uint32_t T, unsigned long long *status,
                                                               uint32_t *err, uint32_t lane) {
    if (c == 0) {
        if (lane == 0)
            atomicExch(&status[0], CST_INC | T);
        return 0;
    }
    if (lane == 0)
        atomicExch(&status[c], CST_AGG | T);
    unsigned long long prefix = 0;
    int64_t t = (int64_t)c - 1;
    uint64_t t0 = 0;
    unsigned ns = 32;
    while (t >= 0) {
        const int64_t idx = t - (int64_t)lane;
        // chunks before the first count as inclusive zeros
        const unsigned long long w =
            idx >= 0 ? (unsigned long long)*(volatile unsigned long long *)&status[idx] : (unsigned long long)CST_INC;
        const unsigned long long flag = w & ~CST_VAL;
        const uint32_t blocked = __ballot_sync(0xFFFFFFFFu, flag == 0);
        const uint32_t inc = __ballot_sync(0xFFFFFFFFu, flag == CST_INC);
        const uint32_t fb = blocked ? (uint32_t)__ffs(blocked) - 1 : 32u;
        const uint32_t fi = inc ? (uint32_t)__ffs(inc) - 1 : 32u;
        const uint32_t take = fi < fb ? fi + 1 : fb;  // lanes summed this step
        unsigned long long v = lane < take ? (w & CST_VAL) : 0ull;
#pragma unroll
        for (int d = 16; d >= 1; d >>= 1)
            v += __shfl_xor_sync(0xFFFFFFFFu, v, d);
        prefix += v;
        if (fi < fb)
            break;
        t -= take;
        if (take == 0) {
            // the nearest predecessor has not published yet
            if (t0 == 0)
                t0 = globaltimer_ns();
            __nanosleep(ns);
            if (ns < 256)
                ns <<= 1;
            const bool give_up = globaltimer_ns() - t0 > WAIT_LIMIT_NS || ld_volatile(err) != 0;
            if (__any_sync(0xFFFFFFFFu, give_up)) {
                if (lane == 0)
                    atomicCAS(err, 0u, DERR_LOOKBACK_TIMEOUT);
                break;
            }
        }
    }
    if (lane == 0)
        atomicExch(&status[c], CST_INC | (prefix + T));
    return prefix;
}

__global__ void __launch_bounds__(BLOCK, 4) compact_kernel(const uint64_t *keys, const uint8_t *vals, uint32_t size,
                                                           uint64_t *dk, uint8_t *dv, unsigned long long *status,
                                                           uint32_t *err) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + 2 * CP_STAGE_BYTES);
    __shared__ uint32_t s_warp[BLOCK / 32];
    __shared__ unsigned long long s_base;
    constexpr uint32_t STEPS = CHUNK / BLOCK;  // 8 steps of 32 consecutive slots per warp
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t chunks = (size + CHUNK - 1) / CHUNK;
    const bool staged = size >= CHUNK;  // whole chunks only: size is a power of two
    if (threadIdx.x == 0 && staged) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init_fence();
    }
    __syncthreads();
    auto issue = [&](uint32_t c, uint32_t st) {
        unsigned char *stage = smem + st * CP_STAGE_BYTES;
        mbar_arrive_expect_tx(&bar[st], CP_STAGE_BYTES);
        bulk_copy_g2s(stage, keys + (size_t)c * CHUNK, CHUNK * 8, &bar[st]);
        bulk_copy_g2s(stage + CHUNK * 8, vals + (size_t)c * CHUNK, CHUNK, &bar[st]);
    };
    uint32_t phases = 0;   // bit st: parity of stage st's next phase
    uint32_t pending = 0;  // thread 0: bit st set while stage st has copies outstanding
    if (staged && threadIdx.x == 0 && blockIdx.x < chunks) {
        issue(blockIdx.x, 0);
        pending |= 1u;
    }
    bool stop = false;
    uint32_t i = 0;
    for (uint32_t c = blockIdx.x; c < chunks; c += gridDim.x, ++i) {
        const uint32_t st = i & 1u;
        uint64_t k[STEPS];
        uint8_t v[STEPS];
        if (staged) {
            if (threadIdx.x == 0 && c + gridDim.x < chunks) {
                issue(c + gridDim.x, st ^ 1u);
                pending |= 2u >> st;  // bit st ^ 1
            }
            const bool landed = mbar_wait(&bar[st], (phases >> st) & 1u, err);
            if (__syncthreads_or(!landed)) {
                stop = true;
                break;
            }
            phases ^= 1u << st;
            pending &= ~(1u << st);
            const uint64_t *sk = reinterpret_cast<const uint64_t *>(smem + st * CP_STAGE_BYTES);
            const uint8_t *sv = smem + st * CP_STAGE_BYTES + CHUNK * 8;
#pragma unroll
            for (uint32_t j = 0; j < STEPS; ++j) {
                const uint32_t t = warp * (32 * STEPS) + 32 * j + lane;
                k[j] = sk[t];
                v[j] = sv[t];
            }
        } else {
            const uint32_t base = c * CHUNK + warp * (32 * STEPS);
#pragma unroll
            for (uint32_t j = 0; j < STEPS; ++j) {
                const uint32_t t = base + 32 * j + lane;
                k[j] = t < size ? keys[t] : KEY_NONE;
                v[j] = t < size ? vals[t] : 0;
            }
        }
        uint32_t mask[STEPS];
        uint32_t total = 0;
#pragma unroll
        for (uint32_t j = 0; j < STEPS; ++j) {
            mask[j] = __ballot_sync(0xFFFFFFFFu, k[j] != KEY_NONE && v[j] != 0);
            total += __popc(mask[j]);
        }
        if (lane == 0)
            s_warp[warp] = total;
        __syncthreads();
        if (warp == 0) {
            // exclusive offsets of the warps, then the chunk's look-back
            const uint32_t x = lane < BLOCK / 32 ? s_warp[lane] : 0u;
            const uint32_t inc_x = warp_incl_scan(x);
            const uint32_t T = __shfl_sync(0xFFFFFFFFu, inc_x, 31);
            __syncwarp();
            if (lane < BLOCK / 32)
                s_warp[lane] = inc_x - x;
            const unsigned long long prefix = compact_lookback(c, T, status, err, lane);
            if (lane == 0) {
                s_base = prefix;
                if (c + 1 == chunks)
                    status[chunks] = prefix + T;
            }
        }
        __syncthreads();
        uint64_t o = s_base + s_warp[warp];
        const uint32_t lt = lanemask_lt();
#pragma unroll
        for (uint32_t j = 0; j < STEPS; ++j) {
            if ((mask[j] >> lane) & 1u) {
                const uint64_t pos = o + __popc(mask[j] & lt);
                dk[pos] = k[j];
                dv[pos] = v[j];
            }
            o += __popc(mask[j]);
        }
        __syncthreads();  // s_warp, s_base and this stage are reused
    }
    // a stop can leave copies in flight: wait for them (bounded) before the
    // CTA's shared memory is released
    if (stop && threadIdx.x == 0) {
        for (uint32_t st = 0; st < 2; ++st)
            if ((pending >> st) & 1u)
                mbar_wait(&bar[st], (phases >> st) & 1u, err);
    }
}

// Redispatch of the whole array [0, size) (size a multiple of CHUNK, segments
// of >= 8 slots) from live[0..L) and pend[0..P), as rebuild_kernel, with the
// sources of each CHUNK-slot output chunk staged by bulk copies: chunk c's
// live range [split[c], split[c + 1]) and its pending range, each widened to
// 16-byte bounds (the arrays' allocations are multiples of 16 bytes, so the
// widened ranges stay inside them), land in one of two stage buffers while
// the CTA merges and writes the previous chunk; the chunk is written in slot
// pairs with 16-byte key stores.
constexpr uint32_t RB_KEY_BYTES = CHUNK * 8 + 64;   // a stage's live + pending keys, each widened
constexpr uint32_t RB_VAL_BYTES = CHUNK + 128;      // a stage's live + pending values, each widened
constexpr uint32_t RB_STAGE_BYTES = RB_KEY_BYTES + RB_VAL_BYTES;
struct RbDesc {
    uint32_t i_lo, nl, np;    // first merged element of the chunk, live and pending counts
    uint32_t lk_off, pk_off;  // byte offsets of the first live / pending key in the stage
    uint32_t lv_off, pv_off;  // byte offsets of the first live / pending value in the stage
    uint32_t ok;              // 0: the chunk failed its bounds check and is skipped
};
constexpr size_t RB_SMEM = 2ull * RB_STAGE_BYTES + CHUNK * 9ull + 2 * sizeof(RbDesc) + 2 * sizeof(uint64_t) + 16;
constexpr uint32_t RB_MIN_SLOTS = 1u << 16;  // smaller arrays take rebuild_kernel

// Thread 0: chunk c's ranges, its descriptor and its copies into `stage`.
__device__ __forceinline__ void rb_issue(uint32_t c, unsigned char *stage, RbDesc *d, uint64_t *bar,
                                         const uint64_t *lk, const uint8_t *lv, uint32_t L, const uint64_t *pk,
                                         const uint8_t *pv, uint32_t P, const uint32_t *split, uint32_t log2seg,
                                         uint32_t log2F, uint32_t *err) {
    const uint64_t M = (uint64_t)L + P;
    const uint32_t t0 = c * CHUNK;
    const uint64_t f_lo = seg_first(t0 >> log2seg, M, log2F), f_hi = seg_first((t0 + CHUNK) >> log2seg, M, log2F);
    const uint32_t i_lo = (uint32_t)(f_lo < M ? f_lo : M), i_hi = (uint32_t)(f_hi < M ? f_hi : M);
    const uint32_t x0 = split[c], x1 = split[c + 1];
    const bool ok = in_bounds(err,
                              x0 <= x1 && x1 <= L && x0 <= i_lo && x1 <= i_hi && i_lo - x0 <= i_hi - x1 &&
                                  i_hi - x1 <= P && i_hi - i_lo <= CHUNK,
                              BS_REBUILD);
    uint32_t bytes = 0;
    RbDesc r{};
    r.ok = ok ? 1u : 0u;
    if (ok) {
        const uint32_t y0 = i_lo - x0, y1 = i_hi - x1;
        r.i_lo = i_lo;
        r.nl = x1 - x0;
        r.np = y1 - y0;
        // [lo, hi) byte ranges widened to 16-byte bounds
        auto widen = [](const void *a, const void *b, uintptr_t &lo, uint32_t &len) {
            lo = reinterpret_cast<uintptr_t>(a) & ~uintptr_t(15);
            const uintptr_t hi = (reinterpret_cast<uintptr_t>(b) + 15) & ~uintptr_t(15);
            len = (uint32_t)(hi - lo);
        };
        uintptr_t lo;
        uint32_t len;
        uint32_t kpos = 0, vpos = RB_KEY_BYTES;
        if (r.nl) {
            widen(lk + x0, lk + x1, lo, len);
            r.lk_off = kpos + (uint32_t)(reinterpret_cast<uintptr_t>(lk + x0) - lo);
            bulk_copy_g2s(stage + kpos, reinterpret_cast<const void *>(lo), len, bar);
            kpos += len;
            bytes += len;
            widen(lv + x0, lv + x1, lo, len);
            r.lv_off = vpos + (uint32_t)(reinterpret_cast<uintptr_t>(lv + x0) - lo);
            bulk_copy_g2s(stage + vpos, reinterpret_cast<const void *>(lo), len, bar);
            vpos += len;
            bytes += len;
        }
        if (r.np) {
            widen(pk + y0, pk + y1, lo, len);
            r.pk_off = kpos + (uint32_t)(reinterpret_cast<uintptr_t>(pk + y0) - lo);
            bulk_copy_g2s(stage + kpos, reinterpret_cast<const void *>(lo), len, bar);
            bytes += len;
            widen(pv + y0, pv + y1, lo, len);
            r.pv_off = vpos + (uint32_t)(reinterpret_cast<uintptr_t>(pv + y0) - lo);
            bulk_copy_g2s(stage + vpos, reinterpret_cast<const void *>(lo), len, bar);
            bytes += len;
        }
    }
    *d = r;
    mbar_arrive_expect_tx(bar, bytes);  // the phase completes once the copies' bytes have landed
}

__global__ void __launch_bounds__(BLOCK, 4) rebuild_bulk_kernel(uint64_t *keys, uint8_t *vals, uint64_t *heads,
                                                                uint32_t *row_offset, uint32_t row_num, uint32_t size,
                                                                uint32_t log2seg, uint32_t log2F, const uint64_t *lk,
                                                                const uint8_t *lv, uint32_t L, const uint64_t *pk,
                                                                const uint8_t *pv, uint32_t P, const uint32_t *split,
                                                                uint64_t gap_key, uint32_t *err) {
    extern __shared__ __align__(16) unsigned char smem[];
    // stage st starts at smem + st * RB_STAGE_BYTES (computed, not indexed
    // from an array, so nothing of the loop lives in local memory)
    uint64_t *mk = reinterpret_cast<uint64_t *>(smem + 2 * RB_STAGE_BYTES);
    uint8_t *mv = reinterpret_cast<uint8_t *>(mk + CHUNK);
    RbDesc *desc = reinterpret_cast<RbDesc *>(mv + CHUNK);
    uint64_t *bar = reinterpret_cast<uint64_t *>((reinterpret_cast<uintptr_t>(desc + 2) + 15) & ~uintptr_t(15));
    const uint64_t M = (uint64_t)L + P;
    const uint32_t seg = 1u << log2seg;
    const uint32_t chunks = size / CHUNK;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init_fence();
    }
    __syncthreads();
    uint32_t pending = 0;  // thread 0: bit st set while stage st has copies outstanding
    if (threadIdx.x == 0 && blockIdx.x < chunks) {
        rb_issue(blockIdx.x, smem, &desc[0], &bar[0], lk, lv, L, pk, pv, P, split, log2seg, log2F, err);
        pending = 1u;
    }
    uint32_t phases = 0;  // bit st: parity of stage st's next phase
    uint32_t i = 0;
    bool stop = false;
    for (uint32_t c = blockIdx.x; c < chunks; c += gridDim.x, ++i) {
        const uint32_t s = i & 1u;
        unsigned char *stage = smem + s * RB_STAGE_BYTES;
        // the next chunk's copies go to the other stage, read last iteration
        if (threadIdx.x == 0 && c + gridDim.x < chunks) {
            rb_issue(c + gridDim.x, smem + (s ^ 1u) * RB_STAGE_BYTES, &desc[s ^ 1u], &bar[s ^ 1u], lk, lv, L, pk, pv,
                     P, split, log2seg, log2F, err);
            pending |= 2u >> s;  // bit s ^ 1
        }
        const bool landed = mbar_wait(&bar[s], (phases >> s) & 1u, err);
        if (__syncthreads_or(!landed)) {
            stop = true;
            break;
        }
        phases ^= 1u << s;
        pending &= ~(1u << s);
        const RbDesc d = desc[s];
        if (!d.ok) {
            // bounds-checked build: the chunk is skipped (the error is recorded)
            __syncthreads();
            continue;
        }
        const uint64_t *sl = reinterpret_cast<const uint64_t *>(stage + d.lk_off);
        const uint64_t *sp = reinterpret_cast<const uint64_t *>(stage + d.pk_off);
        const uint8_t *slv = stage + d.lv_off;
        const uint8_t *spv = stage + d.pv_off;
        const uint32_t nl = d.nl, np = d.np, cnt = nl + np;
        const uint32_t ipt = (cnt + BLOCK - 1) / BLOCK;
        const uint32_t e0 = threadIdx.x * ipt;
        if (e0 < cnt) {
            uint32_t lo = e0 > np ? e0 - np : 0, hi = min(e0, nl);
            while (lo < hi) {
                const uint32_t mid = (lo + hi) >> 1;
                if (sp[e0 - mid - 1] < sl[mid])
                    hi = mid;
                else
                    lo = mid + 1;
            }
            uint32_t x = lo, y = e0 - lo;
            const uint32_t end = min(cnt, e0 + ipt);
            for (uint32_t e = e0; e < end; ++e) {
                const bool take_live = x < nl && (y >= np || sl[x] <= sp[y]);
                if (take_live) {
                    mk[e] = sl[x];
                    mv[e] = slv[x];
                    ++x;
                } else {
                    mk[e] = sp[y];
                    mv[e] = spv[y];
                    ++y;
                }
            }
        }
        __syncthreads();
        // slot pairs: round r, thread t writes slots 2 (r * BLOCK + t) and the
        // next one, so a warp's 16-byte key stores are contiguous (512 B) and
        // its 2-byte value stores too; a pair never straddles a segment
#pragma unroll
        for (uint32_t r = 0; r < CHUNK / (2 * BLOCK); ++r) {
            const uint32_t t = 2 * (r * BLOCK + threadIdx.x);
            const uint32_t slot = c * CHUNK + t;
            const uint32_t sg = slot >> log2seg, ln0 = slot & (seg - 1);
            const uint64_t f0 = seg_first(sg, M, log2F), f1 = seg_first(sg + 1, M, log2F);
            const uint32_t have = (uint32_t)(f1 - f0);
            uint64_t k0 = gap_key, k1 = gap_key;
            uint32_t v0 = 0, v1 = 0;
            if (ln0 < have) {
                const uint32_t e = (uint32_t)(f0 + ln0 - d.i_lo);
                k0 = mk[e];
                v0 = mv[e];
            }
            if (ln0 + 1 < have) {
                const uint32_t e = (uint32_t)(f0 + ln0 + 1 - d.i_lo);
                k1 = mk[e];
                v1 = mv[e];
            }
            *reinterpret_cast<ulonglong2 *>(keys + slot) = make_ulonglong2(k0, k1);
            *reinterpret_cast<uint16_t *>(vals + slot) = (uint16_t)(v0 | (v1 << 8));
            if (ln0 == 0)
                heads[sg] = k0;
            if (is_guard(k0) && (uint32_t)(k0 >> 32) < row_num)
                row_offset[(k0 >> 32) + 1] = slot;
            if (is_guard(k1) && (uint32_t)(k1 >> 32) < row_num)
                row_offset[(k1 >> 32) + 1] = slot + 1;
        }
        __syncthreads();  // mk/mv and this stage are reused
    }
    // a stop can leave copies in flight: wait for them (bounded) before the
    // CTA's shared memory is released
    if (stop && threadIdx.x == 0) {
        for (uint32_t st = 0; st < 2; ++st)
            if ((pending >> st) & 1u)
                mbar_wait(&bar[st], (phases >> st) & 1u, err);
    }
}

// keys[0..L) = live, keys[L..size) = KEY_NONE (values 0): the layout
// resize_gpma leaves when the root rebalance that follows it is rejected.
__global__ void compacted_layout_kernel(uint64_t *keys, uint8_t *vals, uint64_t *heads, uint32_t log2seg,
                                        uint32_t size, const uint64_t *lk, const uint8_t *lv, uint32_t L) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < size; t += gridDim.x * blockDim.x) {
        const uint64_t k = t < L ? lk[t] : KEY_NONE;
        keys[t] = k;
        vals[t] = t < L ? lv[t] : 0;
        if ((t & ((1u << log2seg) - 1)) == 0)
            heads[t >> log2seg] = k;
    }
}

__global__ void heads_kernel(const uint64_t *keys, uint64_t *heads, uint32_t segs, uint32_t log2seg) {
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < segs; s += gridDim.x * blockDim.x)
        heads[s] = keys[(size_t)s << log2seg];
}

__global__ void heads_check_kernel(const uint64_t *keys, const uint64_t *heads, uint32_t segs, uint32_t log2seg,
                                   unsigned long long *bad) {
    unsigned long long c = 0;
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < segs; s += gridDim.x * blockDim.x)
        c += heads[s] != keys[(size_t)s << log2seg];
    if (c)
        atomicAdd(bad, c);
}

int grid_for(uint64_t work, int sms, int per_sm) {
    uint64_t g = (work + BLOCK - 1) / BLOCK;
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(g, (uint64_t)sms * per_sm));
}

// resize_gpma + (root rebalance | significant_insert) of one graph.
gpma_status root_rebuild(gpma_graph *g, bool significant, const uint64_t *pend_k, const uint8_t *pend_v,
                         uint32_t pend_n, cudaStream_t s) {
    const uint32_t size = g->geo.size;
    const uint32_t chunks = (size + CHUNK - 1) / CHUNK;
    prof_mark(g, 0, s);
    g->prof.kernel_launches += 2;
    // 1. stable compaction of the live slots (resize_gpma, gpma.cuh:909-915),
    // one pass with a decoupled look-back; the chunk statuses, the total and
    // the error word live in the graph's chunk buffer (u64 words)
    unsigned long long *cst = reinterpret_cast<unsigned long long *>(g->chunk_cnt);
    uint32_t *cerr = reinterpret_cast<uint32_t *>(cst + chunks + 1);
    GPMA_CUDA(cudaMemsetAsync(cst, 0, sizeof(unsigned long long) * (chunks + 2), s));
    {
        int dev = 0;
        GPMA_CUDA(cudaGetDevice(&dev));
        static int fit[64] = {};
        int &f = fit[dev >= 0 && dev < 64 ? dev : 0];
        if (f == 0) {
            GPMA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&f, compact_kernel, BLOCK, CP_SMEM));
            f = std::max(1, std::min(f, MAX_BLOCKS_PER_SM));
        }
        const uint64_t *ck = g->keys;
        const uint8_t *cv = g->values;
        uint32_t csize = size;
        uint64_t *dk = g->skeys;
        uint8_t *dv = g->svals;
        void *args[] = {&ck, &cv, &csize, &dk, &dv, &cst, &cerr};
        const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(chunks, (uint64_t)g->sms * f));
        GPMA_CUDA(cudaLaunchCooperativeKernel((const void *)compact_kernel, dim3(grid), dim3(BLOCK), args, CP_SMEM, s));
    }
    unsigned long long h_cst[2] = {0, 0};  // total, error word
    GPMA_CUDA(cudaMemcpyAsync(h_cst, cst + chunks, sizeof(h_cst), cudaMemcpyDeviceToHost, s));
    GPMA_CUDA(cudaStreamSynchronize(s));
    if ((uint32_t)h_cst[1])
        return device_error("the compaction of the root rebuild", (uint32_t)h_cst[1]);
    const uint32_t live = (uint32_t)h_cst[0];
    // 2. new geometry (gpma.cuh:917-930)
    uint64_t merge = (uint64_t)live + pend_n;
    uint64_t tree_size = 4;
    while (std::floor(UPPER_ROOT * (double)tree_size) < (double)merge) {
        tree_size *= 2;
        if (tree_size > MAX_SLOTS) {
            set_error("GPMA would need more than 2^31 slots (%llu live + %u insertions)", (unsigned long long)live,
                      pend_n);
            return GPMA_ERR_CAPACITY;
        }
    }
    Geometry geo;
    geo.size = (uint32_t)tree_size;
    geo.seg = 1u << (fls32(fls32(geo.size)) - 1);
    geo.height = fls32(geo.size / geo.seg) - 1;
    recalculate_density(geo);
    // 3. storage
    if (geo.size > g->cap) {
        uint64_t *nk = nullptr;
        uint8_t *nv = nullptr;
        GPMA_TRY(dev_alloc(&nk, geo.size));
        gpma_status st = dev_alloc(&nv, geo.size);
        if (st != GPMA_OK) {
            dev_free(nk);
            return st;
        }
        dev_free(g->keys);
        dev_free(g->values);
        g->keys = nk;
        g->values = nv;
        g->cap = geo.size;
    }
    const uint32_t log2seg = fls32(geo.seg) - 1;
    const uint32_t log2F = fls32(geo.size) - 1 - log2seg;
    const uint32_t out_chunks = (geo.size + CHUNK - 1) / CHUNK;
    // the rebuild kernels write the segment heads of the new geometry
    if ((geo.size >> log2seg) > g->heads_cap || !g->heads) {
        dev_free(g->heads);
        g->heads_cap = 0;
        GPMA_TRY(dev_alloc(&g->heads, geo.size >> log2seg));
        g->heads_cap = geo.size >> log2seg;
    }
    const int rgrid = grid_for((uint64_t)out_chunks * BLOCK, g->sms, 4);
    const size_t rsmem = 2ull * CHUNK * 9;  // staged sources + merged chunk
    // merge splits at every chunk boundary of the new array: the chunk counts
    // of the compaction are spent, so their buffer holds them (grown if the
    // array grew)
    if ((uint64_t)out_chunks + 2 > g->chunk_words) {
        dev_free(g->chunk_cnt);
        g->chunk_words = 0;
        GPMA_TRY(dev_alloc(&g->chunk_cnt, 2ull * (out_chunks + 2) + 4));
        g->chunk_words = 2ull * (out_chunks + 2) + 4;
    }
    uint32_t *split = g->chunk_cnt;
    // the error word of the rebuild (after the splits): bounded waits, and
    // the bounds-checked build's checks
    uint32_t *rebuild_err = g->chunk_cnt + out_chunks + 1;
    GPMA_CUDA(cudaMemsetAsync(rebuild_err, 0, sizeof(uint32_t), s));
    // arrays of RB_MIN_SLOTS slots or more stage each chunk's sources by bulk
    // copies (double-buffered); smaller ones take rebuild_kernel
    auto rebuild = [&](uint64_t gap) -> gpma_status {
        if (geo.size >= RB_MIN_SLOTS) {
            static bool attr_set[64] = {};
            int dev = 0;
            GPMA_CUDA(cudaGetDevice(&dev));
            if (!attr_set[dev >= 0 && dev < 64 ? dev : 0]) {
                GPMA_CUDA(cudaFuncSetAttribute(rebuild_bulk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)RB_SMEM));
                attr_set[dev >= 0 && dev < 64 ? dev : 0] = true;
            }
            const int grid = (int)std::min<uint64_t>((uint64_t)out_chunks, (uint64_t)g->sms * 4);
            rebuild_bulk_kernel<<<grid, BLOCK, RB_SMEM, s>>>(g->keys, g->values, g->heads, g->row_offset, g->row_num,
                                                             geo.size, log2seg, log2F, g->skeys, g->svals, live,
                                                             pend_k, pend_v, pend_n, split, gap, rebuild_err);
        } else {
            rebuild_kernel<<<rgrid, BLOCK, rsmem, s>>>(g->keys, g->values, g->heads, g->row_offset, g->row_num,
                                                        geo.size, log2seg, log2F, g->skeys, g->svals, live, pend_k,
                                                        pend_v, pend_n, split, gap, rebuild_err);
        }
        GPMA_CUDA(cudaGetLastError());
        g->prof.kernel_launches += 1;
        return GPMA_OK;
    };
    auto splits = [&]() {
        merge_split_kernel<<<grid_for((uint64_t)out_chunks + 1, g->sms, 8), BLOCK, 0, s>>>(
            g->skeys, live, pend_k, pend_n, geo.size, log2seg, log2F, split);
        g->prof.kernel_launches += 1;
    };
    if (significant) {
        // significant_insert: everything redispatched, gaps are key 0 / value 0
        splits();
        GPMA_TRY(rebuild(0ull));
        g->stats.significant++;
        g->stats.accepted_windows++;
        g->stats.accepted_slots += geo.size;
    } else {
        const uint32_t h = geo.height;
        if (geo.lower[h] <= merge && merge <= geo.upper[h]) {
            splits();
            GPMA_TRY(rebuild(KEY_NONE));
            g->stats.accepted_windows++;
            g->stats.accepted_slots += geo.size;
        } else {
            // the reference drops the insertions and keeps the compacted array
            compacted_layout_kernel<<<grid_for(geo.size, g->sms, 8), BLOCK, 0, s>>>(
                g->keys, g->values, g->heads, log2seg, geo.size, g->skeys, g->svals, live);
            g->stats.root_drops++;
        }
        g->stats.root_resizes++;
    }
    GPMA_CUDA(cudaGetLastError());
    g->geo = geo;
    prof_mark(g, 1, s);
    GPMA_CUDA(cudaStreamSynchronize(s));
    g->prof.rebuild_ms += prof_elapsed(g, 0, 1);
    {
        uint32_t e = 0;
        GPMA_CUDA(cudaMemcpy(&e, rebuild_err, sizeof(e), cudaMemcpyDeviceToHost));
        if (e)
            return device_error("the bulk rebuild", e);
    }
    // the scratch must cover the whole array for later wide windows
    GPMA_TRY(ensure_scratch(g, geo.size));
    return GPMA_OK;
}

GraphDesc describe(const gpma_graph *g) {
    GraphDesc d{};
    d.keys = g->keys;
    d.vals = g->values;
    d.row_offset = g->row_offset;
    d.skeys = g->skeys;
    d.svals = g->svals;
    d.heads = g->heads;
    d.row_num = g->row_num;
    d.size = g->geo.size;
    d.seg = g->geo.seg;
    d.log2seg = fls32(g->geo.seg) - 1;
    d.height = g->geo.height;
    for (uint32_t i = 0; i <= g->geo.height && i < MAX_LEVELS; ++i) {
        d.lower[i] = g->geo.lower[i];
        d.upper[i] = g->geo.upper[i];
    }
    return d;
}

int g_update_fit[64][2] = {};  // resident CTAs per SM of the two variants, per device

// The variant for a launch of n keys: the tuned CTAs per SM (3 or more
// selects the 3-CTA build), or when left to the library (0) the 3-CTA build
// for launches of at least AUTO_WIDE_KEYS keys.
constexpr uint64_t AUTO_WIDE_KEYS = 1u << 20;
int update_variant(uint64_t n) {
    const uint32_t t = g_tuning.update_blocks_per_sm;
    return t >= 3 || (t == 0 && n >= AUTO_WIDE_KEYS) ? 1 : 0;
}

const void *update_kernel_ptr(int variant) {
    return variant ? (const void *)update_kernel<3> : (const void *)update_kernel<2>;
}

}  // namespace

gpma_status refresh_heads(gpma_graph *g, cudaStream_t s) {
    const uint32_t log2seg = fls32(g->geo.seg) - 1;
    const uint32_t segs = g->geo.size >> log2seg;
    if (segs > g->heads_cap || !g->heads) {
        dev_free(g->heads);
        g->heads_cap = 0;
        GPMA_TRY(dev_alloc(&g->heads, segs));
        g->heads_cap = segs;
    }
    heads_kernel<<<grid_for(segs, g->sms, 8), BLOCK, 0, s>>>(g->keys, g->heads, segs, log2seg);
    GPMA_CUDA(cudaGetLastError());
    g->prof.kernel_launches += 1;
    return GPMA_OK;
}

gpma_status count_bad_heads(gpma_graph *g, cudaStream_t s, uint64_t *bad) {
    const uint32_t log2seg = fls32(g->geo.seg) - 1;
    const uint32_t segs = g->geo.size >> log2seg;
    unsigned long long *d = nullptr;
    GPMA_TRY(dev_alloc(&d, 1));
    gpma_status st = [&]() -> gpma_status {
        GPMA_CUDA(cudaMemsetAsync(d, 0, sizeof(*d), s));
        heads_check_kernel<<<grid_for(segs, g->sms, 8), BLOCK, 0, s>>>(g->keys, g->heads, segs, log2seg, d);
        GPMA_CUDA(cudaGetLastError());
        unsigned long long h = 0;
        GPMA_CUDA(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s));
        GPMA_CUDA(cudaStreamSynchronize(s));
        *bad = h;
        return GPMA_OK;
    }();
    dev_free(d);
    return st;
}

Tuning g_tuning;
TestHooks g_test_hooks;

int update_grid_size(int sms, uint64_t n) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64)
        dev = 0;
    const int v = update_variant(n);
    if (g_update_fit[dev][v] == 0) {
        const void *k = update_kernel_ptr(v);
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)UPDATE_SMEM) != cudaSuccess)
            return 0;
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, BLOCK, UPDATE_SMEM) != cudaSuccess)
            return 0;
        g_update_fit[dev][v] = std::min(per_sm, MAX_BLOCKS_PER_SM);
    }
    return sms * blocks_per_sm(g_update_fit[dev][v], g_tuning.update_blocks_per_sm);
}

gpma_status ensure_scratch(gpma_graph *g, uint32_t slots) {
    if (slots <= g->scratch_cap && g->skeys)
        return GPMA_OK;
    dev_free(g->skeys);
    dev_free(g->svals);
    dev_free(g->chunk_cnt);
    g->scratch_cap = 0;
    // at least 64 slots: both arrays are whole 16-byte units (bulk copies of
    // ranges widened to 16-byte bounds stay inside them)
    GPMA_TRY(dev_alloc(&g->skeys, std::max<uint32_t>(slots, 64)));
    GPMA_TRY(dev_alloc(&g->svals, std::max<uint32_t>(slots, 64)));
    // u64 compaction statuses (chunks + 2), or u32 merge splits
    g->chunk_words = 2ull * (slots / CHUNK + 2) + 4;
    GPMA_TRY(dev_alloc(&g->chunk_cnt, g->chunk_words));
    g->scratch_cap = slots;
    return GPMA_OK;
}

void free_buffers(BatchBuffers &b) {
    for (int i = 0; i < 2; ++i) {
        dev_free(b.bkeys[i]);
        dev_free(b.bvals[i]);
        dev_free(b.ikeys[i]);
        dev_free(b.ivals[i]);
        dev_free(b.wnode[i]);
        dev_free(b.wgraph[i]);
        dev_free(b.wa[i]);
        dev_free(b.wb[i]);
    }
    dev_free(b.leaf);
    dev_free(b.rkeys);
    dev_free(b.rvals);
    dev_free(b.ileaf);
    dev_free(b.igraph);
    dev_free(b.wflag);
    dev_free(b.wlive);
    dev_free(b.sort_tiles);
    dev_free(b.top);
    dev_free(b.sort_status);
    dev_free(b.sort_hist);
    dev_free(b.qcnt);
    dev_free(b.qinfo);
    dev_free(b.qrec);
    dev_free(b.qbound);
    dev_free(b.d_tab);
    dev_free(b.d_stat);
    dev_free(b.chunk_cnt);
    dev_free(b.cta_cnt);
    if (b.h_tab)
        cudaFreeHost(b.h_tab);
    if (b.h_stat)
        cudaFreeHost(b.h_stat);
    b.h_tab = nullptr;
    b.h_stat = nullptr;
    b.gd = nullptr;
    b.boff = b.toff = b.qoff = b.qtoff = nullptr;
    b.stat_slot = 0;
    b.dirty = true;
    b.cap = 0;
    b.gcap = 0;
    b.hist_cap = 0;
    b.chunk_cap = 0;
    b.sort_status_cap = 0;
    b.q_cap = 0;
    b.qrec_cap = 0;
    b.qbound_cap = 0;
    b.tab_shadow_valid = false;
}

gpma_status ensure_buffers(BatchBuffers &b, uint64_t n, uint32_t graphs) {
    if (!b.sort_tiles) {
        GPMA_TRY(dev_alloc(&b.sort_tiles, 8));
        b.dirty = true;
    }
    if (!b.top)
        GPMA_TRY(dev_alloc(&b.top, LOCATE_CACHE));
    if (n > b.cap || !b.bkeys[0]) {
        // a multiple of 16 entries: every buffer is a whole number of 16-byte
        // units, so a bulk copy of a range widened to 16-byte bounds stays inside
        uint64_t cap = (std::max<uint64_t>(n, 1024) + 15) & ~uint64_t(15);
        for (int i = 0; i < 2; ++i) {
            dev_free(b.bkeys[i]);
            dev_free(b.bvals[i]);
            dev_free(b.ikeys[i]);
            dev_free(b.ivals[i]);
            dev_free(b.wnode[i]);
            dev_free(b.wgraph[i]);
            dev_free(b.wa[i]);
            dev_free(b.wb[i]);
        }
        dev_free(b.leaf);
        dev_free(b.rkeys);
        dev_free(b.rvals);
        dev_free(b.ileaf);
        dev_free(b.igraph);
        dev_free(b.wflag);
        dev_free(b.wlive);
        b.cap = 0;
        for (int i = 0; i < 2; ++i) {
            GPMA_TRY(dev_alloc(&b.bkeys[i], cap));
            GPMA_TRY(dev_alloc(&b.bvals[i], cap));
            GPMA_TRY(dev_alloc(&b.ikeys[i], cap));
            GPMA_TRY(dev_alloc(&b.ivals[i], cap));
            GPMA_TRY(dev_alloc(&b.wnode[i], cap));
            GPMA_TRY(dev_alloc(&b.wgraph[i], cap));
            GPMA_TRY(dev_alloc(&b.wa[i], cap));
            GPMA_TRY(dev_alloc(&b.wb[i], cap));
        }
        GPMA_TRY(dev_alloc(&b.leaf, cap));
        GPMA_TRY(dev_alloc(&b.rkeys, cap));
        GPMA_TRY(dev_alloc(&b.rvals, cap));
        GPMA_TRY(dev_alloc(&b.ileaf, cap));
        GPMA_TRY(dev_alloc(&b.igraph, cap));
        GPMA_TRY(dev_alloc(&b.wflag, 2 * cap));  // one array per level parity
        GPMA_TRY(dev_alloc(&b.wlive, cap));
        b.cap = cap;
        // the bucket sort's buffers grow with the batch buffers, so a served
        // round does not meet a first allocation later (a launch of n keys over
        // k graphs uses at most n/16 + k buckets and n/1024 + k items)
        const uint64_t gq = std::max<uint32_t>(graphs, std::max<uint32_t>(b.gcap, 1));
        dev_free(b.qrec);
        dev_free(b.qcnt);
        dev_free(b.qinfo);
        dev_free(b.qbound);
        b.qrec_cap = b.q_cap = b.qbound_cap = 0;
        GPMA_TRY(dev_alloc(&b.qrec, 2 * cap));
        b.qrec_cap = cap;
        GPMA_TRY(dev_alloc(&b.qcnt, cap / 16 + 2 * gq + 64));
        GPMA_TRY(dev_alloc(&b.qinfo, cap / 16 + 2 * gq + 64));
        b.q_cap = cap / 16 + 2 * gq + 64;
        GPMA_TRY(dev_alloc(&b.qbound, cap / 1024 + gq + 64));
        b.qbound_cap = cap / 1024 + gq + 64;
        b.dirty = true;  // the new bucket counts are cleared before the next launch
    }
    if (graphs > b.gcap || !b.d_tab) {
        const uint32_t gc = std::max<uint32_t>(graphs, 1);
        dev_free(b.d_tab);
        dev_free(b.d_stat);
        if (b.h_tab)
            cudaFreeHost(b.h_tab);
        if (b.h_stat)
            cudaFreeHost(b.h_stat);
        b.h_tab = b.h_stat = nullptr;
        b.gd = nullptr;
        b.boff = b.toff = b.qoff = b.qtoff = nullptr;
        b.gcap = 0;
        const size_t tab = sizeof(GraphDesc) * gc + 4 * sizeof(uint32_t) * (gc + 1);
        const size_t slot = (STAT_GS_OFFSET + sizeof(GraphStatus) * gc + 255) & ~size_t(255);
        GPMA_TRY(dev_alloc(&b.d_tab, tab));
        GPMA_TRY(dev_alloc(&b.d_stat, 2 * slot));
        cudaError_t e = cudaMallocHost((void **)&b.h_tab, tab);
        if (e == cudaSuccess)
            e = cudaMallocHost((void **)&b.h_stat, slot);
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaMallocHost(update tables)");
        b.gd = reinterpret_cast<GraphDesc *>(b.d_tab);
        b.tab_shadow_valid = false;
        b.boff = reinterpret_cast<uint32_t *>(b.d_tab + sizeof(GraphDesc) * gc);
        b.toff = b.boff + gc + 1;
        b.qoff = b.toff + gc + 1;
        b.qtoff = b.qoff + gc + 1;
        b.stat_slot = slot;
        b.parity = 0;
        b.dirty = true;
        b.gcap = gc;
    }
    return GPMA_OK;
}

gpma_status update_plan(gpma_graph *const *graphs, const uint64_t *off, uint32_t k, BatchBuffers &buf, int sms,
                        bool check_keys, size_t *tab_bytes, KernelLaunch *L, const uint32_t *abort,
                        const uint64_t *in_k, const uint8_t *in_v) {
    static_assert(sizeof(UpdateArgs) <= KernelLaunch::ARG_BYTES, "update arguments exceed the launch record");
    const uint64_t n = off[k];
    if (n >= (1ull << 31)) {
        // insertion offsets carry a flag in bit 31 in the level loop's copy plan
        set_error("update launch of %llu keys: at most 2^31 - 1 keys per launch", (unsigned long long)n);
        return GPMA_ERR_CAPACITY;
    }
    const int grid = update_grid_size(sms, n);
    if (grid == 0) {
        set_error("update kernel cannot be resident");
        return GPMA_ERR_CUDA;
    }
    GPMA_TRY(ensure_buffers(buf, n, k));
    if (!buf.cta_cnt)
        GPMA_TRY(dev_alloc(&buf.cta_cnt, 8ull * sms * MAX_BLOCKS_PER_SM));  // any tuned grid
    // per-graph tables in the pinned staging copy: descriptors, batch offsets,
    // sort tile offsets (the previous launch's upload finished: it synchronised)
    GraphDesc *h_gd = reinterpret_cast<GraphDesc *>(buf.h_tab);
    uint32_t *h_boff = reinterpret_cast<uint32_t *>(buf.h_tab + sizeof(GraphDesc) * buf.gcap);
    uint32_t *h_toff = h_boff + buf.gcap + 1;
    uint32_t max_height = 0, min_height = UINT32_MAX;
    uint64_t chunk_need = 1;
    for (uint32_t i = 0; i < k; ++i) {
        h_gd[i] = describe(graphs[i]);
        max_height = std::max(max_height, graphs[i]->geo.height);
        min_height = std::min(min_height, graphs[i]->geo.height);
        chunk_need += graphs[i]->geo.size / CHUNK + 1;
        if (i > 0 && graphs[i]->geo.seg < graphs[i - 1]->geo.seg) {
            set_error("update_graphs: graphs must be ordered by segment length");
            return GPMA_ERR_INVALID;
        }
    }
    h_toff[0] = 0;
    for (uint32_t i = 0; i <= k; ++i) {
        h_boff[i] = (uint32_t)off[i];
        if (i > 0) {
            const uint64_t ni = off[i] - off[i - 1];
            h_toff[i] = h_toff[i - 1] + (uint32_t)((ni + SORT_TILE - 1) / SORT_TILE);
        }
    }
    // bucket sort: per graph, 2^qlog equal slot ranges (about BSORT_AVG keys
    // each) and one item per BSORT_ITEM keys
    uint32_t *h_qoff = h_toff + buf.gcap + 1;
    uint32_t *h_qtoff = h_qoff + buf.gcap + 1;
    const bool buckets = g_tuning.update_sort == 0 && (uint32_t)grid <= BSORT_MAX_GRID;
    uint64_t nq = 0;
    h_qoff[0] = h_qtoff[0] = 0;
    for (uint32_t i = 0; i < k; ++i) {
        const uint64_t ni = off[i + 1] - off[i];
        const uint32_t rows = graphs[i]->row_num;
        const uint32_t lsize = graphs[i]->geo.size ? fls32(graphs[i]->geo.size) - 1 : 0;  // size: a power of two
        uint32_t qlog = 0;
        while (qlog < lsize && (uint64_t(BSORT_AVG) << qlog) < ni)
            ++qlog;
        h_gd[i].qbits = std::max<uint32_t>(1, fls32(rows > 2 ? rows - 1 : 1));  // columns < 2^qbits
        h_gd[i].qshift = lsize - qlog;
        h_gd[i].qnbm1 = (1u << qlog) - 1;
        nq += ni ? (1ull << qlog) : 0;
        h_qoff[i + 1] = (uint32_t)nq;
        h_qtoff[i + 1] = h_qtoff[i] + (uint32_t)((ni + BSORT_ITEM - 1) / BSORT_ITEM);
    }
    const bool use_buckets = buckets && n > 0 && nq < BSORT_MAX_BUCKETS;
    if (use_buckets && nq > buf.q_cap) {
        dev_free(buf.qcnt);
        dev_free(buf.qinfo);
        buf.q_cap = 0;
        GPMA_TRY(dev_alloc(&buf.qcnt, nq));
        GPMA_TRY(dev_alloc(&buf.qinfo, nq));
        buf.q_cap = nq;
        buf.dirty = true;
    }
    if (use_buckets && n > buf.qrec_cap) {
        dev_free(buf.qrec);
        buf.qrec_cap = 0;
        GPMA_TRY(dev_alloc(&buf.qrec, 2 * buf.cap));  // 16 bytes per key
        buf.qrec_cap = buf.cap;
    }
    if (use_buckets && h_qtoff[k] > buf.qbound_cap) {
        dev_free(buf.qbound);
        buf.qbound_cap = 0;
        GPMA_TRY(dev_alloc(&buf.qbound, h_qtoff[k]));
        buf.qbound_cap = h_qtoff[k];
    }
    const uint32_t tiles = h_toff[k];
    const uint64_t status_words = 8ull * tiles * 256;
    if (status_words > buf.sort_status_cap) {
        dev_free(buf.sort_status);
        GPMA_TRY(dev_alloc(&buf.sort_status, status_words));
        buf.sort_status_cap = status_words;
        buf.dirty = true;
    }
    const uint32_t hist_rows = k == 1 ? 1 : k + 1;
    if (hist_rows > buf.hist_cap) {
        dev_free(buf.sort_hist);
        GPMA_TRY(dev_alloc(&buf.sort_hist, (size_t)hist_rows * 2048));
        buf.hist_cap = hist_rows;
        buf.dirty = true;
    }
    if (chunk_need > buf.chunk_cap) {
        dev_free(buf.chunk_cnt);
        GPMA_TRY(dev_alloc(&buf.chunk_cnt, chunk_need));
        buf.chunk_cap = chunk_need;
    }
    // the upload covers the tables up to the last tile offset in use
    *tab_bytes = reinterpret_cast<unsigned char *>(h_qtoff + k + 1) - buf.h_tab;
    unsigned char *slot = buf.d_stat + buf.parity * buf.stat_slot;
    unsigned char *next = buf.d_stat + (buf.parity ^ 1) * buf.stat_slot;
    UpdateArgs A;
    memset(&A, 0, sizeof(A));  // padding too: launches are compared byte-wise
    A.gd = buf.gd;
    A.gs = reinterpret_cast<GraphStatus *>(slot + STAT_GS_OFFSET);
    A.G = k;
    A.max_height = max_height;
    A.min_height = min_height;
    A.boff = buf.boff;
    A.toff = buf.toff;
    A.n = (uint32_t)n;
    A.in_k = in_k ? in_k : buf.bkeys[0];
    A.in_v = in_v ? in_v : buf.bvals[0];
    for (int i = 0; i < 2; ++i) {
        A.bk[i] = buf.bkeys[i];
        A.bv[i] = buf.bvals[i];
        A.ikeys[i] = buf.ikeys[i];
        A.ivals[i] = buf.ivals[i];
        A.wnode[i] = buf.wnode[i];
        A.wgraph[i] = buf.wgraph[i];
        A.wa[i] = buf.wa[i];
        A.wb[i] = buf.wb[i];
    }
    A.sort_hist = buf.sort_hist;
    A.sort_tiles = buf.sort_tiles;
    A.sort_status = buf.sort_status;
    if (use_buckets) {
        A.q.qoff = buf.qoff;
        A.q.qtoff = buf.qtoff;
        A.q.nq = (uint32_t)nq;
        A.q.qcnt = buf.qcnt;
        A.q.qinfo = reinterpret_cast<unsigned long long *>(buf.qinfo);
        A.q.rank = buf.ileaf;  // both first written after the sort
        A.q.bkt = buf.igraph;
        A.q.rec = reinterpret_cast<uint4 *>(buf.qrec);
        A.q.bound = buf.qbound;
    }
    A.check_keys = check_keys;
    A.leaf = buf.leaf;
    A.rkeys = buf.rkeys;
    A.rvals = buf.rvals;
    A.ileaf = buf.ileaf;
    A.igraph = buf.igraph;
    A.wflag[0] = buf.wflag;
    A.wflag[1] = buf.wflag + buf.cap;
    A.wlive = buf.wlive;
    A.chunk_cnt = buf.chunk_cnt;
    A.cta_cnt = buf.cta_cnt;
    A.st = reinterpret_cast<DeviceStatus *>(slot);
    A.next_slot = reinterpret_cast<uint32_t *>(next);
    A.next_slot_words = (uint32_t)(buf.stat_slot / sizeof(uint32_t));
    A.hist_words = hist_rows * 2048;
    A.status_words = (uint32_t)status_words;
    A.top = buf.top;
    A.abort = abort;
    A.stall = g_test_hooks.update_stall;
    A.stall_limit_ns = g_test_hooks.update_stall ? g_test_hooks.wait_limit_ns : WAIT_LIMIT_NS;
    L->set(update_kernel_ptr(update_variant(n)), grid, UPDATE_SMEM, &A, sizeof(A));
    return GPMA_OK;
}

gpma_status update_clear(BatchBuffers &buf, cudaStream_t s) {
    if (!buf.dirty)
        return GPMA_OK;
    // first launch, new buffers or an aborted launch: clear everything the
    // kernel otherwise leaves zeroed for its successor
    GPMA_CUDA(cudaMemsetAsync(buf.d_stat, 0, 2 * buf.stat_slot, s));
    GPMA_CUDA(cudaMemsetAsync(buf.sort_hist, 0, sizeof(uint32_t) * buf.hist_cap * 2048, s));
    GPMA_CUDA(cudaMemsetAsync(buf.sort_tiles, 0, 8 * sizeof(uint32_t), s));
    GPMA_CUDA(cudaMemsetAsync(buf.sort_status, 0, buf.sort_status_cap * sizeof(uint32_t), s));
    if (buf.q_cap)
        GPMA_CUDA(cudaMemsetAsync(buf.qcnt, 0, buf.q_cap * sizeof(uint32_t), s));
    buf.dirty = false;
    return GPMA_OK;
}

size_t update_status_bytes(uint32_t k) { return STAT_GS_OFFSET + sizeof(GraphStatus) * k; }

gpma_status update_finish(gpma_graph *const *graphs, uint32_t k, BatchBuffers &buf, const unsigned char *stat,
                          cudaStream_t s, gpma_profile *prof, double kernel_ms) {
    buf.parity ^= 1;
    const DeviceStatus &h = *reinterpret_cast<const DeviceStatus *>(stat);
    const GraphStatus *h_gs = reinterpret_cast<const GraphStatus *>(stat + STAT_GS_OFFSET);
    if (h.err || h.invalid_keys)
        buf.dirty = true;  // the kernel stopped before (or during) its clean-up
    if (prof) {
        prof->kernel_launches += 1;  // the sort runs inside the update kernel
        prof->update_kernels++;
        prof->update_kernel_ms += kernel_ms;
        // phase split from the kernel's own timeline (stamps of an early exit stay 0)
        const unsigned long long *t = h.stamp;
        auto span = [&](int a, int b) { return (t[a] && t[b] && t[b] >= t[a]) ? (t[b] - t[a]) * 1e-6 : 0.0; };
        prof->sort_ms += span(0, 1);
        prof->locate_ms += span(1, 2);
        prof->group_ms += span(2, 3);
        prof->levels_ms += span(3, 4);
        prof->sort_fallbacks += h.sort_fallback != 0;
    }
    if (h.invalid_keys) {
        set_error("update batch holds keys whose column is 0xFFFFFFFF (reserved for row guards and empty slots)");
        return GPMA_ERR_INVALID;
    }
    if (h.err)
        return device_error("the update kernel", h.err);
    for (uint32_t i = 0; i < k; ++i) {
        gpma_graph *g = graphs[i];
        const GraphStatus &gs = h_gs[i];
        const uint32_t inserts = gs.inserts ? gs.inserts - gs.ins_base : 0;  // end - first
        g->stats.last_inserts = h.significant ? h.inserts : inserts;
        g->stats.levels_visited += h.levels;
        if (k == 1) {
            g->stats.accepted_windows += h.accepted_windows;
            g->stats.accepted_slots += h.accepted_slots;
        }
    }
    if (h.significant)
        return root_rebuild(graphs[0], true, buf.ikeys[0], buf.ivals[0], h.inserts, s);
    for (uint32_t i = 0; i < k; ++i) {
        const GraphStatus &gs = h_gs[i];
        if (gs.remaining > 0)
            GPMA_TRY(root_rebuild(graphs[i], false, buf.rkeys + gs.ins_base, buf.rvals + gs.ins_base, gs.remaining,
                                  s));
    }
    return GPMA_OK;
}

bool update_needs_host(const unsigned char *stat, uint32_t k) {
    const DeviceStatus &h = *reinterpret_cast<const DeviceStatus *>(stat);
    const GraphStatus *h_gs = reinterpret_cast<const GraphStatus *>(stat + STAT_GS_OFFSET);
    if (h.err || h.invalid_keys || h.significant)
        return true;
    for (uint32_t i = 0; i < k; ++i)
        if (h_gs[i].remaining > 0)
            return true;
    return false;
}

gpma_status update_graphs(gpma_graph *const *graphs, const uint64_t *off, uint32_t k, BatchBuffers &buf, int sms,
                          cudaStream_t s, bool check_keys, bool profiling, cudaEvent_t *ev, gpma_profile *prof,
                          const uint64_t *in_k, const uint8_t *in_v) {
    if (off[k] == 0)
        return GPMA_OK;
    size_t tab_bytes = 0;
    KernelLaunch L;
    GPMA_TRY(update_plan(graphs, off, k, buf, sms, check_keys, &tab_bytes, &L, nullptr, in_k, in_v));
    // the tables (descriptors, batch and bucket offsets) are the same from
    // one slide step to the next: an identical table is not uploaded again
    if (!buf.tab_shadow_valid || buf.tab_shadow.size() != tab_bytes ||
        memcmp(buf.tab_shadow.data(), buf.h_tab, tab_bytes) != 0) {
        GPMA_CUDA(cudaMemcpyAsync(buf.d_tab, buf.h_tab, tab_bytes, cudaMemcpyHostToDevice, s));
        buf.tab_shadow.assign(buf.h_tab, buf.h_tab + tab_bytes);
        buf.tab_shadow_valid = true;
    }
    GPMA_TRY(update_clear(buf, s));
    prof_mark(profiling, ev, 1, s);
    GPMA_CUDA(L.launch_cooperative(s));
    prof_mark(profiling, ev, 2, s);
    // one read-back: the status and this launch's per-graph results
    GPMA_CUDA(cudaMemcpyAsync(buf.h_stat, buf.d_stat + buf.parity * buf.stat_slot, update_status_bytes(k),
                              cudaMemcpyDeviceToHost, s));
    GPMA_CUDA(cudaStreamSynchronize(s));
    return update_finish(graphs, k, buf, buf.h_stat, s, prof, prof ? prof_elapsed(profiling, ev, 1, 2) : 0.0);
}

// Single-graph update of the n-key batch staged in g->buf.bkeys[0]/bvals[0].
gpma_status update_device(gpma_graph *g, uint64_t n, cudaStream_t s, bool check_keys, const uint64_t *in_k,
                          const uint8_t *in_v) {
    const uint64_t off[2] = {0, n};
    gpma_graph *gs[1] = {g};
    return update_graphs(gs, off, 1, g->buf, g->sms, s, check_keys, g->profiling, g->ev, &g->prof, in_k, in_v);
}

}  // namespace gpma
