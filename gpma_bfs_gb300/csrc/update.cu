// update.cu - GPMA+ batch update on one GB300.
//
// Replaces update_gpma (gpma.cuh:968-1050). After the batch sort (sort.cu)
// one persistent cooperative kernel runs every remaining step on the device,
// separated by bounded grid barriers instead of host round trips:
//   P1 locate: the reference's top-down search over segment first keys, then
//      an equality scan of the leaf with 16-byte loads; hits store the
//      update's value in place (delete/modify/revive, gpma.cuh:188-220);
//   P2 keep the insertions in sorted order (compact_insertions, :836-844);
//   P3 group them by leaf into level-0 windows (group_insertion_by_node,
//      :846-873). A window is (node, [a, b)) into the sorted insertions;
//   level loop (:1012-1029): each window of width W = seg << level counts its
//      live slots, is accepted iff lower <= live + pending <= upper, and an
//      accepted window is rewritten as the stable merge of its live entries
//      and its insertions, redispatched evenly (:636-654) in one coalesced
//      pass. Rejected windows whose parents coincide merge into one parent
//      window (their insertion ranges are adjacent), so insertions are never
//      moved between levels. Windows up to 256 slots go to warp groups, up to
//      2048 slots to one CTA in shared memory, wider ones to the whole grid.
// The host reads one status block at the end. Only the root resize
// (:1034-1044) and the >= 5M-insertion rebuild (:936-966) run host-driven.
#include "gpma_internal.cuh"
#include "sort.cuh"

#include <algorithm>
#include <cmath>

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
    uint64_t *keys;
    uint8_t *vals;
    uint32_t *row_offset;
    uint32_t row_num;
    uint32_t size, seg, log2seg, height;
    const uint32_t *lower;
    const uint32_t *upper;
    uint64_t *bk[2];  // batch, ping-pong buffers of the radix sort (input in [0])
    uint8_t *bv[2];
    uint32_t *sort_hist;    // 8 x 256 digit counts (zeroed per update)
    uint32_t *sort_tiles;   // 8 tile counters (zeroed per update)
    uint32_t *sort_status;  // look-back words, 8 x tiles x 256 (zeroed per update)
    bool check_keys;
    uint32_t n;
    uint32_t *leaf;
    uint64_t *ikeys[2];
    uint8_t *ivals[2];
    uint32_t *ileaf;
    uint32_t *wnode[2];
    uint32_t *wa[2];
    uint32_t *wb[2];
    uint32_t *wflag;
    uint32_t *wlive;
    uint64_t *skeys;
    uint8_t *svals;
    uint32_t *chunk_cnt;
    uint32_t *cta_cnt;
    DeviceStatus *st;
};

// ---- P1: locate ------------------------------------------------------------

// The top levels of the descent read segment first keys at multiples of
// `stride` slots; each CTA copies those (at most LOCATE_CACHE of them) into
// shared memory once, so a key walks the upper levels in shared memory and
// only the last log2(stride/seg) levels in HBM. The comparisons and their
// order are the reference's bit-by-bit descent (gpma.cuh:209-216).
constexpr uint32_t LOCATE_CACHE = 4096;

__device__ __forceinline__ uint32_t locate_one(const UpdateArgs &A, uint64_t key, uint8_t value, const uint64_t *fk,
                                               uint32_t log2stride) {
    const uint32_t seg = A.seg;
    const uint32_t stride = 1u << log2stride;
    uint32_t prefix = 0;
    uint32_t bit = (seg << A.height) >> 1;
    while (stride <= bit) {
        if (fk[(prefix | bit) >> log2stride] <= key)
            prefix |= bit;
        bit >>= 1;
    }
    while (seg <= bit) {
        if (A.keys[prefix | bit] <= key)
            prefix |= bit;
        bit >>= 1;
    }
    uint32_t leaf = value == 0 ? SIZE_NONE : prefix;
    // first equal key of the leaf (handle_del_mod scans all seg slots)
    const ulonglong2 *p = reinterpret_cast<const ulonglong2 *>(A.keys + prefix);
    for (uint32_t j = 0; j < (seg >> 1); ++j) {
        ulonglong2 q = p[j];
        uint32_t hit = q.x == key ? 2 * j : (q.y == key ? 2 * j + 1 : SIZE_NONE);
        if (hit != SIZE_NONE) {
            A.vals[prefix + hit] = value;
            leaf = SIZE_NONE;
            break;
        }
    }
    return leaf;
}

// ---- grid-wide exclusive scan helpers ------------------------------------
// CTA b owns items [lo, hi) of a contiguous split of [0, N).
__device__ __forceinline__ void cta_range(uint32_t N, uint32_t &lo, uint32_t &hi) {
    uint32_t per = (N + gridDim.x - 1) / gridDim.x;
    lo = min(N, blockIdx.x * per);
    hi = min(N, lo + per);
}

// Sum of cnt[0..blockIdx.x) and of cnt[0..gridDim.x).
__device__ __forceinline__ void cta_prefix(const uint32_t *cnt, uint32_t &base, uint32_t &total, uint32_t *tmp) {
    uint32_t a = 0, t = 0;
    for (uint32_t j = threadIdx.x; j < gridDim.x; j += BLOCK) {
        uint32_t c = ld_volatile(cnt + j);
        t += c;
        if (j < blockIdx.x)
            a += c;
    }
    base = block_sum(a, tmp);
    total = block_sum(t, tmp);
}

// ---- redispatch of a chunk of a window ------------------------------------
// Writes slots [t0, t0+len) of the window at `node` (width F << log2seg): slot
// (s, lane) gets element first(s)+lane of the stable merge of live[0..L) and
// pend[0..P) (ties: live first), or gap_key/0 if the segment holds fewer.
// len is a multiple of the segment length; mk/mv hold len entries.
__device__ void redispatch_chunk(uint64_t *keys, uint8_t *vals, uint32_t *row_offset, uint32_t row_num, uint32_t node,
                                 uint32_t log2seg, uint32_t log2F, uint32_t t0, uint32_t len, const uint64_t *lk,
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
__device__ void warp_windows(const UpdateArgs &A, const uint32_t *wn, const uint32_t *wa, const uint32_t *wb,
                             uint32_t nw, uint32_t lo, uint32_t hi, const uint64_t *pk, const uint8_t *pv,
                             unsigned char *smem, unsigned long long &acc) {
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
    const uint32_t seg_mask = A.seg - 1, log2seg = A.log2seg;
    const uint32_t log2F = (31 - __clz(W)) - log2seg;
    const uint32_t total_warps = gridDim.x * (BLOCK / 32);
    for (uint32_t wbase = (blockIdx.x * (BLOCK / 32) + warp) * GPW; wbase < nw; wbase += total_warps * GPW) {
        const uint32_t w = wbase + grp;
        const bool has = w < nw;
        const uint32_t node = has ? wn[w] : 0, a = has ? wa[w] : 0, b = has ? wb[w] : 0;
        const uint32_t t0 = node + gl * K;
        uint64_t k[K];
        uint8_t v[K];
        uint32_t c_l = 0;
        if (has) {
            load_slots<K>(A.keys, A.vals, t0, k, v);
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
            for (uint32_t j = gl; j < p; j += G) {
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
                if (is_guard(k[j])) {
                    const uint32_t row = (uint32_t)(k[j] >> 32);
                    if (row < A.row_num)
                        A.row_offset[row + 1] = node + t;
                }
            }
            store_slots<K>(A.keys, A.vals, t0, k, v);
            if (gl == 0)
                ++acc;
        }
        if (has && gl == 0)
            A.wflag[w] = accept ? 1u : 0u;
        __syncwarp();
    }
}

// ---- windows of 512..CTA_WINDOW_MAX slots: one CTA each ---------------------
template <uint32_t W>
__device__ void cta_windows(const UpdateArgs &A, const uint32_t *wn, const uint32_t *wa, const uint32_t *wb,
                            uint32_t nw, uint32_t lo, uint32_t hi, const uint64_t *pk, const uint8_t *pv,
                            unsigned char *smem, uint32_t *tmp, unsigned long long &acc) {
    constexpr uint32_t K = W / BLOCK;
    uint64_t *sk = reinterpret_cast<uint64_t *>(smem);
    uint64_t *ck = sk + W;
    uint64_t *mk = ck + W;
    uint8_t *sv = reinterpret_cast<uint8_t *>(mk + W);
    uint8_t *cv = sv + W;
    uint8_t *mv = cv + W;
    const uint32_t tid = threadIdx.x;
    const uint32_t seg_mask = A.seg - 1, log2seg = A.log2seg;
    const uint32_t log2F = (31 - __clz(W)) - log2seg;
    for (uint32_t w = blockIdx.x; w < nw; w += gridDim.x) {
        const uint32_t node = wn[w], a = wa[w], b = wb[w];
#pragma unroll
        for (uint32_t j = 0; j < K; ++j) {
            uint32_t t = tid + j * BLOCK;
            sk[t] = A.keys[node + t];
            sv[t] = A.vals[node + t];
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
                A.keys[node + t] = k;
                A.vals[node + t] = v;
                if (is_guard(k)) {
                    uint32_t row = (uint32_t)(k >> 32);
                    if (row < A.row_num)
                        A.row_offset[row + 1] = node + t;
                }
            }
            if (tid == 0)
                ++acc;
        }
        if (tid == 0)
            A.wflag[w] = accept ? 1u : 0u;
        __syncthreads();
    }
}

// ---- windows wider than one CTA: the whole grid, chunk by chunk -------------
__device__ bool grid_windows(const UpdateArgs &A, const uint32_t *wn, const uint32_t *wa, const uint32_t *wb,
                             uint32_t nw, uint32_t W, uint32_t lo, uint32_t hi, const uint64_t *pk,
                             const uint8_t *pv, unsigned char *smem, uint32_t *tmp, unsigned long long &acc) {
    const uint32_t cpw = W / CHUNK;
    const uint32_t total = nw * cpw;
    constexpr uint32_t K = CHUNK / BLOCK;
    // B1: live count of every chunk
    for (uint32_t c = blockIdx.x; c < total; c += gridDim.x) {
        uint32_t w = c / cpw, k = c % cpw;
        uint32_t base = wn[w] + k * CHUNK + threadIdx.x * K;
        uint32_t cl = 0;
#pragma unroll
        for (uint32_t j = 0; j < K; ++j)
            cl += (A.keys[base + j] != KEY_NONE && A.vals[base + j] != 0);
        uint32_t t = block_sum(cl, tmp);
        if (threadIdx.x == 0)
            A.chunk_cnt[c] = t;
    }
    if (!grid_barrier(&A.st->bar, &A.st->err))
        return false;
    // B2: per window, chunk offsets, live total and the density decision
    for (uint32_t w = blockIdx.x; w < nw; w += gridDim.x) {
        uint32_t run = 0;
        for (uint32_t k0 = 0; k0 < cpw; k0 += BLOCK) {
            uint32_t k = k0 + threadIdx.x;
            uint32_t v = k < cpw ? A.chunk_cnt[w * cpw + k] : 0;
            uint32_t tot;
            uint32_t ex = block_excl_scan(v, &tot, tmp);
            if (k < cpw)
                A.chunk_cnt[w * cpw + k] = run + ex;
            run += tot;
        }
        uint32_t M = run + (wb[w] - wa[w]);
        bool accept = lo <= M && M <= hi;
        if (threadIdx.x == 0) {
            A.wflag[w] = accept ? 1u : 0u;
            A.wlive[w] = run;
            if (accept)
                ++acc;
        }
    }
    if (!grid_barrier(&A.st->bar, &A.st->err))
        return false;
    // B3: stable compaction of accepted windows into the scratch arrays
    for (uint32_t c = blockIdx.x; c < total; c += gridDim.x) {
        uint32_t w = c / cpw, k = c % cpw;
        if (!A.wflag[w])
            continue;
        uint32_t node = wn[w];
        uint32_t base = node + k * CHUNK + threadIdx.x * K;
        uint64_t kk[K];
        uint8_t vv[K];
        uint32_t cl = 0;
#pragma unroll
        for (uint32_t j = 0; j < K; ++j) {
            kk[j] = A.keys[base + j];
            vv[j] = A.vals[base + j];
            cl += (kk[j] != KEY_NONE && vv[j] != 0);
        }
        uint32_t tot;
        uint32_t o = node + A.chunk_cnt[c] + block_excl_scan(cl, &tot, tmp);
#pragma unroll
        for (uint32_t j = 0; j < K; ++j) {
            if (kk[j] != KEY_NONE && vv[j] != 0) {
                A.skeys[o] = kk[j];
                A.svals[o] = vv[j];
                ++o;
            }
        }
    }
    if (!grid_barrier(&A.st->bar, &A.st->err))
        return false;
    // B4: merge with the window's insertions and redispatch chunk by chunk
    uint64_t *mk = reinterpret_cast<uint64_t *>(smem);
    uint8_t *mv = reinterpret_cast<uint8_t *>(mk + CHUNK);
    const uint32_t log2F = (31 - __clz(W)) - A.log2seg;
    for (uint32_t c = blockIdx.x; c < total; c += gridDim.x) {
        uint32_t w = c / cpw, k = c % cpw;
        if (!A.wflag[w])
            continue;
        uint32_t node = wn[w], a = wa[w];
        redispatch_chunk(A.keys, A.vals, A.row_offset, A.row_num, node, A.log2seg, log2F, k * CHUNK, CHUNK,
                         A.skeys + node, A.svals + node, A.wlive[w], pk + a, pv + a, wb[w] - a, KEY_NONE,
                         mk, mv);
    }
    return true;
}

template <uint32_t W>
__device__ __forceinline__ void small_dispatch(const UpdateArgs &A, const uint32_t *wn, const uint32_t *wa,
                                               const uint32_t *wb, uint32_t nw, uint32_t lo, uint32_t hi,
                                               const uint64_t *pk, const uint8_t *pv, unsigned char *smem,
                                               uint32_t *tmp, unsigned long long &acc) {
    if constexpr (W <= WARP_WINDOW_MAX)
        warp_windows<W>(A, wn, wa, wb, nw, lo, hi, pk, pv, smem, acc);
    else
        cta_windows<W>(A, wn, wa, wb, nw, lo, hi, pk, pv, smem, tmp, acc);
}

// Minimum resident CTAs per SM the register allocation must allow (build
// option; 2 keeps every path spill-free).
#ifndef GPMA_UPDATE_MIN_BLOCKS
#define GPMA_UPDATE_MIN_BLOCKS 2
#endif

__global__ void __launch_bounds__(BLOCK, GPMA_UPDATE_MIN_BLOCKS) update_kernel(UpdateArgs A) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint32_t tmp[BLOCK / 32 + 1];
    DeviceStatus *st = A.st;

    // S: stable radix sort of the batch (gpma.cuh:977); digit passes are
    // separated by grid barriers, constant digits skipped.
    sort_histogram(A.bk[0], A.n, A.sort_hist, st, A.check_keys, reinterpret_cast<uint32_t *>(smem));
    if (!grid_barrier(&st->bar, &st->err))
        return;
    if (ld_volatile(&st->invalid_keys) != 0)
        return;  // reserved-column keys: reject the batch before any change
    uint32_t sel = 0;
    {
        const uint32_t trivial = sort_trivial_mask(A.sort_hist, A.n);
        const uint32_t tiles = (A.n + SORT_TILE - 1) / SORT_TILE;
        __shared__ uint32_t s_tile;
        for (int p = 0; p < 8; ++p) {
            if (trivial & (1u << p))
                continue;
            const uint64_t *ink = sel ? A.bk[1] : A.bk[0];
            const uint8_t *inv = sel ? A.bv[1] : A.bv[0];
            uint64_t *outk = sel ? A.bk[0] : A.bk[1];
            uint8_t *outv = sel ? A.bv[0] : A.bv[1];
            for (;;) {
                if (threadIdx.x == 0)
                    s_tile = atomicAdd(&A.sort_tiles[p], 1u);
                __syncthreads();
                const uint32_t tile = s_tile;
                __syncthreads();
                if (tile >= tiles)
                    break;
                sort_tile(p, tile, ink, inv, outk, outv, A.n, A.sort_hist, A.sort_status, st, smem, tmp);
            }
            sel ^= 1u;
            if (!grid_barrier(&st->bar, &st->err))
                return;
        }
    }
    const uint64_t *bk = sel ? A.bk[1] : A.bk[0];
    const uint8_t *bv = sel ? A.bv[1] : A.bv[0];
    const uint32_t G = gridDim.x;
    uint32_t scan_id = 0;
#define CNT(id) ((id) ? A.cta_cnt + G : A.cta_cnt)
#define CNTI(id) ((id) ? A.cta_cnt + 3 * G : A.cta_cnt + 2 * G)
    unsigned long long acc = 0, acc_slots = 0;

    // P1: locate every update, applying deletes / modifies in place. The top
    // of the descent comes from a shared-memory copy of the first keys at
    // every `stride`-th slot.
    {
        const uint32_t segs = A.size >> A.log2seg;
        const uint32_t cached = segs < LOCATE_CACHE ? segs : LOCATE_CACHE;
        const uint32_t log2stride = (31 - __clz(A.size / cached));
        uint64_t *fk = reinterpret_cast<uint64_t *>(smem);
        for (uint32_t j = threadIdx.x; j < cached; j += BLOCK)
            fk[j] = A.keys[(size_t)j << log2stride];
        __syncthreads();
        for (uint32_t i = blockIdx.x * BLOCK + threadIdx.x; i < A.n; i += G * BLOCK)
            A.leaf[i] = locate_one(A, bk[i], bv[i], fk, log2stride);
        __syncthreads();
    }
    if (!grid_barrier(&st->bar, &st->err))
        return;

    // P2: stable compaction of the insertions.
    uint32_t lo, hi;
    cta_range(A.n, lo, hi);
    {
        uint32_t cl = 0;
        for (uint32_t i = lo + threadIdx.x; i < hi; i += BLOCK)
            cl += A.leaf[i] != SIZE_NONE;
        uint32_t t = block_sum(cl, tmp);
        if (threadIdx.x == 0)
            CNT(scan_id)[blockIdx.x] = t;
    }
    if (!grid_barrier(&st->bar, &st->err))
        return;
    uint32_t base, m;
    cta_prefix(CNT(scan_id), base, m, tmp);
    for (uint32_t i0 = lo; i0 < hi; i0 += BLOCK) {
        uint32_t i = i0 + threadIdx.x;
        uint32_t f = (i < hi && A.leaf[i] != SIZE_NONE) ? 1u : 0u;
        uint32_t tot;
        uint32_t ex = block_excl_scan(f, &tot, tmp);
        if (f) {
            A.ikeys[0][base + ex] = bk[i];
            A.ivals[0][base + ex] = bv[i];
            A.ileaf[base + ex] = A.leaf[i];
        }
        base += tot;
    }
    scan_id ^= 1;
    if (!grid_barrier(&st->bar, &st->err))
        return;
    if (m >= SIGNIFICANT_INSERTS) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            st->significant = 1;
            st->inserts = m;
        }
        return;
    }

    // P3: run-length grouping of the insertions by leaf -> level-0 windows.
    cta_range(m, lo, hi);
    {
        uint32_t cl = 0;
        for (uint32_t j = lo + threadIdx.x; j < hi; j += BLOCK)
            cl += (j == 0 || A.ileaf[j] != A.ileaf[j - 1]);
        uint32_t t = block_sum(cl, tmp);
        if (threadIdx.x == 0)
            CNT(scan_id)[blockIdx.x] = t;
    }
    if (!grid_barrier(&st->bar, &st->err))
        return;
    uint32_t nw;
    cta_prefix(CNT(scan_id), base, nw, tmp);
    for (uint32_t j0 = lo; j0 < hi; j0 += BLOCK) {
        uint32_t j = j0 + threadIdx.x;
        bool in = j < hi;
        uint32_t head = (in && (j == 0 || A.ileaf[j] != A.ileaf[j - 1])) ? 1u : 0u;
        uint32_t tot;
        uint32_t ex = block_excl_scan(head, &tot, tmp);
        if (in) {
            uint32_t e = base + ex;
            if (head) {
                A.wnode[0][e] = A.ileaf[j];
                A.wa[0][e] = j;
            }
            if (j + 1 == m || A.ileaf[j + 1] != A.ileaf[j])
                A.wb[0][e + head - 1] = j + 1;
        }
        base += tot;
    }
    scan_id ^= 1;
    if (!grid_barrier(&st->bar, &st->err))
        return;

    // Level loop. Windows and their pending insertions live in ping-pong
    // buffers selected by `cur`; each window's insertions are the contiguous
    // range [wa, wb) of the current insertion buffer.
    uint32_t cur = 0, level = 0;
    __shared__ uint32_t s_nb[BLOCK], s_src[BLOCK], s_cnt[BLOCK];
    for (; level <= A.height && nw > 0; ++level) {
        const uint32_t W = A.seg << level;
        const uint32_t lob = A.lower[level], hib = A.upper[level];
        const uint32_t *wn = cur ? A.wnode[1] : A.wnode[0];
        const uint32_t *wa = cur ? A.wa[1] : A.wa[0];
        const uint32_t *wb = cur ? A.wb[1] : A.wb[0];
        const uint64_t *pk = cur ? A.ikeys[1] : A.ikeys[0];
        const uint8_t *pv = cur ? A.ivals[1] : A.ivals[0];
        const unsigned long long before = acc;
        switch (W) {
        case 2: small_dispatch<2>(A, wn, wa, wb, nw, lob, hib, pk, pv, smem, tmp, acc); break;
        case 4: small_dispatch<4>(A, wn, wa, wb, nw, lob, hib, pk, pv, smem, tmp, acc); break;
        case 8: small_dispatch<8>(A, wn, wa, wb, nw, lob, hib, pk, pv, smem, tmp, acc); break;
        case 16: small_dispatch<16>(A, wn, wa, wb, nw, lob, hib, pk, pv, smem, tmp, acc); break;
        case 32: small_dispatch<32>(A, wn, wa, wb, nw, lob, hib, pk, pv, smem, tmp, acc); break;
        case 64: small_dispatch<64>(A, wn, wa, wb, nw, lob, hib, pk, pv, smem, tmp, acc); break;
        case 128: small_dispatch<128>(A, wn, wa, wb, nw, lob, hib, pk, pv, smem, tmp, acc); break;
        case 256: small_dispatch<256>(A, wn, wa, wb, nw, lob, hib, pk, pv, smem, tmp, acc); break;
        case 512: small_dispatch<512>(A, wn, wa, wb, nw, lob, hib, pk, pv, smem, tmp, acc); break;
        case 1024: small_dispatch<1024>(A, wn, wa, wb, nw, lob, hib, pk, pv, smem, tmp, acc); break;
        case 2048: small_dispatch<2048>(A, wn, wa, wb, nw, lob, hib, pk, pv, smem, tmp, acc); break;
        default:
            if (!grid_windows(A, wn, wa, wb, nw, W, lob, hib, pk, pv, smem, tmp, acc))
                return;
        }
        acc_slots += (acc - before) * (unsigned long long)W;
        if (!grid_barrier(&st->bar, &st->err))
            return;
        // Next level. Rejected windows keep their insertions, which are
        // compacted into the other buffer (new offsets from one scan over the
        // windows, as compact_insertions does over insertions, gpma.cuh:1022);
        // a rejected right sibling joins its rejected left sibling in the
        // parent window (up_level, gpma.cuh:881-889 + regrouping).
        const uint32_t nxt = cur ^ 1;
        uint32_t *nwn = nxt ? A.wnode[1] : A.wnode[0];
        uint32_t *nwa = nxt ? A.wa[1] : A.wa[0];
        uint32_t *nwb = nxt ? A.wb[1] : A.wb[0];
        uint64_t *nk = nxt ? A.ikeys[1] : A.ikeys[0];
        uint8_t *nv = nxt ? A.ivals[1] : A.ivals[0];
        cta_range(nw, lo, hi);
        {
            uint32_t ch = 0, ci = 0;
            for (uint32_t w = lo + threadIdx.x; w < hi; w += BLOCK) {
                if (A.wflag[w])
                    continue;
                ci += wb[w] - wa[w];
                uint32_t par = wn[w] & ~W;
                bool merged = w > 0 && !A.wflag[w - 1] && (wn[w - 1] & ~W) == par;
                ch += merged ? 0u : 1u;
            }
            uint32_t th = block_sum(ch, tmp);
            uint32_t ti = block_sum(ci, tmp);
            if (threadIdx.x == 0) {
                CNT(scan_id)[blockIdx.x] = th;
                CNTI(scan_id)[blockIdx.x] = ti;
            }
        }
        if (!grid_barrier(&st->bar, &st->err))
            return;
        uint32_t nw_next, base_i, total_i;
        cta_prefix(CNT(scan_id), base, nw_next, tmp);
        cta_prefix(CNTI(scan_id), base_i, total_i, tmp);
        for (uint32_t w0 = lo; w0 < hi; w0 += BLOCK) {
            const uint32_t w = w0 + threadIdx.x;
            const bool rej = w < hi && !A.wflag[w];
            const uint32_t c = rej ? wb[w] - wa[w] : 0u;
            uint32_t tot_i;
            const uint32_t nb = base_i + block_excl_scan(c, &tot_i, tmp);
            uint32_t head = 0, par = 0;
            if (rej) {
                par = wn[w] & ~W;
                bool merged = w > 0 && !A.wflag[w - 1] && (wn[w - 1] & ~W) == par;
                head = merged ? 0u : 1u;
            }
            uint32_t tot_h;
            const uint32_t ex = block_excl_scan(head, &tot_h, tmp);
            if (head) {
                const uint32_t e = base + ex;
                const bool right = w + 1 < nw && !A.wflag[w + 1] && (wn[w + 1] & ~W) == par;
                nwn[e] = par;
                nwa[e] = nb;
                nwb[e] = nb + c + (right ? wb[w + 1] - wa[w + 1] : 0u);
            }
            s_nb[threadIdx.x] = nb;
            s_src[threadIdx.x] = rej ? wa[w] : 0u;
            s_cnt[threadIdx.x] = c;
            __syncthreads();
            // copy the kept insertions, one warp per window of this tile
            for (uint32_t t = threadIdx.x >> 5; t < BLOCK; t += BLOCK / 32) {
                const uint32_t cc = s_cnt[t], from = s_src[t], to = s_nb[t];
                for (uint32_t e = threadIdx.x & 31; e < cc; e += 32) {
                    nk[to + e] = pk[from + e];
                    nv[to + e] = pv[from + e];
                }
            }
            __syncthreads();
            base += tot_h;
            base_i += tot_i;
        }
        scan_id ^= 1;
        if (!grid_barrier(&st->bar, &st->err))
            return;
        nw = nw_next;
        cur = nxt;
    }

    unsigned long long acc_b = acc;
    // one atomic per CTA for the statistics
    __shared__ unsigned long long s_acc[2];
    if (threadIdx.x == 0) {
        s_acc[0] = 0;
        s_acc[1] = 0;
    }
    __syncthreads();
    if (acc_b)
        atomicAdd(&s_acc[0], acc_b);
    if (acc_slots)
        atomicAdd(&s_acc[1], acc_slots);
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_acc[0])
            atomicAdd(&st->accepted_windows, s_acc[0]);
        if (s_acc[1])
            atomicAdd(&st->accepted_slots, s_acc[1]);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->levels = level;
        st->inserts = m;
        if (nw > 0) {
            const uint32_t ra = (cur ? A.wa[1] : A.wa[0])[0], rb = (cur ? A.wb[1] : A.wb[0])[0];
            st->remaining = rb - ra;
            st->rem_a = ra;
            st->rem_buf = cur;
        }
#undef CNT
#undef CNTI
    }
}

// ---- whole-array kernels for the root resize and the bulk rebuild ----------

// Per-chunk live counts of slots [0, size).
__global__ void __launch_bounds__(BLOCK) chunk_live_kernel(const uint64_t *keys, const uint8_t *vals, uint32_t size,
                                                           uint32_t *chunk_cnt) {
    __shared__ uint32_t tmp[BLOCK / 32 + 1];
    uint32_t chunks = (size + CHUNK - 1) / CHUNK;
    for (uint32_t c = blockIdx.x; c < chunks; c += gridDim.x) {
        uint32_t cl = 0;
        for (uint32_t t = c * CHUNK + threadIdx.x; t < min(size, (c + 1) * CHUNK); t += BLOCK)
            cl += (keys[t] != KEY_NONE && vals[t] != 0);
        uint32_t s = block_sum(cl, tmp);
        if (threadIdx.x == 0)
            chunk_cnt[c] = s;
    }
}

// Exclusive scan of chunk counts in one CTA; writes the total to *total.
__global__ void __launch_bounds__(BLOCK) chunk_scan_kernel(uint32_t *chunk_cnt, uint32_t chunks, uint32_t *total) {
    __shared__ uint32_t tmp[BLOCK / 32 + 1];
    uint32_t run = 0;
    for (uint32_t k0 = 0; k0 < chunks; k0 += BLOCK) {
        uint32_t k = k0 + threadIdx.x;
        uint32_t v = k < chunks ? chunk_cnt[k] : 0;
        uint32_t tot;
        uint32_t ex = block_excl_scan(v, &tot, tmp);
        if (k < chunks)
            chunk_cnt[k] = run + ex;
        run += tot;
    }
    if (threadIdx.x == 0)
        *total = run;
}

// Stable compaction of live slots into dst (thread t owns a contiguous run).
__global__ void __launch_bounds__(BLOCK) chunk_compact_kernel(const uint64_t *keys, const uint8_t *vals, uint32_t size,
                                                              const uint32_t *chunk_off, uint64_t *dk, uint8_t *dv) {
    __shared__ uint32_t tmp[BLOCK / 32 + 1];
    constexpr uint32_t K = CHUNK / BLOCK;
    uint32_t chunks = (size + CHUNK - 1) / CHUNK;
    for (uint32_t c = blockIdx.x; c < chunks; c += gridDim.x) {
        uint32_t base = c * CHUNK + threadIdx.x * K;
        uint32_t cl = 0;
        for (uint32_t j = 0; j < K; ++j) {
            uint32_t t = base + j;
            cl += (t < size && keys[t] != KEY_NONE && vals[t] != 0);
        }
        uint32_t tot;
        uint32_t o = chunk_off[c] + block_excl_scan(cl, &tot, tmp);
        for (uint32_t j = 0; j < K; ++j) {
            uint32_t t = base + j;
            if (t < size && keys[t] != KEY_NONE && vals[t] != 0) {
                dk[o] = keys[t];
                dv[o] = vals[t];
                ++o;
            }
        }
    }
}

// Redispatch of the whole array [0, size) from live[0..L) and pend[0..P).
__global__ void __launch_bounds__(BLOCK) rebuild_kernel(uint64_t *keys, uint8_t *vals, uint32_t *row_offset,
                                                        uint32_t row_num, uint32_t size, uint32_t log2seg,
                                                        uint32_t log2F, const uint64_t *lk, const uint8_t *lv,
                                                        uint32_t L, const uint64_t *pk, const uint8_t *pv, uint32_t P,
                                                        uint64_t gap_key) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint64_t *mk = reinterpret_cast<uint64_t *>(smem);
    uint8_t *mv = reinterpret_cast<uint8_t *>(mk + CHUNK);
    uint32_t chunks = (size + CHUNK - 1) / CHUNK;
    for (uint32_t c = blockIdx.x; c < chunks; c += gridDim.x) {
        uint32_t t0 = c * CHUNK;
        uint32_t len = min(CHUNK, size - t0);
        redispatch_chunk(keys, vals, row_offset, row_num, 0, log2seg, log2F, t0, len, lk, lv, L, pk, pv, P, gap_key,
                         mk, mv);
    }
}

// keys[0..L) = live, keys[L..size) = KEY_NONE (values 0): the layout
// resize_gpma leaves when the root rebalance that follows it is rejected.
__global__ void compacted_layout_kernel(uint64_t *keys, uint8_t *vals, uint32_t size, const uint64_t *lk,
                                        const uint8_t *lv, uint32_t L) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < size; t += gridDim.x * blockDim.x) {
        keys[t] = t < L ? lk[t] : KEY_NONE;
        vals[t] = t < L ? lv[t] : 0;
    }
}

int grid_for(uint64_t work, int sms, int per_sm) {
    uint64_t g = (work + BLOCK - 1) / BLOCK;
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(g, (uint64_t)sms * per_sm));
}

// resize_gpma + (root rebalance | significant_insert) on the device.
gpma_status root_rebuild(gpma_graph *g, bool significant, uint32_t pend_buf, uint32_t pend_a, uint32_t pend_n,
                         cudaStream_t s) {
    const uint64_t *pend_k = g->ikeys[pend_buf] + pend_a;
    const uint8_t *pend_v = g->ivals[pend_buf] + pend_a;
    const uint32_t size = g->geo.size;
    const uint32_t chunks = (size + CHUNK - 1) / CHUNK;
    prof_mark(g, 0, s);
    g->prof.kernel_launches += 4;
    // 1. stable compaction of the live slots (resize_gpma, gpma.cuh:909-915)
    chunk_live_kernel<<<grid_for((uint64_t)chunks * BLOCK, g->sms, 8), BLOCK, 0, s>>>(g->keys, g->values, size,
                                                                                       g->chunk_cnt);
    uint32_t *d_total = reinterpret_cast<uint32_t *>(&g->status->pad);
    chunk_scan_kernel<<<1, BLOCK, 0, s>>>(g->chunk_cnt, chunks, d_total);
    chunk_compact_kernel<<<grid_for((uint64_t)chunks * BLOCK, g->sms, 8), BLOCK, 0, s>>>(g->keys, g->values, size,
                                                                                          g->chunk_cnt, g->skeys,
                                                                                          g->svals);
    GPMA_CUDA(cudaGetLastError());
    uint32_t live = 0;
    GPMA_CUDA(cudaMemcpyAsync(&live, d_total, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    GPMA_CUDA(cudaStreamSynchronize(s));
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
    const int rgrid = grid_for((uint64_t)out_chunks * BLOCK, g->sms, 4);
    const size_t rsmem = CHUNK * 9;
    if (significant) {
        // significant_insert: everything redispatched, gaps are key 0 / value 0
        rebuild_kernel<<<rgrid, BLOCK, rsmem, s>>>(g->keys, g->values, g->row_offset, g->row_num, geo.size, log2seg,
                                                    log2F, g->skeys, g->svals, live, pend_k, pend_v, pend_n, 0ull);
        g->stats.significant++;
        g->stats.accepted_windows++;
        g->stats.accepted_slots += geo.size;
    } else {
        const uint32_t h = geo.height;
        if (geo.lower[h] <= merge && merge <= geo.upper[h]) {
            rebuild_kernel<<<rgrid, BLOCK, rsmem, s>>>(g->keys, g->values, g->row_offset, g->row_num, geo.size,
                                                        log2seg, log2F, g->skeys, g->svals, live, pend_k, pend_v,
                                                        pend_n, KEY_NONE);
            g->stats.accepted_windows++;
            g->stats.accepted_slots += geo.size;
        } else {
            // the reference drops the insertions and keeps the compacted array
            compacted_layout_kernel<<<grid_for(geo.size, g->sms, 8), BLOCK, 0, s>>>(g->keys, g->values, geo.size,
                                                                                     g->skeys, g->svals, live);
            g->stats.root_drops++;
        }
        g->stats.root_resizes++;
    }
    GPMA_CUDA(cudaGetLastError());
    prof_mark(g, 1, s);
    g->geo = geo;
    GPMA_TRY(upload_geometry(g, s));
    GPMA_CUDA(cudaStreamSynchronize(s));
    g->prof.rebuild_ms += prof_elapsed(g, 0, 1);
    // the scratch must cover the whole array for later wide windows
    GPMA_TRY(ensure_scratch(g, geo.size));
    return GPMA_OK;
}

}  // namespace

gpma_status upload_geometry(gpma_graph *g, cudaStream_t s) {
    uint32_t buf[64] = {0};
    for (uint32_t i = 0; i <= g->geo.height && i < 32; ++i) {
        buf[i] = g->geo.lower[i];
        buf[32 + i] = g->geo.upper[i];
    }
    GPMA_CUDA(cudaMemcpyAsync(g->d_lower, buf, 32 * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    GPMA_CUDA(cudaMemcpyAsync(g->d_upper, buf + 32, 32 * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    // the host buffer is on the stack: wait for the copies
    GPMA_CUDA(cudaStreamSynchronize(s));
    return GPMA_OK;
}

gpma_status ensure_scratch(gpma_graph *g, uint32_t slots) {
    if (slots <= g->scratch_cap && g->skeys)
        return GPMA_OK;
    dev_free(g->skeys);
    dev_free(g->svals);
    dev_free(g->chunk_cnt);
    g->scratch_cap = 0;
    GPMA_TRY(dev_alloc(&g->skeys, slots));
    GPMA_TRY(dev_alloc(&g->svals, slots));
    GPMA_TRY(dev_alloc(&g->chunk_cnt, slots / CHUNK + 2));
    g->scratch_cap = slots;
    return GPMA_OK;
}

gpma_status ensure_batch(gpma_graph *g, uint64_t n) {
    if (n <= g->batch_cap && g->bkeys[0])
        return GPMA_OK;
    uint64_t cap = std::max<uint64_t>(n, 1024);
    for (int i = 0; i < 2; ++i) {
        dev_free(g->bkeys[i]);
        dev_free(g->bvals[i]);
        dev_free(g->wnode[i]);
        dev_free(g->wa[i]);
        dev_free(g->wb[i]);
    }
    dev_free(g->leaf);
    for (int i = 0; i < 2; ++i) {
        dev_free(g->ikeys[i]);
        dev_free(g->ivals[i]);
    }
    dev_free(g->ileaf);
    dev_free(g->wflag);
    dev_free(g->wlive);
    g->batch_cap = 0;
    for (int i = 0; i < 2; ++i) {
        GPMA_TRY(dev_alloc(&g->bkeys[i], cap));
        GPMA_TRY(dev_alloc(&g->bvals[i], cap));
        GPMA_TRY(dev_alloc(&g->wnode[i], cap));
        GPMA_TRY(dev_alloc(&g->wa[i], cap));
        GPMA_TRY(dev_alloc(&g->wb[i], cap));
    }
    GPMA_TRY(dev_alloc(&g->leaf, cap));
    for (int i = 0; i < 2; ++i) {
        GPMA_TRY(dev_alloc(&g->ikeys[i], cap));
        GPMA_TRY(dev_alloc(&g->ivals[i], cap));
    }
    GPMA_TRY(dev_alloc(&g->ileaf, cap));
    GPMA_TRY(dev_alloc(&g->wflag, cap));
    GPMA_TRY(dev_alloc(&g->wlive, cap));
    g->batch_cap = cap;
    return GPMA_OK;
}

// Runs the update of the n-key batch already staged in bkeys[0]/bvals[0].
gpma_status update_device(gpma_graph *g, uint64_t n, cudaStream_t s, bool check_keys) {
    if (g->update_grid == 0) {
        GPMA_CUDA(cudaFuncSetAttribute(update_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)UPDATE_SMEM));
        GPMA_CUDA(cudaFuncSetAttribute(rebuild_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(CHUNK * 9)));
        int per_sm = 0;
        GPMA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, update_kernel, BLOCK, UPDATE_SMEM));
        if (per_sm < 1) {
            set_error("update kernel cannot be resident (occupancy 0)");
            return GPMA_ERR_CUDA;
        }
        g->update_grid = g->sms * std::min(per_sm, 4);
        GPMA_TRY(dev_alloc(&g->cta_cnt, 4ull * g->update_grid));
    }
    const uint32_t tiles = (uint32_t)((n + SORT_TILE - 1) / SORT_TILE);
    const uint64_t status_words = 8ull * tiles * 256;
    if (status_words > g->sort_status_cap) {
        dev_free(g->sort_status);
        GPMA_TRY(dev_alloc(&g->sort_status, status_words));
        g->sort_status_cap = status_words;
    }
    GPMA_CUDA(cudaMemsetAsync(g->status, 0, sizeof(DeviceStatus), s));
    GPMA_CUDA(cudaMemsetAsync(g->sort_hist, 0, 8 * 256 * sizeof(uint32_t), s));
    GPMA_CUDA(cudaMemsetAsync(g->sort_tiles, 0, 8 * sizeof(uint32_t), s));
    GPMA_CUDA(cudaMemsetAsync(g->sort_status, 0, status_words * sizeof(uint32_t), s));
    prof_mark(g, 1, s);
    UpdateArgs A;
    A.keys = g->keys;
    A.vals = g->values;
    A.row_offset = g->row_offset;
    A.row_num = g->row_num;
    A.size = g->geo.size;
    A.seg = g->geo.seg;
    A.log2seg = fls32(g->geo.seg) - 1;
    A.height = g->geo.height;
    A.lower = g->d_lower;
    A.upper = g->d_upper;
    A.bk[0] = g->bkeys[0];
    A.bk[1] = g->bkeys[1];
    A.bv[0] = g->bvals[0];
    A.bv[1] = g->bvals[1];
    A.sort_hist = g->sort_hist;
    A.sort_tiles = g->sort_tiles;
    A.sort_status = g->sort_status;
    A.check_keys = check_keys;
    A.n = (uint32_t)n;
    A.leaf = g->leaf;
    for (int i = 0; i < 2; ++i) {
        A.ikeys[i] = g->ikeys[i];
        A.ivals[i] = g->ivals[i];
    }
    A.ileaf = g->ileaf;
    for (int i = 0; i < 2; ++i) {
        A.wnode[i] = g->wnode[i];
        A.wa[i] = g->wa[i];
        A.wb[i] = g->wb[i];
    }
    A.wflag = g->wflag;
    A.wlive = g->wlive;
    A.skeys = g->skeys;
    A.svals = g->svals;
    A.chunk_cnt = g->chunk_cnt;
    A.cta_cnt = g->cta_cnt;
    A.st = g->status;
    void *params[] = {&A};
    GPMA_CUDA(cudaLaunchCooperativeKernel((const void *)update_kernel, dim3(g->update_grid), dim3(BLOCK), params,
                                          UPDATE_SMEM, s));
    prof_mark(g, 2, s);
    GPMA_CUDA(cudaMemcpyAsync(g->h_status, g->status, sizeof(DeviceStatus), cudaMemcpyDeviceToHost, s));
    GPMA_CUDA(cudaStreamSynchronize(s));
    g->prof.kernel_launches += 1;  // the sort runs inside the update kernel
    g->prof.update_kernels++;
    g->prof.update_kernel_ms += prof_elapsed(g, 1, 2);
    const DeviceStatus &h = *g->h_status;
    if (h.invalid_keys) {
        set_error("update batch holds keys whose column is 0xFFFFFFFF (reserved for row guards and empty slots)");
        return GPMA_ERR_INVALID;
    }
    if (h.err) {
        set_error("device-side wait gave up in the update kernel (code %u)", h.err);
        return h.err == DERR_BOUNDS ? GPMA_ERR_DEVICE : GPMA_ERR_TIMEOUT;
    }
    g->stats.levels_visited += h.levels;
    g->stats.accepted_windows += h.accepted_windows;
    g->stats.accepted_slots += h.accepted_slots;
    g->stats.last_inserts = h.inserts;
    if (h.significant)
        return root_rebuild(g, true, 0, 0, h.inserts, s);
    if (h.remaining > 0)
        return root_rebuild(g, false, h.rem_buf, h.rem_a, h.remaining, s);
    return GPMA_OK;
}

}  // namespace gpma
