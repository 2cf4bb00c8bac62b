// msbfs.cu - multi-source BFS over one or many GPMA graphs in one launch.
//
// No reference counterpart (the reference BFS, gpma_bfs.cuh:446-533, takes one
// source of one graph); each of the up to 64 searches per graph has the
// reference's level semantics (levels[src] = 1, a node first reached from
// level L gets L+1, slots with column 0xFFFFFFFF or value 0 are not edges).
//
// The nodes of all graphs form one index space (graph g owns
// [voff[g], voff[g+1])). Each node carries three 64-bit masks, one bit lane
// per source: visited, frontier, next. One persistent cooperative kernel runs
// every level, separated by bounded grid barriers:
//   expand (phase 1): a warp takes 32 consecutive nodes; the rows of those in
//     the frontier are walked as one concatenated slot range (warp-level load
//     balancing) and every edge ORs the source's frontier mask, minus the
//     target's visited lanes, into next[target]; rows longer than 64 slots
//     are queued as 128-slot chunks instead;
//   expand (phase 2): every warp takes chunks;
//   commit: next minus visited becomes the new frontier, joins visited, and
//     gives each newly reached (node, lane) its level.
// The traversed-edge count (edges scanned from reached nodes, per source) is
// summed on the fly for GTEPS.
#include "gpma_internal.cuh"

#include <algorithm>
#include <numeric>

namespace gpma {
namespace {

enum : uint32_t {
    MS_CHANGE = 0,  // 3 rotating counters: CTAs that reached a new (node, lane)
    MS_CHUNKS = 3,  // 3 rotating chunk counters
    MS_ERR = 6,
    MS_LEVELS = 7,
    MS_BAR = 10,    // GridBarrier (2 words)
    MS_FSLOTS = 16, // 3 rotating u64 counters (words 16..21): slots of the rows in the next union frontier
    MS_CTL_WORDS = 24,
};

constexpr uint32_t MS_BIG_ROW = 64;
constexpr uint32_t MS_CHUNK_SLOTS = 128;
// Chunk list entries for `slots` slots over all graphs: rows over MS_BIG_ROW
// slots yield at most len/128 + 1 chunks each, at most slots/65 such rows, so
// a level queues fewer than slots/128 + slots/65 < slots/32 chunks.
inline uint64_t ms_chunk_need(uint64_t slots) { return slots / 32 + 1024; }

struct MsGraph {
    const uint64_t *keys;
    const uint8_t *vals;
    const uint32_t *ro;
    uint32_t *levels;  // [nsrc][n] or null
    uint32_t n, size, nsrc, pad;
};

struct MsArgs {
    const MsGraph *gr;
    uint32_t G;
    const uint32_t *voff;  // G + 1
    const uint32_t *src;   // G * 64
    const uint64_t *soff;  // slot offsets of the concatenated arrays, G + 1 (multiples of 4)
    uint64_t *visited;
    uint64_t *frontier;
    uint64_t *next;
    uint4 *chunks;         // {slot begin, slot end, graph, node}
    uint32_t chunk_cap;
    uint32_t *ctl;
    unsigned long long *reached;  // G * 64
    unsigned long long *traversed;
    uint32_t dense_div;    // a level whose union frontier's rows span >= slots / dense_div slots sweeps every slot (0: never)
    const uint32_t *abort;  // non-zero: return at once (a recorded step after one needing host work)
};

__device__ __forceinline__ uint32_t graph_of_node(const MsArgs &A, uint32_t u) {
    return A.G == 1 ? 0u : segment_of(A.voff, A.G, u);
}

// One slot of graph g scanned with frontier mask fm; returns 1 if it is an edge.
__device__ __forceinline__ uint32_t ms_visit(const MsArgs &A, const MsGraph &Gr, uint32_t g, uint32_t s, uint64_t fm) {
    const uint64_t key = Gr.keys[s];
    const uint32_t w = (uint32_t)key;
    if (w == 0xFFFFFFFFu || Gr.vals[s] == 0 || w >= Gr.n)
        return 0;
    const uint32_t gw = A.voff[g] + w;
    const uint64_t nb = fm & ~A.visited[gw];
    if (nb && (A.next[gw] & nb) != nb)
        atomicOr((unsigned long long *)&A.next[gw], (unsigned long long)nb);
    return 1;
}

// Dense levels: 4 consecutive slots of the sweep over every graph's array
// (node offset vo, n nodes). The key's high word is its source row. The
// frontier masks of all 4, then the visited and next masks of their targets,
// are loaded before any update. Returns the lanes that traverse the 4 slots.
__device__ __forceinline__ uint32_t ms_dense_visit4(const MsArgs &A, uint32_t vo, uint32_t n,
                                                    const uint64_t (&k)[4], uint32_t v4) {
    uint32_t dst[4];
    uint64_t fm[4], nb[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const uint32_t src = (uint32_t)(k[j] >> 32);
        dst[j] = (uint32_t)k[j];
        const bool ok = dst[j] != 0xFFFFFFFFu && ((v4 >> (8 * j)) & 0xFFu) != 0 && src < n && dst[j] < n;
        fm[j] = ok ? A.frontier[vo + src] : 0ull;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j)
        nb[j] = fm[j] ? fm[j] & ~A.visited[vo + dst[j]] : 0ull;
    uint32_t lanes = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        lanes += __popcll(fm[j]);
        if (nb[j] && (A.next[vo + dst[j]] & nb[j]) != nb[j])
            atomicOr((unsigned long long *)&A.next[vo + dst[j]], (unsigned long long)nb[j]);
    }
    return lanes;
}

// Graph of concatenated slot t: the last g with soff[g] <= t.
__device__ __forceinline__ uint32_t graph_of_slot(const MsArgs &A, uint64_t t) {
    uint32_t lo = 0, hi = A.G;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (A.soff[mid] <= t)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

__device__ __forceinline__ unsigned long long *fslots(const MsArgs &A, uint32_t level) {
    return reinterpret_cast<unsigned long long *>(A.ctl + MS_FSLOTS) + level % 3;
}

__device__ __forceinline__ uint32_t ms_row_slots(const MsGraph &Gr, uint32_t v) {
    const uint32_t b = Gr.ro[v], e = min(Gr.ro[v + 1], Gr.size);
    return e > b ? e - b : 0u;
}

__global__ void __launch_bounds__(BLOCK) msbfs_kernel(MsArgs A) {
    if (A.abort && *(const volatile uint32_t *)A.abort)
        return;
    GridBarrier *bar = reinterpret_cast<GridBarrier *>(A.ctl + MS_BAR);
    uint32_t *err = A.ctl + MS_ERR;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gwarp = blockIdx.x * (BLOCK / 32) + (threadIdx.x >> 5);
    const uint32_t nwarps = gridDim.x * (BLOCK / 32);
    const uint32_t gtid = blockIdx.x * BLOCK + threadIdx.x;
    const uint32_t nthreads = gridDim.x * BLOCK;
    const uint32_t N = A.voff[A.G];
    unsigned long long traversed = 0;
    // seed the sources (masks cleared by the host)
    for (uint32_t t = gtid; t < A.G * 64; t += nthreads) {
        const uint32_t g = t >> 6, j = t & 63;
        const MsGraph &Gr = A.gr[g];
        if (j >= Gr.nsrc)
            continue;
        const uint32_t s = A.src[t];
        atomicOr((unsigned long long *)&A.visited[A.voff[g] + s], 1ull << j);
        atomicOr((unsigned long long *)&A.frontier[A.voff[g] + s], 1ull << j);
        atomicAdd(fslots(A, 1), (unsigned long long)ms_row_slots(Gr, s));
        if (Gr.levels)
            Gr.levels[(size_t)j * Gr.n + s] = 1;
    }
    if (!grid_barrier_gen(bar, err))
        return;
    uint32_t level = 1;
    for (;; ++level) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            A.ctl[MS_CHANGE + (level + 1) % 3] = 0;
            A.ctl[MS_CHUNKS + (level + 1) % 3] = 0;
            *fslots(A, level + 2) = 0;
        }
        uint32_t *chunk_cnt = A.ctl + MS_CHUNKS + level % 3;
        __shared__ unsigned long long s_fs;
        __syncthreads();
        if (threadIdx.x == 0)
            s_fs = *reinterpret_cast<volatile unsigned long long *>(fslots(A, level));
        __syncthreads();
        const bool dense = A.dense_div && s_fs * A.dense_div >= A.soff[A.G];
        // expand, dense: every slot of every graph, 4 per thread per step; the
        // frontier masks stay in place until the commit clears them
        const uint64_t quads = dense ? A.soff[A.G] >> 2 : 0;
        for (uint64_t q = gtid; q < quads; q += nthreads) {
            const uint64_t t = q << 2;
            const uint32_t g = A.G == 1 ? 0u : graph_of_slot(A, t);
            const MsGraph &Gr = A.gr[g];
            const uint32_t s = (uint32_t)(t - A.soff[g]);
            const ulonglong2 k01 = *reinterpret_cast<const ulonglong2 *>(Gr.keys + s);
            const ulonglong2 k23 = *reinterpret_cast<const ulonglong2 *>(Gr.keys + s + 2);
            const uint32_t v4 = *reinterpret_cast<const uint32_t *>(Gr.vals + s);
            const uint64_t k[4] = {k01.x, k01.y, k23.x, k23.y};
            traversed += ms_dense_visit4(A, A.voff[g], Gr.n, k, v4);
        }
        // expand, phase 1 (sparse levels)
        for (uint32_t base = gwarp * 32; !dense && base < N; base += nwarps * 32) {
            const uint32_t u = base + lane;
            const uint64_t f = u < N ? A.frontier[u] : 0ull;
            if (__ballot_sync(0xFFFFFFFFu, f != 0ull) == 0)
                continue;
            uint32_t g = 0, b = 0, e = 0, len = 0;
            if (f) {
                A.frontier[u] = 0;  // consumed; the commit phase writes the next frontier
                g = graph_of_node(A, u);
                const MsGraph &Gr = A.gr[g];
                const uint32_t lu = u - A.voff[g];
                const uint32_t r1 = Gr.ro[lu + 1];
                b = Gr.ro[lu];
                e = min(r1, Gr.size);
                if (!in_bounds(err, b <= r1 && r1 <= Gr.size, BS_ROW))
                    b = e;  // an inconsistent row_offset: the row is skipped
                len = e > b ? e - b : 0;
            }
            const uint32_t nch = len > MS_BIG_ROW ? (len + MS_CHUNK_SLOTS - 1) / MS_CHUNK_SLOTS : 0;
            const uint32_t ch_incl = warp_incl_scan(nch);
            const uint32_t ch_total = __shfl_sync(0xFFFFFFFFu, ch_incl, 31);
            if (ch_total) {
                uint32_t cb = 0;
                if (lane == 0)
                    cb = atomicAdd(chunk_cnt, ch_total);
                cb = __shfl_sync(0xFFFFFFFFu, cb, 0);
                if (cb + ch_total <= A.chunk_cap) {
                    const uint32_t pos = cb + ch_incl - nch;
                    for (uint32_t c = 0; c < nch; ++c)
                        A.chunks[pos + c] = make_uint4(b + c * MS_CHUNK_SLOTS, min(e, b + (c + 1) * MS_CHUNK_SLOTS), g, u);
                    if (nch) {
                        // the chunk reads the mask from frontier[u]: keep it until commit
                        A.frontier[u] = f;
                        len = 0;
                    }
                } else {
                    for (uint32_t c = cb + lane; c < min(cb + ch_total, A.chunk_cap); c += 32)
                        A.chunks[c] = make_uint4(0, 0, 0, 0);
                }
            }
            const uint32_t incl = warp_incl_scan(len);
            const uint32_t excl = incl - len;
            const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
            for (uint32_t p0 = 0; p0 < total; p0 += 32) {
                const uint32_t p = p0 + lane;
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
                const uint32_t rg = __shfl_sync(0xFFFFFFFFu, g, r);
                const uint64_t rf = __shfl_sync(0xFFFFFFFFu, f, r);
                if (p < total)
                    traversed += ms_visit(A, A.gr[rg], rg, rb + (p - rex), rf) * (unsigned long long)__popcll(rf);
            }
        }
        if (!dense && !grid_barrier_gen(bar, err))
            return;
        // expand, phase 2: long-row chunks
        const uint32_t nch_all = dense ? 0u : min(cta_broadcast_read(chunk_cnt), A.chunk_cap);
        for (uint32_t c = gwarp; c < nch_all; c += nwarps) {
            const uint4 ch = A.chunks[c];
            if (ch.x >= ch.y)
                continue;
            const uint64_t fm = A.frontier[ch.w];
            const MsGraph &Gr = A.gr[ch.z];
            for (uint32_t s = ch.x + lane; s < ch.y; s += 32)
                traversed += ms_visit(A, Gr, ch.z, s, fm) * (unsigned long long)__popcll(fm);
        }
        if (!grid_barrier_gen(bar, err))
            return;
        // commit
        uint32_t changed = 0;
        unsigned long long fnext = 0;
        for (uint32_t w = gtid; w < N; w += nthreads) {
            const uint64_t nxt = A.next[w];
            const uint64_t vis = A.visited[w];
            const uint64_t nx = nxt & ~vis;
            if (A.frontier[w])
                A.frontier[w] = 0;  // chunked rows kept their mask until now
            if (nxt)
                A.next[w] = 0;
            if (nx) {
                A.frontier[w] = nx;
                A.visited[w] = vis | nx;
                changed = 1;
                const uint32_t g = graph_of_node(A, w);
                const MsGraph &Gr = A.gr[g];
                fnext += ms_row_slots(Gr, w - A.voff[g]);
                if (Gr.levels) {
                    const uint32_t lw = w - A.voff[g];
                    uint64_t m = nx;
                    while (m) {
                        const int bit = __ffsll((long long)m) - 1;
                        m &= m - 1;
                        Gr.levels[(size_t)bit * Gr.n + lw] = level + 1;
                    }
                }
            }
        }
        if (__syncthreads_or(changed) && threadIdx.x == 0)
            atomicAdd(A.ctl + MS_CHANGE + level % 3, 1u);
#pragma unroll
        for (int d = 16; d >= 1; d >>= 1)
            fnext += __shfl_xor_sync(0xFFFFFFFFu, fnext, d);
        if (lane == 0 && fnext)
            atomicAdd(fslots(A, level + 1), fnext);
        if (!grid_barrier_gen(bar, err))
            return;
        if (cta_broadcast_read(A.ctl + MS_CHANGE + level % 3) == 0)
            break;
    }
    // reached (graph, lane) counts: each CTA walks a contiguous node range
    // graph by graph with shared-memory lane counters
    __shared__ unsigned int cnt[64];
    const uint32_t per = (N + gridDim.x - 1) / gridDim.x;
    const uint32_t lo = min(N, blockIdx.x * per), hi = min(N, lo + per);
    uint32_t pos = lo;
    while (__syncthreads_or(pos < hi)) {
        const uint32_t g = graph_of_node(A, pos);
        const uint32_t end = min(hi, A.voff[g + 1]);
        if (threadIdx.x < 64)
            cnt[threadIdx.x] = 0;
        __syncthreads();
        for (uint32_t w = pos + threadIdx.x; w < end; w += BLOCK) {
            uint64_t m = A.visited[w];
            while (m) {
                const int bit = __ffsll((long long)m) - 1;
                m &= m - 1;
                atomicAdd(&cnt[bit], 1u);
            }
        }
        __syncthreads();
        if (threadIdx.x < 64 && cnt[threadIdx.x])
            atomicAdd(&A.reached[(size_t)g * 64 + threadIdx.x], (unsigned long long)cnt[threadIdx.x]);
        pos = end;
    }
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1)
        traversed += __shfl_xor_sync(0xFFFFFFFFu, traversed, d);
    if (lane == 0 && traversed)
        atomicAdd(A.traversed, traversed);
    if (blockIdx.x == 0 && threadIdx.x == 0)
        A.ctl[MS_LEVELS] = level;
}

int g_ms_fit[64] = {};  // resident CTAs per SM, per device

int ms_grid_size(int sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64)
        dev = 0;
    if (g_ms_fit[dev] == 0) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, msbfs_kernel, BLOCK, 0) != cudaSuccess)
            return 0;
        g_ms_fit[dev] = std::min(per_sm, MAX_BLOCKS_PER_SM);
    }
    return sms * blocks_per_sm(g_ms_fit[dev], g_tuning.ms_blocks_per_sm);
}

}  // namespace

void free_batch_bfs(gpma_batch *b) {
    for (int i = 0; i < 3; ++i)
        dev_free(b->ms_mask[i]);
    dev_free(b->ms_tab);
    if (b->h_ms_tab)
        cudaFreeHost(b->h_ms_tab);
    b->h_ms_tab = nullptr;
    dev_free(b->ms_ctl);
    dev_free(b->ms_reached);
    if (b->h_ms_reached)
        cudaFreeHost(b->h_ms_reached);
    b->h_ms_reached = nullptr;
    dev_free(b->ms_chunks);
    b->ms_chunk_cap = 0;
    if (b->h_ms_ctl)
        cudaFreeHost(b->h_ms_ctl);
    b->h_ms_ctl = nullptr;
    b->ms_cap = 0;
    b->ms_gcap = 0;
}

namespace {

// Byte layout of the per-call graph table (device copy and pinned mirror):
// node offsets (k + 1 u32), slot offsets (k + 1 u64), sources (64 k u32),
// graph descriptors (k MsGraph), each part 16-byte aligned.
struct MsTabLayout {
    size_t voff, soff, src, gdesc, bytes;
    explicit MsTabLayout(uint32_t k) {
        auto up = [](size_t x) { return (x + 15) & ~size_t(15); };
        voff = 0;
        soff = up(voff + 4ull * (k + 1));
        src = up(soff + 8ull * (k + 1));
        gdesc = up(src + 4ull * 64 * k);
        bytes = up(gdesc + sizeof(MsGraph) * k);
    }
};

}  // namespace

gpma_status batch_bfs_plan(gpma_batch *b, gpma_graph *const *graphs, const uint32_t *const *srcs,
                           const uint32_t *nsrc, uint32_t k, uint32_t *const *stage, BatchBfsPlan *P,
                           const uint32_t *abort) {
    static_assert(sizeof(MsArgs) <= KernelLaunch::ARG_BYTES, "multi-source BFS arguments exceed the launch record");
    const int grid = ms_grid_size(b->sms);
    if (grid == 0) {
        set_error("multi-source BFS kernel cannot be resident");
        return GPMA_ERR_CUDA;
    }
    uint64_t N = 0, slots = 0;
    for (uint32_t i = 0; i < k; ++i) {
        N += graphs[i]->row_num;
        slots += graphs[i]->geo.size;  // sizes are powers of two >= 4
    }
    if (N > b->ms_cap || !b->ms_mask[0]) {
        for (int i = 0; i < 3; ++i)
            dev_free(b->ms_mask[i]);
        b->ms_cap = 0;
        for (int i = 0; i < 3; ++i)
            GPMA_TRY(dev_alloc(&b->ms_mask[i], std::max<uint64_t>(N, 1)));
        b->ms_cap = std::max<uint64_t>(N, 1);
    }
    const MsTabLayout lay(k);
    if (k > b->ms_gcap || !b->ms_tab) {
        dev_free(b->ms_tab);
        dev_free(b->ms_reached);
        if (b->h_ms_tab)
            cudaFreeHost(b->h_ms_tab);
        if (b->h_ms_reached)
            cudaFreeHost(b->h_ms_reached);
        b->h_ms_tab = nullptr;
        b->h_ms_reached = nullptr;
        b->ms_gcap = 0;
        GPMA_TRY(dev_alloc(&b->ms_tab, lay.bytes));
        GPMA_TRY(dev_alloc(&b->ms_reached, 64ull * k + 1));
        GPMA_CUDA(cudaMallocHost((void **)&b->h_ms_tab, lay.bytes));
        GPMA_CUDA(cudaMallocHost((void **)&b->h_ms_reached, sizeof(unsigned long long) * (64ull * k + 1)));
        b->ms_gcap = k;
    }
    if (ms_chunk_need(slots) > b->ms_chunk_cap) {
        dev_free(b->ms_chunks);
        b->ms_chunk_cap = 0;
        GPMA_TRY(dev_alloc(&b->ms_chunks, 2 * ms_chunk_need(slots)));  // uint4 = 2 x uint2
        b->ms_chunk_cap = ms_chunk_need(slots);
    }
    if (!b->ms_ctl) {
        GPMA_TRY(dev_alloc(&b->ms_ctl, MS_CTL_WORDS));
        GPMA_CUDA(cudaMallocHost((void **)&b->h_ms_ctl, sizeof(uint32_t) * MS_CTL_WORDS));
    }
    // the table, in the pinned mirror (the previous call's upload has finished)
    uint32_t *voff = reinterpret_cast<uint32_t *>(b->h_ms_tab + lay.voff);
    uint64_t *soff = reinterpret_cast<uint64_t *>(b->h_ms_tab + lay.soff);
    uint32_t *src = reinterpret_cast<uint32_t *>(b->h_ms_tab + lay.src);
    MsGraph *gr = reinterpret_cast<MsGraph *>(b->h_ms_tab + lay.gdesc);
    voff[0] = 0;
    soff[0] = 0;
    memset(src, 0, 4ull * 64 * k);
    for (uint32_t i = 0; i < k; ++i) {
        const gpma_graph *g = graphs[i];
        voff[i + 1] = voff[i] + g->row_num;
        soff[i + 1] = soff[i] + g->geo.size;
        gr[i].keys = g->keys;
        gr[i].vals = g->values;
        gr[i].ro = g->row_offset;
        gr[i].n = g->row_num;
        gr[i].size = g->geo.size;
        gr[i].nsrc = nsrc[i];
        gr[i].pad = 0;
        gr[i].levels = stage ? stage[i] : nullptr;
        for (uint32_t j = 0; j < nsrc[i]; ++j)
            src[64ull * i + j] = srcs[i][j];
    }
    P->tab_bytes = lay.bytes;
    void *ptr[BatchBfsPlan::CLEARS] = {b->ms_mask[0], b->ms_mask[1], b->ms_mask[2], b->ms_ctl, b->ms_reached};
    const size_t bytes[BatchBfsPlan::CLEARS] = {8 * N, 8 * N, 8 * N, sizeof(uint32_t) * MS_CTL_WORDS,
                                                sizeof(unsigned long long) * (64ull * k + 1)};
    for (int i = 0; i < BatchBfsPlan::CLEARS; ++i) {
        P->clear_ptr[i] = ptr[i];
        P->clear_bytes[i] = bytes[i];
    }
    MsArgs A;
    memset(&A, 0, sizeof(A));  // padding too: launches are compared byte-wise
    A.gr = reinterpret_cast<const MsGraph *>(b->ms_tab + lay.gdesc);
    A.G = k;
    A.voff = reinterpret_cast<const uint32_t *>(b->ms_tab + lay.voff);
    A.src = reinterpret_cast<const uint32_t *>(b->ms_tab + lay.src);
    A.soff = reinterpret_cast<const uint64_t *>(b->ms_tab + lay.soff);
    A.dense_div = g_tuning.ms_dense_div;
    A.visited = b->ms_mask[0];
    A.frontier = b->ms_mask[1];
    A.next = b->ms_mask[2];
    A.chunks = reinterpret_cast<uint4 *>(b->ms_chunks);
    A.chunk_cap = (uint32_t)std::min<uint64_t>(b->ms_chunk_cap, 0xFFFFFFFFull);
    A.ctl = b->ms_ctl;
    A.reached = reinterpret_cast<unsigned long long *>(b->ms_reached);
    A.traversed = reinterpret_cast<unsigned long long *>(b->ms_reached) + 64ull * k;
    A.abort = abort;
    P->main.set((const void *)msbfs_kernel, grid, 0, &A, sizeof(A));
    P->ctl_bytes = sizeof(uint32_t) * MS_CTL_WORDS;
    P->reached_bytes = sizeof(unsigned long long) * (64ull * k + 1);
    return GPMA_OK;
}

gpma_status batch_bfs_enqueue_readback(gpma_batch *b, const BatchBfsPlan &P, cudaStream_t s) {
    GPMA_CUDA(cudaMemcpyAsync(b->h_ms_ctl, b->ms_ctl, P.ctl_bytes, cudaMemcpyDeviceToHost, s));
    GPMA_CUDA(cudaMemcpyAsync(b->h_ms_reached, b->ms_reached, P.reached_bytes, cudaMemcpyDeviceToHost, s));
    return GPMA_OK;
}

gpma_status batch_bfs_finish(gpma_batch *b, const uint32_t *nsrc, uint32_t k, uint64_t *reached) {
    b->prof.kernel_launches += 1;
    b->prof.bfs_kernels++;
    if (b->h_ms_ctl[MS_ERR])
        return device_error("the multi-source BFS kernel", b->h_ms_ctl[MS_ERR]);
    const unsigned long long *r = b->h_ms_reached;
    if (reached) {
        uint64_t o = 0;
        for (uint32_t i = 0; i < k; ++i)
            for (uint32_t j = 0; j < nsrc[i]; ++j)
                reached[o++] = r[64ull * i + j];
    }
    b->last_traversed = r[64ull * k];
    b->prof.bfs_edges += r[64ull * k];
    return GPMA_OK;
}

// Multi-source BFS of graphs[0..k) with nsrc[i] sources each. Levels (when
// levels != NULL) are written through device staging and copied to the
// caller's pointers; reached receives sum(nsrc) counts.
gpma_status batch_bfs_run(gpma_batch *b, gpma_graph *const *graphs, const uint32_t *const *srcs, const uint32_t *nsrc,
                          uint32_t k, uint32_t *const *levels, uint64_t *reached, cudaStream_t s) {
    // per-graph level staging, only when levels are requested
    std::vector<uint32_t *> stage(k, nullptr);
    auto cleanup = [&]() {
        for (auto *p : stage)
            if (p)
                cudaFree(p);
    };
    auto run = [&]() -> gpma_status {
        if (levels) {
            for (uint32_t i = 0; i < k; ++i) {
                if (!levels[i])
                    continue;
                GPMA_TRY(dev_alloc(&stage[i], (uint64_t)nsrc[i] * graphs[i]->row_num));
                GPMA_CUDA(cudaMemsetAsync(stage[i], 0, sizeof(uint32_t) * nsrc[i] * (uint64_t)graphs[i]->row_num, s));
            }
        }
        BatchBfsPlan P;
        GPMA_TRY(batch_bfs_plan(b, graphs, srcs, nsrc, k, levels ? stage.data() : nullptr, &P));
        GPMA_CUDA(cudaMemcpyAsync(b->ms_tab, b->h_ms_tab, P.tab_bytes, cudaMemcpyHostToDevice, s));
        for (int i = 0; i < BatchBfsPlan::CLEARS; ++i)
            GPMA_CUDA(cudaMemsetAsync(P.clear_ptr[i], 0, P.clear_bytes[i], s));
        prof_mark(b->profiling, b->ev, 0, s);
        GPMA_CUDA(P.main.launch_cooperative(s));
        prof_mark(b->profiling, b->ev, 1, s);
        GPMA_TRY(batch_bfs_enqueue_readback(b, P, s));
        for (uint32_t i = 0; i < k; ++i)
            if (stage[i])
                GPMA_TRY(copy_any(levels[i], stage[i], sizeof(uint32_t) * nsrc[i] * (uint64_t)graphs[i]->row_num, s));
        GPMA_CUDA(cudaStreamSynchronize(s));
        b->prof.bfs_ms += prof_elapsed(b->profiling, b->ev, 0, 1);
        return batch_bfs_finish(b, nsrc, k, reached);
    };
    const gpma_status st = run();
    cleanup();
    return st;
}

}  // namespace gpma
