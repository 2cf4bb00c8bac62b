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
// separated by bounded grid barriers. The frontier is a queue; a warp scans
// the slot range of one frontier node with coalesced 8-byte key and 1-byte
// value loads; the visited set is a bitmap claimed with atomicOr (a plain
// load filters already-visited targets first); new nodes are appended with
// one warp-aggregated atomic per warp step.
//
// Multi-source (k <= 64): one bit lane per source in 64-bit masks
// (visited, frontier, next); per level a warp takes 32 nodes, and for each
// node with a non-empty frontier mask the whole warp scans its row and ORs
// the mask into next[w]; a second sweep turns next into the new frontier and
// writes levels for each newly set lane.
#include "gpma_internal.cuh"

#include <algorithm>
#include <mutex>

namespace gpma {
namespace {

// bfs_ctl layout (u32 words)
enum : uint32_t {
    CTL_CNT = 0,      // 3 rotating queue counters
    CTL_ERR = 4,
    CTL_LEVELS = 5,
    CTL_REACHED = 6,
    CTL_BAR = 8,      // GridBarrier (2 words)
    CTL_WORDS = 16,
};

struct BfsArgs {
    const uint64_t *keys;
    const uint8_t *vals;
    const uint32_t *ro;
    uint32_t n;
    uint32_t size;
    uint32_t *levels;
    uint32_t *visited;
    uint32_t *q0;
    uint32_t *q1;
    uint32_t *ctl;
};

__global__ void __launch_bounds__(BLOCK) bfs_kernel(BfsArgs A) {
    GridBarrier *bar = reinterpret_cast<GridBarrier *>(A.ctl + CTL_BAR);
    uint32_t *err = A.ctl + CTL_ERR;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gwarp = blockIdx.x * (BLOCK / 32) + (threadIdx.x >> 5);
    const uint32_t nwarps = gridDim.x * (BLOCK / 32);
    uint32_t added = 0;
    uint32_t i = 0;
    for (;; ++i) {
        const uint32_t nq = ld_volatile(A.ctl + CTL_CNT + i % 3);
        if (nq == 0)
            break;
        if (blockIdx.x == 0 && threadIdx.x == 0)
            A.ctl[CTL_CNT + (i + 2) % 3] = 0;
        uint32_t *out_cnt = A.ctl + CTL_CNT + (i + 1) % 3;
        const uint32_t *qin = (i & 1) ? A.q1 : A.q0;
        uint32_t *qout = (i & 1) ? A.q0 : A.q1;
        const uint32_t next_level = i + 2;
        for (uint32_t idx = gwarp; idx < nq; idx += nwarps) {
            const uint32_t u = qin[idx];
            uint32_t b = A.ro[u], e = A.ro[u + 1];
            e = min(e, A.size);
            for (uint32_t s0 = b; s0 < e; s0 += 32) {
                const uint32_t s = s0 + lane;
                bool fresh = false;
                uint32_t w = 0;
                if (s < e) {
                    const uint64_t k = A.keys[s];
                    const uint8_t v = A.vals[s];
                    w = (uint32_t)k;
                    if (w != 0xFFFFFFFFu && v != 0 && w < A.n) {
                        const uint32_t bit = 1u << (w & 31);
                        if (!(A.visited[w >> 5] & bit)) {
                            const uint32_t old = atomicOr(&A.visited[w >> 5], bit);
                            fresh = !(old & bit);
                        }
                    }
                }
                const uint32_t ballot = __ballot_sync(0xFFFFFFFFu, fresh);
                if (ballot) {
                    uint32_t basepos = 0;
                    const int leader = __ffs(ballot) - 1;
                    if ((int)lane == leader)
                        basepos = atomicAdd(out_cnt, __popc(ballot));
                    basepos = __shfl_sync(0xFFFFFFFFu, basepos, leader);
                    if (fresh) {
                        A.levels[w] = next_level;
                        qout[basepos + __popc(ballot & lanemask_lt())] = w;
                    }
                    added += (lane == (uint32_t)leader) ? __popc(ballot) : 0;
                }
            }
        }
        if (!grid_barrier(bar, err))
            return;
    }
    if (added)
        atomicAdd(A.ctl + CTL_REACHED, added);
    if (blockIdx.x == 0 && threadIdx.x == 0)
        A.ctl[CTL_LEVELS] = i;
}

__global__ void bfs_init_kernel(uint32_t *levels, uint32_t *visited, uint32_t *q0, uint32_t *ctl, uint32_t src) {
    levels[src] = 1;
    visited[src >> 5] = 1u << (src & 31);
    q0[0] = src;
    ctl[CTL_CNT + 0] = 1;
    ctl[CTL_CNT + 1] = 0;
    ctl[CTL_CNT + 2] = 0;
    ctl[CTL_REACHED] = 1;
}

// ---- multi-source ----------------------------------------------------------

struct MsArgs {
    const uint64_t *keys;
    const uint8_t *vals;
    const uint32_t *ro;
    uint32_t n, size, k;
    const uint32_t *src;
    uint64_t *visited;
    uint64_t *frontier;
    uint64_t *next;
    uint32_t *levels;  // [k][n]
    uint32_t *ctl;
};

__global__ void __launch_bounds__(BLOCK) msbfs_kernel(MsArgs A) {
    GridBarrier *bar = reinterpret_cast<GridBarrier *>(A.ctl + CTL_BAR);
    uint32_t *err = A.ctl + CTL_ERR;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gwarp = blockIdx.x * (BLOCK / 32) + (threadIdx.x >> 5);
    const uint32_t nwarps = gridDim.x * (BLOCK / 32);
    const uint32_t gtid = blockIdx.x * BLOCK + threadIdx.x;
    const uint32_t nthreads = gridDim.x * BLOCK;
    // init: masks cleared by the host; seed the sources
    if (gtid < A.k) {
        uint32_t s = A.src[gtid];
        atomicOr((unsigned long long *)&A.visited[s], 1ull << gtid);
        atomicOr((unsigned long long *)&A.frontier[s], 1ull << gtid);
        A.levels[(uint64_t)gtid * A.n + s] = 1;
    }
    if (!grid_barrier(bar, err))
        return;
    uint32_t level = 1;
    for (;; ++level) {
        // expand: every node with a frontier mask pushes it to its targets
        for (uint32_t base = gwarp * 32; base < A.n; base += nwarps * 32) {
            const uint32_t u = base + lane;
            const uint64_t f = u < A.n ? A.frontier[u] : 0ull;
            uint32_t todo = __ballot_sync(0xFFFFFFFFu, f != 0ull);
            while (todo) {
                const int src_lane = __ffs(todo) - 1;
                todo &= todo - 1;
                const uint32_t uu = base + src_lane;
                const uint64_t fm = __shfl_sync(0xFFFFFFFFu, f, src_lane);
                const uint32_t b = A.ro[uu], e = min(A.ro[uu + 1], A.size);
                for (uint32_t s = b + lane; s < e; s += 32) {
                    const uint64_t key = A.keys[s];
                    const uint32_t w = (uint32_t)key;
                    if (w == 0xFFFFFFFFu || A.vals[s] == 0 || w >= A.n)
                        continue;
                    const uint64_t nb = fm & ~A.visited[w];
                    if (nb && (A.next[w] & nb) != nb)
                        atomicOr((unsigned long long *)&A.next[w], nb);
                }
            }
        }
        if (!grid_barrier(bar, err))
            return;
        // commit: next -> frontier, record levels of newly reached lanes
        uint32_t changed = 0;
        for (uint32_t w = gtid; w < A.n; w += nthreads) {
            const uint64_t nx = A.next[w] & ~A.visited[w];
            A.frontier[w] = nx;
            if (nx) {
                A.next[w] = 0;
                A.visited[w] |= nx;
                uint64_t m = nx;
                while (m) {
                    const int bit = __ffsll((long long)m) - 1;
                    m &= m - 1;
                    A.levels[(uint64_t)bit * A.n + w] = level + 1;
                }
                changed = 1;
            } else if (A.next[w]) {
                A.next[w] = 0;
            }
        }
        const uint32_t any = __syncthreads_or(changed);
        if (any && threadIdx.x == 0)
            atomicAdd(A.ctl + CTL_CNT + (level % 3), 1u);
        if (blockIdx.x == 0 && threadIdx.x == 0)
            A.ctl[CTL_CNT + ((level + 1) % 3)] = 0;
        if (!grid_barrier(bar, err))
            return;
        if (ld_volatile(A.ctl + CTL_CNT + (level % 3)) == 0)
            break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
        A.ctl[CTL_LEVELS] = level;
}

// reached[i] = number of non-zero entries of levels[i][0..n)
__global__ void count_reached_kernel(const uint32_t *levels, uint32_t n, uint32_t k, unsigned long long *reached) {
    __shared__ uint32_t tmp[BLOCK / 32 + 1];
    for (uint32_t i = 0; i < k; ++i) {
        uint32_t c = 0;
        for (uint32_t w = blockIdx.x * BLOCK + threadIdx.x; w < n; w += gridDim.x * BLOCK)
            c += levels[(uint64_t)i * n + w] != 0;
        uint32_t t = block_sum(c, tmp);
        if (threadIdx.x == 0 && t)
            atomicAdd(&reached[i], (unsigned long long)t);
    }
}

gpma_status ensure_bfs(gpma_graph *g) {
    if (g->bfs_cap >= g->row_num && g->bfs_levels)
        return GPMA_OK;
    free_bfs(g);
    uint32_t n = std::max<uint32_t>(g->row_num, 1);
    GPMA_TRY(dev_alloc(&g->bfs_levels, n));
    GPMA_TRY(dev_alloc(&g->bfs_visited, n / 32 + 2));
    GPMA_TRY(dev_alloc(&g->bfs_queue[0], n));
    GPMA_TRY(dev_alloc(&g->bfs_queue[1], n));
    GPMA_TRY(dev_alloc(&g->bfs_ctl, CTL_WORDS + 2 * 64));
    if (!g->h_bfs_ctl) {
        cudaError_t e = cudaMallocHost((void **)&g->h_bfs_ctl, sizeof(uint32_t) * (CTL_WORDS + 2 * 64));
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaMallocHost(bfs ctl)");
    }
    g->bfs_cap = n;
    if (g->bfs_grid == 0) {
        int per_sm = 0;
        GPMA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bfs_kernel, BLOCK, 0));
        int per_sm2 = 0;
        GPMA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm2, msbfs_kernel, BLOCK, 0));
        per_sm = std::min(per_sm, per_sm2);
        if (per_sm < 1) {
            set_error("BFS kernel cannot be resident (occupancy 0)");
            return GPMA_ERR_CUDA;
        }
        g->bfs_grid = g->sms * std::min(per_sm, 8);
    }
    return GPMA_OK;
}

}  // namespace

void free_bfs(gpma_graph *g) {
    dev_free(g->bfs_levels);
    dev_free(g->bfs_visited);
    dev_free(g->bfs_queue[0]);
    dev_free(g->bfs_queue[1]);
    dev_free(g->bfs_ctl);
    for (int i = 0; i < 3; ++i)
        dev_free(g->msbfs_mask[i]);
    dev_free(g->msbfs_levels);
    dev_free(g->msbfs_src);
    g->msbfs_levels_cap = 0;
    g->bfs_cap = 0;
}

// Levels land in g->bfs_levels; *reached is the count of reached nodes.
gpma_status bfs_run(gpma_graph *g, uint32_t src, cudaStream_t s, uint64_t *reached) {
    GPMA_TRY(ensure_bfs(g));
    const uint32_t n = g->row_num;
    GPMA_CUDA(cudaMemsetAsync(g->bfs_levels, 0, sizeof(uint32_t) * n, s));
    GPMA_CUDA(cudaMemsetAsync(g->bfs_visited, 0, sizeof(uint32_t) * (n / 32 + 2), s));
    GPMA_CUDA(cudaMemsetAsync(g->bfs_ctl, 0, sizeof(uint32_t) * CTL_WORDS, s));
    prof_mark(g, 0, s);
    bfs_init_kernel<<<1, 1, 0, s>>>(g->bfs_levels, g->bfs_visited, g->bfs_queue[0], g->bfs_ctl, src);
    BfsArgs A;
    A.keys = g->keys;
    A.vals = g->values;
    A.ro = g->row_offset;
    A.n = n;
    A.size = g->geo.size;
    A.levels = g->bfs_levels;
    A.visited = g->bfs_visited;
    A.q0 = g->bfs_queue[0];
    A.q1 = g->bfs_queue[1];
    A.ctl = g->bfs_ctl;
    void *params[] = {&A};
    GPMA_CUDA(cudaLaunchCooperativeKernel((const void *)bfs_kernel, dim3(g->bfs_grid), dim3(BLOCK), params, 0, s));
    prof_mark(g, 1, s);
    GPMA_CUDA(cudaMemcpyAsync(g->h_bfs_ctl, g->bfs_ctl, sizeof(uint32_t) * CTL_WORDS, cudaMemcpyDeviceToHost, s));
    GPMA_CUDA(cudaStreamSynchronize(s));
    g->prof.kernel_launches += 2;
    g->prof.bfs_kernels++;
    g->prof.bfs_ms += prof_elapsed(g, 0, 1);
    if (g->h_bfs_ctl[CTL_ERR]) {
        set_error("device-side wait gave up in the BFS kernel (code %u)", g->h_bfs_ctl[CTL_ERR]);
        return GPMA_ERR_TIMEOUT;
    }
    if (reached)
        *reached = g->h_bfs_ctl[CTL_REACHED];
    return GPMA_OK;
}

// Levels land in g->msbfs_levels ([k][n]); reached counts in the tail of
// bfs_ctl (read back by the caller).
gpma_status bfs_multi_run(gpma_graph *g, const uint32_t *d_src, uint32_t k, cudaStream_t s) {
    GPMA_TRY(ensure_bfs(g));
    const uint32_t n = g->row_num;
    if (!g->msbfs_mask[0]) {
        for (int i = 0; i < 3; ++i)
            GPMA_TRY(dev_alloc(&g->msbfs_mask[i], std::max<uint32_t>(n, 1)));
    }
    const uint64_t need = (uint64_t)k * n;
    if (need > g->msbfs_levels_cap) {
        dev_free(g->msbfs_levels);
        GPMA_TRY(dev_alloc(&g->msbfs_levels, need));
        g->msbfs_levels_cap = need;
    }
    for (int i = 0; i < 3; ++i)
        GPMA_CUDA(cudaMemsetAsync(g->msbfs_mask[i], 0, sizeof(uint64_t) * n, s));
    GPMA_CUDA(cudaMemsetAsync(g->msbfs_levels, 0, sizeof(uint32_t) * need, s));
    GPMA_CUDA(cudaMemsetAsync(g->bfs_ctl, 0, sizeof(uint32_t) * (CTL_WORDS + 2 * 64), s));
    MsArgs A;
    A.keys = g->keys;
    A.vals = g->values;
    A.ro = g->row_offset;
    A.n = n;
    A.size = g->geo.size;
    A.k = k;
    A.src = d_src;
    A.visited = g->msbfs_mask[0];
    A.frontier = g->msbfs_mask[1];
    A.next = g->msbfs_mask[2];
    A.levels = g->msbfs_levels;
    A.ctl = g->bfs_ctl;
    void *params[] = {&A};
    prof_mark(g, 0, s);
    GPMA_CUDA(cudaLaunchCooperativeKernel((const void *)msbfs_kernel, dim3(g->bfs_grid), dim3(BLOCK), params, 0, s));
    prof_mark(g, 1, s);
    unsigned long long *reached = reinterpret_cast<unsigned long long *>(g->bfs_ctl + CTL_WORDS);
    count_reached_kernel<<<std::max(1, std::min(g->sms * 4, (int)((n + BLOCK - 1) / BLOCK))), BLOCK, 0, s>>>(
        g->msbfs_levels, n, k, reached);
    GPMA_CUDA(cudaGetLastError());
    GPMA_CUDA(cudaMemcpyAsync(g->h_bfs_ctl, g->bfs_ctl, sizeof(uint32_t) * (CTL_WORDS + 2 * 64),
                              cudaMemcpyDeviceToHost, s));
    GPMA_CUDA(cudaStreamSynchronize(s));
    g->prof.kernel_launches += 2;
    g->prof.bfs_kernels++;
    g->prof.bfs_ms += prof_elapsed(g, 0, 1);
    if (g->h_bfs_ctl[CTL_ERR]) {
        set_error("device-side wait gave up in the multi-source BFS kernel (code %u)", g->h_bfs_ctl[CTL_ERR]);
        return GPMA_ERR_TIMEOUT;
    }
    return GPMA_OK;
}

// ---- BFS without device allocation ------------------------------------------
// Some callers cannot allocate device memory on the fly: code that runs under
// a host-side memory arena or a fixed device-memory budget, plug-ins whose
// host process owns every cudaMalloc, or hosts whose pool forbids growth once
// serving starts. For them gpma_bfs_noalloc keeps the BFS working set (visited
// bitmap, two frontier queues, control words) in one file-scope device array
// of a fixed size instead of buffers allocated per graph. Every GPU that loads
// this library holds the array (about 17 MB) until the process exits.
namespace {

constexpr uint32_t NOALLOC_MAX_ROWS = 1u << 21;  // 2,097,152 nodes
constexpr uint32_t NOALLOC_VISITED_WORDS = NOALLOC_MAX_ROWS / 32 + 2;
constexpr size_t NOALLOC_WORDS = CTL_WORDS + NOALLOC_VISITED_WORDS + 2ull * NOALLOC_MAX_ROWS;
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
        g_noalloc_grid[dev] = sms * std::min(per_sm, 8);
        g_noalloc_ptr[dev] = static_cast<uint32_t *>(p);
    }
    *out = g_noalloc_ptr[dev];
    *grid = g_noalloc_grid[dev];
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
    uint32_t *q0 = visited + NOALLOC_VISITED_WORDS;
    uint32_t *q1 = q0 + NOALLOC_MAX_ROWS;
    // the scratch keeps the previous call's contents: clear what must start at zero
    GPMA_CUDA(cudaMemsetAsync(levels, 0, sizeof(uint32_t) * n, s));
    GPMA_CUDA(cudaMemsetAsync(visited, 0, sizeof(uint32_t) * (n / 32 + 2), s));
    GPMA_CUDA(cudaMemsetAsync(ctl, 0, sizeof(uint32_t) * CTL_WORDS, s));
    bfs_init_kernel<<<1, 1, 0, s>>>(levels, visited, q0, ctl, src);
    BfsArgs A;
    A.keys = g->keys;
    A.vals = g->values;
    A.ro = g->row_offset;
    A.n = n;
    A.size = g->geo.size;
    A.levels = levels;
    A.visited = visited;
    A.q0 = q0;
    A.q1 = q1;
    A.ctl = ctl;
    void *params[] = {&A};
    GPMA_CUDA(cudaLaunchCooperativeKernel((const void *)bfs_kernel, dim3(grid), dim3(BLOCK), params, 0, s));
    uint32_t h_ctl[CTL_WORDS];
    GPMA_CUDA(cudaMemcpyAsync(h_ctl, ctl, sizeof(h_ctl), cudaMemcpyDeviceToHost, s));
    GPMA_CUDA(cudaStreamSynchronize(s));
    if (h_ctl[CTL_ERR]) {
        set_error("device-side wait gave up in the BFS kernel (code %u)", h_ctl[CTL_ERR]);
        return GPMA_ERR_TIMEOUT;
    }
    if (reached)
        *reached = h_ctl[CTL_REACHED];
    return GPMA_OK;
}

}  // namespace gpma
