// analytics.cu - PageRank and weakly connected components over the gapped PMA.
//
// No reference counterpart: the reference's only analytic is the BFS
// (gpma_bfs.cuh); GPMA+'s setting also covers connected components and
// PageRank. Both run as persistent cooperative kernels whose hot loop is one
// coalesced sweep over every slot of the array (16-byte key loads, 8 slots
// per thread): a slot is an edge u -> v when its value is non-zero and its
// column is not 0xFFFFFFFF (the BFS's rule), with u = key >> 32 and
// v = low word, both < row_num. No in-edge index is needed.
//
// PageRank (push form of y = d * A^T (x / deg) + teleport): per iteration
//   contrib[u] = rank[u] / outdeg[u] (dangling nodes pool their rank),
//   acc[v]    += contrib[u] for every edge (float atomics),
//   rank'[v]   = (1 - d) / n + d * (acc[v] + dangling / n);
// it stops after `iterations` or when sum |rank' - rank| < tol.
// Weakly connected components: parents start as the node ids; every edge
// hooks the larger of its endpoints' parents under the smaller (atomicMin),
// then pointer jumping shortens every chain; repeated until no edge hooks.
// Parents only decrease and stay inside their component, so each node ends
// labelled with the smallest node id of its component, whatever the order of
// the atomics.
#include "gpma_internal.cuh"

namespace gpma {
namespace {

enum : uint32_t {
    AN_ERR = 0,
    AN_ITERS = 1,
    AN_CHANGED = 2,  // 3 rotating flags (components)
    AN_BAR = 6,      // GridBarrier (2 words)
    AN_DBL = 8,      // doubles from word 8: dangling[3], delta[3]
    AN_WORDS = 8 + 12,
};

struct AnArgs {
    const uint64_t *keys;
    const uint8_t *vals;
    uint32_t n, size;
    uint32_t *deg;     // out-degree (PageRank)
    float *rank, *acc, *contrib;
    uint32_t *parent;  // components
    uint32_t *ctl;
    float damping;
    double tol;
    uint32_t max_iter;
};

// The 8 slots at o*8 as (u, v) edges; edge[j] false where the slot is not an edge.
__device__ __forceinline__ void load8(const AnArgs &A, uint32_t o, uint32_t (&u)[8], uint32_t (&v)[8],
                                      bool (&edge)[8]) {
    const ulonglong2 *kv = reinterpret_cast<const ulonglong2 *>(A.keys);
    const ulonglong2 k0 = kv[4 * o], k1 = kv[4 * o + 1], k2 = kv[4 * o + 2], k3 = kv[4 * o + 3];
    const uint2 vv = reinterpret_cast<const uint2 *>(A.vals)[o];
    const uint64_t k[8] = {k0.x, k0.y, k1.x, k1.y, k2.x, k2.y, k3.x, k3.y};
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        u[j] = (uint32_t)(k[j] >> 32);
        v[j] = (uint32_t)k[j];
        const uint32_t val = ((j < 4 ? vv.x : vv.y) >> (8 * (j & 3))) & 0xFFu;
        edge[j] = v[j] != 0xFFFFFFFFu && val != 0 && u[j] < A.n && v[j] < A.n;
    }
}

// Arrays of 4 slots (the smallest size) as one padded group of 8.
__device__ __forceinline__ void load_small(const AnArgs &A, uint32_t (&u)[8], uint32_t (&v)[8], bool (&edge)[8]) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const uint64_t k = j < 4 ? A.keys[j] : KEY_NONE;
        const uint32_t val = j < 4 ? A.vals[j] : 0u;
        u[j] = (uint32_t)(k >> 32);
        v[j] = (uint32_t)k;
        edge[j] = v[j] != 0xFFFFFFFFu && val != 0 && u[j] < A.n && v[j] < A.n;
    }
}

__device__ __forceinline__ double *an_dbl(const AnArgs &A, int which, uint32_t it) {
    return reinterpret_cast<double *>(A.ctl + AN_DBL) + which * 3 + it % 3;
}

__device__ __forceinline__ double block_sum_f64(double x, double *tmp) {
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1)
        x += __shfl_xor_sync(0xFFFFFFFFu, x, d);
    __syncthreads();
    if ((threadIdx.x & 31) == 0)
        tmp[threadIdx.x >> 5] = x;
    __syncthreads();
    double t = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < BLOCK / 32; ++w)
            t += tmp[w];
    return t;  // valid in thread 0
}

__global__ void __launch_bounds__(BLOCK) pagerank_kernel(AnArgs A) {
    GridBarrier *bar = reinterpret_cast<GridBarrier *>(A.ctl + AN_BAR);
    uint32_t *err = A.ctl + AN_ERR;
    __shared__ double tmp[BLOCK / 32];
    __shared__ double s_val;
    const uint32_t gtid = blockIdx.x * BLOCK + threadIdx.x, nthreads = gridDim.x * BLOCK;
    const uint32_t groups = A.size >> 3;
    const float teleport = (1.0f - A.damping) / (float)A.n;
    // out-degrees: slots are sorted by source, so a thread's 8 slots form a few
    // runs of one source; one atomic per run
    for (uint32_t v = gtid; v < A.n; v += nthreads)
        A.deg[v] = 0;
    if (!grid_barrier(bar, err))
        return;
    for (uint32_t o = gtid; o < groups || (A.size < 8 && o == 0); o += nthreads) {
        uint32_t u[8], v[8];
        bool e[8];
        if (A.size < 8)
            load_small(A, u, v, e);
        else
            load8(A, o, u, v, e);
        uint32_t run_u = 0xFFFFFFFFu, run = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (!e[j])
                continue;
            if (u[j] != run_u) {
                if (run)
                    atomicAdd(&A.deg[run_u], run);
                run_u = u[j];
                run = 0;
            }
            ++run;
        }
        if (run)
            atomicAdd(&A.deg[run_u], run);
        if (A.size < 8)
            break;
    }
    if (!grid_barrier(bar, err))
        return;
    uint32_t it = 0;
    for (; it < A.max_iter; ++it) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            *an_dbl(A, 0, it + 1) = 0.0;  // next iteration's sums start at zero
            *an_dbl(A, 1, it + 1) = 0.0;
        }
        double dang = 0;
        for (uint32_t v = gtid; v < A.n; v += nthreads) {
            const uint32_t d = A.deg[v];
            const float r = A.rank[v];
            A.contrib[v] = d ? r / (float)d : 0.0f;
            if (!d)
                dang += r;
        }
        dang = block_sum_f64(dang, tmp);
        if (threadIdx.x == 0 && dang != 0.0)
            atomicAdd(an_dbl(A, 0, it), dang);
        if (!grid_barrier(bar, err))
            return;
        for (uint32_t o = gtid; o < groups || (A.size < 8 && o == 0); o += nthreads) {
            uint32_t u[8], v[8];
            bool e[8];
            if (A.size < 8)
                load_small(A, u, v, e);
            else
                load8(A, o, u, v, e);
            float c[8];
#pragma unroll
            for (int j = 0; j < 8; ++j)
                c[j] = e[j] ? A.contrib[u[j]] : 0.0f;
#pragma unroll
            for (int j = 0; j < 8; ++j)
                if (e[j] && c[j] != 0.0f)
                    atomicAdd(&A.acc[v[j]], c[j]);
            if (A.size < 8)
                break;
        }
        if (!grid_barrier(bar, err))
            return;
        if (threadIdx.x == 0)
            s_val = *reinterpret_cast<volatile double *>(an_dbl(A, 0, it));
        __syncthreads();
        const float base = teleport + A.damping * (float)(s_val / (double)A.n);
        double delta = 0;
        for (uint32_t v = gtid; v < A.n; v += nthreads) {
            const float nr = base + A.damping * A.acc[v];
            delta += fabs((double)nr - (double)A.rank[v]);
            A.rank[v] = nr;
            A.acc[v] = 0.0f;
        }
        delta = block_sum_f64(delta, tmp);
        if (threadIdx.x == 0)
            atomicAdd(an_dbl(A, 1, it), delta);
        if (!grid_barrier(bar, err))
            return;
        if (threadIdx.x == 0)
            s_val = *reinterpret_cast<volatile double *>(an_dbl(A, 1, it));
        __syncthreads();
        if (s_val < A.tol) {
            ++it;
            break;
        }
    }
    if (gtid == 0)
        A.ctl[AN_ITERS] = it;
}

__global__ void __launch_bounds__(BLOCK) components_kernel(AnArgs A) {
    GridBarrier *bar = reinterpret_cast<GridBarrier *>(A.ctl + AN_BAR);
    uint32_t *err = A.ctl + AN_ERR;
    const uint32_t gtid = blockIdx.x * BLOCK + threadIdx.x, nthreads = gridDim.x * BLOCK;
    const uint32_t groups = A.size >> 3;
    for (uint32_t v = gtid; v < A.n; v += nthreads)
        A.parent[v] = v;
    if (!grid_barrier(bar, err))
        return;
    uint32_t it = 0;
    for (;; ++it) {
        if (blockIdx.x == 0 && threadIdx.x == 0)
            A.ctl[AN_CHANGED + (it + 1) % 3] = 0;
        uint32_t changed = 0;
        // hook: every edge joins its endpoints' parents, the larger under the smaller
        for (uint32_t o = gtid; o < groups || (A.size < 8 && o == 0); o += nthreads) {
            uint32_t u[8], v[8];
            bool e[8];
            if (A.size < 8)
                load_small(A, u, v, e);
            else
                load8(A, o, u, v, e);
            uint32_t pu[8], pv[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                pu[j] = e[j] ? A.parent[u[j]] : 0u;
                pv[j] = e[j] ? A.parent[v[j]] : 0u;
            }
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                if (e[j] && pu[j] != pv[j]) {
                    const uint32_t hi = max(pu[j], pv[j]), lo = min(pu[j], pv[j]);
                    if (atomicMin(&A.parent[hi], lo) > lo)
                        changed = 1;
                }
            }
            if (A.size < 8)
                break;
        }
        if (!grid_barrier(bar, err))
            return;
        // pointer jumping: every node to the end of its (decreasing) chain
        for (uint32_t v = gtid; v < A.n; v += nthreads) {
            uint32_t p = A.parent[v];
            uint32_t q = A.parent[p];
            while (q != p) {
                p = q;
                q = A.parent[p];
            }
            if (A.parent[v] != p)
                A.parent[v] = p;
        }
        if (__syncthreads_or(changed) && threadIdx.x == 0)
            atomicAdd(A.ctl + AN_CHANGED + it % 3, 1u);
        if (!grid_barrier(bar, err))
            return;
        if (cta_broadcast_read(A.ctl + AN_CHANGED + it % 3) == 0)
            break;
    }
    if (gtid == 0)
        A.ctl[AN_ITERS] = it + 1;
}

int an_fit[64] = {};

gpma_status launch(const void *kernel, AnArgs &A, int sms, cudaStream_t s, uint32_t *h_ctl) {
    int dev = 0;
    GPMA_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64)
        dev = 0;
    if (an_fit[dev] == 0) {
        int a = 0, b = 0;
        GPMA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, pagerank_kernel, BLOCK, 0));
        GPMA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, components_kernel, BLOCK, 0));
        an_fit[dev] = std::min(std::min(a, b), 8);
        if (an_fit[dev] < 1) {
            set_error("analytics kernels cannot be resident");
            return GPMA_ERR_CUDA;
        }
    }
    void *params[] = {&A};
    GPMA_CUDA(cudaLaunchCooperativeKernel(kernel, dim3(sms * an_fit[dev]), dim3(BLOCK), params, 0, s));
    GPMA_CUDA(cudaMemcpyAsync(h_ctl, A.ctl, sizeof(uint32_t) * AN_WORDS, cudaMemcpyDeviceToHost, s));
    GPMA_CUDA(cudaStreamSynchronize(s));
    if (h_ctl[AN_ERR])
        return device_error("an analytics kernel", h_ctl[AN_ERR]);
    return GPMA_OK;
}

// The graph's analytics buffer: 4 arrays of row_num words, then the control words.
gpma_status an_buffers(gpma_graph *g, uint32_t **base) {
    const uint32_t n = g->row_num;
    if (!g->an_buf || g->an_cap < n) {
        dev_free(g->an_buf);
        g->an_cap = 0;
        GPMA_TRY(dev_alloc(&g->an_buf, 4ull * n + AN_WORDS + 2));
        g->an_cap = n;
    }
    *base = g->an_buf;
    return GPMA_OK;
}

}  // namespace
}  // namespace gpma

using namespace gpma;

extern "C" {

gpma_status gpma_pagerank(gpma_graph *g, float damping, uint32_t iterations, double tol, float *ranks,
                          uint32_t *iterations_run, void *stream) {
    CallRange range("gpma_pagerank");
    if (!g || !ranks || !(damping >= 0.0f && damping <= 1.0f) || g->row_num == 0) {
        set_error("gpma_pagerank: bad arguments (damping in [0, 1], a graph with nodes, an output array)");
        return GPMA_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t n = g->row_num;
    uint32_t h_ctl[AN_WORDS];
    gpma_status st = [&]() -> gpma_status {
        uint32_t *base = nullptr;
        GPMA_TRY(an_buffers(g, &base));
        uint32_t *deg = base;
        float *rank = reinterpret_cast<float *>(base + n);
        float *acc = reinterpret_cast<float *>(base + 2ull * n);
        float *contrib = reinterpret_cast<float *>(base + 3ull * n);
        // control words 8-byte aligned (they hold doubles)
        uint32_t *ctl = base + ((4ull * n + 1) & ~1ull);
        GPMA_CUDA(cudaMemsetAsync(ctl, 0, sizeof(uint32_t) * AN_WORDS, s));
        GPMA_CUDA(cudaMemsetAsync(acc, 0, sizeof(float) * n, s));
        std::vector<float> init(n, 1.0f / (float)n);
        GPMA_CUDA(cudaMemcpyAsync(rank, init.data(), sizeof(float) * n, cudaMemcpyHostToDevice, s));
        AnArgs A{};
        A.keys = g->keys;
        A.vals = g->values;
        A.n = n;
        A.size = g->geo.size;
        A.deg = deg;
        A.rank = rank;
        A.acc = acc;
        A.contrib = contrib;
        A.ctl = ctl;
        A.damping = damping;
        A.tol = tol;
        A.max_iter = iterations;
        prof_mark(g, 0, s);
        GPMA_TRY(launch((const void *)pagerank_kernel, A, g->sms, s, h_ctl));
        prof_mark(g, 1, s);
        GPMA_TRY(copy_any(ranks, rank, sizeof(float) * n, s));
        GPMA_CUDA(cudaStreamSynchronize(s));
        g->prof.kernel_launches += 1;
        if (iterations_run)
            *iterations_run = h_ctl[AN_ITERS];
        return GPMA_OK;
    }();
    return st;
}

gpma_status gpma_components(gpma_graph *g, uint32_t *labels, uint64_t *components, uint32_t *rounds, void *stream) {
    CallRange range("gpma_components");
    if (!g || !labels) {
        set_error("gpma_components: null argument");
        return GPMA_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t n = g->row_num;
    if (n == 0) {
        if (components)
            *components = 0;
        return GPMA_OK;
    }
    uint32_t h_ctl[AN_WORDS];
    gpma_status st = [&]() -> gpma_status {
        uint32_t *base = nullptr;
        GPMA_TRY(an_buffers(g, &base));
        uint32_t *parent = base;
        uint32_t *ctl = base + ((4ull * n + 1) & ~1ull);
        GPMA_CUDA(cudaMemsetAsync(ctl, 0, sizeof(uint32_t) * AN_WORDS, s));
        AnArgs A{};
        A.keys = g->keys;
        A.vals = g->values;
        A.n = n;
        A.size = g->geo.size;
        A.parent = parent;
        A.ctl = ctl;
        GPMA_TRY(launch((const void *)components_kernel, A, g->sms, s, h_ctl));
        std::vector<uint32_t> host(n);
        GPMA_CUDA(cudaMemcpyAsync(host.data(), parent, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s));
        GPMA_CUDA(cudaStreamSynchronize(s));
        GPMA_TRY(copy_any(labels, host.data(), sizeof(uint32_t) * n, s));
        GPMA_CUDA(cudaStreamSynchronize(s));
        if (components) {
            uint64_t c = 0;
            for (uint32_t v = 0; v < n; ++v)
                c += host[v] == v;
            *components = c;
        }
        if (rounds)
            *rounds = h_ctl[AN_ITERS];
        g->prof.kernel_launches += 1;
        return GPMA_OK;
    }();
    return st;
}

}  // extern "C"
