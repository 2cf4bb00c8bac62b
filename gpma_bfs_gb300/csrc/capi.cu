// capi.cu - the extern "C" boundary of the library (include/gpma_gb300.h).
#include "gpma_internal.cuh"

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

namespace gpma {

static thread_local char g_last_error[512] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

gpma_status device_error(const char *where, uint32_t code) {
    if ((code & 0xFFu) == DERR_BOUNDS) {
        set_error("out-of-range index in %s (bounds-checked build, site %u)", where, code >> 8);
        return GPMA_ERR_DEVICE;
    }
    set_error("device-side wait gave up in %s (code %u)", where, code);
    return GPMA_ERR_TIMEOUT;
}

gpma_status cuda_fail(cudaError_t e, const char *what) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? GPMA_ERR_NOMEM : GPMA_ERR_CUDA;
}

// The device address of page-locked host memory, or null for anything else.
const void *mapped_host_pointer(const void *p) {
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return attr.type == cudaMemoryTypeHost ? attr.devicePointer : nullptr;
}

bool is_device_pointer(const void *p) {
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

gpma_status copy_any(void *dst, const void *src, size_t bytes, cudaStream_t s) {
    if (bytes == 0)
        return GPMA_OK;
    GPMA_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, s));
    return GPMA_OK;
}

namespace {

// Stage a pageable host copy through a pinned buffer so the transfer is a
// true async DMA; device and pinned pointers are copied directly.
gpma_status copy_in(gpma_graph *g, void *dst_dev, const void *src, size_t bytes, cudaStream_t s) {
    if (bytes == 0)
        return GPMA_OK;
    cudaPointerAttributes attr;
    bool known = cudaPointerGetAttributes(&attr, src) == cudaSuccess;
    if (!known)
        cudaGetLastError();
    if (known && attr.type != cudaMemoryTypeUnregistered)
        return copy_any(dst_dev, src, bytes, s);
    (void)g;
    GPMA_CUDA(cudaMemcpyAsync(dst_dev, src, bytes, cudaMemcpyHostToDevice, s));
    return GPMA_OK;
}

void release(gpma_graph *g) {
    dev_free(g->keys);
    dev_free(g->values);
    dev_free(g->heads);
    dev_free(g->row_offset);
    dev_free(g->skeys);
    dev_free(g->svals);
    dev_free(g->chunk_cnt);
    free_buffers(g->buf);
    free_bfs(g);
    dev_free(g->an_buf);
    g->an_cap = 0;
    if (g->own_batch)
        gpma_batch_destroy(g->own_batch);
    g->own_batch = nullptr;
    for (auto &e : g->ev)
        if (e)
            cudaEventDestroy(e);
    if (g->h_bfs_ctl)
        cudaFreeHost(g->h_bfs_ctl);
    g->h_bfs_ctl = nullptr;
}

__global__ void init_layout_kernel(uint64_t *keys, uint8_t *vals) {
    // init_gpma_members (gpma.cuh:54-69): 4 slots, KEY_MAX at 0 and 2
    int t = threadIdx.x;
    if (t < 4) {
        keys[t] = (t == 0 || t == 2) ? KEY_MAX : KEY_NONE;
        vals[t] = (t == 0 || t == 2) ? 1 : 0;
    }
}

__global__ void guard_keys_kernel(uint64_t *keys, uint8_t *vals, uint32_t row_num) {
    // init_gpma_insertions (gpma.cuh:70-78): (r << 32) | 0xFFFFFFFF, value 1
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < row_num; r += gridDim.x * blockDim.x) {
        keys[r] = ((uint64_t)r << 32) + COL_NONE;
        vals[r] = 1;
    }
}

__global__ void mask_values_kernel(const uint64_t *keys, const uint8_t *vals, uint8_t *out, uint32_t size) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < size; t += gridDim.x * blockDim.x)
        out[t] = keys[t] == KEY_NONE ? 0 : vals[t];
}

__global__ void live_flags_kernel(const uint64_t *keys, const uint8_t *vals, uint32_t size, uint32_t *chunk_cnt) {
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

__global__ void scan_chunks_kernel(uint32_t *chunk_cnt, uint32_t chunks, uint32_t *total) {
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

__global__ void gather_live_kernel(const uint64_t *keys, const uint8_t *vals, uint32_t size, const uint32_t *off,
                                   uint64_t *out) {
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
        uint32_t o = off[c] + block_excl_scan(cl, &tot, tmp);
        for (uint32_t j = 0; j < K; ++j) {
            uint32_t t = base + j;
            if (t < size && keys[t] != KEY_NONE && vals[t] != 0)
                out[o++] = keys[t];
        }
    }
}

// Destination segment j (dst_off[j] .. dst_off[j+1]) copied from the source
// starting at src_start[j]: stages batches in segment-length order.
struct GatherArgs {
    uint64_t *dk;
    uint8_t *dv;
    const uint64_t *sk;
    const uint8_t *sv;
    const uint64_t *dst_off;    // m + 1
    const uint64_t *src_start;  // m
    uint32_t m;
    const uint32_t *abort;  // non-zero: return at once (a recorded step after one needing host work)
};
__global__ void gather_segments_kernel(GatherArgs A) {
    if (A.abort && *(const volatile uint32_t *)A.abort)
        return;
    const uint64_t n = A.dst_off[A.m];
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = A.m;
        while (hi - lo > 1) {
            uint32_t mid = (lo + hi) >> 1;
            if (A.dst_off[mid] <= t)
                lo = mid;
            else
                hi = mid;
        }
        const uint64_t src = A.src_start[lo] + (t - A.dst_off[lo]);
        A.dk[t] = A.sk[src];
        A.dv[t] = A.sv[src];
    }
}

int small_grid(uint64_t work, int sms) {
    uint64_t g = (work + BLOCK - 1) / BLOCK;
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(g, (uint64_t)sms * 8));
}

}  // namespace

gpma_status packed_plan(gpma_batch *b, gpma_graph *const *graphs, const uint64_t *keys, const uint8_t *values,
                        const uint64_t *offsets, uint32_t k, PackedPlan *P, const uint32_t *abort) {
    static_assert(sizeof(GatherArgs) <= KernelLaunch::ARG_BYTES, "gather arguments exceed the launch record");
    const uint64_t all = k ? offsets[k] - offsets[0] : 0;
    std::vector<uint32_t> order;
    uint64_t total = 0;
    P->bulk.clear();
    for (uint32_t i = 0; i < k; ++i) {
        const uint64_t c = offsets[i + 1] - offsets[i];
        if (c == 0)
            continue;
        if (c >= SIGNIFICANT_INSERTS) {
            P->bulk.push_back(i);
            continue;
        }
        order.push_back(i);
        total += c;
    }
    P->m = (uint32_t)order.size();
    P->gs.assign(P->m, nullptr);
    P->off.assign(P->m + 1, 0);
    if (P->m == 0)
        return GPMA_OK;
    std::stable_sort(order.begin(), order.end(),
                     [&](uint32_t x, uint32_t y) { return graphs[x]->geo.seg < graphs[y]->geo.seg; });
    GPMA_TRY(ensure_buffers(b->buf, std::max<uint64_t>(total, all), P->m));
    P->upload = !(is_device_pointer(keys) && is_device_pointer(values));
    P->all_keys = all;
    const uint64_t src_base = P->upload ? offsets[0] : 0;
    const uint32_t m = P->m;
    if (m > b->gather_cap || !b->gather_tab) {
        dev_free(b->gather_tab);
        if (b->h_gather_tab)
            cudaFreeHost(b->h_gather_tab);
        b->h_gather_tab = nullptr;
        b->gather_cap = 0;
        GPMA_TRY(dev_alloc(&b->gather_tab, 2ull * m + 1));
        GPMA_CUDA(cudaMallocHost((void **)&b->h_gather_tab, sizeof(uint64_t) * (2ull * m + 1)));
        b->gather_cap = m;
    }
    // destination offsets [0..m], then the source start of each destination segment
    uint64_t *tab = b->h_gather_tab;
    tab[0] = 0;
    for (uint32_t j = 0; j < m; ++j) {
        const uint32_t i = order[j];
        P->gs[j] = graphs[i];
        P->off[j + 1] = P->off[j] + (offsets[i + 1] - offsets[i]);
        tab[j + 1] = P->off[j + 1];
        tab[m + 1 + j] = offsets[i] - src_base;
    }
    P->gtab_bytes = sizeof(uint64_t) * (2ull * m + 1);
    GatherArgs A;
    memset(&A, 0, sizeof(A));
    A.dk = b->buf.bkeys[0];
    A.dv = b->buf.bvals[0];
    A.sk = P->upload ? b->buf.bkeys[1] : keys;
    A.sv = P->upload ? b->buf.bvals[1] : values;
    A.dst_off = b->gather_tab;
    A.src_start = b->gather_tab + m + 1;
    A.m = m;
    A.abort = abort;
    P->gather.set((const void *)gather_segments_kernel, small_grid(total, b->sms), 0, &A, sizeof(A));
    return GPMA_OK;
}

gpma_status packed_stage(gpma_batch *b, const PackedPlan &P, const uint64_t *keys, const uint8_t *values,
                         const uint64_t *offsets, cudaStream_t s, bool with_table) {
    (void)P;
    if (P.upload) {
        // one upload of the packed range into the second sort buffer
        const uint64_t first = offsets[0];
        const uint64_t all = P.all_keys;
        GPMA_TRY(copy_any(b->buf.bkeys[1], keys + first, all * sizeof(uint64_t), s));
        GPMA_TRY(copy_any(b->buf.bvals[1], values + first, all, s));
    }
    if (with_table)
        GPMA_CUDA(cudaMemcpyAsync(b->gather_tab, b->h_gather_tab, P.gtab_bytes, cudaMemcpyHostToDevice, s));
    return GPMA_OK;
}

namespace {

}  // namespace
}  // namespace gpma

using namespace gpma;

extern "C" {

const char *gpma_version(void) { return "gpma_gb300 0.1 (sm_103a)"; }

const char *gpma_last_error(void) { return g_last_error; }

const char *gpma_status_string(gpma_status s) {
    switch (s) {
    case GPMA_OK: return "ok";
    case GPMA_ERR_INVALID: return "invalid argument";
    case GPMA_ERR_CUDA: return "CUDA runtime error";
    case GPMA_ERR_NOMEM: return "out of memory";
    case GPMA_ERR_CAPACITY: return "capacity exceeded";
    case GPMA_ERR_TIMEOUT: return "device wait timed out";
    case GPMA_ERR_IO: return "I/O error";
    case GPMA_ERR_DEVICE: return "device-side check failed";
    case GPMA_ERR_BUSY: return "server queue full";
    case GPMA_ERR_BUDGET: return "HBM admission budget exceeded";
    }
    return "unknown status";
}

gpma_status gpma_create(uint32_t row_num, void *stream, gpma_graph **out) {
    CallRange range("gpma_create");
    if (!out) {
        set_error("gpma_create: out is NULL");
        return GPMA_ERR_INVALID;
    }
    *out = nullptr;
    if (row_num >= 0xFFFFFFFFu) {
        set_error("gpma_create: row_num %u leaves no room for the reserved column", row_num);
        return GPMA_ERR_INVALID;
    }
    gpma_graph *g = new (std::nothrow) gpma_graph();
    if (!g) {
        set_error("gpma_create: host allocation failed");
        return GPMA_ERR_NOMEM;
    }
    cudaStream_t s = (cudaStream_t)stream;
    gpma_status st = [&]() -> gpma_status {
        GPMA_CUDA(cudaGetDevice(&g->device));
        GPMA_CUDA(cudaDeviceGetAttribute(&g->sms, cudaDevAttrMultiProcessorCount, g->device));
        g->row_num = row_num;
        g->cap = 4;
        GPMA_TRY(dev_alloc(&g->keys, 4));
        GPMA_TRY(dev_alloc(&g->values, 4));
        GPMA_TRY(dev_alloc(&g->row_offset, (uint64_t)row_num + 1));
        GPMA_TRY(ensure_scratch(g, 4));
        GPMA_CUDA(cudaMemsetAsync(g->row_offset, 0, sizeof(uint32_t) * ((uint64_t)row_num + 1), s));
        init_layout_kernel<<<1, 32, 0, s>>>(g->keys, g->values);
        GPMA_CUDA(cudaGetLastError());
        g->geo.size = 4;
        g->geo.seg = 2;
        g->geo.height = 1;
        recalculate_density(g->geo);
        GPMA_TRY(refresh_heads(g, s));
        if (row_num == 0)
            return GPMA_OK;
        GPMA_TRY(ensure_buffers(g->buf, row_num, 1));
        guard_keys_kernel<<<small_grid(row_num, g->sms), BLOCK, 0, s>>>(g->buf.bkeys[0], g->buf.bvals[0], row_num);
        GPMA_CUDA(cudaGetLastError());
        return update_device(g, row_num, s, /*check_keys=*/false);  // the guards use the reserved column
    }();
    if (st != GPMA_OK) {
        release(g);
        delete g;
        return st;
    }
    g->stats = gpma_stats{};
    g->prof = gpma_profile{};
    *out = g;
    return GPMA_OK;
}

gpma_status gpma_destroy(gpma_graph *g) {
    if (!g)
        return GPMA_OK;
    cudaDeviceSynchronize();
    release(g);
    delete g;
    return GPMA_OK;
}

gpma_status gpma_update(gpma_graph *g, const uint64_t *keys, const uint8_t *values, uint64_t n, void *stream) {
    CallRange range("gpma_update");
    if (!g || (n && (!keys || !values))) {
        set_error("gpma_update: null argument");
        return GPMA_ERR_INVALID;
    }
    if (n >= (1ull << 30)) {
        set_error("gpma_update: batch of %llu keys exceeds 2^30", (unsigned long long)n);
        return GPMA_ERR_CAPACITY;
    }
    g->stats.updates++;
    g->stats.submitted += n;
    if (n == 0)
        return GPMA_OK;
    cudaStream_t s = (cudaStream_t)stream;
    GPMA_TRY(ensure_buffers(g->buf, n, 1));
    if (is_device_pointer(keys) && is_device_pointer(values))
        return update_device(g, n, s, true, keys, values);  // the kernel reads the caller's batch in place
    {
        // page-locked host batches: the kernel reads them over the host link
        // itself (the keys twice: ranks, then the scatter), no staging copy
        const void *dk = mapped_host_pointer(keys), *dv = mapped_host_pointer(values);
        if (dk && dv)
            return update_device(g, n, s, true, static_cast<const uint64_t *>(dk), static_cast<const uint8_t *>(dv));
    }
    GPMA_TRY(copy_in(g, g->buf.bkeys[0], keys, n * sizeof(uint64_t), s));
    GPMA_TRY(copy_in(g, g->buf.bvals[0], values, n, s));
    return update_device(g, n, s);
}

gpma_status gpma_bfs(gpma_graph *g, uint32_t src, uint32_t *levels, uint64_t *reached, void *stream) {
    CallRange range("gpma_bfs");
    if (!g || !levels) {
        set_error("gpma_bfs: null argument");
        return GPMA_ERR_INVALID;
    }
    if (src >= g->row_num) {
        set_error("gpma_bfs: start node %u out of range (row_num %u)", src, g->row_num);
        return GPMA_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    GPMA_TRY(bfs_run(g, src, s, reached));
    GPMA_TRY(copy_any(levels, g->bfs_levels, sizeof(uint32_t) * g->row_num, s));
    GPMA_CUDA(cudaStreamSynchronize(s));
    return GPMA_OK;
}

gpma_status gpma_validate(gpma_graph *g, uint64_t *bad, void *stream) {
    CallRange range("gpma_validate");
    if (!g || !bad) {
        set_error("gpma_validate: null argument");
        return GPMA_ERR_INVALID;
    }
    return count_bad_heads(g, (cudaStream_t)stream, bad);
}

gpma_status gpma_bfs_noalloc(gpma_graph *g, uint32_t src, uint32_t *levels, uint64_t *reached, void *stream) {
    if (!g || !levels) {
        set_error("gpma_bfs_noalloc: null argument");
        return GPMA_ERR_INVALID;
    }
    if (src >= g->row_num) {
        set_error("gpma_bfs_noalloc: start node %u out of range (row_num %u)", src, g->row_num);
        return GPMA_ERR_INVALID;
    }
    if (!is_device_pointer(levels)) {
        set_error("gpma_bfs_noalloc: levels must be device memory (no staging buffer can be allocated)");
        return GPMA_ERR_INVALID;
    }
    return bfs_noalloc_run(g, src, levels, reached, (cudaStream_t)stream);
}

gpma_status gpma_bfs_multi(gpma_graph *g, const uint32_t *srcs, uint32_t k, uint32_t *levels, uint64_t *reached,
                           void *stream) {
    CallRange range("gpma_bfs_multi");
    if (!g || !srcs || !levels || k == 0 || k > 64) {
        set_error("gpma_bfs_multi: bad arguments (k must be 1..64)");
        return GPMA_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t hs[64];
    GPMA_TRY(copy_any(hs, srcs, sizeof(uint32_t) * k, s));
    GPMA_CUDA(cudaStreamSynchronize(s));
    for (uint32_t i = 0; i < k; ++i) {
        if (hs[i] >= g->row_num) {
            set_error("gpma_bfs_multi: source %u out of range (row_num %u)", hs[i], g->row_num);
            return GPMA_ERR_INVALID;
        }
    }
    if (!g->own_batch)
        GPMA_TRY(gpma_batch_create(&g->own_batch));
    gpma_graph *gl[1] = {g};
    const uint32_t *sl[1] = {hs};
    uint32_t *ll[1] = {levels};
    const uint32_t nl[1] = {k};
    g->own_batch->profiling = g->profiling;
    if (g->profiling && !g->own_batch->ev[0])
        for (auto &e : g->own_batch->ev)
            GPMA_CUDA(cudaEventCreate(&e));
    const gpma_profile before = g->own_batch->prof;
    GPMA_TRY(batch_bfs_run(g->own_batch, gl, sl, nl, 1, ll, reached, s));
    const gpma_profile &after = g->own_batch->prof;
    g->prof.bfs_ms += after.bfs_ms - before.bfs_ms;
    g->prof.bfs_kernels += after.bfs_kernels - before.bfs_kernels;
    g->prof.kernel_launches += after.kernel_launches - before.kernel_launches;
    g->prof.bfs_edges += after.bfs_edges - before.bfs_edges;
    return GPMA_OK;
}

// ---- many graphs per launch ---------------------------------------------------

gpma_status gpma_batch_create(gpma_batch **out) {
    if (!out) {
        set_error("gpma_batch_create: out is NULL");
        return GPMA_ERR_INVALID;
    }
    gpma_batch *b = new (std::nothrow) gpma_batch();
    if (!b) {
        set_error("gpma_batch_create: host allocation failed");
        return GPMA_ERR_NOMEM;
    }
    cudaError_t e = cudaGetDevice(&b->device);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    if (e != cudaSuccess) {
        delete b;
        return cuda_fail(e, "gpma_batch_create");
    }
    *out = b;
    return GPMA_OK;
}

gpma_status gpma_batch_destroy(gpma_batch *b) {
    if (!b)
        return GPMA_OK;
    cudaDeviceSynchronize();
    free_buffers(b->buf);
    free_batch_bfs(b);
    dev_free(b->gather_tab);
    if (b->h_gather_tab)
        cudaFreeHost(b->h_gather_tab);
    b->h_gather_tab = nullptr;
    for (auto &e : b->ev)
        if (e)
            cudaEventDestroy(e);
    delete b;
    return GPMA_OK;
}

gpma_status gpma_batch_update(gpma_batch *b, gpma_graph *const *graphs, const uint64_t *const *keys,
                              const uint8_t *const *values, const uint64_t *counts, uint32_t k, void *stream) {
    CallRange range("gpma_batch_update");
    if (!b || (k && (!graphs || !keys || !values || !counts))) {
        set_error("gpma_batch_update: null argument");
        return GPMA_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<uint32_t> order;
    uint64_t total = 0;
    for (uint32_t i = 0; i < k; ++i) {
        if (!graphs[i] || (counts[i] && (!keys[i] || !values[i]))) {
            set_error("gpma_batch_update: null graph or batch %u", i);
            return GPMA_ERR_INVALID;
        }
        for (uint32_t j = 0; j < i; ++j)
            if (graphs[j] == graphs[i]) {
                set_error("gpma_batch_update: graph %u appears twice", i);
                return GPMA_ERR_INVALID;
            }
        if (counts[i] >= (1ull << 30)) {
            set_error("gpma_batch_update: batch %u of %llu keys exceeds 2^30", i, (unsigned long long)counts[i]);
            return GPMA_ERR_CAPACITY;
        }
    }
    for (uint32_t i = 0; i < k; ++i) {
        graphs[i]->stats.updates++;
        graphs[i]->stats.submitted += counts[i];
        if (counts[i] == 0)
            continue;
        if (counts[i] >= SIGNIFICANT_INSERTS) {
            // a possible bulk rebuild: the single-graph path, on the graph's own buffers
            GPMA_TRY(ensure_buffers(graphs[i]->buf, counts[i], 1));
            GPMA_TRY(copy_in(graphs[i], graphs[i]->buf.bkeys[0], keys[i], counts[i] * sizeof(uint64_t), s));
            GPMA_TRY(copy_in(graphs[i], graphs[i]->buf.bvals[0], values[i], counts[i], s));
            GPMA_TRY(update_device(graphs[i], counts[i], s));
            continue;
        }
        order.push_back(i);
        total += counts[i];
    }
    if (order.empty())
        return GPMA_OK;
    if (total >= (1ull << 31)) {
        set_error("gpma_batch_update: %llu keys in one call exceed 2^31", (unsigned long long)total);
        return GPMA_ERR_CAPACITY;
    }
    // the kernel wants graphs ordered by segment length
    std::stable_sort(order.begin(), order.end(),
                     [&](uint32_t x, uint32_t y) { return graphs[x]->geo.seg < graphs[y]->geo.seg; });
    GPMA_TRY(ensure_buffers(b->buf, total, (uint32_t)order.size()));
    std::vector<gpma_graph *> gs(order.size());
    std::vector<uint64_t> off(order.size() + 1, 0);
    for (size_t j = 0; j < order.size(); ++j) {
        const uint32_t i = order[j];
        gs[j] = graphs[i];
        off[j + 1] = off[j] + counts[i];
        GPMA_TRY(copy_in(graphs[i], b->buf.bkeys[0] + off[j], keys[i], counts[i] * sizeof(uint64_t), s));
        GPMA_TRY(copy_in(graphs[i], b->buf.bvals[0] + off[j], values[i], counts[i], s));
    }
    return update_graphs(gs.data(), off.data(), (uint32_t)gs.size(), b->buf, b->sms, s, true, b->profiling, b->ev,
                         &b->prof);
}

gpma_status gpma_batch_update_packed(gpma_batch *b, gpma_graph *const *graphs, const uint64_t *keys,
                                     const uint8_t *values, const uint64_t *offsets, uint32_t k, void *stream) {
    CallRange range("gpma_batch_update_packed");
    if (!b || (k && (!graphs || !offsets || !keys || !values))) {
        set_error("gpma_batch_update_packed: null argument");
        return GPMA_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const uint64_t all = k ? offsets[k] - offsets[0] : 0;
    for (uint32_t i = 0; i < k; ++i) {
        if (!graphs[i] || offsets[i + 1] < offsets[i]) {
            set_error("gpma_batch_update_packed: null graph or decreasing offsets at %u", i);
            return GPMA_ERR_INVALID;
        }
        for (uint32_t j = 0; j < i; ++j)
            if (graphs[j] == graphs[i]) {
                set_error("gpma_batch_update_packed: graph %u appears twice", i);
                return GPMA_ERR_INVALID;
            }
    }
    if (all >= (1ull << 31)) {
        set_error("gpma_batch_update_packed: %llu keys in one call exceed 2^31", (unsigned long long)all);
        return GPMA_ERR_CAPACITY;
    }
    for (uint32_t i = 0; i < k; ++i) {
        graphs[i]->stats.updates++;
        graphs[i]->stats.submitted += offsets[i + 1] - offsets[i];
    }
    PackedPlan P;
    GPMA_TRY(packed_plan(b, graphs, keys, values, offsets, k, &P));
    for (uint32_t i : P.bulk) {
        // a possible bulk rebuild: the single-graph path, on the graph's own buffers
        const uint64_t c = offsets[i + 1] - offsets[i];
        GPMA_TRY(ensure_buffers(graphs[i]->buf, c, 1));
        GPMA_TRY(copy_any(graphs[i]->buf.bkeys[0], keys + offsets[i], c * sizeof(uint64_t), s));
        GPMA_TRY(copy_any(graphs[i]->buf.bvals[0], values + offsets[i], c, s));
        GPMA_TRY(update_device(graphs[i], c, s));
    }
    if (P.m == 0)
        return GPMA_OK;
    GPMA_TRY(packed_stage(b, P, keys, values, offsets, s));
    GPMA_CUDA(P.gather.launch(s));
    b->prof.kernel_launches += 1;
    return update_graphs(P.gs.data(), P.off.data(), P.m, b->buf, b->sms, s, true, b->profiling, b->ev, &b->prof);
}

gpma_status gpma_batch_bfs_multi(gpma_batch *b, gpma_graph *const *graphs, const uint32_t *const *srcs,
                                 const uint32_t *nsrc, uint32_t k, uint32_t *const *levels, uint64_t *reached,
                                 void *stream) {
    CallRange range("gpma_batch_bfs_multi");
    if (!b || (k && (!graphs || !srcs || !nsrc))) {
        set_error("gpma_batch_bfs_multi: null argument");
        return GPMA_ERR_INVALID;
    }
    if (k == 0)
        return GPMA_OK;
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<std::vector<uint32_t>> hs(k);
    std::vector<const uint32_t *> hp(k);
    uint64_t nodes = 0;
    for (uint32_t i = 0; i < k; ++i) {
        if (!graphs[i] || !srcs[i] || nsrc[i] == 0 || nsrc[i] > 64) {
            set_error("gpma_batch_bfs_multi: graph %u: null pointer or source count not in 1..64", i);
            return GPMA_ERR_INVALID;
        }
        hs[i].resize(nsrc[i]);
        GPMA_TRY(copy_any(hs[i].data(), srcs[i], sizeof(uint32_t) * nsrc[i], s));
        nodes += graphs[i]->row_num;
    }
    GPMA_CUDA(cudaStreamSynchronize(s));
    if (nodes >= (1ull << 32)) {
        set_error("gpma_batch_bfs_multi: %llu nodes in one call exceed 2^32", (unsigned long long)nodes);
        return GPMA_ERR_CAPACITY;
    }
    for (uint32_t i = 0; i < k; ++i) {
        for (uint32_t v : hs[i])
            if (v >= graphs[i]->row_num) {
                set_error("gpma_batch_bfs_multi: graph %u: source %u out of range (row_num %u)", i, v,
                          graphs[i]->row_num);
                return GPMA_ERR_INVALID;
            }
        hp[i] = hs[i].data();
    }
    return batch_bfs_run(b, graphs, hp.data(), nsrc, k, levels, reached, s);
}

gpma_status gpma_batch_set_profiling(gpma_batch *b, int enabled) {
    if (!b) {
        set_error("gpma_batch_set_profiling: null argument");
        return GPMA_ERR_INVALID;
    }
    if (enabled && !b->ev[0])
        for (auto &e : b->ev)
            GPMA_CUDA(cudaEventCreate(&e));
    b->profiling = enabled != 0;
    return GPMA_OK;
}

gpma_status gpma_batch_get_profile(const gpma_batch *b, gpma_profile *out) {
    if (!b || !out) {
        set_error("gpma_batch_get_profile: null argument");
        return GPMA_ERR_INVALID;
    }
    *out = b->prof;
    return GPMA_OK;
}

gpma_status gpma_batch_reset_profile(gpma_batch *b) {
    if (!b) {
        set_error("gpma_batch_reset_profile: null argument");
        return GPMA_ERR_INVALID;
    }
    b->prof = gpma_profile{};
    return GPMA_OK;
}

// ---- snapshot ------------------------------------------------------------------
// File: "GPMASNP1", then u32 version (1), row_num, size, segment_length,
// tree_height, u32 0, u64 payload checksum; payload: keys (size x u64),
// masked values (size x u8), row_offset ((row_num + 1) x u32). Integers are
// little-endian, written byte by byte.
}  // extern "C"

namespace gpma {
namespace {

const char SNAP_MAGIC[8] = {'G', 'P', 'M', 'A', 'S', 'N', 'P', '1'};
constexpr size_t SNAP_HEADER = 40;

void put_le(unsigned char *b, uint64_t v, int bytes) {
    for (int i = 0; i < bytes; ++i)
        b[i] = (unsigned char)(v >> (8 * i));
}

uint64_t get_le(const unsigned char *b, int bytes) {
    uint64_t v = 0;
    for (int i = 0; i < bytes; ++i)
        v |= (uint64_t)b[i] << (8 * i);
    return v;
}

// 64-bit multiply-xorshift mix over the payload bytes (not cryptographic:
// it detects truncation and corruption).
struct SnapHash {
    uint64_t h = 0x243F6A8885A308D3ull;
    void add(const unsigned char *p, size_t n) {
        for (size_t i = 0; i < n; ++i) {
            h = (h ^ p[i]) * 0x100000001B3ull;
            h ^= h >> 29;
        }
    }
};

// Host byte order independent serialisation of a u64 / u32 array chunk.
template <typename T>
void to_le(const T *a, size_t n, unsigned char *out) {
    for (size_t i = 0; i < n; ++i)
        put_le(out + i * sizeof(T), (uint64_t)a[i], (int)sizeof(T));
}

template <typename T>
void from_le(const unsigned char *in, size_t n, T *a) {
    for (size_t i = 0; i < n; ++i)
        a[i] = (T)get_le(in + i * sizeof(T), (int)sizeof(T));
}

bool valid_geometry(uint32_t size, uint32_t seg, uint32_t height) {
    if (size < 4 || (size & (size - 1)) != 0 || size > MAX_SLOTS)
        return false;
    // gpma.cuh:921-922
    const uint32_t want_seg = 1u << (fls32(fls32(size)) - 1);
    return seg == want_seg && height == fls32(size / seg) - 1;
}

// The structure the device code walks without further checks: row_offset
// starts at 0 and never decreases, row r's guard (r << 32 | 0xFFFFFFFF) sits
// at slot row_offset[r + 1] < size, and the live slots hold keys in
// ascending order. A file whose checksum matches but whose layout breaks one
// of these (written by another program, or edited) is refused before
// anything reaches the GPU: the BFS would otherwise walk row ranges outside
// the array.
const char *snapshot_layout_error(uint32_t row_num, uint32_t size, const uint64_t *keys, const unsigned char *vals,
                                  const uint32_t *ro) {
    if (ro[0] != 0)
        return "row_offset[0] is not 0";
    for (uint64_t r = 0; r < row_num; ++r) {
        const uint32_t at = ro[r + 1];
        if (at < ro[r] || at >= size)
            return "row_offset is not a non-decreasing list of slots inside the array";
        if (keys[at] != ((r << 32) | 0xFFFFFFFFull))
            return "a row guard is not at its row_offset slot";
    }
    bool any = false;
    uint64_t prev = 0;
    for (uint32_t i = 0; i < size; ++i) {
        if (keys[i] == KEY_NONE || vals[i] == 0)
            continue;
        if (any && keys[i] < prev)
            return "live slots are not in ascending key order";
        prev = keys[i];
        any = true;
    }
    return nullptr;
}

}  // namespace
}  // namespace gpma

extern "C" {

gpma_status gpma_save(gpma_graph *g, const char *path, void *stream) {
    CallRange range("gpma_save");
    if (!g || !path) {
        set_error("gpma_save: null argument");
        return GPMA_ERR_INVALID;
    }
    const uint32_t size = g->geo.size;
    const uint64_t ro_n = (uint64_t)g->row_num + 1;
    std::vector<uint64_t> keys(size);
    std::vector<uint8_t> vals(size);
    std::vector<uint32_t> ro(ro_n);
    GPMA_TRY(gpma_export_layout(g, keys.data(), vals.data(), ro.data(), stream));
    std::vector<unsigned char> payload(size * 9ull + ro_n * 4);
    to_le(keys.data(), size, payload.data());
    std::memcpy(payload.data() + size * 8ull, vals.data(), size);
    to_le(ro.data(), ro_n, payload.data() + size * 9ull);
    SnapHash hash;
    hash.add(payload.data(), payload.size());
    unsigned char hdr[SNAP_HEADER];
    std::memcpy(hdr, SNAP_MAGIC, 8);
    put_le(hdr + 8, 1, 4);
    put_le(hdr + 12, g->row_num, 4);
    put_le(hdr + 16, size, 4);
    put_le(hdr + 20, g->geo.seg, 4);
    put_le(hdr + 24, g->geo.height, 4);
    put_le(hdr + 28, 0, 4);
    put_le(hdr + 32, hash.h, 8);
    FILE *f = std::fopen(path, "wb");
    if (!f) {
        set_error("gpma_save: cannot open %s", path);
        return GPMA_ERR_IO;
    }
    bool bad = std::fwrite(hdr, 1, SNAP_HEADER, f) != SNAP_HEADER ||
               std::fwrite(payload.data(), 1, payload.size(), f) != payload.size();
    bad |= std::fclose(f) != 0;
    if (bad) {
        set_error("gpma_save: write to %s failed", path);
        return GPMA_ERR_IO;
    }
    return GPMA_OK;
}

gpma_status gpma_load(const char *path, void *stream, gpma_graph **out) {
    CallRange range("gpma_load");
    if (!path || !out) {
        set_error("gpma_load: null argument");
        return GPMA_ERR_INVALID;
    }
    *out = nullptr;
    FILE *f = std::fopen(path, "rb");
    if (!f) {
        set_error("gpma_load: cannot open %s", path);
        return GPMA_ERR_IO;
    }
    unsigned char hdr[SNAP_HEADER];
    if (std::fread(hdr, 1, SNAP_HEADER, f) != SNAP_HEADER || std::memcmp(hdr, SNAP_MAGIC, 8) != 0 ||
        get_le(hdr + 8, 4) != 1) {
        std::fclose(f);
        set_error("gpma_load: %s is not a snapshot of this version", path);
        return GPMA_ERR_IO;
    }
    const uint32_t row_num = (uint32_t)get_le(hdr + 12, 4), size = (uint32_t)get_le(hdr + 16, 4);
    const uint32_t seg = (uint32_t)get_le(hdr + 20, 4), height = (uint32_t)get_le(hdr + 24, 4);
    if (!valid_geometry(size, seg, height) || row_num >= 0xFFFFFFFFu) {
        std::fclose(f);
        set_error("gpma_load: %s holds an impossible geometry (size %u, segment %u, height %u)", path, size, seg,
                  height);
        return GPMA_ERR_IO;
    }
    const uint64_t ro_n = (uint64_t)row_num + 1;
    std::vector<unsigned char> payload(size * 9ull + ro_n * 4);
    const bool short_read = std::fread(payload.data(), 1, payload.size(), f) != payload.size();
    const bool trailing = !short_read && std::fgetc(f) != EOF;
    std::fclose(f);
    SnapHash hash;
    if (!short_read)
        hash.add(payload.data(), payload.size());
    if (short_read || trailing || hash.h != get_le(hdr + 32, 8)) {
        set_error("gpma_load: %s is truncated or corrupt", path);
        return GPMA_ERR_IO;
    }
    std::vector<uint64_t> keys(size);
    std::vector<uint32_t> ro(ro_n);
    from_le(payload.data(), size, keys.data());
    from_le(payload.data() + size * 9ull, ro_n, ro.data());
    if (const char *why = snapshot_layout_error(row_num, size, keys.data(), payload.data() + size * 8ull, ro.data())) {
        set_error("gpma_load: %s is not a valid layout: %s", path, why);
        return GPMA_ERR_IO;
    }
    gpma_graph *g = new (std::nothrow) gpma_graph();
    if (!g) {
        set_error("gpma_load: host allocation failed");
        return GPMA_ERR_NOMEM;
    }
    cudaStream_t s = (cudaStream_t)stream;
    gpma_status st = [&]() -> gpma_status {
        GPMA_CUDA(cudaGetDevice(&g->device));
        GPMA_CUDA(cudaDeviceGetAttribute(&g->sms, cudaDevAttrMultiProcessorCount, g->device));
        g->row_num = row_num;
        g->cap = size;
        GPMA_TRY(dev_alloc(&g->keys, size));
        GPMA_TRY(dev_alloc(&g->values, size));
        GPMA_TRY(dev_alloc(&g->row_offset, ro_n));
        GPMA_TRY(ensure_scratch(g, size));
        g->geo.size = size;
        g->geo.seg = seg;
        g->geo.height = height;
        recalculate_density(g->geo);
        GPMA_CUDA(cudaMemcpyAsync(g->keys, keys.data(), size * 8ull, cudaMemcpyHostToDevice, s));
        GPMA_CUDA(cudaMemcpyAsync(g->values, payload.data() + size * 8ull, size, cudaMemcpyHostToDevice, s));
        GPMA_CUDA(cudaMemcpyAsync(g->row_offset, ro.data(), ro_n * 4, cudaMemcpyHostToDevice, s));
        GPMA_TRY(refresh_heads(g, s));
        GPMA_CUDA(cudaStreamSynchronize(s));
        return GPMA_OK;
    }();
    if (st != GPMA_OK) {
        release(g);
        delete g;
        return st;
    }
    *out = g;
    return GPMA_OK;
}

gpma_status gpma_get_tuning(gpma_tuning *out) {
    if (!out) {
        set_error("gpma_get_tuning: null argument");
        return GPMA_ERR_INVALID;
    }
    *out = gpma_tuning{};
    out->bfs_dense_div = g_tuning.bfs_dense_div;
    out->bfs_blocks_per_sm = g_tuning.bfs_blocks_per_sm;
    out->ms_dense_div = g_tuning.ms_dense_div;
    out->ms_blocks_per_sm = g_tuning.ms_blocks_per_sm;
    out->update_blocks_per_sm = g_tuning.update_blocks_per_sm;
    out->update_sort = g_tuning.update_sort;
    return GPMA_OK;
}

gpma_status gpma_set_tuning(const gpma_tuning *t) {
    if (!t) {
        set_error("gpma_set_tuning: null argument");
        return GPMA_ERR_INVALID;
    }
    if (t->bfs_blocks_per_sm > MAX_BLOCKS_PER_SM || t->ms_blocks_per_sm > MAX_BLOCKS_PER_SM ||
        t->update_blocks_per_sm > MAX_BLOCKS_PER_SM) {
        set_error("gpma_set_tuning: CTAs per SM above %d", MAX_BLOCKS_PER_SM);
        return GPMA_ERR_INVALID;
    }
    if (t->update_sort > 1) {
        set_error("gpma_set_tuning: update_sort %u is not 0 (buckets) or 1 (digit passes)", t->update_sort);
        return GPMA_ERR_INVALID;
    }
    g_tuning.bfs_dense_div = t->bfs_dense_div;
    g_tuning.bfs_blocks_per_sm = t->bfs_blocks_per_sm;
    g_tuning.ms_dense_div = t->ms_dense_div;
    g_tuning.ms_blocks_per_sm = t->ms_blocks_per_sm;
    g_tuning.update_blocks_per_sm = t->update_blocks_per_sm;
    g_tuning.update_sort = t->update_sort;
    return GPMA_OK;
}

gpma_status gpma_get_test_hooks(gpma_test_hooks *out) {
    if (!out) {
        set_error("gpma_get_test_hooks: null argument");
        return GPMA_ERR_INVALID;
    }
    *out = gpma_test_hooks{};
    out->update_stall = g_test_hooks.update_stall;
    out->bfs_stall = g_test_hooks.bfs_stall;
    out->wait_limit_us = g_test_hooks.wait_limit_ns == WAIT_LIMIT_NS ? 0u
                                                                     : (uint32_t)(g_test_hooks.wait_limit_ns / 1000);
    out->noalloc_chunk_cap = g_test_hooks.noalloc_chunk_cap;
    out->noalloc_overflows = g_test_hooks.noalloc_overflows;
    return GPMA_OK;
}

gpma_status gpma_set_test_hooks(const gpma_test_hooks *h) {
    if (!h) {
        set_error("gpma_set_test_hooks: null argument");
        return GPMA_ERR_INVALID;
    }
    if (h->update_stall > 1 || h->bfs_stall > 1) {
        set_error("gpma_set_test_hooks: stall flags are 0 or 1");
        return GPMA_ERR_INVALID;
    }
    if (h->noalloc_chunk_cap > 65536) {
        set_error("gpma_set_test_hooks: noalloc_chunk_cap above 65536");
        return GPMA_ERR_INVALID;
    }
    g_test_hooks.update_stall = h->update_stall;
    g_test_hooks.bfs_stall = h->bfs_stall;
    g_test_hooks.wait_limit_ns = h->wait_limit_us ? 1000ull * h->wait_limit_us : WAIT_LIMIT_NS;
    g_test_hooks.noalloc_chunk_cap = h->noalloc_chunk_cap;
    return GPMA_OK;
}

gpma_status gpma_get_geometry(const gpma_graph *g, gpma_geometry *out) {
    if (!g || !out) {
        set_error("gpma_get_geometry: null argument");
        return GPMA_ERR_INVALID;
    }
    out->size = g->geo.size;
    out->segment_length = g->geo.seg;
    out->tree_height = g->geo.height;
    out->row_num = g->row_num;
    return GPMA_OK;
}

gpma_status gpma_get_thresholds(const gpma_graph *g, uint32_t *lower, uint32_t *upper) {
    if (!g) {
        set_error("gpma_get_thresholds: null argument");
        return GPMA_ERR_INVALID;
    }
    for (uint32_t i = 0; i <= g->geo.height; ++i) {
        if (lower)
            lower[i] = g->geo.lower[i];
        if (upper)
            upper[i] = g->geo.upper[i];
    }
    return GPMA_OK;
}

gpma_status gpma_export_layout(gpma_graph *g, uint64_t *keys, uint8_t *masked_values, uint32_t *row_offset,
                               void *stream) {
    CallRange range("gpma_export_layout");
    if (!g) {
        set_error("gpma_export_layout: null argument");
        return GPMA_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t size = g->geo.size;
    if (keys)
        GPMA_TRY(copy_any(keys, g->keys, sizeof(uint64_t) * size, s));
    if (masked_values) {
        uint8_t *tmp = nullptr;
        GPMA_TRY(dev_alloc(&tmp, size));
        mask_values_kernel<<<small_grid(size, g->sms), BLOCK, 0, s>>>(g->keys, g->values, tmp, size);
        gpma_status st = copy_any(masked_values, tmp, size, s);
        cudaStreamSynchronize(s);
        dev_free(tmp);
        GPMA_TRY(st);
    }
    if (row_offset)
        GPMA_TRY(copy_any(row_offset, g->row_offset, sizeof(uint32_t) * ((uint64_t)g->row_num + 1), s));
    GPMA_CUDA(cudaStreamSynchronize(s));
    return GPMA_OK;
}

gpma_status gpma_export_compact(gpma_graph *g, uint64_t *keys, uint64_t capacity, uint64_t *count, void *stream) {
    CallRange range("gpma_export_compact");
    if (!g || !count) {
        set_error("gpma_export_compact: null argument");
        return GPMA_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t size = g->geo.size;
    const uint32_t chunks = (size + CHUNK - 1) / CHUNK;
    uint32_t *off = nullptr;
    GPMA_TRY(dev_alloc(&off, chunks + 1));
    live_flags_kernel<<<small_grid((uint64_t)chunks * BLOCK, g->sms), BLOCK, 0, s>>>(g->keys, g->values, size, off);
    scan_chunks_kernel<<<1, BLOCK, 0, s>>>(off, chunks, off + chunks);
    uint32_t total = 0;
    cudaMemcpyAsync(&total, off + chunks, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        dev_free(off);
        return cuda_fail(e, "gpma_export_compact");
    }
    *count = total;
    gpma_status st = GPMA_OK;
    if (keys) {
        if (capacity < total) {
            set_error("gpma_export_compact: capacity %llu < %u live keys", (unsigned long long)capacity, total);
            st = GPMA_ERR_INVALID;
        } else {
            uint64_t *tmp = nullptr;
            st = dev_alloc(&tmp, total);
            if (st == GPMA_OK) {
                gather_live_kernel<<<small_grid((uint64_t)chunks * BLOCK, g->sms), BLOCK, 0, s>>>(g->keys, g->values,
                                                                                                 size, off, tmp);
                st = copy_any(keys, tmp, sizeof(uint64_t) * total, s);
                cudaStreamSynchronize(s);
                dev_free(tmp);
            }
        }
    }
    dev_free(off);
    return st;
}

gpma_status gpma_device_arrays(gpma_graph *g, const uint64_t **keys, const uint8_t **values,
                               const uint32_t **row_offset) {
    if (!g) {
        set_error("gpma_device_arrays: null argument");
        return GPMA_ERR_INVALID;
    }
    if (keys)
        *keys = g->keys;
    if (values)
        *values = g->values;
    if (row_offset)
        *row_offset = g->row_offset;
    return GPMA_OK;
}

gpma_status gpma_set_profiling(gpma_graph *g, int enabled) {
    if (!g) {
        set_error("gpma_set_profiling: null argument");
        return GPMA_ERR_INVALID;
    }
    if (enabled && !g->ev[0]) {
        for (auto &e : g->ev)
            GPMA_CUDA(cudaEventCreate(&e));
    }
    g->profiling = enabled != 0;
    return GPMA_OK;
}

gpma_status gpma_get_profile(const gpma_graph *g, gpma_profile *out) {
    if (!g || !out) {
        set_error("gpma_get_profile: null argument");
        return GPMA_ERR_INVALID;
    }
    *out = g->prof;
    return GPMA_OK;
}

gpma_status gpma_reset_profile(gpma_graph *g) {
    if (!g) {
        set_error("gpma_reset_profile: null argument");
        return GPMA_ERR_INVALID;
    }
    g->prof = gpma_profile{};
    return GPMA_OK;
}

gpma_status gpma_get_stats(const gpma_graph *g, gpma_stats *out) {
    if (!g || !out) {
        set_error("gpma_get_stats: null argument");
        return GPMA_ERR_INVALID;
    }
    *out = g->stats;
    return GPMA_OK;
}

}  // extern "C"
