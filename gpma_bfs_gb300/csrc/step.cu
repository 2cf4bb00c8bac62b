// step.cu - one sliding-window step of a graph (update_gpma of a batch, then
// BFS from one source) recorded once as a CUDA graph and replayed per step.
//
// The reference's demo loop (gpma_bfs_demo.cu, main loop) calls update_gpma
// and then gpma_bfs for every slide step; each call is a chain of launches,
// copies and host synchronisations. Here the device work of a whole step is
// one graph launch:
//   table upload -> update kernel (cooperative) -> 5 BFS clears -> BFS init ->
//   BFS kernel (cooperative) -> status and BFS control read-back
// with a single host synchronisation. The batch upload and the optional copy
// of the levels go on the same stream outside the graph, so the caller's
// buffers may be pageable, pinned or device memory.
//
// The graph is rebuilt only when something baked into its nodes changes
// (buffers reallocated, the kernel variant or grid, the array geometry
// enlarging the BFS buffers); the per-step arguments (batch size, status
// slot, source) are updated in place with cudaGraphExecKernelNodeSetParams.
// When the update kernel asks for host work (root resize, the bulk rebuild
// of a large batch) or fails, the step finishes on the host exactly as
// update_gpma does and the BFS is run again on the final array, so results
// are always those of update_gpma followed by gpma_bfs.
#include "gpma_internal.cuh"

#include <new>
#include <vector>

struct gpma_step {
    gpma_graph *g = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t n_update = nullptr, n_init = nullptr, n_bfs = nullptr;
    // what the nodes were built with
    gpma::KernelLaunch upd, bfs;
    uint32_t *init_args[4] = {};
    uint32_t init_src = 0;
    struct Baked {
        const void *h_tab, *d_tab, *d_stat, *bfs_ctl, *h_bfs_ctl;
        size_t tab_bytes, stat_slot, ctl_bytes;
        const void *upd_func, *bfs_func;
        unsigned upd_grid, bfs_grid;
        size_t upd_smem;
        void *clear_ptr[gpma::BfsPlan::CLEARS];
        size_t clear_bytes[gpma::BfsPlan::CLEARS];
    } baked{};
    unsigned char *h_stat = nullptr;  // pinned copy of both status slots
    size_t h_stat_bytes = 0;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    gpma_step_stats stats{};
};

namespace gpma {
namespace {

void drop_graph(gpma_step *st) {
    if (st->exec)
        cudaGraphExecDestroy(st->exec);
    if (st->graph)
        cudaGraphDestroy(st->graph);
    st->exec = nullptr;
    st->graph = nullptr;
    st->n_update = st->n_init = st->n_bfs = nullptr;
}

gpma_step::Baked bake(const gpma_graph *g, size_t tab_bytes, const KernelLaunch &upd, const BfsPlan &bp) {
    gpma_step::Baked b;
    memset(&b, 0, sizeof(b));  // compared byte-wise
    b.h_tab = g->buf.h_tab;
    b.d_tab = g->buf.d_tab;
    b.d_stat = g->buf.d_stat;
    b.bfs_ctl = g->bfs_ctl;
    b.h_bfs_ctl = g->h_bfs_ctl;
    b.tab_bytes = tab_bytes;
    b.stat_slot = g->buf.stat_slot;
    b.ctl_bytes = bp.ctl_bytes;
    b.upd_func = upd.func;
    b.bfs_func = bp.main.func;
    b.upd_grid = upd.grid.x;
    b.bfs_grid = bp.main.grid.x;
    b.upd_smem = upd.smem;
    for (int i = 0; i < BfsPlan::CLEARS; ++i) {
        b.clear_ptr[i] = bp.clear_ptr[i];
        b.clear_bytes[i] = bp.clear_bytes[i];
    }
    return b;
}

bool same_baked(const gpma_step::Baked &a, const gpma_step::Baked &b) { return memcmp(&a, &b, sizeof(a)) == 0; }

gpma_status set_cooperative(cudaGraphNode_t node) {
    cudaLaunchAttributeValue v{};
    v.cooperative = 1;
    GPMA_CUDA(cudaGraphKernelNodeSetAttribute(node, cudaLaunchAttributeCooperative, &v));
    return GPMA_OK;
}

// Appends nodes to a chain (each depends on the previous one).
struct Chain {
    cudaGraph_t graph;
    cudaGraphNode_t prev = nullptr;
    gpma_status copy(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind) {
        cudaGraphNode_t n;
        GPMA_CUDA(cudaGraphAddMemcpyNode1D(&n, graph, prev ? &prev : nullptr, prev ? 1 : 0, dst, src, bytes, kind));
        prev = n;
        return GPMA_OK;
    }
    gpma_status zero(void *dst, size_t bytes) {  // bytes: a multiple of 4
        cudaMemsetParams mp{};
        mp.dst = dst;
        mp.value = 0;
        mp.elementSize = 4;
        mp.width = bytes / 4;
        mp.height = 1;
        mp.pitch = 0;
        cudaGraphNode_t n;
        GPMA_CUDA(cudaGraphAddMemsetNode(&n, graph, prev ? &prev : nullptr, prev ? 1 : 0, &mp));
        prev = n;
        return GPMA_OK;
    }
    gpma_status kernel(KernelLaunch &L, bool cooperative, cudaGraphNode_t *out) {
        cudaKernelNodeParams kp = L.node();
        GPMA_CUDA(cudaGraphAddKernelNode(out, graph, prev ? &prev : nullptr, prev ? 1 : 0, &kp));
        if (cooperative)
            GPMA_TRY(set_cooperative(*out));
        prev = *out;
        return GPMA_OK;
    }
};

// Updates a kernel node's arguments in place when they changed.
gpma_status refresh_kernel(cudaGraphExec_t exec, cudaGraphNode_t node, KernelLaunch &now, KernelLaunch &built,
                           uint64_t *updates) {
    if (now.same(built))
        return GPMA_OK;
    cudaKernelNodeParams kp = now.node();
    GPMA_CUDA(cudaGraphExecKernelNodeSetParams(exec, node, &kp));
    built = now;
    ++*updates;
    return GPMA_OK;
}

// Builds and instantiates the step's graph from the current plans (one chain).
gpma_status build_graph(gpma_step *st, size_t tab_bytes, KernelLaunch &upd, BfsPlan &bp) {
    drop_graph(st);
    gpma_graph *g = st->g;
    const size_t stat_bytes = 2 * g->buf.stat_slot;
    if (stat_bytes > st->h_stat_bytes) {
        if (st->h_stat)
            cudaFreeHost(st->h_stat);
        st->h_stat = nullptr;
        st->h_stat_bytes = 0;
        GPMA_CUDA(cudaMallocHost((void **)&st->h_stat, stat_bytes));
        st->h_stat_bytes = stat_bytes;
    }
    GPMA_CUDA(cudaGraphCreate(&st->graph, 0));
    cudaGraphNode_t prev = nullptr, node = nullptr;
    auto deps = [&]() { return prev ? &prev : (const cudaGraphNode_t *)nullptr; };
    auto ndeps = [&]() { return prev ? (size_t)1 : (size_t)0; };
    GPMA_CUDA(cudaGraphAddMemcpyNode1D(&node, st->graph, deps(), ndeps(), g->buf.d_tab, g->buf.h_tab, tab_bytes,
                                       cudaMemcpyHostToDevice));
    prev = node;
    cudaKernelNodeParams kp = upd.node();
    GPMA_CUDA(cudaGraphAddKernelNode(&st->n_update, st->graph, deps(), ndeps(), &kp));
    GPMA_TRY(set_cooperative(st->n_update));
    prev = st->n_update;
    for (int i = 0; i < BfsPlan::CLEARS; ++i) {
        cudaMemsetParams mp{};
        mp.dst = bp.clear_ptr[i];
        mp.value = 0;
        mp.elementSize = 4;  // every cleared buffer is 32-bit words
        mp.width = bp.clear_bytes[i] / 4;
        mp.height = 1;
        mp.pitch = 0;
        GPMA_CUDA(cudaGraphAddMemsetNode(&node, st->graph, deps(), ndeps(), &mp));
        prev = node;
    }
    bp.bind_init();
    cudaKernelNodeParams ip{};
    ip.func = const_cast<void *>(bp.init_func);
    ip.gridDim = dim3(1, 1, 1);
    ip.blockDim = dim3(1, 1, 1);
    ip.sharedMemBytes = 0;
    ip.kernelParams = bp.init_params;
    GPMA_CUDA(cudaGraphAddKernelNode(&st->n_init, st->graph, deps(), ndeps(), &ip));
    prev = st->n_init;
    kp = bp.main.node();
    GPMA_CUDA(cudaGraphAddKernelNode(&st->n_bfs, st->graph, deps(), ndeps(), &kp));
    GPMA_TRY(set_cooperative(st->n_bfs));
    prev = st->n_bfs;
    GPMA_CUDA(cudaGraphAddMemcpyNode1D(&node, st->graph, deps(), ndeps(), st->h_stat, g->buf.d_stat, stat_bytes,
                                       cudaMemcpyDeviceToHost));
    prev = node;
    GPMA_CUDA(cudaGraphAddMemcpyNode1D(&node, st->graph, deps(), ndeps(), g->h_bfs_ctl, g->bfs_ctl, bp.ctl_bytes,
                                       cudaMemcpyDeviceToHost));
    GPMA_CUDA(cudaGraphInstantiate(&st->exec, st->graph, 0));
    st->upd = upd;
    st->bfs = bp.main;
    st->init_args[0] = bp.init_levels;
    st->init_args[1] = bp.init_visited;
    st->init_args[2] = bp.init_front0;
    st->init_args[3] = bp.init_ctl;
    st->init_src = bp.init_src;
    st->baked = bake(g, tab_bytes, upd, bp);
    st->stats.builds++;
    return GPMA_OK;
}

// Brings the instantiated graph's per-step arguments up to date.
gpma_status refresh_params(gpma_step *st, KernelLaunch &upd, BfsPlan &bp) {
    if (!upd.same(st->upd)) {
        cudaKernelNodeParams kp = upd.node();
        GPMA_CUDA(cudaGraphExecKernelNodeSetParams(st->exec, st->n_update, &kp));
        st->upd = upd;
        st->stats.param_updates++;
    }
    const uint32_t *ia[4] = {bp.init_levels, bp.init_visited, bp.init_front0, bp.init_ctl};
    bool init_same = bp.init_src == st->init_src;
    for (int i = 0; i < 4; ++i)
        init_same = init_same && ia[i] == st->init_args[i];
    if (!init_same) {
        bp.bind_init();
        cudaKernelNodeParams ip{};
        ip.func = const_cast<void *>(bp.init_func);
        ip.gridDim = dim3(1, 1, 1);
        ip.blockDim = dim3(1, 1, 1);
        ip.kernelParams = bp.init_params;
        GPMA_CUDA(cudaGraphExecKernelNodeSetParams(st->exec, st->n_init, &ip));
        st->init_args[0] = bp.init_levels;
        st->init_args[1] = bp.init_visited;
        st->init_args[2] = bp.init_front0;
        st->init_args[3] = bp.init_ctl;
        st->init_src = bp.init_src;
        st->stats.param_updates++;
    }
    if (!bp.main.same(st->bfs)) {
        cudaKernelNodeParams kp = bp.main.node();
        GPMA_CUDA(cudaGraphExecKernelNodeSetParams(st->exec, st->n_bfs, &kp));
        st->bfs = bp.main;
        st->stats.param_updates++;
    }
    return GPMA_OK;
}

}  // namespace

gpma_status step_run(gpma_step *st, const uint64_t *keys, const uint8_t *values, uint64_t n, uint32_t src,
                     uint32_t *levels, uint64_t *reached, cudaStream_t s) {
    gpma_graph *g = st->g;
    g->stats.updates++;
    g->stats.submitted += n;
    st->stats.runs++;
    if (n == 0) {
        // nothing to update: the step is the BFS alone
        st->stats.host_runs++;
        GPMA_TRY(bfs_run(g, src, s, reached));
    } else {
        GPMA_TRY(ensure_buffers(g->buf, n, 1));
        GPMA_TRY(copy_any(g->buf.bkeys[0], keys, n * sizeof(uint64_t), s));
        GPMA_TRY(copy_any(g->buf.bvals[0], values, n, s));
        const uint64_t off[2] = {0, n};
        gpma_graph *gl[1] = {g};
        size_t tab_bytes = 0;
        KernelLaunch upd;
        GPMA_TRY(update_plan(gl, off, 1, g->buf, g->sms, true, &tab_bytes, &upd));
        BfsPlan bp;
        const bool profiling = g->profiling;
        g->profiling = false;  // no per-level stamps inside a recorded step
        const gpma_status ps = bfs_plan(g, src, &bp);
        g->profiling = profiling;
        GPMA_TRY(ps);
        if (!st->exec || !same_baked(bake(g, tab_bytes, upd, bp), st->baked))
            GPMA_TRY(build_graph(st, tab_bytes, upd, bp));
        else
            GPMA_TRY(refresh_params(st, upd, bp));
        GPMA_TRY(update_clear(g->buf, s));
        const unsigned char *stat = st->h_stat + g->buf.parity * g->buf.stat_slot;
        GPMA_CUDA(cudaEventRecord(st->ev[0], s));
        g->buf.tab_shadow_valid = false;  // the graph uploads its own table
        GPMA_CUDA(cudaGraphLaunch(st->exec, s));
        GPMA_CUDA(cudaEventRecord(st->ev[1], s));
        GPMA_CUDA(cudaStreamSynchronize(s));
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, st->ev[0], st->ev[1]) != cudaSuccess) {
            cudaGetLastError();
            ms = 0.f;
        }
        st->stats.last_ms = ms;
        st->stats.total_ms += ms;
        st->stats.graph_launches++;
        g->prof.kernel_launches += 3;  // update, BFS init, BFS
        const bool host_work = update_needs_host(stat, 1);
        GPMA_TRY(update_finish(gl, 1, g->buf, stat, s, nullptr, 0.0));
        if (host_work) {
            // the array changed on the host after the recorded BFS ran: redo it
            st->stats.host_runs++;
            GPMA_TRY(bfs_run(g, src, s, reached));
        } else {
            GPMA_TRY(bfs_finish(g, reached));
        }
    }
    if (levels) {
        GPMA_TRY(copy_any(levels, g->bfs_levels, sizeof(uint32_t) * g->row_num, s));
        GPMA_CUDA(cudaStreamSynchronize(s));
    }
    return GPMA_OK;
}

}  // namespace gpma

// ---- recorded steps of a batch of graphs ------------------------------------
// The batched form's step: one packed update of every graph of the step (the
// gather of the batches into segment-length order, then the persistent
// update kernel) and one multi-source BFS over all of them, as one graph:
//   gather table upload -> gather kernel -> update table upload -> update
//   kernel (cooperative) -> BFS table upload -> 5 BFS clears -> multi-source
//   BFS kernel (cooperative) -> status, control and count read-back.
// A step whose batch holds an empty or a bulk-sized (>= 5M keys) part, or
// whose update needs host work, runs or finishes through the eager calls,
// which give the same results.

struct gpma_batch_step {
    gpma_batch *b = nullptr;
    std::vector<gpma_graph *> graphs;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t n_gather = nullptr, n_update = nullptr, n_ms = nullptr;
    gpma::KernelLaunch gather, upd, ms;
    std::vector<unsigned char> baked;  // the pointers, sizes and launch shapes the nodes hold
    unsigned char *h_stat = nullptr;   // pinned copy of both status slots
    size_t h_stat_bytes = 0;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    gpma_step_stats stats{};
    // several steps recorded in one graph (gpma_batch_step_run_many)
    struct Multi {
        uint32_t steps = 0;
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        std::vector<cudaGraphNode_t> n_gather, n_update, n_ms;
        std::vector<gpma::KernelLaunch> gather, upd, ms;
        std::vector<unsigned char> baked;
        // pinned: the BFS table once, then per step its gather table, update
        // table, status slot, BFS control words and BFS counts
        unsigned char *h_buf = nullptr;
        size_t h_bytes = 0;
        size_t mtab = 0, gtab = 0, utab = 0, stat = 0, ctl = 0, reach = 0, per_step = 0;
        uint32_t *d_abort = nullptr;  // set by the first step that needs host work
    } multi;
};

namespace gpma {
namespace {

// After a recorded step's update: a status that asks for host work (root
// rebalance, bulk rebuild, invalid keys, an error) or a launch that did not
// run sets the abort word, and every later gather, update and BFS launch of
// the recording returns at once.
struct GateArgs {
    const unsigned char *stat;
    uint32_t k;
    uint32_t *abort;
};
__global__ void step_gate_kernel(GateArgs A) {
    const DeviceStatus &h = *reinterpret_cast<const DeviceStatus *>(A.stat);
    const GraphStatus *gs = reinterpret_cast<const GraphStatus *>(A.stat + STAT_GS_OFFSET);
    uint32_t need = 0;
    for (uint32_t i = threadIdx.x; i < A.k; i += blockDim.x)
        need |= (uint32_t)(gs[i].remaining > 0);
    need = __syncthreads_or(need);
    if (threadIdx.x == 0 && (need || h.err || h.invalid_keys || h.significant || h.stamp[0] == 0))
        *A.abort = 1u;
}

void drop_multi_graph(gpma_batch_step *st) {
    if (st->multi.exec)
        cudaGraphExecDestroy(st->multi.exec);
    if (st->multi.graph)
        cudaGraphDestroy(st->multi.graph);
    st->multi.exec = nullptr;
    st->multi.graph = nullptr;
    st->multi.steps = 0;
    st->multi.baked.clear();
}

void drop_batch_graph(gpma_batch_step *st) {
    if (st->exec)
        cudaGraphExecDestroy(st->exec);
    if (st->graph)
        cudaGraphDestroy(st->graph);
    st->exec = nullptr;
    st->graph = nullptr;
}

template <typename T>
void put(std::vector<unsigned char> &v, const T &x) {
    const unsigned char *p = reinterpret_cast<const unsigned char *>(&x);
    v.insert(v.end(), p, p + sizeof(T));
}

std::vector<unsigned char> bake_batch(const gpma_batch *b, const PackedPlan &pp, size_t tab_bytes,
                                      const KernelLaunch &upd, const BatchBfsPlan &bp) {
    std::vector<unsigned char> v;
    put(v, (const void *)b->h_gather_tab);
    put(v, (const void *)b->gather_tab);
    put(v, pp.gtab_bytes);
    put(v, pp.gather.func);
    put(v, pp.gather.grid.x);
    put(v, (const void *)b->buf.h_tab);
    put(v, (const void *)b->buf.d_tab);
    put(v, tab_bytes);
    put(v, upd.func);
    put(v, upd.grid.x);
    put(v, upd.smem);
    put(v, (const void *)b->h_ms_tab);
    put(v, (const void *)b->ms_tab);
    put(v, bp.tab_bytes);
    for (int i = 0; i < BatchBfsPlan::CLEARS; ++i) {
        put(v, bp.clear_ptr[i]);
        put(v, bp.clear_bytes[i]);
    }
    put(v, bp.main.func);
    put(v, bp.main.grid.x);
    put(v, (const void *)b->buf.d_stat);
    put(v, b->buf.stat_slot);
    put(v, (const void *)b->ms_ctl);
    put(v, (const void *)b->h_ms_ctl);
    put(v, (const void *)b->ms_reached);
    put(v, (const void *)b->h_ms_reached);
    put(v, bp.reached_bytes);
    return v;
}

gpma_status build_batch_graph(gpma_batch_step *st, PackedPlan &pp, size_t tab_bytes, KernelLaunch &upd,
                              BatchBfsPlan &bp) {
    drop_batch_graph(st);
    gpma_batch *b = st->b;
    const size_t stat_bytes = 2 * b->buf.stat_slot;
    if (stat_bytes > st->h_stat_bytes) {
        if (st->h_stat)
            cudaFreeHost(st->h_stat);
        st->h_stat = nullptr;
        st->h_stat_bytes = 0;
        GPMA_CUDA(cudaMallocHost((void **)&st->h_stat, stat_bytes));
        st->h_stat_bytes = stat_bytes;
    }
    GPMA_CUDA(cudaGraphCreate(&st->graph, 0));
    Chain c{st->graph};
    GPMA_TRY(c.copy(b->gather_tab, b->h_gather_tab, pp.gtab_bytes, cudaMemcpyHostToDevice));
    GPMA_TRY(c.kernel(pp.gather, false, &st->n_gather));
    GPMA_TRY(c.copy(b->buf.d_tab, b->buf.h_tab, tab_bytes, cudaMemcpyHostToDevice));
    GPMA_TRY(c.kernel(upd, true, &st->n_update));
    GPMA_TRY(c.copy(b->ms_tab, b->h_ms_tab, bp.tab_bytes, cudaMemcpyHostToDevice));
    for (int i = 0; i < BatchBfsPlan::CLEARS; ++i)
        GPMA_TRY(c.zero(bp.clear_ptr[i], bp.clear_bytes[i]));
    GPMA_TRY(c.kernel(bp.main, true, &st->n_ms));
    GPMA_TRY(c.copy(st->h_stat, b->buf.d_stat, stat_bytes, cudaMemcpyDeviceToHost));
    GPMA_TRY(c.copy(b->h_ms_ctl, b->ms_ctl, bp.ctl_bytes, cudaMemcpyDeviceToHost));
    GPMA_TRY(c.copy(b->h_ms_reached, b->ms_reached, bp.reached_bytes, cudaMemcpyDeviceToHost));
    GPMA_CUDA(cudaGraphInstantiate(&st->exec, st->graph, 0));
    st->gather = pp.gather;
    st->upd = upd;
    st->ms = bp.main;
    st->baked = bake_batch(b, pp, tab_bytes, upd, bp);
    st->stats.builds++;
    return GPMA_OK;
}

}  // namespace

gpma_status batch_step_run(gpma_batch_step *st, const uint64_t *keys, const uint8_t *values, const uint64_t *offsets,
                           const uint32_t *const *srcs, const uint32_t *nsrc, uint64_t *reached, cudaStream_t s) {
    gpma_batch *b = st->b;
    gpma_graph *const *graphs = st->graphs.data();
    const uint32_t k = (uint32_t)st->graphs.size();
    st->stats.runs++;
    bool eager = false;
    for (uint32_t i = 0; i < k; ++i) {
        const uint64_t c = offsets[i + 1] - offsets[i];
        eager = eager || c == 0 || c >= SIGNIFICANT_INSERTS;
    }
    if (eager) {
        st->stats.host_runs++;
        GPMA_TRY(gpma_batch_update_packed(b, graphs, keys, values, offsets, k, s));
        return batch_bfs_run(b, graphs, srcs, nsrc, k, nullptr, reached, s);
    }
    for (uint32_t i = 0; i < k; ++i) {
        graphs[i]->stats.updates++;
        graphs[i]->stats.submitted += offsets[i + 1] - offsets[i];
    }
    PackedPlan pp;
    GPMA_TRY(packed_plan(b, graphs, keys, values, offsets, k, &pp));
    GPMA_TRY(packed_stage(b, pp, keys, values, offsets, s, /*with_table=*/false));
    size_t tab_bytes = 0;
    KernelLaunch upd;
    GPMA_TRY(update_plan(pp.gs.data(), pp.off.data(), pp.m, b->buf, b->sms, true, &tab_bytes, &upd));
    BatchBfsPlan bp;
    GPMA_TRY(batch_bfs_plan(b, graphs, srcs, nsrc, k, nullptr, &bp));
    if (!st->exec || bake_batch(b, pp, tab_bytes, upd, bp) != st->baked) {
        GPMA_TRY(build_batch_graph(st, pp, tab_bytes, upd, bp));
    } else {
        GPMA_TRY(refresh_kernel(st->exec, st->n_gather, pp.gather, st->gather, &st->stats.param_updates));
        GPMA_TRY(refresh_kernel(st->exec, st->n_update, upd, st->upd, &st->stats.param_updates));
        GPMA_TRY(refresh_kernel(st->exec, st->n_ms, bp.main, st->ms, &st->stats.param_updates));
    }
    GPMA_TRY(update_clear(b->buf, s));
    const unsigned char *stat = st->h_stat + b->buf.parity * b->buf.stat_slot;
    GPMA_CUDA(cudaEventRecord(st->ev[0], s));
    b->buf.tab_shadow_valid = false;  // the graph uploads its own table
    GPMA_CUDA(cudaGraphLaunch(st->exec, s));
    GPMA_CUDA(cudaEventRecord(st->ev[1], s));
    GPMA_CUDA(cudaStreamSynchronize(s));
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, st->ev[0], st->ev[1]) != cudaSuccess) {
        cudaGetLastError();
        ms = 0.f;
    }
    st->stats.last_ms = ms;
    st->stats.total_ms += ms;
    st->stats.graph_launches++;
    b->prof.kernel_launches += 2;  // gather and update; the BFS is counted by its finish
    const bool host_work = update_needs_host(stat, pp.m);
    GPMA_TRY(update_finish(pp.gs.data(), pp.m, b->buf, stat, s, nullptr, 0.0));
    if (host_work) {
        // the arrays changed on the host after the recorded BFS ran: redo it
        st->stats.host_runs++;
        return batch_bfs_run(b, graphs, srcs, nsrc, k, nullptr, reached, s);
    }
    return batch_bfs_finish(b, nsrc, k, reached);
}

namespace {
size_t pad16(size_t x) { return (x + 15) & ~size_t(15); }
}  // namespace

// S steps in one graph launch. Step t's batch is keys[t]/values[t] (device)
// with offsets at offsets + t * (k + 1); every step searches from the same
// sources; reached receives S x sum(nsrc) counts. Steps whose parts are empty
// or bulk-sized, or host batches, run one by one through batch_step_run.
// Each recorded step is: gather-table upload, gather, update-table upload,
// update kernel, status copy, gate, BFS clears, multi-source BFS, BFS
// read-back. A step whose update needs host work stops the rest of the
// recording (the gate's abort word); its host work, its BFS and the steps
// after it then run as batch_step_run would, so the results are always those
// of the per-step calls.
gpma_status batch_step_run_many(gpma_batch_step *st, uint32_t S, const uint64_t *const *keys,
                                const uint8_t *const *values, const uint64_t *offsets, const uint32_t *const *srcs,
                                const uint32_t *nsrc, uint64_t *reached, cudaStream_t s) {
    gpma_batch *b = st->b;
    gpma_graph *const *graphs = st->graphs.data();
    const uint32_t k = (uint32_t)st->graphs.size();
    uint64_t per_src = 0;
    for (uint32_t i = 0; i < k; ++i)
        per_src += nsrc[i];
    auto off_of = [&](uint32_t t) { return offsets + (size_t)t * (k + 1); };
    auto reach_of = [&](uint32_t t) { return reached ? reached + (size_t)t * per_src : nullptr; };
    auto one_by_one = [&](uint32_t from) -> gpma_status {
        for (uint32_t t = from; t < S; ++t)
            GPMA_TRY(batch_step_run(st, keys[t], values[t], off_of(t), srcs, nsrc, reach_of(t), s));
        return GPMA_OK;
    };
    bool eligible = S > 1;
    for (uint32_t t = 0; t < S && eligible; ++t) {
        eligible = is_device_pointer(keys[t]) && is_device_pointer(values[t]);
        const uint64_t *o = off_of(t);
        for (uint32_t i = 0; i < k && eligible; ++i) {
            const uint64_t c = o[i + 1] - o[i];
            eligible = c > 0 && c < SIGNIFICANT_INSERTS;
        }
    }
    if (!eligible)
        return one_by_one(0);
    auto &M = st->multi;
    if (!M.d_abort)
        GPMA_TRY(dev_alloc(&M.d_abort, 1));
    // Plans of every step: the first pass grows the buffers to what all steps
    // need, the second records pointers that no later plan moves. Step t's
    // status goes to slot parity[t], as consecutive launches alternate.
    std::vector<PackedPlan> pp(S);
    std::vector<size_t> tabb(S);
    std::vector<KernelLaunch> upd(S);
    std::vector<int> parity(S);
    BatchBfsPlan bp;
    const int p0 = b->buf.parity;
    for (int pass = 0; pass < 2; ++pass) {
        b->buf.parity = p0;
        for (uint32_t t = 0; t < S; ++t) {
            GPMA_TRY(packed_plan(b, graphs, keys[t], values[t], off_of(t), k, &pp[t], M.d_abort));
            GPMA_TRY(update_plan(pp[t].gs.data(), pp[t].off.data(), pp[t].m, b->buf, b->sms, true, &tabb[t], &upd[t],
                                 M.d_abort));
            parity[t] = b->buf.parity;
            b->buf.parity ^= 1;
            if (pass == 1) {
                unsigned char *hs = M.h_buf + pad16(M.mtab) + (size_t)t * M.per_step;
                memcpy(hs, b->h_gather_tab, pp[t].gtab_bytes);
                memcpy(hs + pad16(M.gtab), b->buf.h_tab, tabb[t]);
            }
        }
        GPMA_TRY(batch_bfs_plan(b, graphs, srcs, nsrc, k, nullptr, &bp, M.d_abort));
        if (pass == 0) {
            size_t gtab = 0, utab = 0;
            for (uint32_t t = 0; t < S; ++t) {
                gtab = std::max(gtab, pp[t].gtab_bytes);
                utab = std::max(utab, tabb[t]);
            }
            M.mtab = bp.tab_bytes;
            M.gtab = gtab;
            M.utab = utab;
            M.stat = b->buf.stat_slot;
            M.ctl = bp.ctl_bytes;
            M.reach = bp.reached_bytes;
            M.per_step = pad16(M.gtab) + pad16(M.utab) + pad16(M.stat) + pad16(M.ctl) + pad16(M.reach);
            const size_t need = pad16(M.mtab) + (size_t)S * M.per_step;
            if (need > M.h_bytes) {
                drop_multi_graph(st);  // its nodes point into the old staging
                if (M.h_buf)
                    cudaFreeHost(M.h_buf);
                M.h_buf = nullptr;
                M.h_bytes = 0;
                GPMA_CUDA(cudaMallocHost((void **)&M.h_buf, need));
                M.h_bytes = need;
            }
        } else {
            memcpy(M.h_buf, b->h_ms_tab, bp.tab_bytes);
        }
    }
    b->buf.parity = p0;
    const size_t o_utab = pad16(M.gtab), o_stat = o_utab + pad16(M.utab), o_ctl = o_stat + pad16(M.stat),
                 o_reach = o_ctl + pad16(M.ctl);
    // what the nodes hold besides kernel arguments
    std::vector<unsigned char> baked;
    put(baked, S);
    put(baked, (const void *)M.h_buf);
    put(baked, (const void *)M.d_abort);
    put(baked, M.per_step);
    put(baked, (const void *)b->ms_tab);
    put(baked, (const void *)b->ms_ctl);
    put(baked, (const void *)b->ms_reached);
    put(baked, bp.tab_bytes);
    put(baked, bp.ctl_bytes);
    put(baked, bp.reached_bytes);
    for (int i = 0; i < BatchBfsPlan::CLEARS; ++i) {
        put(baked, bp.clear_ptr[i]);
        put(baked, bp.clear_bytes[i]);
    }
    put(baked, bp.main.func);
    put(baked, bp.main.grid.x);
    put(baked, (const void *)b->gather_tab);
    put(baked, (const void *)b->buf.d_tab);
    put(baked, (const void *)b->buf.d_stat);
    put(baked, b->buf.stat_slot);
    for (uint32_t t = 0; t < S; ++t) {  // (grids are kernel arguments too: refreshed in place)
        put(baked, pp[t].gtab_bytes);
        put(baked, pp[t].gather.func);
        put(baked, tabb[t]);
        put(baked, upd[t].func);
        put(baked, upd[t].smem);
        put(baked, parity[t]);
        put(baked, pp[t].m);
    }
    if (!M.exec || baked != M.baked) {
        drop_multi_graph(st);
        GPMA_CUDA(cudaGraphCreate(&M.graph, 0));
        Chain c{M.graph};
        GPMA_TRY(c.zero(M.d_abort, sizeof(uint32_t)));
        GPMA_TRY(c.copy(b->ms_tab, M.h_buf, bp.tab_bytes, cudaMemcpyHostToDevice));
        M.n_gather.assign(S, nullptr);
        M.n_update.assign(S, nullptr);
        M.n_ms.assign(S, nullptr);
        M.gather.assign(pp.size(), KernelLaunch());
        M.upd.assign(S, KernelLaunch());
        M.ms.assign(S, KernelLaunch());
        for (uint32_t t = 0; t < S; ++t) {
            unsigned char *hs = M.h_buf + pad16(M.mtab) + (size_t)t * M.per_step;
            unsigned char *slot = b->buf.d_stat + parity[t] * b->buf.stat_slot;
            GPMA_TRY(c.copy(b->gather_tab, hs, pp[t].gtab_bytes, cudaMemcpyHostToDevice));
            GPMA_TRY(c.kernel(pp[t].gather, false, &M.n_gather[t]));
            GPMA_TRY(c.copy(b->buf.d_tab, hs + o_utab, tabb[t], cudaMemcpyHostToDevice));
            GPMA_TRY(c.kernel(upd[t], true, &M.n_update[t]));
            GPMA_TRY(c.copy(hs + o_stat, slot, b->buf.stat_slot, cudaMemcpyDeviceToHost));
            GateArgs ga{slot, pp[t].m, M.d_abort};
            KernelLaunch gate;
            gate.set((const void *)step_gate_kernel, 1, 0, &ga, sizeof(ga));
            cudaGraphNode_t gn = nullptr;
            GPMA_TRY(c.kernel(gate, false, &gn));
            for (int i = 0; i < BatchBfsPlan::CLEARS; ++i)
                GPMA_TRY(c.zero(bp.clear_ptr[i], bp.clear_bytes[i]));
            GPMA_TRY(c.kernel(bp.main, true, &M.n_ms[t]));
            GPMA_TRY(c.copy(hs + o_ctl, b->ms_ctl, bp.ctl_bytes, cudaMemcpyDeviceToHost));
            GPMA_TRY(c.copy(hs + o_reach, b->ms_reached, bp.reached_bytes, cudaMemcpyDeviceToHost));
            M.gather[t] = pp[t].gather;
            M.upd[t] = upd[t];
            M.ms[t] = bp.main;
        }
        GPMA_CUDA(cudaGraphInstantiate(&M.exec, M.graph, 0));
        M.steps = S;
        M.baked = baked;
        st->stats.builds++;
    } else {
        for (uint32_t t = 0; t < S; ++t) {
            GPMA_TRY(refresh_kernel(M.exec, M.n_gather[t], pp[t].gather, M.gather[t], &st->stats.param_updates));
            GPMA_TRY(refresh_kernel(M.exec, M.n_update[t], upd[t], M.upd[t], &st->stats.param_updates));
            GPMA_TRY(refresh_kernel(M.exec, M.n_ms[t], bp.main, M.ms[t], &st->stats.param_updates));
        }
    }
    GPMA_TRY(update_clear(b->buf, s));
    GPMA_CUDA(cudaEventRecord(st->ev[0], s));
    b->buf.tab_shadow_valid = false;  // the graph uploads its own tables
    GPMA_CUDA(cudaGraphLaunch(M.exec, s));
    GPMA_CUDA(cudaEventRecord(st->ev[1], s));
    GPMA_CUDA(cudaStreamSynchronize(s));
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, st->ev[0], st->ev[1]) != cudaSuccess) {
        cudaGetLastError();
        ms = 0.f;
    }
    st->stats.last_ms = ms;
    st->stats.total_ms += ms;
    st->stats.graph_launches++;
    // the steps in order, exactly as batch_step_run finishes one
    for (uint32_t t = 0; t < S; ++t) {
        const unsigned char *hs = M.h_buf + pad16(M.mtab) + (size_t)t * M.per_step;
        const unsigned char *stat = hs + o_stat;
        if (reinterpret_cast<const DeviceStatus *>(stat)->stamp[0] == 0) {
            set_error("gpma_batch_step_run_many: recorded step %u did not run", t);
            b->buf.dirty = true;
            return GPMA_ERR_DEVICE;
        }
        st->stats.runs++;
        const uint64_t *o = off_of(t);
        for (uint32_t i = 0; i < k; ++i) {
            graphs[i]->stats.updates++;
            graphs[i]->stats.submitted += o[i + 1] - o[i];
        }
        b->prof.kernel_launches += 2;  // gather and update; the BFS is counted by its finish
        const bool host_work = update_needs_host(stat, pp[t].m);
        GPMA_TRY(update_finish(pp[t].gs.data(), pp[t].m, b->buf, stat, s, nullptr, 0.0));
        if (host_work) {
            // the recording stopped after this update: its BFS and the later
            // steps run on the array the host work left
            st->stats.host_runs++;
            GPMA_TRY(batch_bfs_run(b, graphs, srcs, nsrc, k, nullptr, reach_of(t), s));
            return one_by_one(t + 1);
        }
        memcpy(b->h_ms_ctl, hs + o_ctl, bp.ctl_bytes);
        memcpy(b->h_ms_reached, hs + o_reach, bp.reached_bytes);
        GPMA_TRY(batch_bfs_finish(b, nsrc, k, reach_of(t)));
    }
    return GPMA_OK;
}

}  // namespace gpma

extern "C" {

gpma_status gpma_step_create(gpma_graph *g, gpma_step **out) {
    if (!g || !out) {
        gpma::set_error("gpma_step_create: null argument");
        return GPMA_ERR_INVALID;
    }
    *out = nullptr;
    gpma_step *st = new (std::nothrow) gpma_step();
    if (!st) {
        gpma::set_error("gpma_step_create: out of host memory");
        return GPMA_ERR_NOMEM;
    }
    st->g = g;
    for (int i = 0; i < 2; ++i) {
        cudaError_t e = cudaEventCreate(&st->ev[i]);
        if (e != cudaSuccess) {
            gpma_step_destroy(st);
            return gpma::cuda_fail(e, "cudaEventCreate");
        }
    }
    *out = st;
    return GPMA_OK;
}

gpma_status gpma_step_destroy(gpma_step *st) {
    if (!st)
        return GPMA_OK;
    gpma::drop_graph(st);
    for (int i = 0; i < 2; ++i)
        if (st->ev[i])
            cudaEventDestroy(st->ev[i]);
    if (st->h_stat)
        cudaFreeHost(st->h_stat);
    delete st;
    return GPMA_OK;
}

gpma_status gpma_step_run(gpma_step *st, const uint64_t *keys, const uint8_t *values, uint64_t n, uint32_t src,
                          uint32_t *levels, uint64_t *reached, void *stream) {
    gpma::CallRange range("gpma_step_run");
    if (!st || (n && (!keys || !values))) {
        gpma::set_error("gpma_step_run: null argument");
        return GPMA_ERR_INVALID;
    }
    if (n >= (1ull << 30)) {
        gpma::set_error("gpma_step_run: batch of %llu keys exceeds 2^30", (unsigned long long)n);
        return GPMA_ERR_CAPACITY;
    }
    if (src >= st->g->row_num) {
        gpma::set_error("gpma_step_run: start node %u out of range (row_num %u)", src, st->g->row_num);
        return GPMA_ERR_INVALID;
    }
    return gpma::step_run(st, keys, values, n, src, levels, reached, (cudaStream_t)stream);
}

gpma_status gpma_step_get_stats(const gpma_step *st, gpma_step_stats *out) {
    if (!st || !out) {
        gpma::set_error("gpma_step_get_stats: null argument");
        return GPMA_ERR_INVALID;
    }
    *out = st->stats;
    return GPMA_OK;
}

gpma_status gpma_batch_step_create(gpma_batch *b, gpma_graph *const *graphs, uint32_t k, gpma_batch_step **out) {
    if (!b || !out || (k && !graphs) || k == 0) {
        gpma::set_error("gpma_batch_step_create: null argument or no graphs");
        return GPMA_ERR_INVALID;
    }
    *out = nullptr;
    for (uint32_t i = 0; i < k; ++i) {
        if (!graphs[i]) {
            gpma::set_error("gpma_batch_step_create: graph %u is null", i);
            return GPMA_ERR_INVALID;
        }
        for (uint32_t j = 0; j < i; ++j)
            if (graphs[j] == graphs[i]) {
                gpma::set_error("gpma_batch_step_create: graph %u appears twice", i);
                return GPMA_ERR_INVALID;
            }
    }
    gpma_batch_step *st = new (std::nothrow) gpma_batch_step();
    if (!st) {
        gpma::set_error("gpma_batch_step_create: out of host memory");
        return GPMA_ERR_NOMEM;
    }
    st->b = b;
    st->graphs.assign(graphs, graphs + k);
    for (int i = 0; i < 2; ++i) {
        cudaError_t e = cudaEventCreate(&st->ev[i]);
        if (e != cudaSuccess) {
            gpma_batch_step_destroy(st);
            return gpma::cuda_fail(e, "cudaEventCreate");
        }
    }
    *out = st;
    return GPMA_OK;
}

gpma_status gpma_batch_step_destroy(gpma_batch_step *st) {
    if (!st)
        return GPMA_OK;
    gpma::drop_batch_graph(st);
    gpma::drop_multi_graph(st);
    if (st->multi.h_buf)
        cudaFreeHost(st->multi.h_buf);
    gpma::dev_free(st->multi.d_abort);
    for (int i = 0; i < 2; ++i)
        if (st->ev[i])
            cudaEventDestroy(st->ev[i]);
    if (st->h_stat)
        cudaFreeHost(st->h_stat);
    delete st;
    return GPMA_OK;
}

namespace {

// Arguments of one batched step (`who` names the entry point in messages).
gpma_status check_batch_step(const char *who, const gpma_batch_step *st, const uint64_t *keys, const uint8_t *values,
                             const uint64_t *offsets, const uint32_t *const *srcs, const uint32_t *nsrc) {
    const uint32_t k = (uint32_t)st->graphs.size();
    if (offsets[k] > offsets[0] && (!keys || !values)) {
        gpma::set_error("%s: null keys or values", who);
        return GPMA_ERR_INVALID;
    }
    if (offsets[k] - offsets[0] >= (1ull << 31)) {
        gpma::set_error("%s: %llu keys in one step exceed 2^31", who, (unsigned long long)(offsets[k] - offsets[0]));
        return GPMA_ERR_CAPACITY;
    }
    uint64_t nodes = 0;
    for (uint32_t i = 0; i < k; ++i) {
        if (offsets[i + 1] < offsets[i]) {
            gpma::set_error("%s: decreasing offsets at %u", who, i);
            return GPMA_ERR_INVALID;
        }
        if (!srcs[i] || nsrc[i] == 0 || nsrc[i] > 64) {
            gpma::set_error("%s: graph %u: null sources or source count not in 1..64", who, i);
            return GPMA_ERR_INVALID;
        }
        for (uint32_t j = 0; j < nsrc[i]; ++j)
            if (srcs[i][j] >= st->graphs[i]->row_num) {
                gpma::set_error("%s: graph %u: source %u out of range (row_num %u)", who, i, srcs[i][j],
                                st->graphs[i]->row_num);
                return GPMA_ERR_INVALID;
            }
        nodes += st->graphs[i]->row_num;
    }
    if (nodes >= (1ull << 32)) {
        gpma::set_error("%s: %llu nodes in one step exceed 2^32", who, (unsigned long long)nodes);
        return GPMA_ERR_CAPACITY;
    }
    return GPMA_OK;
}

}  // namespace

gpma_status gpma_batch_step_run(gpma_batch_step *st, const uint64_t *keys, const uint8_t *values,
                                const uint64_t *offsets, const uint32_t *const *srcs, const uint32_t *nsrc,
                                uint64_t *reached, void *stream) {
    gpma::CallRange range("gpma_batch_step_run");
    if (!st || !offsets || !srcs || !nsrc) {
        gpma::set_error("gpma_batch_step_run: null argument");
        return GPMA_ERR_INVALID;
    }
    GPMA_TRY(check_batch_step("gpma_batch_step_run", st, keys, values, offsets, srcs, nsrc));
    return gpma::batch_step_run(st, keys, values, offsets, srcs, nsrc, reached, (cudaStream_t)stream);
}

gpma_status gpma_batch_step_run_many(gpma_batch_step *st, uint32_t steps, const uint64_t *const *keys,
                                     const uint8_t *const *values, const uint64_t *offsets,
                                     const uint32_t *const *srcs, const uint32_t *nsrc, uint64_t *reached,
                                     void *stream) {
    gpma::CallRange range("gpma_batch_step_run_many");
    if (!st || !offsets || !srcs || !nsrc || (steps && (!keys || !values))) {
        gpma::set_error("gpma_batch_step_run_many: null argument");
        return GPMA_ERR_INVALID;
    }
    const uint32_t k = (uint32_t)st->graphs.size();
    for (uint32_t t = 0; t < steps; ++t)
        GPMA_TRY(check_batch_step("gpma_batch_step_run_many", st, keys[t], values[t], offsets + (size_t)t * (k + 1),
                                  srcs, nsrc));
    if (steps == 0)
        return GPMA_OK;
    return gpma::batch_step_run_many(st, steps, keys, values, offsets, srcs, nsrc, reached, (cudaStream_t)stream);
}

gpma_status gpma_batch_step_get_stats(const gpma_batch_step *st, gpma_step_stats *out) {
    if (!st || !out) {
        gpma::set_error("gpma_batch_step_get_stats: null argument");
        return GPMA_ERR_INVALID;
    }
    *out = st->stats;
    return GPMA_OK;
}

}  // extern "C"
