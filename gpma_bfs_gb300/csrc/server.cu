// server.cu - served form: many resident graphs, update batches and BFS
// queries served with continuous batching (no reference counterpart; the
// reference applies one update_gpma call at a time, gpma.cuh:968).
//
// Scheduling (host): one FIFO queue per graph. A round visits the graphs in
// order of their queue head's arrival and takes, per graph, at most one update
// batch (its keys counted against max_round_keys and its worst-case growth
// against the HBM budget) and then the BFS queries queued directly behind it,
// packed as source lanes up to 64. Execution (device): the round's updates in
// one batched update launch (gpma_batch_update_packed), then its searches in
// one multi-source BFS launch (gpma_batch_bfs_multi). Because a graph's
// requests only ever run in queue order and a search runs after the update in
// front of it, each result equals the one the same requests give on the graph
// alone.
#include "gpma_internal.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <limits>
#include <memory>
#include <unordered_map>
#include <vector>

namespace {

struct Request {
    uint64_t id = 0;
    uint32_t graph = 0;
    uint32_t kind = 0;  // 0 update, 1 BFS
    uint32_t state = GPMA_REQ_QUEUED;
    int32_t status = GPMA_OK;
    double arrival = 0, start = 0, done = 0;
    uint64_t round = 0;
    std::vector<uint64_t> keys;
    std::vector<uint8_t> vals;
    uint64_t n = 0;
    uint64_t inserts = 0;  // non-zero values: the batch's possible insertions
    uint32_t nsrc = 0;
    uint32_t lane = 0;
    uint32_t src[64] = {};
    uint64_t reached[64] = {};
    uint32_t *levels_out = nullptr;
};

struct Graph {
    gpma_graph *g = nullptr;
    uint32_t row_num = 0;
    uint64_t charged = 0;      // bytes charged against the budget
    uint64_t plan_size = 0;    // plan-only mode: the array size the graph is assumed to have
    std::deque<uint64_t> queue;
};

constexpr double UPPER_ROOT_DENSITY = 0.84;  // root upper density bound (gpma.cuh:147-168)

// Smallest power-of-two array (>= 4 slots) whose root upper bound holds `live`
// entries, as the reference sizes the array on resize (gpma.cuh:906-934).
uint64_t slots_for(uint64_t live) {
    uint64_t s = 4;
    while ((uint64_t)std::floor(UPPER_ROOT_DENSITY * (double)s) < live)
        s <<= 1;
    return s;
}

// Device bytes of a graph with `slots` slots: keys + values, the same again as
// wide-window scratch, row_offset, BFS bitmaps and levels.
uint64_t graph_bytes(uint64_t slots, uint32_t row_num) {
    return slots * 18ull + 4ull * ((uint64_t)row_num + 1) + 4ull * row_num + 3ull * ((uint64_t)row_num / 8 + 16);
}

uint64_t actual_bytes(const gpma_graph *g) {
    return (uint64_t)g->cap * 9ull + (uint64_t)g->scratch_cap * 9ull + 4ull * ((uint64_t)g->row_num + 1) +
           (uint64_t)g->bfs_cap * 4ull + 3ull * ((uint64_t)g->row_num / 8 + 16);
}

}  // namespace

struct gpma_server {
    gpma_server_config cfg{};
    bool plan_only = false;
    cudaStream_t stream = nullptr;
    gpma_batch *batch = nullptr;
    std::vector<Graph> graphs;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
    uint64_t next_id = 1;
    uint64_t rounds = 0;
    uint64_t queued = 0, queued_keys = 0;
    uint64_t fixed_bytes = 0;  // round buffers charged against the budget
    std::vector<uint64_t> last_round;
    // pinned staging of a round's update keys
    uint64_t *h_keys = nullptr;
    uint8_t *h_vals = nullptr;
    uint64_t staging_cap = 0;

    uint64_t committed() const {
        uint64_t c = fixed_bytes;
        for (const Graph &g : graphs)
            c += g.charged;
        return c;
    }
};

using namespace gpma;

namespace {

// Bytes a graph is charged: the larger of its admission estimate and what it
// holds now.
void recharge(gpma_server *s, Graph &G) {
    if (G.g)
        G.charged = std::max(G.charged, actual_bytes(G.g));
}

// Worst-case bytes of the graph after an update with `inserts` insertions.
uint64_t grown_bytes(const gpma_server *s, const Graph &G, uint64_t inserts) {
    const uint64_t size = G.g ? G.g->geo.size : G.plan_size;
    const uint64_t live_max = (uint64_t)std::floor(UPPER_ROOT_DENSITY * (double)size);
    const uint64_t need = slots_for(live_max + inserts);
    return std::max(G.charged, graph_bytes(std::max<uint64_t>(need, size), G.row_num));
}

gpma_status ensure_staging(gpma_server *s, uint64_t n) {
    if (n <= s->staging_cap)
        return GPMA_OK;
    if (s->h_keys)
        cudaFreeHost(s->h_keys);
    if (s->h_vals)
        cudaFreeHost(s->h_vals);
    s->h_keys = nullptr;
    s->h_vals = nullptr;
    s->staging_cap = 0;
    const uint64_t cap = std::max<uint64_t>(n, 1u << 20);
    GPMA_CUDA(cudaMallocHost((void **)&s->h_keys, cap * sizeof(uint64_t)));
    GPMA_CUDA(cudaMallocHost((void **)&s->h_vals, cap));
    s->staging_cap = cap;
    return GPMA_OK;
}

struct BfsEntry {
    uint32_t graph;
    std::vector<uint64_t> reqs;
    uint32_t lanes = 0;
    bool want_levels = false;
};

}  // namespace

extern "C" {

gpma_status gpma_server_create(const gpma_server_config *cfg, void *stream, gpma_server **out) {
    if (!cfg || !out) {
        set_error("gpma_server_create: null argument");
        return GPMA_ERR_INVALID;
    }
    *out = nullptr;
    if (cfg->max_round_keys == 0 || cfg->max_round_bfs_graphs == 0 || cfg->max_queued == 0) {
        set_error("gpma_server_create: max_round_keys, max_round_bfs_graphs and max_queued must be positive");
        return GPMA_ERR_INVALID;
    }
    gpma_server *s = new (std::nothrow) gpma_server();
    if (!s) {
        set_error("gpma_server_create: host allocation failed");
        return GPMA_ERR_NOMEM;
    }
    s->cfg = *cfg;
    s->plan_only = (cfg->flags & GPMA_SERVER_PLAN_ONLY) != 0;
    s->stream = (cudaStream_t)stream;
    // the round's update buffers (about 110 bytes per key) are charged up front
    s->fixed_bytes = 110ull * cfg->max_round_keys;
    if (s->fixed_bytes > cfg->hbm_budget_bytes) {
        delete s;
        set_error("gpma_server_create: round buffers for %llu keys exceed the budget",
                  (unsigned long long)cfg->max_round_keys);
        return GPMA_ERR_BUDGET;
    }
    if (!s->plan_only) {
        gpma_status st = gpma_batch_create(&s->batch);
        if (st == GPMA_OK)
            st = gpma_batch_set_profiling(s->batch, 1);
        if (st != GPMA_OK) {
            gpma_batch_destroy(s->batch);
            delete s;
            return st;
        }
    }
    *out = s;
    return GPMA_OK;
}

gpma_status gpma_server_destroy(gpma_server *s) {
    if (!s)
        return GPMA_OK;
    for (Graph &G : s->graphs)
        gpma_destroy(G.g);
    gpma_batch_destroy(s->batch);
    if (s->h_keys)
        cudaFreeHost(s->h_keys);
    if (s->h_vals)
        cudaFreeHost(s->h_vals);
    delete s;
    return GPMA_OK;
}

gpma_status gpma_server_add_graph(gpma_server *s, uint32_t row_num, uint64_t reserve_edges, uint32_t *graph_id) {
    if (!s || !graph_id) {
        set_error("gpma_server_add_graph: null argument");
        return GPMA_ERR_INVALID;
    }
    const uint64_t slots = slots_for(reserve_edges + row_num + 2);
    const uint64_t est = graph_bytes(slots, row_num);
    if (s->committed() + est > s->cfg.hbm_budget_bytes) {
        set_error("gpma_server_add_graph: %llu bytes for %u nodes / %llu edges exceed the budget (%llu of %llu "
                  "committed)",
                  (unsigned long long)est, row_num, (unsigned long long)reserve_edges,
                  (unsigned long long)s->committed(), (unsigned long long)s->cfg.hbm_budget_bytes);
        return GPMA_ERR_BUDGET;
    }
    Graph G;
    G.row_num = row_num;
    G.charged = est;
    G.plan_size = slots;
    if (!s->plan_only)
        GPMA_TRY(gpma_create(row_num, s->stream, &G.g));
    s->graphs.push_back(std::move(G));
    *graph_id = (uint32_t)(s->graphs.size() - 1);
    return GPMA_OK;
}

gpma_status gpma_server_graph(gpma_server *s, uint32_t graph_id, gpma_graph **out) {
    if (!s || !out || graph_id >= s->graphs.size()) {
        set_error("gpma_server_graph: bad arguments");
        return GPMA_ERR_INVALID;
    }
    *out = s->graphs[graph_id].g;
    return GPMA_OK;
}

static gpma_status admit(gpma_server *s, uint32_t graph_id, uint64_t keys, const char *what) {
    if (graph_id >= s->graphs.size()) {
        set_error("%s: no graph %u", what, graph_id);
        return GPMA_ERR_INVALID;
    }
    if (s->queued >= s->cfg.max_queued || (keys && s->queued_keys + keys > s->cfg.max_queued_keys)) {
        set_error("%s: queue full (%llu requests, %llu keys waiting)", what, (unsigned long long)s->queued,
                  (unsigned long long)s->queued_keys);
        return GPMA_ERR_BUSY;
    }
    return GPMA_OK;
}

gpma_status gpma_server_submit_update(gpma_server *s, uint32_t graph_id, const uint64_t *keys, const uint8_t *values,
                                      uint64_t n, double arrival, uint64_t *request_id) {
    if (!s || !request_id || (n && (!keys || !values))) {
        set_error("gpma_server_submit_update: null argument");
        return GPMA_ERR_INVALID;
    }
    if (n >= (1ull << 30)) {
        set_error("gpma_server_submit_update: batch of %llu keys exceeds 2^30", (unsigned long long)n);
        return GPMA_ERR_CAPACITY;
    }
    GPMA_TRY(admit(s, graph_id, n, "gpma_server_submit_update"));
    auto r = std::make_unique<Request>();
    r->id = s->next_id++;
    r->graph = graph_id;
    r->kind = 0;
    r->arrival = arrival;
    r->n = n;
    r->keys.assign(keys, keys + n);
    r->vals.assign(values, values + n);
    for (uint64_t i = 0; i < n; ++i)
        r->inserts += values[i] != 0;
    *request_id = r->id;
    s->graphs[graph_id].queue.push_back(r->id);
    s->queued++;
    s->queued_keys += n;
    s->reqs.emplace(r->id, std::move(r));
    return GPMA_OK;
}

gpma_status gpma_server_submit_bfs(gpma_server *s, uint32_t graph_id, const uint32_t *sources, uint32_t k,
                                   double arrival, uint32_t *levels, uint64_t *request_id) {
    if (!s || !request_id || !sources || k == 0 || k > 64) {
        set_error("gpma_server_submit_bfs: bad arguments (1..64 sources)");
        return GPMA_ERR_INVALID;
    }
    GPMA_TRY(admit(s, graph_id, 0, "gpma_server_submit_bfs"));
    for (uint32_t i = 0; i < k; ++i)
        if (sources[i] >= s->graphs[graph_id].row_num) {
            set_error("gpma_server_submit_bfs: source %u out of range (row_num %u)", sources[i],
                      s->graphs[graph_id].row_num);
            return GPMA_ERR_INVALID;
        }
    auto r = std::make_unique<Request>();
    r->id = s->next_id++;
    r->graph = graph_id;
    r->kind = 1;
    r->arrival = arrival;
    r->nsrc = k;
    std::memcpy(r->src, sources, sizeof(uint32_t) * k);
    r->levels_out = levels;
    *request_id = r->id;
    s->graphs[graph_id].queue.push_back(r->id);
    s->queued++;
    s->reqs.emplace(r->id, std::move(r));
    return GPMA_OK;
}

gpma_status gpma_server_run_round(gpma_server *s, double now, gpma_round_info *info) {
    CallRange range("gpma_server_run_round");
    if (!s) {
        set_error("gpma_server_run_round: null argument");
        return GPMA_ERR_INVALID;
    }
    const auto t0 = std::chrono::steady_clock::now();
    gpma_round_info ri{};
    ri.start = now;
    s->last_round.clear();

    // ---- plan: graphs by the arrival of their queue head --------------------
    std::vector<uint32_t> order;
    for (uint32_t i = 0; i < s->graphs.size(); ++i)
        if (!s->graphs[i].queue.empty() && s->reqs[s->graphs[i].queue.front()]->arrival <= now)
            order.push_back(i);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        return s->reqs[s->graphs[a].queue.front()]->arrival < s->reqs[s->graphs[b].queue.front()]->arrival;
    });
    std::vector<uint64_t> upd;       // update requests of the round
    std::vector<uint32_t> upd_graph;
    std::vector<size_t> skip(s->graphs.size(), 0);  // queue entries taken by the update
    std::vector<Request *> failed;
    uint64_t round_keys = 0;
    const uint64_t base = s->committed();
    uint64_t committed = base;
    for (uint32_t gi : order) {
        Graph &G = s->graphs[gi];
        Request *r = s->reqs[G.queue.front()].get();
        if (r->kind != 0)
            continue;
        if (round_keys > 0 && round_keys + r->n > s->cfg.max_round_keys)
            continue;  // waits for a later round
        const uint64_t grown = grown_bytes(s, G, r->inserts);
        if (base - G.charged + grown > s->cfg.hbm_budget_bytes) {
            // does not fit even if no other graph grows: it never will
            r->state = GPMA_REQ_FAILED;
            r->status = GPMA_ERR_BUDGET;
            failed.push_back(r);
            continue;
        }
        if (committed - G.charged + grown > s->cfg.hbm_budget_bytes)
            continue;  // other graphs grow this round: wait
        committed += grown - G.charged;
        G.charged = grown;
        upd.push_back(r->id);
        upd_graph.push_back(gi);
        skip[gi] = 1;
        round_keys += r->n;
    }
    for (Request *r : failed) {
        Graph &G = s->graphs[r->graph];
        G.queue.pop_front();
        s->queued--;
        s->queued_keys -= r->n;
        r->start = now;
        r->done = now;
        r->round = s->rounds + 1;
        r->keys.clear();
        r->keys.shrink_to_fit();
        r->vals.clear();
        r->vals.shrink_to_fit();
        ri.failed++;
    }
    std::vector<BfsEntry> bfs;
    for (uint32_t gi : order) {
        if (bfs.size() >= s->cfg.max_round_bfs_graphs)
            break;
        Graph &G = s->graphs[gi];
        if (G.queue.empty())
            continue;
        Request *head = s->reqs[G.queue.front()].get();
        if (head->kind == 0 && skip[gi] == 0)
            continue;  // an update in front of the searches waits: so do they
        BfsEntry e;
        e.graph = gi;
        for (size_t q = skip[gi]; q < G.queue.size(); ++q) {
            Request *r = s->reqs[G.queue[q]].get();
            if (r->kind != 1 || r->arrival > now || e.lanes + r->nsrc > 64)
                break;
            r->lane = e.lanes;
            e.lanes += r->nsrc;
            e.want_levels |= r->levels_out != nullptr;
            e.reqs.push_back(r->id);
        }
        if (!e.reqs.empty())
            bfs.push_back(std::move(e));
    }
    if (upd.empty() && bfs.empty()) {
        if (info) {
            ri.round = s->rounds;
            *info = ri;
        }
        return GPMA_OK;
    }
    const uint64_t round_no = ++s->rounds;
    ri.round = round_no;

    // ---- execute -------------------------------------------------------------
    gpma_status st = GPMA_OK;
    std::vector<uint64_t> reached;
    double upd_seconds = 0.0, lone_update_ms = 0.0;
    if (!s->plan_only) {
        gpma_profile p0{};
        gpma_batch_get_profile(s->batch, &p0);
        if (upd.size() == 1) {
            // a lone update: the single-graph call straight from the request's
            // own buffer (no staging copy, no gather)
            Request *r = s->reqs[upd[0]].get();
            gpma_graph *g = s->graphs[upd_graph[0]].g;
            gpma_profile q0{}, q1{};
            st = gpma_set_profiling(g, 1);
            gpma_get_profile(g, &q0);
            if (st == GPMA_OK)
                st = gpma_update(g, r->keys.data(), r->vals.data(), r->n, s->stream);
            upd_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            gpma_get_profile(g, &q1);
            lone_update_ms = (q1.update_kernel_ms + q1.rebuild_ms) - (q0.update_kernel_ms + q0.rebuild_ms);
        } else if (!upd.empty()) {
            st = ensure_staging(s, round_keys);
            std::vector<gpma_graph *> gs(upd.size());
            std::vector<uint64_t> off(upd.size() + 1, 0);
            for (size_t j = 0; st == GPMA_OK && j < upd.size(); ++j) {
                Request *r = s->reqs[upd[j]].get();
                gs[j] = s->graphs[upd_graph[j]].g;
                std::memcpy(s->h_keys + off[j], r->keys.data(), r->n * sizeof(uint64_t));
                std::memcpy(s->h_vals + off[j], r->vals.data(), r->n);
                off[j + 1] = off[j] + r->n;
            }
            if (st == GPMA_OK)
                st = gpma_batch_update_packed(s->batch, gs.data(), s->h_keys, s->h_vals, off.data(),
                                              (uint32_t)gs.size(), s->stream);
            // the call returns once the update is on the device: its requests
            // are done here, before the round's searches run
            upd_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        }
        std::vector<std::vector<uint32_t>> lvl(bfs.size());
        if (st == GPMA_OK && !bfs.empty()) {
            std::vector<gpma_graph *> gs(bfs.size());
            std::vector<std::vector<uint32_t>> srcs(bfs.size());
            std::vector<const uint32_t *> sp(bfs.size());
            std::vector<uint32_t> ns(bfs.size());
            std::vector<uint32_t *> lp(bfs.size(), nullptr);
            bool any_levels = false;
            uint64_t lanes = 0;
            for (size_t j = 0; j < bfs.size(); ++j) {
                gs[j] = s->graphs[bfs[j].graph].g;
                for (uint64_t id : bfs[j].reqs) {
                    Request *r = s->reqs[id].get();
                    srcs[j].insert(srcs[j].end(), r->src, r->src + r->nsrc);
                }
                sp[j] = srcs[j].data();
                ns[j] = bfs[j].lanes;
                lanes += bfs[j].lanes;
                if (bfs[j].want_levels) {
                    lvl[j].resize((size_t)bfs[j].lanes * gs[j]->row_num);
                    lp[j] = lvl[j].data();
                    any_levels = true;
                }
            }
            reached.assign(lanes, 0);
            st = gpma_batch_bfs_multi(s->batch, gs.data(), sp.data(), ns.data(), (uint32_t)gs.size(),
                                      any_levels ? lp.data() : nullptr, reached.data(), s->stream);
            if (st == GPMA_OK)
                ri.edges = s->batch->last_traversed;
        }
        if (st == GPMA_OK) {
            // hand each search its lanes (levels rows [lane, lane + nsrc))
            for (size_t j = 0; j < bfs.size(); ++j) {
                if (!bfs[j].want_levels)
                    continue;
                const uint32_t n = s->graphs[bfs[j].graph].row_num;
                for (uint64_t id : bfs[j].reqs) {
                    Request *r = s->reqs[id].get();
                    if (r->levels_out)
                        std::memcpy(r->levels_out, lvl[j].data() + (size_t)r->lane * n,
                                    sizeof(uint32_t) * r->nsrc * (size_t)n);
                }
            }
        }
        gpma_profile p1{};
        gpma_batch_get_profile(s->batch, &p1);
        ri.update_ms = (p1.update_kernel_ms + p1.rebuild_ms) - (p0.update_kernel_ms + p0.rebuild_ms) + lone_update_ms;
        ri.bfs_ms = p1.bfs_ms - p0.bfs_ms;
        for (uint32_t gi : upd_graph)
            recharge(s, s->graphs[gi]);
    } else {
        uint64_t lanes = 0;
        for (const BfsEntry &e : bfs)
            lanes += e.lanes;
        reached.assign(lanes, 0);
    }
    const double seconds = s->plan_only
                               ? 0.0
                               : std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    ri.seconds = seconds;

    // ---- complete --------------------------------------------------------------
    auto finish = [&](Request *r, double took) {
        r->state = st == GPMA_OK ? GPMA_REQ_DONE : GPMA_REQ_FAILED;
        r->status = st;
        r->start = now;
        r->done = now + took;
        r->round = round_no;
        s->last_round.push_back(r->id);
    };
    for (size_t j = 0; j < upd.size(); ++j) {
        Request *r = s->reqs[upd[j]].get();
        Graph &G = s->graphs[upd_graph[j]];
        G.queue.pop_front();
        s->queued--;
        s->queued_keys -= r->n;
        ri.updates++;
        ri.keys += r->n;
        r->keys.clear();
        r->keys.shrink_to_fit();
        r->vals.clear();
        r->vals.shrink_to_fit();
        finish(r, upd_seconds);
    }
    uint64_t lane_base = 0;
    for (const BfsEntry &e : bfs) {
        Graph &G = s->graphs[e.graph];
        for (uint64_t id : e.reqs) {
            Request *r = s->reqs[id].get();
            // the entries taken are the front of the queue now that the update left
            G.queue.pop_front();
            s->queued--;
            for (uint32_t j = 0; j < r->nsrc; ++j)
                r->reached[j] = reached[lane_base + r->lane + j];
            ri.bfs_requests++;
            ri.sources += r->nsrc;
            finish(r, seconds);
        }
        lane_base += e.lanes;
        ri.bfs_graphs++;
    }
    if (st != GPMA_OK)
        ri.failed += ri.updates + ri.bfs_requests;
    if (info)
        *info = ri;
    return st;
}

gpma_status gpma_server_poll(gpma_server *s, uint64_t request_id, int release, gpma_request_info *out) {
    if (!s || !out) {
        set_error("gpma_server_poll: null argument");
        return GPMA_ERR_INVALID;
    }
    auto it = s->reqs.find(request_id);
    if (it == s->reqs.end()) {
        set_error("gpma_server_poll: unknown request %llu", (unsigned long long)request_id);
        return GPMA_ERR_INVALID;
    }
    const Request *r = it->second.get();
    std::memset(out, 0, sizeof(*out));
    out->id = r->id;
    out->graph = r->graph;
    out->kind = r->kind;
    out->state = r->state;
    out->status = r->status;
    out->arrival = r->arrival;
    out->start = r->start;
    out->done = r->done;
    out->round = r->round;
    out->keys = r->n;
    out->nsrc = r->nsrc;
    out->lane = r->lane;
    std::memcpy(out->reached, r->reached, sizeof(out->reached));
    if (release && r->state != GPMA_REQ_QUEUED)
        s->reqs.erase(it);
    return GPMA_OK;
}

gpma_status gpma_server_cancel(gpma_server *s, uint64_t request_id) {
    if (!s) {
        set_error("gpma_server_cancel: null argument");
        return GPMA_ERR_INVALID;
    }
    auto it = s->reqs.find(request_id);
    if (it == s->reqs.end()) {
        set_error("gpma_server_cancel: unknown request %llu", (unsigned long long)request_id);
        return GPMA_ERR_INVALID;
    }
    Request *r = it->second.get();
    if (r->state != GPMA_REQ_QUEUED) {
        set_error("gpma_server_cancel: request %llu has already run", (unsigned long long)request_id);
        return GPMA_ERR_INVALID;
    }
    // a queued request sits in its graph's queue until a round takes it
    std::deque<uint64_t> &q = s->graphs[r->graph].queue;
    const auto qi = std::find(q.begin(), q.end(), request_id);
    if (qi == q.end()) {
        set_error("gpma_server_cancel: request %llu is not in its graph's queue", (unsigned long long)request_id);
        return GPMA_ERR_INVALID;
    }
    q.erase(qi);
    s->queued--;
    s->queued_keys -= r->n;
    r->state = GPMA_REQ_CANCELLED;
    r->levels_out = nullptr;
    r->keys.clear();
    r->keys.shrink_to_fit();
    r->vals.clear();
    r->vals.shrink_to_fit();
    return GPMA_OK;
}

gpma_status gpma_server_last_round(const gpma_server *s, uint64_t *ids, uint32_t capacity, uint32_t *count) {
    if (!s || !count || (capacity && !ids)) {
        set_error("gpma_server_last_round: null argument");
        return GPMA_ERR_INVALID;
    }
    *count = (uint32_t)s->last_round.size();
    std::copy_n(s->last_round.begin(), std::min<size_t>(capacity, s->last_round.size()), ids);
    return GPMA_OK;
}

gpma_status gpma_server_queued(const gpma_server *s, uint64_t *requests, uint64_t *keys, double *next_arrival) {
    if (!s) {
        set_error("gpma_server_queued: null argument");
        return GPMA_ERR_INVALID;
    }
    if (requests)
        *requests = s->queued;
    if (keys)
        *keys = s->queued_keys;
    if (next_arrival) {
        double t = std::numeric_limits<double>::infinity();
        for (const Graph &G : s->graphs)
            if (!G.queue.empty())
                t = std::min(t, s->reqs.at(G.queue.front())->arrival);
        *next_arrival = t;
    }
    return GPMA_OK;
}

gpma_status gpma_server_committed_bytes(const gpma_server *s, uint64_t *bytes) {
    if (!s || !bytes) {
        set_error("gpma_server_committed_bytes: null argument");
        return GPMA_ERR_INVALID;
    }
    *bytes = s->committed();
    return GPMA_OK;
}

}  // extern "C"
