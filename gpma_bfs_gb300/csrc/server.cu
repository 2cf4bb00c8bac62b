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
//
// Lanes: up to four rounds in flight, each with its own stream, gpma_batch and
// pinned staging. Planning and completion run under the server's mutex; a
// round's device work runs outside it on its lane. A graph with requests in a
// round in flight is skipped by other rounds' planning, and the requests a
// round takes leave their queue (state RUNNING) when it is planned.
#include "gpma_internal.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <limits>
#include <memory>
#include <condition_variable>
#include <mutex>
#include <thread>
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
    // the batch: in the pinned input ring (ring_block >= 0) or in the vectors
    std::vector<uint64_t> keys;
    std::vector<uint8_t> vals;
    const uint64_t *k = nullptr;
    const uint8_t *v = nullptr;
    int64_t ring_block = -1;
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
    bool inflight = false;     // its requests are in a round that has not completed
    std::deque<uint64_t> queue;
};

// One round in flight: its stream, batch buffers and pinned staging.
struct Lane {
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    gpma_batch *batch = nullptr;
    bool busy = false;
    uint64_t *h_keys = nullptr;
    uint8_t *h_vals = nullptr;
    uint64_t staging_cap = 0;
};

constexpr uint32_t MAX_LANES = 4;

// Pinned host ring for queued update batches: blocks are taken at the tail
// (wrapping to the start when the end is short) and given back when their
// request completes; the head advances over the given-back blocks in
// allocation order.
struct InputRing {
    unsigned char *base = nullptr;
    uint64_t cap = 0, head = 0, tail = 0, used = 0;
    struct Block {
        uint64_t off, size;
        bool done;
    };
    std::deque<Block> blocks;
    uint64_t first_id = 0;  // id of blocks.front()

    // offset of a free block of `size` bytes, or -1
    int64_t take(uint64_t size, uint64_t *id) {
        size = (size + 15) & ~uint64_t(15);
        if (!base || size == 0 || size > cap)
            return -1;
        uint64_t off;
        if (blocks.empty()) {
            head = tail = 0;
            off = 0;
        } else if (tail >= head) {  // free space: [tail, cap) and [0, head)
            if (cap - tail >= size)
                off = tail;
            else if (head > size)  // wrap (strictly below head: a full ring never looks empty)
                off = 0;
            else
                return -1;
        } else {  // free space: [tail, head)
            if (head - tail > size)
                off = tail;
            else
                return -1;
        }
        if (off == 0 && !blocks.empty() && tail != 0 && tail >= head)
            blocks.push_back({tail, cap - tail, true});  // the skipped end, given back at once
        blocks.push_back({off, size, false});
        tail = off + size;
        used += size;
        *id = first_id + blocks.size() - 1;
        return (int64_t)off;
    }
    void give_back(uint64_t id) {
        if (id < first_id || id - first_id >= blocks.size())
            return;
        Block &b = blocks[id - first_id];
        if (b.done)
            return;
        b.done = true;
        used -= b.size;
        while (!blocks.empty() && blocks.front().done) {
            head = blocks.front().off + blocks.front().size;
            blocks.pop_front();
            ++first_id;
        }
        if (blocks.empty())
            head = tail = 0;
    }
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
    std::vector<Lane> lanes;
    std::mutex mu;  // queues, requests, graphs' flags and charges, lanes' busy flags
    // serving loop (gpma_server_start): one worker thread per lane on the
    // server's own clock; woken by submissions and completed rounds
    std::condition_variable cv;
    std::vector<std::thread> workers;
    bool stopping = false;
    bool started = false;
    std::chrono::steady_clock::time_point epoch;
    uint64_t running = 0;       // requests taken by rounds in flight
    gpma_status loop_status = GPMA_OK;  // first failing round of the serving loop
    gpma_server_stats stats{};
    std::vector<Graph> graphs;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
    uint64_t next_id = 1;
    uint64_t rounds = 0;
    uint64_t queued = 0, queued_keys = 0;
    uint64_t fixed_bytes = 0;  // round buffers charged against the budget
    InputRing ring;

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

gpma_status ensure_staging(Lane &L, uint64_t n) {
    if (n <= L.staging_cap)
        return GPMA_OK;
    if (L.h_keys)
        cudaFreeHost(L.h_keys);
    if (L.h_vals)
        cudaFreeHost(L.h_vals);
    L.h_keys = nullptr;
    L.h_vals = nullptr;
    L.staging_cap = 0;
    const uint64_t cap = std::max<uint64_t>(n, 1u << 20);
    GPMA_CUDA(cudaMallocHost((void **)&L.h_keys, cap * sizeof(uint64_t)));
    GPMA_CUDA(cudaMallocHost((void **)&L.h_vals, cap));
    L.staging_cap = cap;
    return GPMA_OK;
}

// Drops a request's batch: its ring block or its vectors.
void drop_batch(gpma_server *s, Request *r) {
    if (r->ring_block >= 0)
        s->ring.give_back((uint64_t)r->ring_block);
    r->ring_block = -1;
    r->k = nullptr;
    r->v = nullptr;
    r->keys.clear();
    r->keys.shrink_to_fit();
    r->vals.clear();
    r->vals.shrink_to_fit();
}

void release_lane(Lane &L) {
    gpma_batch_destroy(L.batch);
    L.batch = nullptr;
    if (L.h_keys)
        cudaFreeHost(L.h_keys);
    if (L.h_vals)
        cudaFreeHost(L.h_vals);
    L.h_keys = nullptr;
    L.h_vals = nullptr;
    if (L.own_stream && L.stream)
        cudaStreamDestroy(L.stream);
    L.stream = nullptr;
}

// Ids of the requests of the last round each host thread ran, per server.
thread_local const gpma_server *t_last_server = nullptr;
thread_local std::vector<uint64_t> t_last_round;

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
    if (cfg->lanes > MAX_LANES) {
        set_error("gpma_server_create: %u lanes requested, at most %u", cfg->lanes, MAX_LANES);
        return GPMA_ERR_INVALID;
    }
    const uint32_t lanes = cfg->lanes ? cfg->lanes : 1u;
    gpma_server *s = new (std::nothrow) gpma_server();
    if (!s) {
        set_error("gpma_server_create: host allocation failed");
        return GPMA_ERR_NOMEM;
    }
    s->cfg = *cfg;
    s->plan_only = (cfg->flags & GPMA_SERVER_PLAN_ONLY) != 0;
    s->stream = (cudaStream_t)stream;
    // each lane's round update buffers (about 120 bytes per key) are charged up front
    s->fixed_bytes = 120ull * cfg->max_round_keys * lanes;
    if (s->fixed_bytes > cfg->hbm_budget_bytes) {
        delete s;
        set_error("gpma_server_create: round buffers for %llu keys exceed the budget",
                  (unsigned long long)cfg->max_round_keys);
        return GPMA_ERR_BUDGET;
    }
    s->lanes.resize(lanes);
    if (cfg->input_ring_bytes) {
        // pinned for uploads; plain host memory in plan-only mode (no device)
        const uint64_t cap = (cfg->input_ring_bytes + 15) & ~uint64_t(15);
        if (s->plan_only) {
            s->ring.base = static_cast<unsigned char *>(std::malloc(cap));
            if (!s->ring.base) {
                delete s;
                set_error("gpma_server_create: input ring of %llu bytes", (unsigned long long)cap);
                return GPMA_ERR_NOMEM;
            }
        } else {
            cudaError_t e = cudaMallocHost((void **)&s->ring.base, cap);
            if (e != cudaSuccess) {
                s->ring.base = nullptr;
                cudaGetLastError();
                delete s;
                set_error("gpma_server_create: pinned input ring of %llu bytes: %s", (unsigned long long)cap,
                          cudaGetErrorString(e));
                return GPMA_ERR_NOMEM;
            }
        }
        s->ring.cap = cap;
    }
    if (!s->plan_only) {
        gpma_status st = GPMA_OK;
        for (uint32_t i = 0; i < lanes && st == GPMA_OK; ++i) {
            Lane &L = s->lanes[i];
            if (i == 0) {
                L.stream = s->stream;  // the first lane runs on the caller's stream
            } else {
                cudaError_t e = cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking);
                if (e != cudaSuccess) {
                    st = cuda_fail(e, "cudaStreamCreateWithFlags(server lane)");
                    break;
                }
                L.own_stream = true;
            }
            st = gpma_batch_create(&L.batch);
            if (st == GPMA_OK)
                st = gpma_batch_set_profiling(L.batch, 1);
        }
        if (st != GPMA_OK) {
            for (Lane &L : s->lanes)
                release_lane(L);
            if (s->ring.base)
                cudaFreeHost(s->ring.base);  // not plan-only here
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
    gpma_server_stop(s);
    for (Lane &L : s->lanes)
        if (L.stream)
            cudaStreamSynchronize(L.stream);
    for (Graph &G : s->graphs)
        gpma_destroy(G.g);
    for (Lane &L : s->lanes)
        release_lane(L);
    if (s->ring.base) {
        if (s->plan_only)
            std::free(s->ring.base);
        else
            cudaFreeHost(s->ring.base);
    }
    if (t_last_server == s)
        t_last_server = nullptr;
    delete s;
    return GPMA_OK;
}

gpma_status gpma_server_add_graph(gpma_server *s, uint32_t row_num, uint64_t reserve_edges, uint32_t *graph_id) {
    if (!s || !graph_id) {
        set_error("gpma_server_add_graph: null argument");
        return GPMA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(s->mu);
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
    if (!s || !out) {
        set_error("gpma_server_graph: bad arguments");
        return GPMA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(s->mu);
    if (graph_id >= s->graphs.size()) {
        set_error("gpma_server_graph: no graph %u", graph_id);
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
    std::lock_guard<std::mutex> lock(s->mu);
    GPMA_TRY(admit(s, graph_id, n, "gpma_server_submit_update"));
    auto r = std::make_unique<Request>();
    r->id = s->next_id++;
    r->graph = graph_id;
    r->kind = 0;
    r->arrival = arrival;
    r->n = n;
    uint64_t block = 0;
    const int64_t off = n ? s->ring.take(n * 9ull, &block) : -1;
    if (off >= 0) {
        uint64_t *rk = reinterpret_cast<uint64_t *>(s->ring.base + off);
        uint8_t *rv = s->ring.base + off + n * 8ull;
        std::memcpy(rk, keys, n * sizeof(uint64_t));
        std::memcpy(rv, values, n);
        r->k = rk;
        r->v = rv;
        r->ring_block = (int64_t)block;
    } else {
        r->keys.assign(keys, keys + n);
        r->vals.assign(values, values + n);
        r->k = r->keys.data();
        r->v = r->vals.data();
    }
    for (uint64_t i = 0; i < n; ++i)
        r->inserts += values[i] != 0;
    *request_id = r->id;
    s->graphs[graph_id].queue.push_back(r->id);
    s->queued++;
    s->queued_keys += n;
    s->reqs.emplace(r->id, std::move(r));
    s->cv.notify_all();
    return GPMA_OK;
}

gpma_status gpma_server_submit_bfs(gpma_server *s, uint32_t graph_id, const uint32_t *sources, uint32_t k,
                                   double arrival, uint32_t *levels, uint64_t *request_id) {
    if (!s || !request_id || !sources || k == 0 || k > 64) {
        set_error("gpma_server_submit_bfs: bad arguments (1..64 sources)");
        return GPMA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(s->mu);
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
    s->cv.notify_all();
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
    t_last_server = s;
    t_last_round.clear();

    // ---- plan (under the lock): a free lane, graphs by their queue head's arrival
    std::unique_lock<std::mutex> lock(s->mu);
    uint32_t lane = MAX_LANES;
    for (uint32_t i = 0; i < s->lanes.size(); ++i)
        if (!s->lanes[i].busy) {
            lane = i;
            break;
        }
    if (lane == MAX_LANES) {
        // every lane has a round in flight: nothing to run now
        if (info) {
            ri.round = s->rounds;
            *info = ri;
        }
        return GPMA_OK;
    }
    std::vector<uint32_t> order;
    for (uint32_t i = 0; i < s->graphs.size(); ++i)
        if (!s->graphs[i].inflight && !s->graphs[i].queue.empty() &&
            s->reqs[s->graphs[i].queue.front()]->arrival <= now)
            order.push_back(i);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        return s->reqs[s->graphs[a].queue.front()]->arrival < s->reqs[s->graphs[b].queue.front()]->arrival;
    });
    std::vector<Request *> upd;      // update requests of the round
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
        upd.push_back(r);
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
        drop_batch(s, r);
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
    // take the round's requests out of their queues (updates first, then the
    // searches behind them) and its graphs out of other rounds' planning
    std::vector<std::vector<Request *>> bfs_reqs(bfs.size());
    for (size_t j = 0; j < upd.size(); ++j) {
        Graph &G = s->graphs[upd_graph[j]];
        G.queue.pop_front();
        G.inflight = true;
        s->queued--;
        upd[j]->state = GPMA_REQ_RUNNING;
    }
    for (size_t j = 0; j < bfs.size(); ++j) {
        Graph &G = s->graphs[bfs[j].graph];
        G.inflight = true;
        for (uint64_t id : bfs[j].reqs) {
            Request *r = s->reqs[id].get();
            G.queue.pop_front();  // the entries taken are the queue's front now
            s->queued--;
            r->state = GPMA_REQ_RUNNING;
            bfs_reqs[j].push_back(r);
        }
    }
    Lane &L = s->lanes[lane];
    L.busy = true;
    uint64_t taken = upd.size();
    for (const auto &v : bfs_reqs)
        taken += v.size();
    s->running += taken;
    {
        uint32_t busy = 0;
        for (const Lane &x : s->lanes)
            busy += x.busy ? 1u : 0u;
        s->stats.max_inflight_rounds = std::max(s->stats.max_inflight_rounds, busy);
    }
    std::vector<gpma_graph *> upd_g(upd.size()), bfs_g(bfs.size());
    for (size_t j = 0; j < upd.size(); ++j)
        upd_g[j] = s->graphs[upd_graph[j]].g;
    for (size_t j = 0; j < bfs.size(); ++j)
        bfs_g[j] = s->graphs[bfs[j].graph].g;
    lock.unlock();

    // ---- execute on the lane (no lock: the round owns its graphs, its
    // requests and the lane) -------------------------------------------------
    gpma_status st = GPMA_OK;
    std::vector<uint64_t> reached;
    double upd_seconds = 0.0, lone_update_ms = 0.0;
    if (!s->plan_only) {
        gpma_profile p0{};
        gpma_batch_get_profile(L.batch, &p0);
        if (upd.size() == 1) {
            // a lone update: the single-graph call straight from the request's
            // own buffer (no staging copy, no gather)
            Request *r = upd[0];
            gpma_graph *g = upd_g[0];
            gpma_profile q0{}, q1{};
            st = gpma_set_profiling(g, 1);
            gpma_get_profile(g, &q0);
            if (st == GPMA_OK)
                st = gpma_update(g, r->k, r->v, r->n, L.stream);
            upd_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            gpma_get_profile(g, &q1);
            lone_update_ms = (q1.update_kernel_ms + q1.rebuild_ms) - (q0.update_kernel_ms + q0.rebuild_ms);
        } else if (!upd.empty()) {
            st = ensure_staging(L, round_keys);
            std::vector<uint64_t> off(upd.size() + 1, 0);
            for (size_t j = 0; st == GPMA_OK && j < upd.size(); ++j) {
                Request *r = upd[j];
                std::memcpy(L.h_keys + off[j], r->k, r->n * sizeof(uint64_t));
                std::memcpy(L.h_vals + off[j], r->v, r->n);
                off[j + 1] = off[j] + r->n;
            }
            if (st == GPMA_OK)
                st = gpma_batch_update_packed(L.batch, upd_g.data(), L.h_keys, L.h_vals, off.data(),
                                              (uint32_t)upd_g.size(), L.stream);
            // the call returns once the update is on the device: its requests
            // are done here, before the round's searches run
            upd_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        }
        std::vector<std::vector<uint32_t>> lvl(bfs.size());
        if (st == GPMA_OK && !bfs.empty()) {
            std::vector<std::vector<uint32_t>> srcs(bfs.size());
            std::vector<const uint32_t *> sp(bfs.size());
            std::vector<uint32_t> ns(bfs.size());
            std::vector<uint32_t *> lp(bfs.size(), nullptr);
            bool any_levels = false;
            uint64_t lanes = 0;
            for (size_t j = 0; j < bfs.size(); ++j) {
                for (Request *r : bfs_reqs[j])
                    srcs[j].insert(srcs[j].end(), r->src, r->src + r->nsrc);
                sp[j] = srcs[j].data();
                ns[j] = bfs[j].lanes;
                lanes += bfs[j].lanes;
                if (bfs[j].want_levels) {
                    lvl[j].resize((size_t)bfs[j].lanes * bfs_g[j]->row_num);
                    lp[j] = lvl[j].data();
                    any_levels = true;
                }
            }
            reached.assign(lanes, 0);
            st = gpma_batch_bfs_multi(L.batch, bfs_g.data(), sp.data(), ns.data(), (uint32_t)bfs_g.size(),
                                      any_levels ? lp.data() : nullptr, reached.data(), L.stream);
            if (st == GPMA_OK)
                ri.edges = L.batch->last_traversed;
        }
        if (st == GPMA_OK) {
            // hand each search its lanes (levels rows [lane, lane + nsrc))
            for (size_t j = 0; j < bfs.size(); ++j) {
                if (!bfs[j].want_levels)
                    continue;
                const uint32_t n = bfs_g[j]->row_num;
                for (Request *r : bfs_reqs[j])
                    if (r->levels_out)
                        std::memcpy(r->levels_out, lvl[j].data() + (size_t)r->lane * n,
                                    sizeof(uint32_t) * r->nsrc * (size_t)n);
            }
        }
        gpma_profile p1{};
        gpma_batch_get_profile(L.batch, &p1);
        ri.update_ms = (p1.update_kernel_ms + p1.rebuild_ms) - (p0.update_kernel_ms + p0.rebuild_ms) + lone_update_ms;
        ri.bfs_ms = p1.bfs_ms - p0.bfs_ms;
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

    // ---- complete (under the lock) ----------------------------------------------
    lock.lock();
    auto finish = [&](Request *r, double took) {
        r->state = st == GPMA_OK ? GPMA_REQ_DONE : GPMA_REQ_FAILED;
        r->status = st;
        r->start = now;
        r->done = now + took;
        r->round = round_no;
        t_last_round.push_back(r->id);
    };
    for (size_t j = 0; j < upd.size(); ++j) {
        Request *r = upd[j];
        s->queued_keys -= r->n;
        ri.updates++;
        ri.keys += r->n;
        drop_batch(s, r);
        finish(r, upd_seconds);
        Graph &G = s->graphs[upd_graph[j]];
        G.inflight = false;
        if (!s->plan_only)
            recharge(s, G);
    }
    uint64_t lane_base = 0;
    for (size_t j = 0; j < bfs.size(); ++j) {
        for (Request *r : bfs_reqs[j]) {
            for (uint32_t q = 0; q < r->nsrc; ++q)
                r->reached[q] = reached[lane_base + r->lane + q];
            ri.bfs_requests++;
            ri.sources += r->nsrc;
            finish(r, seconds);
        }
        lane_base += bfs[j].lanes;
        s->graphs[bfs[j].graph].inflight = false;
        ri.bfs_graphs++;
    }
    L.busy = false;
    s->running -= taken;
    if (st != GPMA_OK)
        ri.failed += ri.updates + ri.bfs_requests;
    s->stats.rounds++;
    s->stats.requests += taken;
    s->stats.keys += ri.keys;
    s->stats.edges += ri.edges;
    s->stats.busy_seconds += ri.seconds;
    s->stats.update_ms += ri.update_ms;
    s->stats.bfs_ms += ri.bfs_ms;
    s->stats.max_round_requests = std::max<uint32_t>(s->stats.max_round_requests, (uint32_t)taken);
    lock.unlock();
    s->cv.notify_all();
    if (info)
        *info = ri;
    return st;
}

gpma_status gpma_server_poll(gpma_server *s, uint64_t request_id, int release, gpma_request_info *out) {
    if (!s || !out) {
        set_error("gpma_server_poll: null argument");
        return GPMA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(s->mu);
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
    if (release && r->state != GPMA_REQ_QUEUED && r->state != GPMA_REQ_RUNNING)
        s->reqs.erase(it);
    return GPMA_OK;
}

gpma_status gpma_server_cancel(gpma_server *s, uint64_t request_id) {
    if (!s) {
        set_error("gpma_server_cancel: null argument");
        return GPMA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->reqs.find(request_id);
    if (it == s->reqs.end()) {
        set_error("gpma_server_cancel: unknown request %llu", (unsigned long long)request_id);
        return GPMA_ERR_INVALID;
    }
    Request *r = it->second.get();
    if (r->state != GPMA_REQ_QUEUED) {
        set_error("gpma_server_cancel: request %llu has already run or is running", (unsigned long long)request_id);
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
    drop_batch(s, r);
    return GPMA_OK;
}

gpma_status gpma_server_last_round(const gpma_server *s, uint64_t *ids, uint32_t capacity, uint32_t *count) {
    if (!s || !count || (capacity && !ids)) {
        set_error("gpma_server_last_round: null argument");
        return GPMA_ERR_INVALID;
    }
    const std::vector<uint64_t> empty;
    const std::vector<uint64_t> &last = t_last_server == s ? t_last_round : empty;
    *count = (uint32_t)last.size();
    std::copy_n(last.begin(), std::min<size_t>(capacity, last.size()), ids);
    return GPMA_OK;
}

gpma_status gpma_server_queued(const gpma_server *s, uint64_t *requests, uint64_t *keys, double *next_arrival) {
    if (!s) {
        set_error("gpma_server_queued: null argument");
        return GPMA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(const_cast<gpma_server *>(s)->mu);
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

static double server_clock(const gpma_server *s) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - s->epoch).count();
}

// One lane's worker of the serving loop.
static void serve_loop(gpma_server *s) {
    bool idle = false;  // the last round found nothing it could take
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (idle)
                // runnable by arrival but held back (budget, round limits, a
                // graph in another lane): wait for a round to complete
                s->cv.wait_for(lk, std::chrono::milliseconds(1));
            for (;;) {
                if (s->stopping)
                    return;
                bool free_lane = false;
                for (const Lane &L : s->lanes)
                    free_lane |= !L.busy;
                double next = std::numeric_limits<double>::infinity();
                if (free_lane)
                    for (const Graph &G : s->graphs)
                        if (!G.inflight && !G.queue.empty())
                            next = std::min(next, s->reqs.at(G.queue.front())->arrival);
                const double now = server_clock(s);
                if (next <= now)
                    break;
                if (next == std::numeric_limits<double>::infinity())
                    s->cv.wait_for(lk, std::chrono::milliseconds(10));
                else
                    s->cv.wait_for(lk, std::chrono::duration<double>(std::min(next - now, 0.01)));
            }
        }
        gpma_round_info ri{};
        const gpma_status st = gpma_server_run_round(s, server_clock(s), &ri);
        idle = ri.updates + ri.bfs_requests + ri.failed == 0;
        if (st != GPMA_OK) {
            std::lock_guard<std::mutex> lk(s->mu);
            if (s->loop_status == GPMA_OK)
                s->loop_status = st;
        }
    }
}

gpma_status gpma_server_start(gpma_server *s) {
    if (!s) {
        set_error("gpma_server_start: null argument");
        return GPMA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->started) {
        set_error("gpma_server_start: the serving loop is already running");
        return GPMA_ERR_INVALID;
    }
    int dev = -1;  // plan-only mode: no device
    if (!s->plan_only)
        GPMA_CUDA(cudaGetDevice(&dev));
    if (!s->plan_only) {
        // each lane's update buffers for a full round (max_round_keys keys, as
        // charged to the budget) and its search state for every graph added so
        // far, allocated now rather than by the first rounds that need them
        // (an allocation inside a round stalls it and the other lanes)
        std::vector<gpma_graph *> all;
        for (Graph &G : s->graphs)
            all.push_back(G.g);
        const uint32_t k = (uint32_t)all.size();
        std::vector<uint32_t> zero(k, 0u), one(k, 1u);
        std::vector<const uint32_t *> srcs(k);
        for (uint32_t i = 0; i < k; ++i)
            srcs[i] = &zero[i];
        for (Lane &L : s->lanes) {
            GPMA_TRY(ensure_buffers(L.batch->buf, s->cfg.max_round_keys, std::max<uint32_t>(k, 1)));
            if (k) {
                BatchBfsPlan P;
                GPMA_TRY(batch_bfs_plan(L.batch, all.data(), srcs.data(), one.data(), k, nullptr, &P));
            }
        }
    }
    s->epoch = std::chrono::steady_clock::now();
    s->stopping = false;
    s->loop_status = GPMA_OK;
    s->started = true;
    try {
        for (size_t i = 0; i < s->lanes.size(); ++i)
            s->workers.emplace_back([s, dev]() {
                if (dev >= 0)
                    cudaSetDevice(dev);
                serve_loop(s);
            });
    } catch (...) {
        s->stopping = true;
        set_error("gpma_server_start: could not start the worker threads");
        return GPMA_ERR_NOMEM;
    }
    return GPMA_OK;
}

gpma_status gpma_server_clock(const gpma_server *s, double *now) {
    if (!s || !now) {
        set_error("gpma_server_clock: null argument");
        return GPMA_ERR_INVALID;
    }
    *now = s->started ? server_clock(s) : 0.0;
    return GPMA_OK;
}

gpma_status gpma_server_drain(gpma_server *s, double timeout_seconds) {
    if (!s) {
        set_error("gpma_server_drain: null argument");
        return GPMA_ERR_INVALID;
    }
    std::unique_lock<std::mutex> lk(s->mu);
    const auto until = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_seconds);
    while (s->queued > 0 || s->running > 0) {
        if (!s->started) {
            set_error("gpma_server_drain: the serving loop is not running");
            return GPMA_ERR_INVALID;
        }
        if (s->cv.wait_until(lk, until) == std::cv_status::timeout && (s->queued > 0 || s->running > 0)) {
            set_error("gpma_server_drain: %llu requests queued and %llu running after %.3f s",
                      (unsigned long long)s->queued, (unsigned long long)s->running, timeout_seconds);
            return GPMA_ERR_TIMEOUT;
        }
    }
    if (s->loop_status != GPMA_OK)
        set_error("gpma_server_drain: a round of the serving loop failed (%s)", gpma_status_string(s->loop_status));
    return s->loop_status;
}

gpma_status gpma_server_stop(gpma_server *s) {
    if (!s) {
        set_error("gpma_server_stop: null argument");
        return GPMA_ERR_INVALID;
    }
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
    }
    s->cv.notify_all();
    for (std::thread &t : s->workers)
        if (t.joinable())
            t.join();
    s->workers.clear();
    std::lock_guard<std::mutex> lk(s->mu);
    s->started = false;
    return GPMA_OK;
}

gpma_status gpma_server_get_stats(const gpma_server *s, gpma_server_stats *out) {
    if (!s || !out) {
        set_error("gpma_server_get_stats: null argument");
        return GPMA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(const_cast<gpma_server *>(s)->mu);
    *out = s->stats;
    return GPMA_OK;
}

gpma_status gpma_server_committed_bytes(const gpma_server *s, uint64_t *bytes) {
    if (!s || !bytes) {
        set_error("gpma_server_committed_bytes: null argument");
        return GPMA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(const_cast<gpma_server *>(s)->mu);
    *bytes = s->committed();
    return GPMA_OK;
}

}  // extern "C"
