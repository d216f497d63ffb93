// g5_server.cpp -- BFS query serving with continuous batching.
//
// The reference answers one root at a time (cpu_2d/main.cpp:419-462).  Here a
// server keeps several graphs resident and answers single-root queries as
// they arrive: a worker thread steps the batched level loop of all graphs
// one level at a time; between steps, finished roots retire (their frontier
// became empty, so their parent arrays are complete) and queued queries are
// admitted into free root slots.  A query therefore starts at the next level
// boundary instead of waiting for a whole batch, and its work shares every
// adjacency read with the other queries of its graph that are in flight.
//
// Two slot kinds: one-root search workspaces on their own streams (queries
// start as soon as a workspace is free and run concurrently), or root bits
// of the bit-sliced level loop (queries join at the next level boundary and
// share every adjacency read with the other roots of their graph).  The
// automatic mode gives the large graphs, whose one-root searches would
// saturate the GPU first, the level slots and the small ones the stream
// workspaces, each kind with its own worker thread.
// A third kind, cohorts, runs the batched kernel itself: a graph holds a few
// batch workspaces (sharing one degree-ordered copy of the graph), and when a
// workspace is free the queries queued for that graph -- up to the
// workspace's root slots -- start together as one bit-sliced search.  Under
// light load a cohort holds one or two queries and starts at once; under
// heavy load queries gather while the workspaces are busy, so the cohorts
// grow and one adjacency read serves up to 64 queries.
// Admission is by device memory: a graph gets as many slots (at most 64) as
// its share of the budget holds.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "g5_internal.h"
#include "g5bfs.h"

namespace {

using Clock = std::chrono::steady_clock;

// Automatic mode: graphs of at least this many vertices get level slots.
constexpr int64_t kAutoLevelsVertices = int64_t(1) << 25;
// Cohort mode: graphs of at least this many vertices get cohorts, smaller
// ones (whose one-root searches are short) stream workspaces.
constexpr int64_t kCohortVertices = int64_t(1) << 21;
constexpr int kCohortWorkspaces = 2;  // batch workspaces per cohort graph
constexpr int kCohortPlain = 2;       // one-root workspaces per cohort graph
// Cohort policy (defaults; g5_server_cohort_policy changes them): a batched
// search of a few roots costs several one-root searches (at scale 26 one
// root alone takes 4x, 16 roots 13x, 64 roots 17x a one-root search), so a
// cohort starts once kCohortMin queries wait or the oldest has waited
// kCohortWaitMs; a query runs alone on a one-root workspace while fewer than
// kPlainMax wait and no cohort of its graph is running.  At 5000 queries/s
// over graphs of scales 20-26, full cohorts with a 30 ms deadline gave the
// lowest p99 (113 ms, against 125-156 ms for 8-32 roots or 5-20 ms).
constexpr int kCohortMinDefault = 64;
constexpr double kCohortWaitMsDefault = 30.0;
constexpr size_t kPlainMax = 4;

// One batch workspace of a cohort graph and the queries it runs.
struct Cohort {
    g5_batch *bt = nullptr;
    uint32_t *pred = nullptr;      // vertex-major [v][nroots]
    int cap = 0;                   // root slots
    int nroots = 0;                // roots of the running or finished cohort
    int state = 0;                 // 0 free, 1 running, 2 finished (results held)
    int held = 0;                  // finished queries whose results are not yet released
    std::vector<uint64_t> tickets; // ticket of each root
    std::vector<int64_t> roots;
};

struct Query {
    int graph = 0;
    int64_t root = 0;
    int slot = -1;
    int cohort = -1;  // cohort graphs: batch workspace index (slot = root index in it), or -1 for a
                      // one-root workspace (slot = its index)
    int state = 0;  // 0 queued, 1 running, 2 done, 3 released
    Clock::time_point t_submit, t_start, t_done;
};

}  // namespace

struct g5_server {
    std::vector<g5_graph *> graphs;
    int mode = G5_SERVE_STREAMS;
    std::vector<int> kind;                  // per graph: G5_SERVE_STREAMS or G5_SERVE_LEVELS
    std::vector<int> levels_graphs;         // graphs in the batch, in batch order
    std::vector<int> bidx;                  // per graph: index in the batch (-1 if none)
    std::vector<std::vector<g5_bfs *>> ws;  // streams mode: workspaces per graph
    std::vector<std::vector<Cohort>> cohorts;  // cohort graphs: batch workspaces
    std::vector<std::vector<uint64_t>> plain_query;  // cohort graphs: ticket per one-root workspace (0 free)
    int cohort_min = kCohortMinDefault;      // queued queries that start a cohort at once
    double cohort_wait_ms = kCohortWaitMsDefault;  // ... or the oldest query's wait that does
    uint32_t *col_buf = nullptr;          // one root's uint32 parents, gathered for a result
    std::vector<uint32_t> col_host;
    std::mutex result_mu;                 // guards col_buf / col_host
    cudaStream_t rstream = nullptr;       // result gathers
    g5_batch *bt = nullptr;
    uint32_t *pred = nullptr;             // parents of every slot (device)
    std::vector<uint64_t> pred_base;      // per graph
    std::vector<int> slots;               // per graph
    std::vector<std::vector<uint64_t>> slot_query;  // ticket per slot (0 free)
    std::vector<uint64_t> retire;         // per graph: slots to clear next step
    std::vector<std::deque<uint64_t>> queue;
    std::unordered_map<uint64_t, Query> queries;
    uint64_t next_ticket = 1;
    int keep_results = 1;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::thread worker, worker2, worker3; // stream-workspace, level-slot and cohort workers
    std::atomic<bool> stop{false};
    g5_status error = G5_OK;
    // statistics
    uint64_t steps = 0, completed = 0;
    double device_ms = 0;
};

namespace {

// Streams mode: every slot is a one-root search workspace with its own
// stream; launched searches run concurrently and are polled for completion.
void worker_streams(g5_server *sv)
{
    cudaSetDevice(sv->graphs[0]->device);
    const int ng = (int)sv->graphs.size();
    std::vector<std::vector<int>> running(ng);
    for (int g = 0; g < ng; ++g) running[g].assign(sv->kind[g] == G5_SERVE_STREAMS ? sv->slots[g] : 0, 0);
    int nrun = 0;
    while (!sv->stop.load()) {
        {
            std::unique_lock<std::mutex> lk(sv->mu);
            for (int g = 0; g < ng; ++g) {
                if (sv->kind[g] != G5_SERVE_STREAMS) continue;
                for (int s = 0; s < sv->slots[g] && !sv->queue[g].empty(); ++s) {
                    if (sv->slot_query[g][s] != 0) continue;
                    const uint64_t t = sv->queue[g].front();
                    sv->queue[g].pop_front();
                    Query &q = sv->queries[t];
                    q.slot = s;
                    q.state = 1;
                    q.t_start = Clock::now();
                    sv->slot_query[g][s] = t;
                    const g5_status st = g5_bfs_launch(sv->ws[g][s], q.root);
                    if (st != G5_OK) {
                        sv->error = st;
                        sv->stop.store(true);
                        sv->cv_done.notify_all();
                        return;
                    }
                    running[g][s] = 1;
                    ++nrun;
                }
            }
            if (nrun == 0) {
                sv->cv_work.wait_for(lk, std::chrono::milliseconds(2));
                continue;
            }
        }
        bool any_done = false;
        for (int g = 0; g < ng; ++g) {
            if (sv->kind[g] != G5_SERVE_STREAMS) continue;
            for (int s = 0; s < sv->slots[g]; ++s) {
                if (!running[g][s]) continue;
                int done = 0;
                double ms = 0;
                const g5_status st = g5_bfs_poll(sv->ws[g][s], &done, &ms);
                if (!done) continue;
                running[g][s] = 0;
                --nrun;
                any_done = true;
                std::lock_guard<std::mutex> lk(sv->mu);
                if (st != G5_OK) {
                    sv->error = st;
                    sv->stop.store(true);
                    sv->cv_done.notify_all();
                    return;
                }
                sv->steps += 1;
                sv->device_ms += ms;
                const uint64_t t = sv->slot_query[g][s];
                Query &q = sv->queries[t];
                q.state = 2;
                q.t_done = Clock::now();
                sv->completed += 1;
                if (!sv->keep_results) {
                    q.state = 3;
                    sv->slot_query[g][s] = 0;
                }
            }
        }
        if (any_done) {
            std::lock_guard<std::mutex> lk(sv->mu);
            sv->cv_done.notify_all();
        } else {
            std::this_thread::sleep_for(std::chrono::microseconds(20));
        }
    }
}

// Levels mode: every slot is a root bit of the graph's bit-sliced level
// loop, stepped one level at a time.
void worker_loop(g5_server *sv)
{
    cudaSetDevice(sv->graphs[0]->device);
    const std::vector<int> &lg = sv->levels_graphs;  // batch index -> graph
    const int nb = (int)lg.size();
    std::vector<int32_t> ag, as;
    std::vector<int64_t> ar;
    std::vector<uint64_t> active(nb, 0), retire(nb, 0), inflight(nb, 0);
    while (!sv->stop.load()) {
        ag.clear();
        as.clear();
        ar.clear();
        {
            std::unique_lock<std::mutex> lk(sv->mu);
            // admit queued queries into free slots (a slot retired in the last
            // step is cleared by this step before its new root starts)
            for (int i = 0; i < nb; ++i) {
                const int g = lg[i];
                for (int s = 0; s < sv->slots[g] && !sv->queue[g].empty(); ++s) {
                    if (sv->slot_query[g][s] != 0 || (sv->retire[g] >> s) & 1ull) continue;
                    const uint64_t t = sv->queue[g].front();
                    sv->queue[g].pop_front();
                    Query &q = sv->queries[t];
                    q.slot = s;
                    q.state = 1;
                    q.t_start = Clock::now();
                    sv->slot_query[g][s] = t;
                    ag.push_back(i);
                    as.push_back(s);
                    ar.push_back(q.root);
                    inflight[i] |= 1ull << s;
                }
                retire[i] = sv->retire[g];
                sv->retire[g] = 0;
            }
            bool any_inflight = false, any_retire = false;
            for (int i = 0; i < nb; ++i) {
                any_inflight |= inflight[i] != 0;
                any_retire |= retire[i] != 0;
            }
            if (!any_inflight && ag.empty() && !any_retire) {
                sv->cv_work.wait_for(lk, std::chrono::milliseconds(2));
                continue;
            }
        }
        double ms = 0;
        g5_status st = g5_batch_serve_step(sv->bt, ag.data(), as.data(), ar.data(), (int)ag.size(), retire.data(),
                                           active.data(), &ms);
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->steps += 1;
        sv->device_ms += ms;
        if (st != G5_OK) {
            sv->error = st;
            sv->stop.store(true);
            sv->cv_done.notify_all();
            return;
        }
        const Clock::time_point now = Clock::now();
        for (int i = 0; i < nb; ++i) {
            const int g = lg[i];
            const uint64_t fin = inflight[i] & ~active[i];
            if (!fin) continue;
            inflight[i] &= ~fin;
            for (int s = 0; s < sv->slots[g]; ++s) {
                if (!((fin >> s) & 1ull)) continue;
                const uint64_t t = sv->slot_query[g][s];
                Query &q = sv->queries[t];
                q.state = 2;
                q.t_done = now;
                sv->completed += 1;
                if (!sv->keep_results) {
                    // results are not kept: the slot is free at once
                    q.state = 3;
                    sv->slot_query[g][s] = 0;
                    sv->retire[g] |= 1ull << s;
                }
            }
        }
        sv->cv_done.notify_all();
    }
}

// Cohorts: when a batch workspace of a graph is free, the queries queued
// for that graph (up to its root slots) start together as one batched
// search; finished cohorts are polled and their queries completed.
void worker_cohorts(g5_server *sv)
{
    cudaSetDevice(sv->graphs[0]->device);
    const int ng = (int)sv->graphs.size();
    int nrun = 0;
    std::vector<std::vector<int>> plain_run(ng);
    for (int g = 0; g < ng; ++g) plain_run[g].assign(sv->plain_query[g].size(), 0);
    auto fail = [&](g5_status st) {
        sv->error = st;
        sv->stop.store(true);
        sv->cv_done.notify_all();
    };
    while (!sv->stop.load()) {
        {
            std::unique_lock<std::mutex> lk(sv->mu);
            for (int g = 0; g < ng; ++g) {
                if (sv->kind[g] != G5_SERVE_COHORTS) continue;
                // a short queue runs on one-root workspaces while no cohort
                // of the graph runs (a lone query finishes sooner alone than
                // as a batch); otherwise queries gather into cohorts
                bool cohort_running = false;
                for (const Cohort &c : sv->cohorts[g]) cohort_running |= c.state == 1;
                for (int s = 0; s < (int)sv->plain_query[g].size(); ++s) {
                    if (sv->queue[g].empty() || sv->queue[g].size() >= kPlainMax || cohort_running) break;
                    if (sv->plain_query[g][s] != 0) continue;
                    const uint64_t t = sv->queue[g].front();
                    sv->queue[g].pop_front();
                    Query &q = sv->queries[t];
                    q.cohort = -1;
                    q.slot = s;
                    q.state = 1;
                    q.t_start = Clock::now();
                    sv->plain_query[g][s] = t;
                    const g5_status st = g5_bfs_launch(sv->ws[g][s], q.root);
                    if (st != G5_OK) return fail(st);
                    plain_run[g][s] = 1;
                    ++nrun;
                }
                bool start = !sv->queue[g].empty();
                if (start && (int)sv->queue[g].size() < sv->cohort_min) {
                    // too few to share well: wait for more, up to the oldest's deadline
                    const Query &oldest = sv->queries[sv->queue[g].front()];
                    const double waited = std::chrono::duration<double, std::milli>(Clock::now() - oldest.t_submit).count();
                    start = waited >= sv->cohort_wait_ms;
                }
                for (int w = 0; w < (int)sv->cohorts[g].size() && start && !sv->queue[g].empty(); ++w) {
                    Cohort &c = sv->cohorts[g][w];
                    if (c.state != 0) continue;
                    c.tickets.clear();
                    c.roots.clear();
                    const Clock::time_point now = Clock::now();
                    while (!sv->queue[g].empty() && (int)c.tickets.size() < c.cap) {
                        const uint64_t t = sv->queue[g].front();
                        sv->queue[g].pop_front();
                        Query &q = sv->queries[t];
                        q.cohort = w;
                        q.slot = (int)c.tickets.size();
                        q.state = 1;
                        q.t_start = now;
                        c.tickets.push_back(t);
                        c.roots.push_back(q.root);
                    }
                    c.nroots = (int)c.tickets.size();
                    const g5_status st = g5_batch_launch(c.bt, c.roots.data(), &c.nroots, c.pred);
                    if (st != G5_OK) return fail(st);
                    c.state = 1;
                    ++nrun;
                }
            }
            if (nrun == 0) {
                sv->cv_work.wait_for(lk, std::chrono::milliseconds(2));
                continue;
            }
        }
        bool any_done = false;
        for (int g = 0; g < ng; ++g) {
            if (sv->kind[g] != G5_SERVE_COHORTS) continue;
            for (int s = 0; s < (int)plain_run[g].size(); ++s) {
                if (!plain_run[g][s]) continue;
                int done = 0;
                double ms = 0;
                const g5_status st = g5_bfs_poll(sv->ws[g][s], &done, &ms);
                if (!done) continue;
                plain_run[g][s] = 0;
                --nrun;
                any_done = true;
                std::lock_guard<std::mutex> lk(sv->mu);
                if (st != G5_OK) return fail(st);
                sv->steps += 1;
                sv->device_ms += ms;
                Query &q = sv->queries[sv->plain_query[g][s]];
                q.state = sv->keep_results ? 2 : 3;
                q.t_done = Clock::now();
                sv->completed += 1;
                if (!sv->keep_results) sv->plain_query[g][s] = 0;
            }
            for (Cohort &c : sv->cohorts[g]) {
                if (c.state != 1) continue;
                int done = 0;
                double ms = 0;
                const g5_status st = g5_batch_poll(c.bt, 0, &done, &ms);
                if (!done) continue;
                --nrun;
                any_done = true;
                std::lock_guard<std::mutex> lk(sv->mu);
                if (st != G5_OK) return fail(st);
                sv->steps += 1;
                sv->device_ms += ms;
                const Clock::time_point now = Clock::now();
                for (uint64_t t : c.tickets) {
                    Query &q = sv->queries[t];
                    q.state = sv->keep_results ? 2 : 3;
                    q.t_done = now;
                    sv->completed += 1;
                }
                // without kept results the workspace is free at once; with
                // them it is held until every query's result is released
                c.held = sv->keep_results ? c.nroots : 0;
                c.state = c.held ? 2 : 0;
            }
        }
        if (any_done) {
            std::lock_guard<std::mutex> lk(sv->mu);
            sv->cv_done.notify_all();
        } else {
            std::this_thread::sleep_for(std::chrono::microseconds(20));
        }
    }
}

}  // namespace

extern "C" {

g5_status g5_server_create_modes(g5_graph *const *graphs, int ngraphs, size_t mem_budget, int keep_results,
                                 const int *modes, g5_server **out)
{
    if (!graphs || ngraphs < 1 || ngraphs > 64 || !out || !modes) return G5_ERR_INVALID_ARG;
    *out = nullptr;
    for (int i = 0; i < ngraphs; ++i)
        if (!graphs[i] || (modes[i] != G5_SERVE_STREAMS && modes[i] != G5_SERVE_LEVELS && modes[i] != G5_SERVE_COHORTS))
            return G5_ERR_INVALID_ARG;
    g5_server *sv = new g5_server();
    sv->keep_results = keep_results ? 1 : 0;
    sv->mode = G5_SERVE_AUTO;
    for (int i = 0; i < ngraphs; ++i) {
        sv->graphs.push_back(graphs[i]);
        sv->kind.push_back(modes[i]);
    }
    auto fail = [&](g5_status st) {
        for (auto &v : sv->ws)
            for (g5_bfs *b : v) g5_bfs_destroy(b);
        for (auto &v : sv->cohorts)  // borrowers first: the first workspace owns the graph copy
            for (int w = (int)v.size() - 1; w >= 0; --w) {
                if (v[w].bt) g5_batch_destroy(v[w].bt);
                cudaFree(v[w].pred);
            }
        if (sv->bt) g5_batch_destroy(sv->bt);
        cudaFree(sv->pred);
        cudaFree(sv->col_buf);
        if (sv->rstream) cudaStreamDestroy(sv->rstream);
        delete sv;
        return st;
    };
    // memory-based admission from an equal share of the budget per graph:
    // one-root workspaces (their footprint estimated per vertex and edge), or
    // root slots of 4 bytes per vertex
    g5_bfs_config cfg;
    g5_bfs_config_default(&cfg);
    cfg.alpha = 40.0;
    cfg.beta = 200.0;
    const uint64_t share = mem_budget / (uint64_t)ngraphs;
    // cohort graphs get what the other graphs leave of the budget, in
    // proportion to their vertex counts (their parents take 4 bytes per
    // vertex and root slot)
    uint64_t cohort_n = 0, other_used = 0;
    for (int i = 0; i < ngraphs; ++i)
        if (sv->kind[i] == G5_SERVE_COHORTS) cohort_n += (uint64_t)graphs[i]->n;
    sv->ws.resize(ngraphs);
    sv->cohorts.resize(ngraphs);
    sv->plain_query.resize(ngraphs);
    sv->pred_base.assign(ngraphs, 0);
    sv->bidx.assign(ngraphs, -1);
    std::vector<g5_graph *> bgraphs;
    std::vector<int> bslots;
    uint64_t pb = 0;
    for (int i = 0; i < ngraphs; ++i) {
        const uint64_t n = (uint64_t)graphs[i]->n;
        uint64_t k;
        if (sv->kind[i] == G5_SERVE_COHORTS) {
            sv->slots.push_back(0);  // set below, once the other graphs' use is known
            sv->slot_query.emplace_back();
            continue;
        }
        if (sv->kind[i] == G5_SERVE_STREAMS) {
            const uint64_t per = 48ull * n + (uint64_t)graphs[i]->nnz / 64 + (1u << 20);
            k = std::min<uint64_t>(64, share / per);
            if (k == 0) return fail(G5_ERR_OOM);
            other_used += k * per;
            for (uint64_t j = 0; j < k; ++j) {
                g5_bfs *b = nullptr;
                const g5_status st = g5_bfs_create(graphs[i], &cfg, &b);
                if (st != G5_OK) return fail(st);
                sv->ws[i].push_back(b);
            }
        } else {
            k = std::min<uint64_t>(64, share / (4ull * n));
            if (k == 0) return fail(G5_ERR_OOM);
            other_used += k * 4ull * n;
            sv->bidx[i] = (int)bgraphs.size();
            sv->levels_graphs.push_back(i);
            bgraphs.push_back(graphs[i]);
            bslots.push_back((int)k);
            sv->pred_base[i] = pb;  // batch order: the layout g5_batch_serve_begin uses
            pb += k * n;
        }
        sv->slots.push_back((int)k);
        sv->slot_query.emplace_back(k, 0);
    }
    const uint64_t left = mem_budget > other_used ? mem_budget - other_used : 0;
    uint64_t col_n = 0;
    for (int i = 0; i < ngraphs; ++i) {
        if (sv->kind[i] == G5_SERVE_LEVELS) col_n = std::max<uint64_t>(col_n, (uint64_t)graphs[i]->n);
        if (sv->kind[i] != G5_SERVE_COHORTS) continue;
        const uint64_t n = (uint64_t)graphs[i]->n;
        col_n = std::max(col_n, n);
        const uint64_t gshare = (uint64_t)((double)left * (double)n / (double)cohort_n);
        const uint64_t per_plain = 48ull * n + (uint64_t)graphs[i]->nnz / 64 + (1u << 20);
        const uint64_t fixed = g5::batch_copy_bytes(graphs[i]) + kCohortPlain * per_plain;
        const uint64_t per_ws = g5::batch_workspace_bytes(graphs[i]);
        // as many workspaces (up to kCohortWorkspaces) as leave room for at
        // least 8 root slots each, and every workspace the slots that fit
        int nw = kCohortWorkspaces;
        uint64_t cap = 0;
        for (; nw >= 1; --nw) {
            const uint64_t need = fixed + (uint64_t)nw * per_ws;
            cap = gshare > need ? (gshare - need) / ((uint64_t)nw * 4ull * n) : 0;
            if (cap >= 8 || (nw == 1 && cap >= 1)) break;
        }
        if (nw < 1 || cap < 1) return fail(G5_ERR_OOM);
        cap = std::min<uint64_t>(64, cap);
        sv->slots[i] = (int)cap * nw;
        for (int p = 0; p < kCohortPlain; ++p) {
            g5_bfs *b = nullptr;
            const g5_status st = g5_bfs_create(graphs[i], &cfg, &b);
            if (st != G5_OK) return fail(st);
            sv->ws[i].push_back(b);
        }
        sv->plain_query[i].assign(kCohortPlain, 0);
        for (int w = 0; w < nw; ++w) {
            Cohort c;
            c.cap = (int)cap;
            const g5_status st = w == 0 ? g5_batch_create(&sv->graphs[i], 1, &c.bt)
                                        : g5::batch_create_sharing(sv->cohorts[i][0].bt, &c.bt);
            if (st == G5_OK && cudaMalloc(&c.pred, sizeof(uint32_t) * cap * n) != cudaSuccess) {
                cudaGetLastError();
                c.pred = nullptr;
                sv->cohorts[i].push_back(c);
                return fail(G5_ERR_OOM);
            }
            sv->cohorts[i].push_back(c);
            if (st != G5_OK) return fail(st);
        }
    }
    if (col_n) {
        if (cudaMalloc(&sv->col_buf, sizeof(uint32_t) * col_n) != cudaSuccess) {
            cudaGetLastError();
            sv->col_buf = nullptr;
            return fail(G5_ERR_OOM);
        }
        sv->col_host.resize(col_n);
    }
    if (cudaStreamCreateWithFlags(&sv->rstream, cudaStreamNonBlocking) != cudaSuccess) return fail(G5_ERR_CUDA);
    sv->retire.assign(ngraphs, 0);
    sv->queue.resize(ngraphs);
    if (!bgraphs.empty()) {
        if (cudaMalloc(&sv->pred, sizeof(uint32_t) * pb) != cudaSuccess) {
            cudaGetLastError();
            sv->pred = nullptr;
            return fail(G5_ERR_OOM);
        }
        g5_status st = g5_batch_create(bgraphs.data(), (int)bgraphs.size(), &sv->bt);
        if (st == G5_OK) st = g5_batch_serve_begin(sv->bt, sv->pred, bslots.data());
        if (st != G5_OK) return fail(st);
        sv->worker2 = std::thread(worker_loop, sv);
    }
    bool any_streams = false, any_cohorts = false;
    for (int i = 0; i < ngraphs; ++i) {
        any_streams |= sv->kind[i] == G5_SERVE_STREAMS;
        any_cohorts |= sv->kind[i] == G5_SERVE_COHORTS;
    }
    if (any_streams) sv->worker = std::thread(worker_streams, sv);
    if (any_cohorts) sv->worker3 = std::thread(worker_cohorts, sv);
    *out = sv;
    return G5_OK;
}

g5_status g5_server_create(g5_graph *const *graphs, int ngraphs, size_t mem_budget, int keep_results, int mode,
                           g5_server **out)
{
    if (!graphs || ngraphs < 1 || ngraphs > 64 || !out) return G5_ERR_INVALID_ARG;
    if (mode != G5_SERVE_STREAMS && mode != G5_SERVE_LEVELS && mode != G5_SERVE_AUTO && mode != G5_SERVE_COHORTS)
        return G5_ERR_INVALID_ARG;
    std::vector<int> modes(ngraphs, mode);
    for (int i = 0; i < ngraphs; ++i) {
        if (!graphs[i]) return G5_ERR_INVALID_ARG;
        if (mode == G5_SERVE_AUTO)
            modes[i] = graphs[i]->n >= kAutoLevelsVertices ? G5_SERVE_LEVELS : G5_SERVE_STREAMS;
        if (mode == G5_SERVE_COHORTS)
            modes[i] = graphs[i]->n >= kCohortVertices ? G5_SERVE_COHORTS : G5_SERVE_STREAMS;
    }
    g5_status st = g5_server_create_modes(graphs, ngraphs, mem_budget, keep_results, modes.data(), out);
    if (st == G5_OK) (*out)->mode = mode;
    return st;
}

g5_status g5_server_cohort_policy(g5_server *sv, int min_roots, double max_wait_ms)
{
    if (!sv || min_roots < 1 || min_roots > 64 || !(max_wait_ms >= 0)) return G5_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->cohort_min = min_roots;
    sv->cohort_wait_ms = max_wait_ms;
    sv->cv_work.notify_all();
    return G5_OK;
}

g5_status g5_server_slots(g5_server *sv, int *slots)
{
    if (!sv || !slots) return G5_ERR_INVALID_ARG;
    for (size_t i = 0; i < sv->slots.size(); ++i) slots[i] = sv->slots[i];
    return G5_OK;
}

g5_status g5_server_submit(g5_server *sv, int graph, int64_t root, uint64_t *ticket)
{
    if (!sv || !ticket || graph < 0 || graph >= (int)sv->graphs.size()) return G5_ERR_INVALID_ARG;
    if (root < 0 || root >= sv->graphs[graph]->n) return G5_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(sv->mu);
    if (sv->error != G5_OK) return sv->error;
    const uint64_t t = sv->next_ticket++;
    Query q;
    q.graph = graph;
    q.root = root;
    q.t_submit = Clock::now();
    sv->queries[t] = q;
    sv->queue[graph].push_back(t);
    *ticket = t;
    sv->cv_work.notify_all();
    return G5_OK;
}

g5_status g5_server_wait(g5_server *sv, uint64_t ticket, double timeout_s, int *done)
{
    if (!sv || !done) return G5_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->queries.find(ticket);
    if (it == sv->queries.end()) return G5_ERR_INVALID_ARG;
    const auto deadline = Clock::now() + std::chrono::duration<double>(timeout_s);
    while (sv->queries[ticket].state < 2 && sv->error == G5_OK) {
        if (sv->cv_done.wait_until(lk, deadline) == std::cv_status::timeout) break;
    }
    *done = sv->queries[ticket].state >= 2;
    return sv->error;
}

g5_status g5_server_result(g5_server *sv, uint64_t ticket, int64_t *pred_host, double *latency_ms,
                           double *queue_ms)
{
    // copies a finished query's parents (int64, -1 unvisited; may be NULL)
    // and frees its slot
    if (!sv) return G5_ERR_INVALID_ARG;
    cudaSetDevice(sv->graphs[0]->device);
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->queries.find(ticket);
    if (it == sv->queries.end() || it->second.state < 2) return G5_ERR_INVALID_ARG;
    Query q = it->second;
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(q.t_done - q.t_submit).count();
    if (queue_ms) *queue_ms = std::chrono::duration<double, std::milli>(q.t_start - q.t_submit).count();
    g5_status rc = G5_OK;
    const bool one_root = sv->kind[q.graph] == G5_SERVE_STREAMS ||
                          (sv->kind[q.graph] == G5_SERVE_COHORTS && q.cohort < 0);
    if (q.state == 2 && pred_host && one_root) {
        const int64_t n = sv->graphs[q.graph]->n;
        const int64_t *src = nullptr;
        g5_bfs_device_pred(sv->ws[q.graph][q.slot], &src);
        lk.unlock();
        if (cudaMemcpy(pred_host, src, sizeof(int64_t) * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = G5_ERR_CUDA;
        lk.lock();
    } else if (q.state == 2 && pred_host) {
        // a column of a vertex-major uint32 array (level slots or a cohort):
        // gathered into the server's column buffer, copied out and widened;
        // the slot is not reused before it is released below
        const int64_t n = sv->graphs[q.graph]->n;
        const uint32_t *src;
        int R;
        if (sv->kind[q.graph] == G5_SERVE_COHORTS) {
            const Cohort &c = sv->cohorts[q.graph][q.cohort];
            src = c.pred;
            R = c.nroots;
        } else {
            src = sv->pred + sv->pred_base[q.graph];
            R = sv->slots[q.graph];
        }
        lk.unlock();
        {
            std::lock_guard<std::mutex> rl(sv->result_mu);
            rc = g5_batch_root_parents(src, n, R, q.slot, sv->col_buf, sv->rstream);
            if (rc == G5_OK &&
                (cudaMemcpyAsync(sv->col_host.data(), sv->col_buf, sizeof(uint32_t) * (size_t)n,
                                 cudaMemcpyDeviceToHost, sv->rstream) != cudaSuccess ||
                 cudaStreamSynchronize(sv->rstream) != cudaSuccess))
                rc = G5_ERR_CUDA;
            if (rc == G5_OK)
                for (int64_t v = 0; v < n; ++v)
                    pred_host[v] = sv->col_host[v] == 0xFFFFFFFFu ? -1 : (int64_t)sv->col_host[v];
        }
        lk.lock();
    }
    if (rc != G5_OK) return rc;
    Query &qq = sv->queries[ticket];
    if (qq.state == 2) {
        if (sv->kind[qq.graph] == G5_SERVE_COHORTS && qq.cohort < 0) {
            sv->plain_query[qq.graph][qq.slot] = 0;
        } else if (sv->kind[qq.graph] == G5_SERVE_COHORTS) {
            Cohort &c = sv->cohorts[qq.graph][qq.cohort];
            if (c.held > 0 && --c.held == 0) c.state = 0;
        } else {
            sv->slot_query[qq.graph][qq.slot] = 0;
            if (sv->kind[qq.graph] == G5_SERVE_LEVELS) sv->retire[qq.graph] |= 1ull << qq.slot;
        }
        qq.state = 3;
        sv->cv_work.notify_all();
    }
    sv->queries.erase(ticket);
    return G5_OK;
}

g5_status g5_server_stats(g5_server *sv, uint64_t *steps, uint64_t *completed, double *device_ms)
{
    if (!sv) return G5_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(sv->mu);
    if (steps) *steps = sv->steps;
    if (completed) *completed = sv->completed;
    if (device_ms) *device_ms = sv->device_ms;
    return sv->error;
}

g5_status g5_server_destroy(g5_server *sv)
{
    if (!sv) return G5_ERR_INVALID_ARG;
    sv->stop.store(true);
    sv->cv_work.notify_all();
    if (sv->worker.joinable()) sv->worker.join();
    if (sv->worker2.joinable()) sv->worker2.join();
    if (sv->worker3.joinable()) sv->worker3.join();
    for (auto &v : sv->ws)
        for (g5_bfs *b : v) g5_bfs_destroy(b);
    for (auto &v : sv->cohorts)  // borrowers first: the first workspace owns the graph copy
        for (int w = (int)v.size() - 1; w >= 0; --w) {
            if (v[w].bt) g5_batch_destroy(v[w].bt);
            cudaFree(v[w].pred);
        }
    if (sv->bt) g5_batch_destroy(sv->bt);
    cudaFree(sv->pred);
    cudaFree(sv->col_buf);
    if (sv->rstream) cudaStreamDestroy(sv->rstream);
    delete sv;
    return G5_OK;
}

}  // extern "C"
