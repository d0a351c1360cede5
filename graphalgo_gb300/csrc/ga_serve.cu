// Request server: triangle-count, k-truss and BC queries on device-resident
// graphs, taken as they arrive by worker threads that each own a context
// (and so a stream); work of different workers overlaps on the device.
//
// Admission. Every request carries an upper bound on the device bytes its
// call allocates (request_bytes_bound). A worker starts the oldest queued
// request only while the bounds of the calls in flight plus its own fit in
// the server's HBM budget; a request whose bound alone exceeds the budget
// is refused with GA_ERR_ADMISSION.
//
// Continuous batching. When a worker takes a request on a small graph, it
// also takes the other queued requests of the same type on small graphs and
// runs them as one batched call over the block-diagonal union of their
// graphs: TC requests share a slot per graph, k-truss requests per (graph,
// k) with one k per graph, and every BC request has its own slot and
// sources. The batched calls give every request the result it gets alone.
#include "ga_internal.cuh"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>

namespace ga {

// ------------------------------------------------------------ byte bounds
// Upper bounds on the bytes one call allocates from its context, following
// the allocations of tc_device / ktruss_impl / bc_device (requested sizes;
// 1 MiB covers the scan scratch, flags and other small buffers).
static int64_t bound_tc(int64_t m, int64_t nnz, int64_t sval) {
    // lower triangle (<= nnz entries) + its unit copy + values + scratch
    return 64 * (m + 2) + nnz * (4 + sval + 8 + 4 + 16) + (1 << 20);
}

static int64_t bound_ktruss(int64_t m, int64_t nnz) {
    // copy of C, support, compaction, SpGEMM scratch, mirror index arrays
    return 32 * (m + 2) + 60 * (nnz + 1) + (1 << 20);
}

static int64_t bound_bc(int64_t m, int64_t nnz, int64_t ns) {
    const int64_t words = (ns + 31) / 32;
    // FP64 copy (and transpose), entry store, dense W, per-vertex state
    return 40 * (m + 1) * (ns + 1) + 4 * m * words + 80 * (m + 2) + 32 * nnz + (1 << 20);
}

// ns: the union's sources; ncols: the largest source count of one graph
// (batched BC keeps state for union vertices x ncols, plus one level-0
// entry and its column per source).
static int64_t bound_batch(int type, int64_t m, int64_t nnz, int64_t count, int64_t ns, int64_t ncols) {
    // union (int32 values), per-graph arrays, then the call on the union
    const int64_t u = 4 * (m + 1) + 8 * nnz + 64 * (count + 1) + 16 * (m + 2) + 4 * ns;
    return u + (type == GA_REQ_TC      ? bound_tc(m, nnz, 4)
                : type == GA_REQ_KTRUSS ? bound_ktruss(m, nnz)
                                        : bound_bc(m, nnz, ncols) + 48 * ns + 16 * (count + 1));
}

int64_t request_bytes_bound(int type, int64_t m, int64_t nnz, int64_t param) {
    switch (type) {
    case GA_REQ_TC: return bound_tc(m, nnz, 4);
    case GA_REQ_KTRUSS: return bound_ktruss(m, nnz);
    case GA_REQ_BC: return bound_bc(m, nnz, param);
    }
    return -1;
}

// ------------------------------------------------------------------ server
struct SrvGraph {
    ga_csr A = nullptr;
    int64_t m = 0, nnz = 0;
};

struct SrvReq {
    int64_t id = 0;
    int type = 0, graph = 0, k = 0, want_edges = 0;
    std::vector<int32_t> sources;
    int64_t bound = 0;
    bool done = false;
    ga_server_result res{};
    std::vector<int32_t> trst, tcol;
    std::vector<double> bc;
    std::string error;
};

constexpr size_t kMaxGraphs = 1 << 16;  // graph slots reserved up front (no reallocation under readers)

using Clock = std::chrono::steady_clock;

struct Server {
    int device = 0;
    ga_server_config cfg{};
    int64_t budget = 0;
    ga_ctx home = nullptr;
    std::vector<ga_ctx> wctx;
    std::vector<SrvGraph> graphs;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<SrvReq*> queue;
    std::unordered_map<int64_t, std::unique_ptr<SrvReq>> reqs;
    int64_t next_id = 1;
    int64_t reserved = 0;
    int in_flight = 0;
    bool stop = false;
    ga_server_stats st{};
    std::vector<std::thread> threads;
    Clock::time_point t0;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

static bool coalescible(const Server* s, const SrvReq* r) {
    return s->cfg.coalesce && s->graphs[(size_t)r->graph].nnz <= s->cfg.coalesce_nnz;
}

// One slot of a batched call: a graph copy in the union and the requests it
// serves. TC requests share a slot per graph, k-truss requests per (graph,
// k); every BC request has its own slot (its own sources).
static int64_t slot_key(const SrvReq* r) {
    if (r->type == GA_REQ_TC) return r->graph;
    if (r->type == GA_REQ_KTRUSS) return ((int64_t)r->graph << 20) | (int64_t)(r->k & 0xfffff);
    return -r->id;
}

// Batched BC keeps state per (union vertex, source column), a column being
// the j-th source of every graph: union vertices x (largest source count +
// 1) + sources at most cfg.bc_group_pairs.
constexpr int64_t kBcMaxSrc = 1024;                   // sources of one BC request

// Picks the calls to run next (under the lock): the queue head and, when it
// can be batched, the requests of the same type behind it. Returns the group
// and its byte reservation; an empty group means nothing can start now.
static std::vector<SrvReq*> take_group(Server* s, int64_t* reserve) {
    std::vector<SrvReq*> group;
    while (!s->queue.empty()) {
        SrvReq* head = s->queue.front();
        if (head->bound > s->budget) {  // can never run: refuse
            s->queue.pop_front();
            head->res.status = GA_ERR_ADMISSION;
            head->res.t_start = head->res.t_end = s->now();
            head->done = true;
            s->st.rejected += 1;
            s->cv_done.notify_all();
            continue;
        }
        if (s->reserved + head->bound > s->budget) return group;  // wait for memory
        group.push_back(head);
        *reserve = head->bound;
        s->queue.pop_front();
        if (!coalescible(s, head)) return group;
        // gather same-type requests on small graphs, keeping queue order for the rest
        std::unordered_map<int64_t, int> slots{{slot_key(head), 0}};
        const SrvGraph& hg = s->graphs[(size_t)head->graph];
        int64_t um = hg.m, unz = hg.nnz, ns = (int64_t)head->sources.size(), nslots = 1;
        int64_t ncols = ns;
        for (auto it = s->queue.begin(); it != s->queue.end() && (int64_t)group.size() < s->cfg.coalesce_max_requests;) {
            SrvReq* r = *it;
            if (r->type != head->type || !coalescible(s, r)) { ++it; continue; }
            const bool fresh = slots.find(slot_key(r)) == slots.end();
            const SrvGraph& g = s->graphs[(size_t)r->graph];
            const int64_t m2 = um + (fresh ? g.m : 0), z2 = unz + (fresh ? g.nnz : 0);
            const int64_t ns2 = ns + (int64_t)r->sources.size();
            const int64_t nc2 = std::max<int64_t>(ncols, (int64_t)r->sources.size());
            if (z2 > s->cfg.coalesce_max_nnz) { ++it; continue; }
            if (r->type == GA_REQ_BC && (nc2 > kBcMaxSrc || m2 * (nc2 + 1) + ns2 > s->cfg.bc_group_pairs)) {
                ++it;
                continue;
            }
            const int64_t b2 = bound_batch(head->type, m2, z2, nslots + (fresh ? 1 : 0), ns2, nc2);
            if (s->reserved + b2 > s->budget) { ++it; continue; }
            if (fresh) slots[slot_key(r)] = (int)nslots++;
            um = m2; unz = z2; ns = ns2; ncols = nc2;
            *reserve = b2;
            group.push_back(r);
            it = s->queue.erase(it);
        }
        if (group.size() > 1) *reserve = std::max(*reserve, bound_batch(head->type, um, unz, nslots, ns, ncols));
        return group;
    }
    return group;
}

static void fill_error(SrvReq* r, int rc, ga_ctx ctx) {
    r->res.status = rc;
    if (rc != GA_OK) r->error = ga_last_error(ctx);
}

static void run_single(Server* s, ga_ctx ctx, SrvReq* r) {
    const SrvGraph& g = s->graphs[(size_t)r->graph];
    int rc = GA_OK;
    if (r->type == GA_REQ_TC) {
        int64_t total = 0;
        rc = ga_tc(ctx, (ga_algo)s->cfg.tc_algo, g.A, &total, nullptr);
        r->res.tc_total = total;
    } else if (r->type == GA_REQ_KTRUSS) {
        ga_csr C = nullptr;
        int iters = 0;
        rc = ga_ktruss(ctx, (ga_algo)s->cfg.ktruss_algo, g.A, r->k, &C, &iters);
        if (rc == GA_OK) {
            r->res.iters = iters;
            r->res.truss_nnz = C->nnz;
            if (r->want_edges) {
                r->trst.resize((size_t)C->m + 1);
                r->tcol.resize((size_t)std::max<int64_t>(C->nnz, 1));
                rc = ga_csr_download(ctx, C, r->trst.data(), r->tcol.data(), nullptr);
            }
            ga_csr_free(ctx, C);
        }
    } else {
        r->bc.assign((size_t)std::max<int64_t>(g.m, 1), 0.0);
        rc = ga_bc(ctx, g.A, r->sources.data(), (int64_t)r->sources.size(), r->bc.data());
    }
    fill_error(r, rc, ctx);
}

// Batched calls run on unions whose sizes change from call to call: with
// GA_AUTO they use MSA rather than tune each new union.
// Batched calls under GA_AUTO use triangle listing (unions of symmetric 0/1
// graphs; other matrices fall back inside the call).
static ga_algo group_algo(int a) { return a == GA_AUTO ? GA_TRI : (ga_algo)a; }

static void run_group(Server* s, ga_ctx ctx, std::vector<SrvReq*>& group) {
    // slots of the union, in first-seen order
    std::vector<int64_t> order;
    std::vector<SrvReq*> first;
    std::unordered_map<int64_t, int> slot;
    for (SrvReq* r : group)
        if (slot.emplace(slot_key(r), (int)order.size()).second) {
            order.push_back(slot_key(r));
            first.push_back(r);
        }
    std::vector<ga_csr> parts;
    for (SrvReq* r : first) parts.push_back(s->graphs[(size_t)r->graph].A);
    const int64_t count = (int64_t)parts.size();
    std::vector<int64_t> voff((size_t)count + 1);
    ga_csr U = nullptr;
    int rc = ga_csr_block_diag(ctx, count, parts.data(), &U, voff.data());
    const int type = group[0]->type;
    if (rc == GA_OK && type == GA_REQ_TC) {
        std::vector<int64_t> totals((size_t)count);
        rc = ga_batch_tc(ctx, group_algo(s->cfg.tc_algo), U, count, voff.data(), totals.data());
        if (rc == GA_OK)
            for (SrvReq* r : group) r->res.tc_total = totals[(size_t)slot[slot_key(r)]];
    } else if (rc == GA_OK && type == GA_REQ_KTRUSS) {
        ga_csr C = nullptr;
        std::vector<int> iters((size_t)count), ks((size_t)count);
        for (int64_t g = 0; g < count; ++g) ks[(size_t)g] = first[(size_t)g]->k;
        rc = ga_batch_ktruss_k(ctx, group_algo(s->cfg.ktruss_algo), U, count, voff.data(), ks.data(), &C,
                               iters.data());
        if (rc == GA_OK) {
            bool edges = false;
            for (SrvReq* r : group) edges = edges || r->want_edges;
            std::vector<int32_t> crst((size_t)C->m + 1), ccol;
            if (edges) ccol.resize((size_t)std::max<int64_t>(C->nnz, 1));
            rc = ga_csr_download(ctx, C, crst.data(), edges ? ccol.data() : nullptr, nullptr);
            if (rc == GA_OK) {
                for (SrvReq* r : group) {
                    const int g = slot[slot_key(r)];
                    const int64_t b = voff[(size_t)g], e = voff[(size_t)g + 1];
                    r->res.iters = iters[(size_t)g];
                    r->res.truss_nnz = crst[(size_t)e] - crst[(size_t)b];
                    if (r->want_edges) {
                        r->trst.resize((size_t)(e - b + 1));
                        for (int64_t i = b; i <= e; ++i) r->trst[(size_t)(i - b)] = crst[(size_t)i] - crst[(size_t)b];
                        r->tcol.resize((size_t)std::max<int64_t>(r->res.truss_nnz, 1));
                        for (int64_t q = crst[(size_t)b]; q < crst[(size_t)e]; ++q)
                            r->tcol[(size_t)(q - crst[(size_t)b])] = ccol[(size_t)q] - (int32_t)b;
                    }
                }
            }
            ga_csr_free(ctx, C);
        }
    } else if (rc == GA_OK) {  // BC: every request its own slot and sources
        std::vector<int64_t> soff((size_t)count + 1, 0);
        std::vector<int32_t> src;
        for (int64_t g = 0; g < count; ++g) {
            const auto& sv = first[(size_t)g]->sources;
            src.insert(src.end(), sv.begin(), sv.end());
            soff[(size_t)g + 1] = (int64_t)src.size();
        }
        std::vector<double> bc((size_t)std::max<int64_t>(U->m, 1));
        rc = ga_batch_bc(ctx, U, count, voff.data(), soff.data(), src.data(), bc.data());
        if (rc == GA_OK)
            for (SrvReq* r : group) {
                const int g = slot[slot_key(r)];
                r->bc.assign(bc.begin() + voff[(size_t)g], bc.begin() + voff[(size_t)g + 1]);
                if (r->bc.empty()) r->bc.assign(1, 0.0);
            }
    }
    if (U) ga_csr_free(ctx, U);
    for (SrvReq* r : group) fill_error(r, rc, ctx);
}

static void worker_main(Server* s, int w) {
    cudaSetDevice(s->device);
    ga_ctx ctx = s->wctx[(size_t)w];
    for (;;) {
        std::vector<SrvReq*> group;
        int64_t reserve = 0;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            for (;;) {
                group = take_group(s, &reserve);
                if (!group.empty()) break;
                if (s->stop && s->queue.empty()) return;
                s->cv_work.wait(lk);
            }
            s->reserved += reserve;
            s->st.peak_reserved = std::max(s->st.peak_reserved, s->reserved);
            s->in_flight += 1;
            s->st.max_in_flight = std::max<int64_t>(s->st.max_in_flight, s->in_flight);
            s->st.calls += 1;
            if (group.size() > 1) {
                s->st.batched_calls += 1;
                s->st.batched_requests += (int64_t)group.size();
            }
            s->st.max_group = std::max<int64_t>(s->st.max_group, (int64_t)group.size());
            const double t = s->now();
            for (SrvReq* r : group) {
                r->res.t_start = t;
                r->res.batch_size = (int)group.size();
                r->res.worker = w;
            }
        }
        if (group.size() == 1) run_single(s, ctx, group[0]);
        else run_group(s, ctx, group);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            const double t = s->now();
            for (SrvReq* r : group) {
                r->res.t_end = t;
                r->done = true;
                if (r->res.status == GA_OK) s->st.completed += 1;
                else s->st.failed += 1;
            }
            s->reserved -= reserve;
            s->in_flight -= 1;
        }
        s->cv_done.notify_all();
        s->cv_work.notify_all();
    }
}

}  // namespace ga

struct ga_server_s : ga::Server {};

using namespace ga;

extern "C" {

int ga_request_bytes_bound(int type, int64_t m, int64_t nnz, int64_t param, int64_t* bytes) {
    if (!bytes || m < 0 || nnz < 0 || param < 0) return GA_ERR_INVALID_ARG;
    const int64_t b = request_bytes_bound(type, m, nnz, param);
    if (b < 0) return GA_ERR_INVALID_ARG;
    *bytes = b;
    return GA_OK;
}

int ga_server_create(int device, const ga_server_config* cfg, ga_server* out) {
    if (!out) return GA_ERR_INVALID_ARG;
    *out = nullptr;
    std::unique_ptr<ga_server_s> s(new (std::nothrow) ga_server_s());
    if (!s) return GA_ERR_OOM;
    s->device = device;
    ga_server_config c{};
    if (cfg) c = *cfg;
    if (c.workers <= 0) c.workers = 4;
    if (c.coalesce_nnz <= 0) c.coalesce_nnz = 1 << 20;
    if (c.coalesce_max_nnz <= 0) c.coalesce_max_nnz = 1 << 22;
    if (c.coalesce_max_requests <= 0) c.coalesce_max_requests = 4096;
    if (c.bc_group_pairs <= 0) c.bc_group_pairs = (int64_t)1 << 25;
    if (c.workers > 64) return GA_ERR_INVALID_ARG;
    s->cfg = c;
    int rc = ga_ctx_create(device, nullptr, &s->home);
    if (rc != GA_OK) return rc;
    s->graphs.reserve(kMaxGraphs);
    for (int w = 0; w < c.workers; ++w) {
        ga_ctx x = nullptr;
        rc = ga_ctx_create(device, nullptr, &x);
        if (rc != GA_OK) {
            for (ga_ctx y : s->wctx) ga_ctx_destroy(y);
            ga_ctx_destroy(s->home);
            return rc;
        }
        s->wctx.push_back(x);
    }
    int64_t f = 0, t = 0;
    ga_mem_info(s->home, &f, &t);
    s->budget = c.hbm_budget > 0 ? c.hbm_budget : (int64_t)(0.8 * (double)f);
    s->st.budget = s->budget;
    s->t0 = Clock::now();
    ga_server_s* raw = s.get();
    for (int w = 0; w < c.workers; ++w) raw->threads.emplace_back(worker_main, raw, w);
    *out = s.release();
    return GA_OK;
}

// Registers A (owned by the home context from now on); the caller holds
// srv->mu. Frees A when it is refused.
static int add_resident(ga_server srv, ga_csr A, int* graph_id) {
    const int64_t m = A->m, nnz = A->nnz;
    try {
        GA_REQUIRE(A->dtype == GA_INT32 && A->m == A->n, GA_ERR_INVALID_ARG,
                   "server graphs must be square int32 adjacency matrices");
        // settle the cached flags now: workers only read them afterwards
        csr_unit_values(srv->home, A);
        csr_is_symmetric(srv->home, A);
        GA_REQUIRE(A->sym == 1, GA_ERR_INVALID_ARG, "server graphs must be symmetric adjacency matrices");
    } catch (const Error& e) {
        srv->home->last_error = e.msg;
        ga_csr_free(srv->home, A);
        return e.code;
    }
    SrvGraph g;
    g.A = A;
    g.m = m;
    g.nnz = nnz;
    srv->graphs.push_back(g);
    srv->budget -= 4 * (m + 1) + 8 * nnz;  // the resident graph comes out of the budget
    srv->st.budget = srv->budget;
    *graph_id = (int)srv->graphs.size() - 1;
    return GA_OK;
}

int ga_server_add_graph(ga_server srv, int64_t m, const int32_t* rst, const int32_t* col, int* graph_id) {
    if (!srv || !graph_id || m < 0 || !rst) return GA_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(srv->mu);
    if (srv->graphs.size() >= kMaxGraphs) return GA_ERR_UNSUPPORTED;
    ga_csr A = nullptr;
    int rc = ga_csr_upload(srv->home, m, m, rst[m], rst, col, nullptr, GA_INT32, &A);
    if (rc != GA_OK) return rc;
    return add_resident(srv, A, graph_id);
}

int ga_server_add_graph_device(ga_server srv, ga_ctx ctx, ga_csr A, int* graph_id) {
    if (!srv || !ctx || !A || !graph_id || ctx->device != srv->device) return GA_ERR_INVALID_ARG;
    int rc = ga_ctx_sync(ctx);  // A complete before the home stream copies it
    if (rc != GA_OK) return rc;
    std::lock_guard<std::mutex> lk(srv->mu);
    if (srv->graphs.size() >= kMaxGraphs) return GA_ERR_UNSUPPORTED;
    ga_csr C = nullptr;
    rc = ga_csr_from_device(srv->home, A->m, A->n, A->nnz, A->rst, A->col, A->val, A->dtype, &C);
    if (rc != GA_OK) return rc;
    return add_resident(srv, C, graph_id);
}

int ga_server_add_graph_file(ga_server srv, const char* path, int* graph_id) {
    if (!srv || !path || !graph_id) return GA_ERR_INVALID_ARG;
    const size_t len = strlen(path);
    const bool mtx = len > 4 && strcmp(path + len - 4, ".mtx") == 0;
    const bool bin = len > 4 && strcmp(path + len - 4, ".bin") == 0;
    if (!mtx && !bin) return GA_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lk(srv->mu);
    if (srv->graphs.size() >= kMaxGraphs) return GA_ERR_UNSUPPORTED;
    ga_csr A = nullptr;
    // the reference CLI's preparation for TC and k-truss: adjacency, lower-triangle symmetrisation
    const int flags = GA_EDGES_LOWER_SYMM | GA_EDGES_UNIT;
    int rc = mtx ? ga_read_mtx(srv->home, path, flags, nullptr, &A) : ga_read_bin(srv->home, path, flags, nullptr, &A);
    if (rc != GA_OK) return rc;
    return add_resident(srv, A, graph_id);
}

int ga_server_graph_info(ga_server srv, int graph, int64_t* m, int64_t* nnz) {
    if (!srv) return GA_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(srv->mu);
    if (graph < 0 || graph >= (int)srv->graphs.size()) return GA_ERR_INVALID_ARG;
    const SrvGraph& g = srv->graphs[(size_t)graph];
    if (m) *m = g.m;
    if (nnz) *nnz = g.nnz;
    return GA_OK;
}

int ga_server_submit(ga_server srv, int type, int graph, int k, const int32_t* sources, int nsrc, int want_edges,
                     int64_t* req_id) {
    if (!srv || !req_id) return GA_ERR_INVALID_ARG;
    std::unique_ptr<SrvReq> r(new SrvReq());
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        if (srv->stop) return GA_ERR_INVALID_ARG;
        if (graph < 0 || graph >= (int)srv->graphs.size()) return GA_ERR_INVALID_ARG;
        if (type != GA_REQ_TC && type != GA_REQ_KTRUSS && type != GA_REQ_BC) return GA_ERR_INVALID_ARG;
        if (type == GA_REQ_BC && (nsrc < 0 || (nsrc > 0 && !sources))) return GA_ERR_INVALID_ARG;
        const SrvGraph& g = srv->graphs[(size_t)graph];
        r->id = srv->next_id++;
        r->type = type;
        r->graph = graph;
        r->k = k;
        r->want_edges = want_edges;
        if (type == GA_REQ_BC) r->sources.assign(sources, sources + nsrc);
        r->bound = request_bytes_bound(type, g.m, g.nnz, nsrc);
        r->res.type = type;
        r->res.graph = graph;
        r->res.bytes_bound = r->bound;
        r->res.status = -1;
        r->res.t_submit = srv->now();
        *req_id = r->id;
        srv->queue.push_back(r.get());
        srv->reqs.emplace(r->id, std::move(r));
        srv->st.submitted += 1;
    }
    srv->cv_work.notify_one();
    return GA_OK;
}

int ga_server_wait(ga_server srv, int64_t req_id, double timeout_s, ga_server_result* res) {
    if (!srv) return GA_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(req_id);
    if (it == srv->reqs.end()) return GA_ERR_INVALID_ARG;
    SrvReq* r = it->second.get();
    const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                              std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 1e9));
    while (!r->done) {
        if (srv->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !r->done) return GA_ERR_TIMEOUT;
    }
    if (res) {
        *res = r->res;
        res->truss_rst = r->trst.empty() ? nullptr : r->trst.data();
        res->truss_col = r->tcol.empty() ? nullptr : r->tcol.data();
        res->bc = r->bc.empty() ? nullptr : r->bc.data();
        res->error = r->error.empty() ? nullptr : r->error.c_str();
    }
    return GA_OK;
}

int ga_server_cancel(ga_server srv, int64_t req_id) {
    if (!srv) return GA_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(req_id);
    if (it == srv->reqs.end()) return GA_ERR_INVALID_ARG;
    SrvReq* r = it->second.get();
    auto q = std::find(srv->queue.begin(), srv->queue.end(), r);
    if (q == srv->queue.end()) return GA_ERR_UNSUPPORTED;  // started or done: it runs to completion
    srv->queue.erase(q);
    r->res.status = GA_ERR_CANCELLED;
    r->res.t_start = r->res.t_end = srv->now();
    r->error = "cancelled before it started";
    r->done = true;
    srv->st.cancelled += 1;
    srv->cv_done.notify_all();
    return GA_OK;
}

int ga_server_release(ga_server srv, int64_t req_id) {
    if (!srv) return GA_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(req_id);
    if (it == srv->reqs.end() || !it->second->done) return GA_ERR_INVALID_ARG;
    srv->reqs.erase(it);
    return GA_OK;
}

int ga_server_drain(ga_server srv, double timeout_s) {
    if (!srv) return GA_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(srv->mu);
    const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                              std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 1e9));
    while (!srv->queue.empty() || srv->in_flight > 0) {
        if (srv->cv_done.wait_until(lk, deadline) == std::cv_status::timeout &&
            (!srv->queue.empty() || srv->in_flight > 0))
            return GA_ERR_TIMEOUT;
    }
    return GA_OK;
}

int ga_server_get_stats(ga_server srv, ga_server_stats* out) {
    if (!srv || !out) return GA_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(srv->mu);
    *out = srv->st;
    out->reserved = srv->reserved;
    out->queued = (int64_t)srv->queue.size();
    return GA_OK;
}

int ga_server_destroy(ga_server srv) {
    if (!srv) return GA_ERR_INVALID_ARG;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->stop = true;
    }
    srv->cv_work.notify_all();
    for (auto& t : srv->threads) t.join();
    for (auto& g : srv->graphs) ga_csr_free(srv->home, g.A);
    for (ga_ctx x : srv->wctx) ga_ctx_destroy(x);
    ga_ctx_destroy(srv->home);
    delete srv;
    return GA_OK;
}

}  // extern "C"
