// Serving runtime: continuous batching of PPR / RWR queries (no reference
// counterpart; the reference runs one query per process).
//
// State that stays resident between ticks:
//   - the graph (owned by the ptw_graph handle);
//   - a device arena of count-table slots, carved by a buddy allocator into
//     power-of-two tables, one per active query (admission by device memory);
//   - a device plan block (the tick's query table) and its pinned host mirror.
// A tick gives every active query a share of the tick's walkers (its walker
// ranks j0 .. j0+share-1) and runs them all in one k_batch launch; walkers
// finish within the tick, so a query is done once all its ranks have run.
// Draws depend on (query id, rank) only: a query's counts are the same
// however its ranks are split across ticks and whatever runs beside it.
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <deque>
#include <string>
#include <map>
#include <vector>

#include "batch_kernels.cuh"

namespace ptw {
namespace {

// Buddy allocator over [0, 2^max_order) slots, minimum block 2^min_order.
class Buddy {
public:
    void init(uint64_t total_slots, int min_order)
    {
        min_order_ = min_order;
        max_order_ = min_order;
        while ((2ull << max_order_) <= total_slots) ++max_order_;
        if ((1ull << max_order_) > total_slots) max_order_ = -1;  // arena smaller than one block
        free_.assign(64, {});
        if (max_order_ >= min_order_) free_[max_order_].push_back(0);
    }
    bool alloc(uint64_t slots, uint64_t *off)
    {
        int o = min_order_;
        while ((1ull << o) < slots) ++o;
        if (max_order_ < 0 || o > max_order_) return false;
        int k = o;
        while (k <= max_order_ && free_[k].empty()) ++k;
        if (k > max_order_) return false;
        uint64_t b = free_[k].back();
        free_[k].pop_back();
        while (k > o) {
            --k;
            free_[k].push_back(b + (1ull << k));  // upper half stays free
        }
        *off = b;
        used_[b] = o;
        return true;
    }
    void release(uint64_t off)
    {
        auto it = used_.find(off);
        if (it == used_.end()) return;
        int o = it->second;
        used_.erase(it);
        uint64_t b = off;
        while (o < max_order_) {
            const uint64_t buddy = b ^ (1ull << o);
            auto &fl = free_[o];
            auto f = std::find(fl.begin(), fl.end(), buddy);
            if (f == fl.end()) break;
            fl.erase(f);
            b = std::min(b, buddy);
            ++o;
        }
        free_[o].push_back(b);
    }
    uint64_t capacity() const { return max_order_ < 0 ? 0 : 1ull << max_order_; }

private:
    int min_order_ = 8, max_order_ = -1;
    std::vector<std::vector<uint64_t>> free_;
    std::map<uint64_t, int> used_;
};

struct Pending {
    ptw_query q;
    uint32_t src;  // internal id
    double submit_s;
    bool full;     // re-run with a table that cannot fill
};

struct Active {
    Pending p;
    uint64_t cap, off;  // table slots, arena offset
    bool dense;         // dense array of n counters instead of a hash table
    uint64_t started;   // ranks run so far
    double admit_s;
};

// Pinned host memory that completed results are copied into by the device;
// a block is reused once no pending result refers to it.
struct PinnedBlock {
    uint32_t *p = nullptr;
    uint64_t words = 0;
    ~PinnedBlock()
    {
        if (p) cudaFreeHost(p);
    }
};

struct Done {
    ptw_serve_result r;
    std::shared_ptr<PinnedBlock> blk;  // keeps names / counts alive
    const uint32_t *names = nullptr, *counts = nullptr;
};

}  // namespace
}  // namespace ptw

struct ptw_server {
    ptw_graph *g = nullptr;
    ptw_serve_cfg cfg{};
    uint64_t thr = 0;
    std::chrono::steady_clock::time_point t0;
    ptw::Buddy buddy;
    unsigned long long *arena = nullptr;
    uint32_t S = 0;                  // plan capacity (max_active)
    uint32_t D = 0;                  // descriptor capacity per tick
    std::vector<uint64_t> take;      // walker ranks given to each active query this tick
    void *d_plan = nullptr, *h_plan = nullptr;
    size_t plan_bytes = 0, ret_off = 0, ret_bytes = 0;
    std::deque<ptw::Pending> pending;
    std::vector<ptw::Active> active;
    std::deque<ptw::Done> done;
    ptw::BatchArgs args{};
    unsigned grid = 1;
    const void *kfn = nullptr;        // k_batch<false> or k_batch<true> (extended columns)
    bool uses_ext = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t knode = nullptr;
    cudaKernelNodeParams kparams{};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    std::vector<std::shared_ptr<ptw::PinnedBlock>> pinned;  // result staging pool
    ptw_serve_stats st{};
};

namespace ptw {
namespace {

double now_s(const ptw_server *s)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - s->t0).count();
}

// Plan block layout (identical on host and device), S query slots and D
// walker descriptors:
//   tab[S] u64 | src[S] u32 | qid[S] u32 | mask[S] u32 | desc[D] uint3 |
//   flag[S] u32 | (pad to 16) ctrl[2] u64
// The tail from flag on is what a tick copies back.
struct PlanView {
    unsigned long long *tab, *ctrl;
    uint32_t *src, *qid, *mask, *flag;
    uint3 *desc;
};

PlanView view(void *base, uint32_t S, uint32_t D)
{
    PlanView v;
    char *p = (char *)base;
    v.tab = (unsigned long long *)p;
    p += 8ull * S;
    v.src = (uint32_t *)p;
    p += 4ull * S;
    v.qid = (uint32_t *)p;
    p += 4ull * S;
    v.mask = (uint32_t *)p;
    p += 4ull * S;
    v.desc = (uint3 *)p;
    p += sizeof(uint3) * (size_t)D;
    v.flag = (uint32_t *)p;
    p += 4ull * S;
    p = (char *)(((uintptr_t)p + 15) & ~(uintptr_t)15);
    v.ctrl = (unsigned long long *)p;
    return v;
}

size_t plan_size(uint32_t S, uint32_t D)
{
    size_t b = 20ull * S + sizeof(uint3) * (size_t)D + 4ull * S;
    return ((b + 15) & ~(size_t)15) + 16;
}

int build_tick_graph(ptw_server *s)
{
    cudaStream_t st = s->g->stream;
    PTW_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    cudaError_t e1 = cudaMemcpyAsync(s->d_plan, s->h_plan, s->plan_bytes, cudaMemcpyHostToDevice, st);
    void *kargs[] = {&s->args};
    cudaError_t e2 = cudaLaunchKernel(s->kfn, dim3(s->grid), dim3(256), kargs, 0, st);
    cudaError_t e3 = cudaMemcpyAsync((char *)s->h_plan + s->ret_off, (char *)s->d_plan + s->ret_off,
                                     s->ret_bytes, cudaMemcpyDeviceToHost, st);
    cudaError_t e4 = cudaStreamEndCapture(st, &s->graph);
    if (e1 != cudaSuccess) return cuda_fail(e1, "tick graph copy-in");
    if (e2 != cudaSuccess) return cuda_fail(e2, "tick graph kernel");
    if (e3 != cudaSuccess) return cuda_fail(e3, "tick graph copy-out");
    if (e4 != cudaSuccess) return cuda_fail(e4, "cudaStreamEndCapture");
    size_t nn = 0;
    PTW_CUDA(cudaGraphGetNodes(s->graph, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    PTW_CUDA(cudaGraphGetNodes(s->graph, nodes.data(), &nn));
    for (auto nd : nodes) {
        cudaGraphNodeType t;
        PTW_CUDA(cudaGraphNodeGetType(nd, &t));
        if (t == cudaGraphNodeTypeKernel) s->knode = nd;
    }
    if (!s->knode) return fail(PTW_ECUDA, "tick graph has no kernel node");
    PTW_CUDA(cudaGraphKernelNodeGetParams(s->knode, &s->kparams));
    PTW_CUDA(cudaGraphInstantiate(&s->exec, s->graph, 0));
    return PTW_OK;
}

// A free pinned block of at least `words` words: reuses one that no pending
// result refers to, else allocates (blocks grow geometrically).
std::shared_ptr<PinnedBlock> pinned_block(ptw_server *s, uint64_t words)
{
    std::shared_ptr<PinnedBlock> *spare = nullptr;
    for (auto &b : s->pinned) {
        if (b.use_count() != 1) continue;
        if (b->words >= words) return b;
        spare = &b;  // free but too small: replace it
    }
    auto nb = std::make_shared<PinnedBlock>();
    uint64_t w = std::max<uint64_t>(words, 1ull << 23);
    if (spare) w = std::max(w, 2 * (*spare)->words);
    if (cudaMallocHost(&nb->p, w * 4) != cudaSuccess) {
        nb->p = nullptr;
        return nullptr;
    }
    nb->words = w;
    if (spare) *spare = nb;
    else s->pinned.push_back(nb);
    return nb;
}

// Turns the tables of finished queries (indices into s->active) into results
// and releases the tables; the caller removes them from s->active.
int collect(ptw_server *s, const std::vector<size_t> &fin)
{
    NvtxRange nvtx("serve_collect");
    if (fin.empty()) return PTW_OK;
    std::vector<unsigned long long> base(fin.size());
    std::vector<uint32_t> cap(fin.size());
    std::vector<uint8_t> dense(fin.size());
    std::vector<Done> out(fin.size());
    for (size_t i = 0; i < fin.size(); ++i) {
        base[i] = s->active[fin[i]].off;
        dense[i] = s->active[fin[i]].dense ? 1 : 0;
        cap[i] = dense[i] ? s->g->dg.n : (uint32_t)s->active[fin[i]].cap;
    }
    Compacted c;
    c.top_k = s->cfg.top_k;
    std::shared_ptr<PinnedBlock> blk;
    c.sink = [&](uint64_t n) -> uint32_t * {
        blk = pinned_block(s, 2 * n);
        return blk ? blk->p : nullptr;
    };
    int rc = compact_tables(s->g, s->arena, base.data(), cap.data(), dense.data(), (uint32_t)fin.size(), &c);
    if (rc) return rc;
    for (size_t i = 0; i < fin.size(); ++i) {
        out[i].blk = blk;
        out[i].names = c.h_names + c.seg[i];
        out[i].counts = c.h_counts + c.seg[i];
    }
    s->st.entries += c.n;
    const double t = now_s(s);
    for (size_t i = 0; i < fin.size(); ++i) {
        const Active &a = s->active[fin[i]];
        out[i].r.query_id = a.p.q.query_id;
        out[i].r.source = a.p.q.source;
        out[i].r.budget = a.p.q.budget;
        out[i].r.n_entries = c.seg[i + 1] - c.seg[i];
        out[i].r.submit_s = a.p.submit_s;
        out[i].r.admit_s = a.admit_s;
        out[i].r.done_s = t;
        s->buddy.release(a.off);
        s->done.push_back(std::move(out[i]));
    }
    return PTW_OK;
}

}  // namespace
}  // namespace ptw

using namespace ptw;

extern "C" int ptw_serve_open(ptw_graph *g, const ptw_serve_cfg *cfg, ptw_server **out)
try {
    NvtxRange nvtx("ptw_serve_open");
    if (!cfg) return fail(PTW_EINVAL, "null argument");
    if (const int rc0 = check_stop(cfg->sp, cfg->max_moves)) return rc0;
    if (!g || !out) return fail(PTW_EINVAL, "null argument");
    *out = nullptr;
    if (cfg->app != PTW_APP_VISITS && cfg->app != PTW_APP_ENDPOINT) return fail(PTW_EINVAL, "unknown app");
    PTW_CUDA(cudaSetDevice(g->device));
    ptw_server *s = new (std::nothrow) ptw_server();
    if (!s) return fail(PTW_ENOMEM, "host allocation failed");
    s->g = g;
    s->cfg = *cfg;
    if (!s->cfg.tick_walkers) s->cfg.tick_walkers = 1ull << 23;
    if (!s->cfg.max_active) s->cfg.max_active = 4096;
    s->S = s->cfg.max_active;
    s->thr = stop_threshold(cfg->sp);
    s->t0 = std::chrono::steady_clock::now();
    uint64_t bytes = cfg->table_bytes;
    if (!bytes) {
        size_t fr = 0, tot = 0;
        cudaError_t e = cudaMemGetInfo(&fr, &tot);
        if (e != cudaSuccess) {
            delete s;
            return cuda_fail(e, "cudaMemGetInfo");
        }
        bytes = fr / 4;
    }
    s->buddy.init(bytes / 8, 8);
    int rc = PTW_OK;
    cudaError_t e = device_malloc(&s->arena, std::max<uint64_t>(s->buddy.capacity(), 1) * 8);
    // every query's share splits into at most share/kDescWalkers + 1 descriptors
    s->D = (uint32_t)std::min<uint64_t>(0xFFFFFFFFull, s->cfg.tick_walkers / kDescWalkers + 2ull * s->S + 1);
    s->plan_bytes = plan_size(s->S, s->D);
    if (e == cudaSuccess) e = device_malloc(&s->d_plan, s->plan_bytes);
    if (e == cudaSuccess) e = cudaMallocHost(&s->h_plan, s->plan_bytes);
    if (e != cudaSuccess) {
        rc = cuda_fail(e, "server allocation");
    } else {
        std::memset(s->h_plan, 0, s->plan_bytes);
        PlanView dv = view(s->d_plan, s->S, s->D);
        PlanView hv = view(s->h_plan, s->S, s->D);
        s->ret_off = (char *)hv.flag - (char *)s->h_plan;
        s->ret_bytes = s->plan_bytes - s->ret_off;
        BatchArgs &a = s->args;
        a.adj = g->dg.adj;
        a.col = g->dg.col;
        a.int2idx = g->dg.int2idx;
        a.ext_idx = g->dg.id_bound == g->dg.n ? 1u : 0u;  // names 0..n-1
        a.desc = dv.desc;
        a.q_src = dv.src;
        a.q_qid = dv.qid;
        a.q_tab = dv.tab;
        a.q_mask = dv.mask;
        a.q_flag = dv.flag;
        a.slots = s->arena;
        a.ctrl = dv.ctrl;
        a.check = g->sc.ctrl + 7;
        a.n_slots = s->buddy.capacity();
        a.m = g->dg.m;
        a.n = g->dg.n;
        a.nq = s->S;
        a.ndesc = 0;
        a.thr = s->thr;
        a.key0 = (uint32_t)cfg->seed;
        a.key1 = (uint32_t)(cfg->seed >> 32);
        a.max_moves = cfg->max_moves;
        a.app = cfg->app;
        int per_sm = 0;
        const bool ext = (g->tune.ext_columns & 1) && ensure_ext_columns(g);
        a.col_ext = g->dg.col_ext;
        s->kfn = ext ? (const void *)k_batch<true> : (const void *)k_batch<false>;
        s->uses_ext = ext;
        if (ext) ++g->ext_users;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, s->kfn, 256, 0);
        if (e != cudaSuccess) rc = cuda_fail(e, "occupancy");
        s->grid = (unsigned)std::max(1, g->num_sms * std::max(per_sm, 1));
        if (rc == PTW_OK) {
            e = cudaEventCreate(&s->ev[0]);
            if (e == cudaSuccess) e = cudaEventCreate(&s->ev[1]);
            if (e != cudaSuccess) rc = cuda_fail(e, "server events");
        }
        if (rc == PTW_OK && cfg->use_graph) rc = build_tick_graph(s);
        // one staging block up front (cfg.staging_mb), so the first results do not wait for it
        const uint64_t staging_words = (uint64_t)cfg->staging_mb << 18;  // MiB -> 4-byte words
        if (rc == PTW_OK && !pinned_block(s, std::max<uint64_t>(staging_words, 1)))
            rc = fail(PTW_ENOMEM, "pinned result staging");
    }
    if (rc != PTW_OK) {
        ptw_serve_close(s);
        return rc;
    }
    *out = s;
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_serve_submit(ptw_server *s, const ptw_query *q)
try {
    if (!s || !q) return fail(PTW_EINVAL, "null argument");
    if (q->budget < 1 || q->budget > (1ull << 28)) return fail(PTW_EINVAL, "budget must be in [1, 2^28]");
    const uint32_t n = s->g->dg.n;
    const uint32_t *p = std::lower_bound(s->g->h_names, s->g->h_names + n, q->source);
    if (p == s->g->h_names + n || *p != q->source)
        return fail(PTW_EINVAL, "source " + std::to_string(q->source) + " is not a vertex of the graph");
    Pending pd;
    pd.q = *q;
    pd.src = s->g->h_idx2int[p - s->g->h_names];
    pd.submit_s = now_s(s);
    pd.full = false;
    s->pending.push_back(pd);
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_serve_step(ptw_server *s, uint32_t *n_done, uint32_t *n_active, uint32_t *n_pending)
try {
    NvtxRange nvtx("ptw_serve_step");
    if (!s) return fail(PTW_EINVAL, "null server");
    PTW_CUDA(cudaSetDevice(s->g->device));
    const double t_enter = now_s(s);
    cudaStream_t st = s->g->stream;
    const uint32_t n = s->g->dg.n;
    const size_t done_before = s->done.size();
    // 1. admission: FIFO while a slot and a table fit
    while (!s->pending.empty() && s->active.size() < s->S) {
        Pending &pd = s->pending.front();
        const TableSize ts = pd.full ? dense_table(n)
                                     : count_table(s->cfg.sp, s->cfg.max_moves, s->cfg.app, s->cfg.table_factor,
                                                   pd.q.budget, n, 1u);
        const uint64_t cap = ts.slots;
        uint64_t off = 0;
        if (!s->buddy.alloc(cap, &off)) {
            if (s->active.empty() && cap > s->buddy.capacity())
                return fail(PTW_ENOMEM, "a query's count table is larger than the whole table arena");
            break;
        }
        PTW_CUDA(cudaMemsetAsync(s->arena + off, 0, cap * 8, st));
        Active a;
        a.p = pd;
        a.cap = cap;
        a.dense = ts.dense;
        a.off = off;
        a.started = 0;
        a.admit_s = now_s(s);
        s->active.push_back(a);
        s->pending.pop_front();
    }
    uint32_t nd = 0;
    if (!s->active.empty()) {
        // 2. plan: a fair share of the tick's walkers per active query
        PlanView hv = view(s->h_plan, s->S, s->D);
        const uint32_t na = (uint32_t)s->active.size();
        // a fair share per query, rounded to whole descriptors so the plan
        // never holds more than D of them
        uint64_t share = std::max<uint64_t>(1024, s->cfg.tick_walkers / na);
        share = (share + kDescWalkers - 1) / kDescWalkers * kDescWalkers;
        std::vector<uint64_t> j0(na);
        s->take.assign(na, 0);
        for (uint32_t i = 0; i < na; ++i) {
            const Active &a = s->active[i];
            s->take[i] = std::min<uint64_t>(share, a.p.q.budget - a.started);
            j0[i] = a.started;
            hv.tab[i] = a.off;
            hv.src[i] = a.p.src;
            hv.qid[i] = a.p.q.query_id;
            hv.mask[i] = a.dense ? kDenseMask : (uint32_t)(a.cap - 1);
            hv.flag[i] = 0;
        }
        std::vector<uint3> desc;
        std::vector<uint64_t> tbytes(na);
        for (uint32_t i = 0; i < na; ++i) tbytes[i] = s->active[i].cap * 8;
        interleave_descriptors(j0, s->take, tbytes, kGroupBytes, desc);
        if (desc.size() > s->D) {
            // more active queries than the plan holds descriptors for: keep
            // the first D (whole queries stay consistent: trim their takes)
            desc.resize(s->D);
            std::vector<uint64_t> got(na, 0);
            for (const uint3 &d : desc) got[d.x] += d.z;
            s->take = got;
        }
        std::memcpy(hv.desc, desc.data(), desc.size() * sizeof(uint3));
        hv.ctrl[0] = hv.ctrl[1] = 0;
        s->args.ndesc = (uint32_t)desc.size();
        // 3. the tick
        PTW_CUDA(cudaEventRecord(s->ev[0], st));
        if (s->exec) {
            void *kp[] = {&s->args};
            cudaKernelNodeParams p = s->kparams;
            p.kernelParams = kp;
            PTW_CUDA(cudaGraphExecKernelNodeSetParams(s->exec, s->knode, &p));
            PTW_CUDA(cudaGraphLaunch(s->exec, st));
        } else {
            PTW_CUDA(cudaMemcpyAsync(s->d_plan, s->h_plan, s->plan_bytes, cudaMemcpyHostToDevice, st));
            void *kargs[] = {&s->args};
            PTW_CUDA(cudaLaunchKernel(s->kfn, dim3(s->grid), dim3(256), kargs, 0, st));
            PTW_CUDA(cudaMemcpyAsync((char *)s->h_plan + s->ret_off, (char *)s->d_plan + s->ret_off,
                                     s->ret_bytes, cudaMemcpyDeviceToHost, st));
        }
        PTW_CUDA(cudaEventRecord(s->ev[1], st));
        PTW_CUDA(cudaStreamSynchronize(st));
        if (const int rc0 = check_word_status(s->g)) return rc0;
        float dev_ms = 0;
        PTW_CUDA(cudaEventElapsedTime(&dev_ms, s->ev[0], s->ev[1]));
        s->st.device_ms += dev_ms;
        ++s->st.ticks;
        s->st.moves += hv.ctrl[1];
        // 4. progress; completed queries become results; a query whose table
        //    filled is queued again (first) with a table that cannot fill
        std::vector<size_t> fin;
        std::vector<char> drop(na, 0);
        std::vector<Pending> retry;
        for (uint32_t i = 0; i < na; ++i) {
            Active &a = s->active[i];
            if (hv.flag[i]) {
                ++s->st.retries;
                retry.push_back(a.p);
                retry.back().full = true;
                s->buddy.release(a.off);
                drop[i] = 1;
                continue;
            }
            a.started += s->take[i];
            s->st.walkers += s->take[i];
            if (a.started == a.p.q.budget) {
                fin.push_back(i);
                drop[i] = 1;
            }
        }
        const double t_collect = now_s(s);
        int rc = collect(s, fin);
        if (rc) return rc;
        s->st.collect_ms += 1e3 * (now_s(s) - t_collect);
        s->st.completed += fin.size();
        std::vector<Active> keep;
        for (uint32_t i = 0; i < na; ++i)
            if (!drop[i]) keep.push_back(s->active[i]);
        s->active.swap(keep);
        for (auto it = retry.rbegin(); it != retry.rend(); ++it) s->pending.push_front(*it);
        nd = (uint32_t)(s->done.size() - done_before);
    }
    s->st.step_ms += 1e3 * (now_s(s) - t_enter);
    if (n_done) *n_done = nd;
    if (n_active) *n_active = (uint32_t)s->active.size();
    if (n_pending) *n_pending = (uint32_t)s->pending.size();
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_serve_poll(ptw_server *s, ptw_serve_result *r)
try {
    if (!s || !r) return fail(PTW_EINVAL, "null argument");
    if (s->done.empty()) return 0;
    *r = s->done.front().r;
    return 1;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_serve_take(ptw_server *s, uint32_t *h_names, uint32_t *h_counts)
try {
    if (!s) return fail(PTW_EINVAL, "null server");
    if (s->done.empty()) return fail(PTW_EINVAL, "no completed result");
    Done &d = s->done.front();
    const size_t ne = d.r.n_entries;
    if (h_names && ne) std::memcpy(h_names, d.names, ne * 4);
    if (h_counts && ne) std::memcpy(h_counts, d.counts, ne * 4);
    s->done.pop_front();
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_serve_view(const ptw_server *s, const uint32_t **names, const uint32_t **counts)
try {
    if (!s || !names || !counts) return fail(PTW_EINVAL, "null argument");
    if (s->done.empty()) return fail(PTW_EINVAL, "no completed result");
    *names = s->done.front().names;
    *counts = s->done.front().counts;
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_serve_get_stats(const ptw_server *s, ptw_serve_stats *out)
try {
    if (!s || !out) return fail(PTW_EINVAL, "null argument");
    *out = s->st;
    out->active = (uint32_t)s->active.size();
    out->pending = (uint32_t)s->pending.size();
    out->pinned_bytes = 0;
    for (const auto &b : s->pinned) out->pinned_bytes += b->words * 4;
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" double ptw_serve_clock(const ptw_server *s) { return s ? now_s(s) : 0.0; }

extern "C" void ptw_serve_close(ptw_server *s)
try {
    if (!s) return;
    cudaSetDevice(s->g->device);
    cudaStreamSynchronize(s->g->stream);
    if (s->uses_ext) --s->g->ext_users;
    s->done.clear();
    s->pinned.clear();
    for (cudaEvent_t e : s->ev)
        if (e) cudaEventDestroy(e);
    if (s->exec) cudaGraphExecDestroy(s->exec);
    if (s->graph) cudaGraphDestroy(s->graph);
    cudaFree(s->arena);
    cudaFree(s->d_plan);
    if (s->h_plan) cudaFreeHost(s->h_plan);
    delete s;
} catch (...) {
    host_exception();
}

// ---- checkpoint / resume ------------------------------------------------------
//
// File: magic "PTWSRV1\0", a 64-bit key of the graph (n, m, id bound, names),
// the configuration (ptw_serve_cfg), the server clock and statistics, then
//   pending queries: ptw_query, u8 full, f64 submit_s
//   active queries:  ptw_query, u8 full, f64 submit_s, f64 admit_s,
//                    u64 ranks run, u8 dense, u64 table slots, the table
//   finished results not taken: ptw_serve_result, names[n], counts[n]
// and a closing magic.

namespace ptw {
namespace {

const char kSrvMagic[8] = {'P', 'T', 'W', 'S', 'R', 'V', '1', '\0'};

uint64_t graph_key(const ptw_graph *g)
{
    uint64_t h = 1469598103934665603ull;
    auto add = [&](const void *p, size_t n) {
        const unsigned char *c = (const unsigned char *)p;
        for (size_t i = 0; i < n; ++i) h = (h ^ c[i]) * 1099511628211ull;
    };
    add(&g->dg.n, sizeof g->dg.n);
    add(&g->dg.m, sizeof g->dg.m);
    add(&g->dg.id_bound, sizeof g->dg.id_bound);
    add(g->h_names, (size_t)g->dg.n * 4);
    return h;
}

struct File {
    FILE *f = nullptr;
    bool ok = true;
    ~File()
    {
        if (f) std::fclose(f);
    }
    template <typename T> void put(const T *p, size_t n = 1)
    {
        ok = ok && std::fwrite(p, sizeof(T), n, f) == n;
    }
    template <typename T> void get(T *p, size_t n = 1)
    {
        ok = ok && std::fread(p, sizeof(T), n, f) == n;
    }
};

}  // namespace
}  // namespace ptw

extern "C" int ptw_serve_save(const ptw_server *s, const char *path)
try {
    NvtxRange nvtx("ptw_serve_save");
    if (!s || !path) return fail(PTW_EINVAL, "null argument");
    PTW_CUDA(cudaSetDevice(s->g->device));
    PTW_CUDA(cudaStreamSynchronize(s->g->stream));
    const std::string tmp = std::string(path) + ".tmp";
    File out;
    out.f = std::fopen(tmp.c_str(), "wb");
    if (!out.f) return fail(PTW_EIO, "cannot create " + tmp);
    const uint64_t key = graph_key(s->g);
    const double clock = now_s(s);
    const uint64_t counts[3] = {s->pending.size(), s->active.size(), s->done.size()};
    out.put(kSrvMagic, 8);
    out.put(&key);
    out.put(&s->cfg);
    out.put(&clock);
    out.put(&s->st);
    out.put(counts, 3);
    for (const Pending &p : s->pending) {
        const uint8_t full = p.full ? 1 : 0;
        out.put(&p.q);
        out.put(&full);
        out.put(&p.submit_s);
    }
    std::vector<unsigned long long> tab;
    for (const Active &a : s->active) {
        const uint8_t full = a.p.full ? 1 : 0, dense = a.dense ? 1 : 0;
        out.put(&a.p.q);
        out.put(&full);
        out.put(&a.p.submit_s);
        out.put(&a.admit_s);
        out.put(&a.started);
        out.put(&dense);
        out.put(&a.cap);
        tab.resize(a.cap);
        PTW_CUDA(cudaMemcpy(tab.data(), s->arena + a.off, a.cap * 8, cudaMemcpyDeviceToHost));
        out.put(tab.data(), tab.size());
    }
    for (const Done &d : s->done) {
        out.put(&d.r);
        out.put(d.names, d.r.n_entries);
        out.put(d.counts, d.r.n_entries);
    }
    out.put(kSrvMagic, 8);
    out.ok = out.ok && std::fflush(out.f) == 0 && fsync(fileno(out.f)) == 0;
    std::fclose(out.f);
    out.f = nullptr;
    if (!out.ok || std::rename(tmp.c_str(), path) != 0) {
        std::remove(tmp.c_str());
        return fail(PTW_EIO, std::string("cannot write the server checkpoint ") + path);
    }
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_serve_restore(ptw_graph *g, const char *path, ptw_server **out)
try {
    NvtxRange nvtx("ptw_serve_restore");
    if (!g || !path || !out) return fail(PTW_EINVAL, "null argument");
    *out = nullptr;
    File in;
    in.f = std::fopen(path, "rb");
    if (!in.f) return fail(PTW_EIO, std::string("cannot open ") + path);
    char magic[8];
    uint64_t key = 0, counts[3] = {0, 0, 0};
    ptw_serve_cfg cfg{};
    double clock = 0;
    ptw_serve_stats st{};
    in.get(magic, 8);
    if (!in.ok || std::memcmp(magic, kSrvMagic, 8)) return fail(PTW_EINVAL, std::string(path) + " is not a server checkpoint");
    in.get(&key);
    if (!in.ok || key != graph_key(g))
        return fail(PTW_EINVAL, std::string(path) + " was saved from a server on another graph");
    in.get(&cfg);
    in.get(&clock);
    in.get(&st);
    in.get(counts, 3);
    if (!in.ok) return fail(PTW_EIO, std::string("truncated server checkpoint ") + path);
    ptw_server *s = nullptr;
    int rc = ptw_serve_open(g, &cfg, &s);
    if (rc) return rc;
    auto bail = [&](int code) {
        ptw_serve_close(s);
        return code;
    };
    // the clock continues from the saved one (latencies leave the downtime out)
    s->t0 = std::chrono::steady_clock::now() -
            std::chrono::duration_cast<std::chrono::steady_clock::duration>(std::chrono::duration<double>(clock));
    s->st = st;
    const uint32_t n = g->dg.n;
    auto source_id = [&](uint32_t name, uint32_t *id) -> bool {
        const uint32_t *p = std::lower_bound(g->h_names, g->h_names + n, name);
        if (p == g->h_names + n || *p != name) return false;
        *id = g->h_idx2int[p - g->h_names];
        return true;
    };
    for (uint64_t i = 0; i < counts[0]; ++i) {
        Pending p;
        uint8_t full = 0;
        in.get(&p.q);
        in.get(&full);
        in.get(&p.submit_s);
        p.full = full != 0;
        if (!in.ok || !source_id(p.q.source, &p.src)) return bail(fail(PTW_EIO, "bad pending query in checkpoint"));
        s->pending.push_back(p);
    }
    std::vector<unsigned long long> tab;
    for (uint64_t i = 0; i < counts[1]; ++i) {
        Active a;
        uint8_t full = 0, dense = 0;
        in.get(&a.p.q);
        in.get(&full);
        in.get(&a.p.submit_s);
        in.get(&a.admit_s);
        in.get(&a.started);
        in.get(&dense);
        in.get(&a.cap);
        a.p.full = full != 0;
        a.dense = dense != 0;
        if (!in.ok || !source_id(a.p.q.source, &a.p.src) || a.started > a.p.q.budget || a.cap == 0 ||
            a.cap > s->buddy.capacity())
            return bail(fail(PTW_EIO, "bad active query in checkpoint"));
        tab.resize(a.cap);
        in.get(tab.data(), tab.size());
        if (!in.ok) return bail(fail(PTW_EIO, "truncated server checkpoint"));
        if (s->active.size() >= s->S || !s->buddy.alloc(a.cap, &a.off))
            return bail(fail(PTW_ENOMEM, "the restored server's table arena cannot hold the saved active queries"));
        cudaError_t e = cudaMemcpy(s->arena + a.off, tab.data(), a.cap * 8, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return bail(cuda_fail(e, "restoring a count table"));
        s->active.push_back(a);
    }
    // finished results: read, then staged together in one pinned block
    std::vector<ptw_serve_result> rs(counts[2]);
    std::vector<std::vector<uint32_t>> lists(counts[2]);
    uint64_t words = 0;
    for (uint64_t i = 0; i < counts[2]; ++i) {
        in.get(&rs[i]);
        if (!in.ok || rs[i].n_entries > n) return bail(fail(PTW_EIO, "truncated server checkpoint"));
        lists[i].resize(2 * rs[i].n_entries);
        in.get(lists[i].data(), lists[i].size());
        words += lists[i].size();
    }
    if (!in.ok) return bail(fail(PTW_EIO, "truncated server checkpoint"));
    if (counts[2]) {
        std::shared_ptr<PinnedBlock> blk = pinned_block(s, std::max<uint64_t>(words, 1));
        if (!blk) return bail(fail(PTW_ENOMEM, "pinned result staging"));
        uint64_t at = 0;
        for (uint64_t i = 0; i < counts[2]; ++i) {
            Done d;
            d.r = rs[i];
            d.blk = blk;
            std::memcpy(blk->p + at, lists[i].data(), lists[i].size() * 4);
            d.names = blk->p + at;
            d.counts = blk->p + at + rs[i].n_entries;
            at += lists[i].size();
            s->done.push_back(std::move(d));
        }
    }
    in.get(magic, 8);
    if (!in.ok || std::memcmp(magic, kSrvMagic, 8)) return bail(fail(PTW_EIO, "truncated server checkpoint"));
    *out = s;
    return PTW_OK;
} catch (...) {
    return host_exception();
}
