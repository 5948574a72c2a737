// Batched single-source PPR / RWR (K4).
//
// The reference answers one source per process (src/core/ppr.cpp:121-138,
// source hard-coded to internal id 0; RWR.cpp:109-128 records (start, end)
// pairs).  Here thousands of queries run in one persistent launch per wave:
//
//   device query table   q_off[q]  first global walker index of query q
//                         q_src[q]  source (internal id), q_qid[q] its query id
//                         q_tab[q], q_mask[q]  its count table (slot offset, size-1)
//   global walker index g -> query q = last q with q_off[q] <= g (binary search),
//   walker id (q_qid[q] << 32) + (g - q_off[q]): every draw depends on the
//   query id and the walker's rank in its query only, so a query's counts are
//   the same alone or in any batch and wave.
//
// Per-query counts of a small query are kept sparse in an open-addressing
// table of 64-bit slots (vertex internal id + 1 in the high half, count in the
// low half), sized from the query's budget; a query that finds no free slot
// within the probe limit raises its flag and the host runs it again with a
// dense array.  A query whose table would take at least 4n bytes counts into
// a dense array of n 32-bit counters indexed by canonical vertex index: a
// visit is one fire-and-forget reduction instead of a probe, and the array
// is already in name order, so its compaction needs no sort.  Waves take
// queries in order while their tables fit the table budget (admission by
// device memory).  After a wave the tables are compacted into (name, count)
// lists sorted by name (or each query's top k by count) and copied to the
// host.
#include <cub/cub.cuh>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include <sys/mman.h>
#include <unistd.h>

#include "batch_kernels.cuh"

struct ptw_batch {
    uint32_t nq = 0;
    std::vector<ptw_query> queries;
    std::vector<uint64_t> offsets;  // [nq + 1]
    ptw::HostArray names, counts;
    ptw_walk_stats stats{};
    uint32_t top_k = 0;  // results hold each query's top_k largest counts only
    // Device-resident results (PTW_BATCH_DEVICE_RESULTS): lists and offsets
    // in the library's device pool instead of names / counts.
    bool device = false;
    int device_id = 0;
    ptw::PoolArray d_names, d_counts, d_offsets;  // d_offsets holds nq + 1 uint64 (as 2 words each)
    ptw_batch_phases phases{};
};

namespace ptw {
namespace {
// Result of one wave: its queries (caller indices, in wave order), their
// compacted entries, and which of them overflowed (entries to be replaced).
struct WaveResult {
    std::vector<uint32_t> idx;
    Compacted c;
    std::vector<char> overflow;
};
}  // namespace
}  // namespace ptw

namespace ptw {

int PhaseTimer::begin(int phase, cudaStream_t s)
{
    Span sp{phase, nullptr, nullptr};
    if (cudaEventCreate(&sp.a) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    if (cudaEventCreate(&sp.b) != cudaSuccess) {
        cudaGetLastError();
        cudaEventDestroy(sp.a);
        return -1;
    }
    if (cudaEventRecord(sp.a, s) != cudaSuccess) cudaGetLastError();
    spans.push_back(sp);
    return (int)spans.size() - 1;
}

void PhaseTimer::end(int span, cudaStream_t s)
{
    if (span < 0) return;
    if (cudaEventRecord(spans[span].b, s) != cudaSuccess) cudaGetLastError();
    if (spans[span].phase == kPlace) last_place = span;
    if (spans[span].phase == kCopy) last_copy = span;
}

void PhaseTimer::sums(double out[kPhases], double *copy_tail_ms) const
{
    for (int k = 0; k < kPhases; ++k) out[k] = 0;
    for (const Span &sp : spans) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, sp.a, sp.b) == cudaSuccess) out[sp.phase] += ms;
        else cudaGetLastError();
    }
    *copy_tail_ms = 0;
    if (last_place >= 0 && last_copy >= 0) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, spans[last_place].b, spans[last_copy].b) == cudaSuccess)
            *copy_tail_ms = std::max(0.0f, ms);
        else
            cudaGetLastError();
    }
}

PhaseTimer::~PhaseTimer()
{
    for (Span &sp : spans) {
        cudaEventDestroy(sp.a);
        cudaEventDestroy(sp.b);
    }
}

namespace {

constexpr uint64_t kMaxBudget = 1ull << 28;

// Effective batch launch parameters (zero fields of ptw_batch_tune take the
// defaults).
struct BatchTune {
    uint32_t desc_walkers, blocks_per_sm, dense_ratio;
    uint64_t group_bytes;
    bool ext;
};

BatchTune effective_tune(const ptw_graph *g)
{
    const ptw_batch_tune &t = g->btune;
    BatchTune e;
    e.desc_walkers = t.desc_walkers ? t.desc_walkers : kDescWalkers;
    e.blocks_per_sm = t.blocks_per_sm;
    e.dense_ratio = t.dense_ratio ? t.dense_ratio : 1u;
    e.group_bytes = t.group_bytes == 0 ? kGroupBytes : t.group_bytes == ~0ull ? 0ull : t.group_bytes;
    e.ext = t.ext_columns == 1 ? true : t.ext_columns == 2 ? false : (g->tune.ext_columns & 1) != 0;
    return e;
}

// Faults in the pages of fresh host buffers from several threads.  A
// device-to-host copy into pages the process has never touched takes the
// faults one by one inside the copy (about 6x slower than the copy itself
// for gigabytes); touching one byte per page first, while the device is
// still busy, leaves the copy at link speed.  With pin, the buffers are
// then registered with CUDA (page-locked): copies into pageable pages that
// had been faulted in still took 2-3.6x longer in about one call in three,
// copies into registered pages did not.  One coordinator thread runs the
// touching threads and the registration, so both overlap the walk.
class Prefault {
public:
    void start(std::initializer_list<std::pair<void *, size_t>> bufs, bool pin = false)
    {
        size_t total = 0;
        for (auto &b : bufs) total += b.second;
        if (total < (64u << 20)) return;  // small: the copy absorbs it
        std::vector<std::pair<void *, size_t>> v(bufs);
        pinned_.assign(v.size(), false);
        coord_ = std::thread([this, v, pin] {
            const long pg = sysconf(_SC_PAGESIZE);
            const size_t page = pg > 0 ? (size_t)pg : 4096;
            const unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
            try {
                parallel_for_threads(nt * (unsigned)v.size(), [&](unsigned i) {
                    char *p = (char *)v[i / nt].first;
                    const size_t len = v[i / nt].second, t = i % nt;
                    const size_t lo = len * t / nt, hi = len * (t + 1) / nt;
                    for (size_t x = lo - lo % page; x < hi; x += page)
                        if (x >= lo) ((volatile char *)p)[x] = 0;
                });
            } catch (...) {
                return;  // pages not touched yet fault in during the copy
            }
            if (pin)
                for (size_t b = 0; b < v.size(); ++b) pinned_[b] = host_pin((uint32_t *)v[b].first, v[b].second);
        });
    }
    void join()
    {
        if (coord_.joinable()) coord_.join();
    }
    // Whether every buffer was registered (valid after join).
    bool pinned() const
    {
        if (pinned_.empty()) return false;
        for (bool b : pinned_)
            if (!b) return false;
        return true;
    }
    ~Prefault() { join(); }

private:
    std::thread coord_;
    std::vector<bool> pinned_;
};

// Page-locked host arrays (base pointer -> bytes) and the host cache live
// in objects that are never destroyed: nothing of theirs runs at exit,
// when the CUDA runtime may already be gone.
struct PinRegistry {
    std::mutex mu;
    std::map<const void *, uint64_t> arrays;
    uint64_t bytes = 0;
};
PinRegistry &pins()
{
    static PinRegistry *r = new PinRegistry;
    return *r;
}

uint64_t pin_limit()
{
    const long pages = sysconf(_SC_PHYS_PAGES), pg = sysconf(_SC_PAGESIZE);
    return pages > 0 && pg > 0 ? (uint64_t)pages * (uint64_t)pg / 4 : 0;
}

}  // namespace

bool host_pin(uint32_t *p, uint64_t bytes)
{
    if (!p || !bytes) return false;
    PinRegistry &r = pins();
    {
        std::lock_guard<std::mutex> lk(r.mu);
        if (r.arrays.count(p) || r.bytes + bytes > pin_limit()) return false;
        r.bytes += bytes;  // reserved while registering
    }
    // portable: the registering thread's current device need not be the graph's
    const bool ok = cudaHostRegister(p, bytes, cudaHostRegisterPortable) == cudaSuccess;
    std::lock_guard<std::mutex> lk(r.mu);
    if (ok) {
        r.arrays[p] = bytes;
    } else {
        cudaGetLastError();
        r.bytes -= bytes;
    }
    return ok;
}

void HostArrayDelete::operator()(uint32_t *p) const
{
    if (!p) return;
    PinRegistry &r = pins();
    bool was = false;
    {
        std::lock_guard<std::mutex> lk(r.mu);
        auto it = r.arrays.find(p);
        if (it != r.arrays.end()) {
            r.bytes -= it->second;
            r.arrays.erase(it);
            was = true;
        }
    }
    if (was && cudaHostUnregister(p) != cudaSuccess) cudaGetLastError();
    delete[] p;
}

namespace {

// Hands the whole pages of [p + used, p + cap) back to the system; the
// range stays valid (it reads as zeros if touched again).
void release_tail(void *p, size_t used, size_t cap)
{
    const long pg = sysconf(_SC_PAGESIZE);
    const uintptr_t page = pg > 0 ? (uintptr_t)pg : 4096;
    const uintptr_t lo = ((uintptr_t)p + used + page - 1) & ~(page - 1);
    const uintptr_t hi = ((uintptr_t)p + cap) & ~(page - 1);
    if (hi > lo) madvise((void *)lo, hi - lo, MADV_DONTNEED);
}

struct DevBuf {
    cudaStream_t st;
    std::vector<void *> ptrs;
    explicit DevBuf(cudaStream_t s) : st(s) {}
    template <typename T> cudaError_t alloc(T **p, uint64_t count)
    {
        void *q = nullptr;
        cudaError_t e = pooled_alloc_async(&q, std::max<uint64_t>(count, 1) * sizeof(T), st);
        if (e == cudaSuccess) ptrs.push_back(q);
        *p = (T *)q;
        return e;
    }
    ~DevBuf()
    {
        for (void *q : ptrs) cudaFreeAsync(q, st);
    }
};

template <typename F> cudaError_t cub_call(F f, cudaStream_t st)
{
    size_t bytes = 0;
    cudaError_t e = f(nullptr, bytes);
    if (e != cudaSuccess) return e;
    void *tmp = nullptr;
    e = pooled_alloc_async(&tmp, std::max<size_t>(bytes, 16), st);
    if (e != cudaSuccess) return e;
    e = f(tmp, bytes);
    cudaFreeAsync(tmp, st);
    return e;
}

struct WaveQuery {
    uint32_t index;  // position in the caller's array
    uint32_t src;    // internal id
    uint32_t qid;
    uint64_t budget;
    uint64_t cap;    // 64-bit slots of its table (a power of two for a hash table)
    bool dense;      // dense array of n counters instead of a hash table
};

}  // namespace

// Splits [j0, j0 + count) of every entry into descriptors of at most
// dw ranks.  Entries are cut into consecutive groups whose tables
// add up to about group_bytes (0 = one group); descriptors go round-robin
// over the entries of a group, and groups follow one another.  Warps take
// descriptors in order, so the count tables being written at any moment are
// those of about one group: a few hundred MB stay largely in L2 where the
// tables of thousands of queries at once would not (1.6x faster walk kernel
// on 4096 queries at R-MAT scale 22 with 384 MB groups).
uint64_t interleave_descriptors(const std::vector<uint64_t> &j0, const std::vector<uint64_t> &count,
                                const std::vector<uint64_t> &table_bytes, uint64_t group_bytes,
                                std::unique_ptr<uint3[]> &desc, unsigned threads, uint32_t dw)
{
    const uint32_t ne = (uint32_t)count.size();
    std::vector<uint32_t> gb;  // first entry of each group, then ne
    for (uint32_t g0 = 0; g0 < ne;) {
        uint64_t bytes = 0;
        uint32_t g1 = g0;
        while (g1 < ne && (g1 == g0 || group_bytes == 0 || bytes + table_bytes[g1] <= group_bytes)) {
            bytes += table_bytes[g1];
            ++g1;
        }
        gb.push_back(g0);
        g0 = g1;
    }
    gb.push_back(ne);
    const size_t ng = gb.size() - 1;
    std::vector<uint64_t> goff(ng + 1, 0);  // first descriptor of each group
    for (size_t k = 0; k < ng; ++k) {
        uint64_t d = 0;
        for (uint32_t i = gb[k]; i < gb[k + 1]; ++i) d += (count[i] + dw - 1) / dw;
        goff[k + 1] = goff[k] + d;
    }
    desc.reset(new uint3[std::max<uint64_t>(goff[ng], 1)]);  // not value-initialised
    uint3 *out = desc.get();
    auto fill = [&](size_t k) {
        std::vector<uint32_t> live;
        for (uint32_t i = gb[k]; i < gb[k + 1]; ++i)
            if (count[i]) live.push_back(i);
        uint3 *o = out + goff[k];
        for (uint64_t r = 0; !live.empty(); ++r) {
            size_t keep = 0;
            const uint64_t off = r * dw;
            for (uint32_t i : live) {
                const uint64_t c = std::min<uint64_t>(dw, count[i] - off);
                *o++ = make_uint3(i, (uint32_t)(j0[i] + off), (uint32_t)c);
                if (off + c < count[i]) live[keep++] = i;
            }
            live.resize(keep);
        }
    };
    // groups are independent: fill them on host threads when there are many descriptors
    const unsigned nth = goff[ng] >= (1u << 18) ? (unsigned)std::min<size_t>(ng, std::max(1u, threads)) : 1u;
    if (nth <= 1) {
        for (size_t k = 0; k < ng; ++k) fill(k);
    } else {
        std::atomic<size_t> next{0};
        parallel_for_threads(nth, [&](unsigned) {
            for (size_t k; (k = next.fetch_add(1)) < ng;) fill(k);
        });
    }
    return goff[ng];
}

void interleave_descriptors(const std::vector<uint64_t> &j0, const std::vector<uint64_t> &count,
                            const std::vector<uint64_t> &table_bytes, uint64_t group_bytes,
                            std::vector<uint3> &desc)
{
    std::unique_ptr<uint3[]> buf;
    const uint64_t n = interleave_descriptors(j0, count, table_bytes, group_bytes, buf, 1, kDescWalkers);
    desc.assign(buf.get(), buf.get() + n);
}

namespace {

// Runs one wave; stores each query's sorted entries in per-query host lists.
int run_wave(ptw_graph *g, const std::vector<WaveQuery> &wq, const ptw_batch_cfg *cfg, uint64_t thr,
             std::vector<WaveResult> &waves, std::vector<uint32_t> &overflow, uint64_t *moves_out,
             float *walk_ms, PhaseTimer *ph)
{
    NvtxRange nvtx("run_wave");
    cudaStream_t st = g->stream;
    const uint32_t nq = (uint32_t)wq.size();
    const BatchTune bt = effective_tune(g);
    const bool device_results = (cfg->flags & PTW_BATCH_DEVICE_RESULTS) != 0;
    const bool timing = std::getenv("PTW_TIMING") != nullptr;
    auto clk = [] { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); };
    const double t_enter = clk();
    double t_plan = 0, t_setup = 0;
    std::vector<unsigned long long> h_tab(nq + 1);
    std::vector<uint32_t> h_src(nq), h_qid(nq), h_mask(nq), h_cap(nq);
    std::vector<uint8_t> h_dense(nq);
    std::vector<uint64_t> j0(nq, 0), cnt(nq);
    for (uint32_t i = 0; i < nq; ++i) {
        h_tab[i + 1] = h_tab[i] + ((wq[i].cap + 15) & ~15ull);  // tables start on 128-byte lines
        h_src[i] = wq[i].src;
        h_qid[i] = wq[i].qid;
        h_dense[i] = wq[i].dense ? 1 : 0;
        h_mask[i] = wq[i].dense ? kDenseMask : (uint32_t)(wq[i].cap - 1);
        h_cap[i] = wq[i].dense ? g->dg.n : (uint32_t)wq[i].cap;
        cnt[i] = wq[i].budget;
    }
    std::unique_ptr<uint3[]> h_desc;
    std::vector<uint64_t> tbytes(nq);
    for (uint32_t i = 0; i < nq; ++i) tbytes[i] = wq[i].cap * 8;
    const uint64_t nd = interleave_descriptors(j0, cnt, tbytes, bt.group_bytes, h_desc,
                                               std::min(16u, std::max(1u, std::thread::hardware_concurrency())),
                                               bt.desc_walkers);
    t_plan = clk();
    ph->plan_ms += 1e3 * (t_plan - t_enter);
    const uint64_t n_slots = h_tab[nq];
    const int sp_up = ph->begin(PhaseTimer::kUpload, st);
    DevBuf db(st);
    unsigned long long *d_tab, *d_slots, *d_ctrl;
    uint32_t *d_src, *d_qid, *d_mask, *d_flag;
    uint3 *d_desc;
    PTW_CUDA(db.alloc(&d_tab, nq + 1));
    PTW_CUDA(db.alloc(&d_src, nq));
    PTW_CUDA(db.alloc(&d_qid, nq));
    PTW_CUDA(db.alloc(&d_mask, nq));
    PTW_CUDA(db.alloc(&d_flag, nq));
    PTW_CUDA(db.alloc(&d_ctrl, 2));
    PTW_CUDA(db.alloc(&d_desc, nd));
    PTW_CUDA(db.alloc(&d_slots, n_slots));
    PTW_CUDA(cudaMemcpyAsync(d_tab, h_tab.data(), (nq + 1) * 8ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_src, h_src.data(), nq * 4ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_qid, h_qid.data(), nq * 4ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_mask, h_mask.data(), nq * 4ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_desc, h_desc.get(), nd * sizeof(uint3), cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemsetAsync(d_flag, 0, nq * 4ull, st));
    PTW_CUDA(cudaMemsetAsync(d_ctrl, 0, 16, st));
    PTW_CUDA(cudaMemsetAsync(d_slots, 0, n_slots * 8, st));
    ph->end(sp_up, st);
    if (timing) {
        PTW_CUDA(cudaStreamSynchronize(st));
        t_setup = clk();
    }

    BatchArgs a;
    a.adj = g->dg.adj;
    a.col = g->dg.col;
    const bool ext = bt.ext && ensure_ext_columns(g);
    a.col_ext = g->dg.col_ext;
    a.int2idx = g->dg.int2idx;
    a.ext_idx = g->dg.id_bound == g->dg.n ? 1u : 0u;  // names 0..n-1
    a.desc = d_desc;
    a.q_src = d_src;
    a.q_qid = d_qid;
    a.q_tab = d_tab;
    a.q_mask = d_mask;
    a.q_flag = d_flag;
    a.slots = d_slots;
    a.ctrl = d_ctrl;
    a.check = g->sc.ctrl + 7;
    a.n_slots = n_slots;
    a.m = g->dg.m;
    a.n = g->dg.n;
    a.nq = nq;
    a.ndesc = (uint32_t)nd;
    a.thr = thr;
    a.key0 = (uint32_t)cfg->seed;
    a.key1 = (uint32_t)(cfg->seed >> 32);
    a.max_moves = cfg->max_moves;
    a.app = cfg->app;
    if (nd >= (1ull << 32)) return fail(PTW_EINVAL, "wave too large");
    int per_sm = 0;
    const void *kfn = ext ? (const void *)k_batch<true> : (const void *)k_batch<false>;
    PTW_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, 256, 0));
    per_sm = std::max(per_sm, 1);
    if (bt.blocks_per_sm) per_sm = std::min<int>(per_sm, (int)bt.blocks_per_sm);
    uint64_t grid = (uint64_t)g->num_sms * per_sm;
    grid = std::min<uint64_t>(grid, std::max<uint64_t>(1, (nd + 7) / 8));
    // Full lists: host buffers of an estimated size are faulted in on host
    // threads while the walk runs (about 1.1 distinct entries per walker on
    // R-MAT at sp 0.2; 1.5 leaves room); compaction adopts them if the lists
    // fit.
    WaveResult wr;
    wr.c.top_k = cfg->top_k;
    wr.c.device = device_results;
    wr.c.ph = ph;
    Prefault early;
    if (cfg->top_k == 0 && !device_results) {
        uint64_t est = 0;
        for (uint32_t i = 0; i < nq; ++i)
            est += std::min<uint64_t>(g->dg.n, (uint64_t)(1.5 * (double)wq[i].budget) + 64);
        if (est * 8 >= (64ull << 20)) {
            // Fresh arrays every call, faulted in and page-locked on host
            // threads while the device walks.  Arrays kept from an earlier
            // batch and reused (registered once) took copies 2-40x slower in
            // some calls on some hosts (5 of 12 calls on one host, where 12
            // calls into fresh arrays all copied at 193 GB/s).
            wr.c.pre_names.reset(new (std::nothrow) uint32_t[est]);
            wr.c.pre_counts.reset(new (std::nothrow) uint32_t[est]);
            wr.c.pre_cap = est;
            wr.c.pre_pinned = false;
            if (wr.c.pre_names && wr.c.pre_counts) {
                early.start({{wr.c.pre_names.get(), est * 4}, {wr.c.pre_counts.get(), est * 4}}, true);
                wr.c.pre_join = [&early, &wr] {
                    early.join();
                    wr.c.pre_pinned = early.pinned();
                };
            } else {
                wr.c.pre_names.reset();
                wr.c.pre_counts.reset();
                wr.c.pre_cap = 0;
            }
        }
    }
    PTW_CUDA(cudaEventRecord(g->ev[0], st));
    const int sp_walk = ph->begin(PhaseTimer::kWalk, st);
    {
        void *kargs[] = {&a};
        PTW_CUDA(cudaLaunchKernel(kfn, dim3((unsigned)grid), dim3(256), kargs, 0, st));
    }
    ph->end(sp_walk, st);
    PTW_CUDA(cudaEventRecord(g->ev[1], st));
    PTW_CUDA(cudaGetLastError());
    std::vector<uint32_t> h_flag(nq);
    unsigned long long h_moves = 0;
    PTW_CUDA(cudaMemcpyAsync(h_flag.data(), d_flag, nq * 4ull, cudaMemcpyDeviceToHost, st));
    PTW_CUDA(cudaMemcpyAsync(&h_moves, d_ctrl + 1, 8, cudaMemcpyDeviceToHost, st));
    int rc = compact_tables(g, d_slots, h_tab.data(), h_cap.data(), h_dense.data(), nq, &wr.c);
    if (!rc) rc = check_word_status(g);
    early.join();
    wr.c.pre_join = nullptr;
    wr.c.pre_names.reset();
    wr.c.pre_counts.reset();
    if (rc) return rc;
    float ms = 0;
    PTW_CUDA(cudaEventElapsedTime(&ms, g->ev[0], g->ev[1]));
    *walk_ms += ms;
    *moves_out += h_moves;
    if (timing)
        std::fprintf(stderr,
                     "[ptw] wave of %u queries, %llu descriptors, %llu slots: plan %.1f ms, setup %.1f ms, "
                     "walk kernel %.1f ms, wave %.1f ms\n",
                     nq, (unsigned long long)nd, (unsigned long long)n_slots, 1e3 * (t_plan - t_enter),
                     1e3 * (t_setup - t_plan), ms, 1e3 * (clk() - t_enter));
    wr.idx.resize(nq);
    wr.overflow.assign(nq, 0);
    for (uint32_t i = 0; i < nq; ++i) {
        wr.idx[i] = wq[i].index;
        if (h_flag[i]) {
            overflow.push_back(wq[i].index);
            wr.overflow[i] = 1;
        }
    }
    waves.push_back(std::move(wr));
    return PTW_OK;
}

// Concatenates the waves' entries in caller query order.  One wave holding
// every query in order (the common case) is adopted without a copy.
// Device-resident results are concatenated on the device (one copy per
// query segment when there is more than one wave).
int assemble(ptw_graph *g, ptw_batch *b, std::vector<WaveResult> &waves)
{
    const uint32_t nq = b->nq;
    std::vector<const WaveResult *> src_w(nq, nullptr);
    std::vector<uint32_t> src_i(nq, 0);
    for (const WaveResult &w : waves)
        for (uint32_t k = 0; k < w.idx.size(); ++k)
            if (!w.overflow[k]) {
                src_w[w.idx[k]] = &w;
                src_i[w.idx[k]] = k;
            }
    b->offsets.assign(nq + 1, 0);
    for (uint32_t i = 0; i < nq; ++i) {
        const WaveResult *w = src_w[i];
        const uint64_t len = w ? w->c.seg[src_i[i] + 1] - w->c.seg[src_i[i]] : 0;
        b->offsets[i + 1] = b->offsets[i] + len;
    }
    const uint64_t total = b->offsets[nq];
    bool adopt = waves.size() == 1 && waves[0].idx.size() == nq;
    if (adopt)
        for (uint32_t k = 0; k < nq; ++k) adopt = adopt && waves[0].idx[k] == k && !waves[0].overflow[k];
    if (b->device) {
        cudaStream_t st = g->stream;
        if (adopt) {
            b->d_names = std::move(waves[0].c.d_names);
            b->d_counts = std::move(waves[0].c.d_counts);
        } else if (total) {
            PTW_CUDA(b->d_names.alloc(total, st));
            PTW_CUDA(b->d_counts.alloc(total, st));
            for (uint32_t i = 0; i < nq; ++i) {
                const WaveResult *w = src_w[i];
                const uint64_t len = b->offsets[i + 1] - b->offsets[i];
                if (!w || !len) continue;
                const uint64_t a = w->c.seg[src_i[i]];
                PTW_CUDA(cudaMemcpyAsync(b->d_names.p + b->offsets[i], w->c.d_names.p + a, len * 4,
                                         cudaMemcpyDeviceToDevice, st));
                PTW_CUDA(cudaMemcpyAsync(b->d_counts.p + b->offsets[i], w->c.d_counts.p + a, len * 4,
                                         cudaMemcpyDeviceToDevice, st));
            }
        }
        PTW_CUDA(b->d_offsets.alloc(2ull * (nq + 1), st));
        PTW_CUDA(cudaMemcpyAsync(b->d_offsets.p, b->offsets.data(), (nq + 1) * 8ull, cudaMemcpyHostToDevice, st));
        return PTW_OK;
    }
    if (adopt) {
        b->names = std::move(waves[0].c.names);
        b->counts = std::move(waves[0].c.counts);
        return PTW_OK;
    }
    if (!total) return PTW_OK;
    b->names.reset(new (std::nothrow) uint32_t[total]);
    b->counts.reset(new (std::nothrow) uint32_t[total]);
    if (!b->names || !b->counts) return fail(PTW_ENOMEM, "host allocation of batch results failed");
    for (uint32_t i = 0; i < nq; ++i) {
        const WaveResult *w = src_w[i];
        if (!w) continue;
        const uint64_t a = w->c.seg[src_i[i]], len = b->offsets[i + 1] - b->offsets[i];
        std::memcpy(b->names.get() + b->offsets[i], w->c.names.get() + a, len * 4);
        std::memcpy(b->counts.get() + b->offsets[i], w->c.counts.get() + a, len * 4);
    }
    return PTW_OK;
}

uint64_t next_pow2(uint64_t x)
{
    uint64_t p = 1;
    while (p < x) p <<= 1;
    return p;
}

}  // namespace

const ptw_query *batch_queries(const ptw_batch *b) { return b->queries.data(); }
uint32_t batch_top_k(const ptw_batch *b) { return b->top_k; }
bool batch_device(const ptw_batch *b) { return b->device; }

int compact_tables(ptw_graph *g, unsigned long long *d_slots, const unsigned long long *h_base,
                   const uint32_t *h_cap, const uint8_t *h_dense, uint32_t nt, Compacted *out)
{
    NvtxRange nvtx("compact_tables");
    out->n = 0;
    out->seg.assign(nt + 1, 0);
    out->names.reset();
    out->counts.reset();
    out->h_names = out->h_counts = nullptr;
    if (nt == 0) return PTW_OK;
    cudaStream_t st = g->stream;
    const bool timing = std::getenv("PTW_TIMING") != nullptr;
    auto clk = [] { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); };
    const double t0 = timing ? (cudaStreamSynchronize(st), clk()) : 0.0;
    double t1 = 0, t2 = 0, t_join = 0;
    PhaseTimer no_timer;
    PhaseTimer *ph = out->ph ? out->ph : &no_timer;
    struct PagesWait {  // host time spent waiting for result pages, added up on every return
        PhaseTimer *ph;
        double &ms;
        ~PagesWait() { ph->host_pages_ms += 1e3 * ms; }
    } pages_wait{ph, t_join};
    Prefault prefault;  // joined before the copies (and on any early return)
    std::vector<uint8_t> dense_flags(nt, 0);
    if (h_dense) dense_flags.assign(h_dense, h_dense + nt);
    uint64_t n_dense = 0;
    for (uint32_t i = 0; i < nt; ++i) n_dense += dense_flags[i] ? 1 : 0;
    const uint32_t k = out->top_k;
    // Block chunks of kChunkBytes per table, in table order.
    std::vector<unsigned long long> tch(nt + 1, 0);
    for (uint32_t i = 0; i < nt; ++i) {
        if (h_base[i] & 1) return fail(PTW_EINVAL, "count table not 16-byte aligned");
        const uint64_t bytes = (uint64_t)h_cap[i] * (dense_flags[i] ? 4 : 8);
        tch[i + 1] = tch[i] + (bytes + kChunkBytes - 1) / kChunkBytes;
    }
    const uint64_t nch = tch[nt];
    if (nch >= (1ull << 31)) return fail(PTW_EINVAL, "count tables too large to compact in one call");
    DevBuf db(st);
    unsigned long long *d_base, *d_cnt, *d_seg, *d_fill, *d_tch, *d_cc, *d_hc, *d_pos = nullptr, *d_hpos = nullptr;
    uint32_t *d_cap, *d_hist = nullptr;
    uint8_t *d_dense;
    PTW_CUDA(db.alloc(&d_base, nt));
    PTW_CUDA(db.alloc(&d_cap, nt));
    PTW_CUDA(db.alloc(&d_dense, nt));
    PTW_CUDA(db.alloc(&d_cnt, nt));
    PTW_CUDA(db.alloc(&d_seg, nt + 1));
    PTW_CUDA(db.alloc(&d_fill, nt));
    PTW_CUDA(db.alloc(&d_tch, nt + 1));
    const uint64_t npc = nch * 8;  // warp pieces: 8 per chunk
    PTW_CUDA(db.alloc(&d_cc, std::max<uint64_t>(npc, 1)));
    PTW_CUDA(db.alloc(&d_hc, std::max<uint64_t>(npc, 1)));
    const int sp_count = ph->begin(PhaseTimer::kCount, st);
    PTW_CUDA(cudaMemcpyAsync(d_base, h_base, nt * 8ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_cap, h_cap, nt * 4ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_dense, dense_flags.data(), nt, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemcpyAsync(d_tch, tch.data(), (nt + 1) * 8ull, cudaMemcpyHostToDevice, st));
    PTW_CUDA(cudaMemsetAsync(d_cnt, 0, nt * 8ull, st));
    PTW_CUDA(cudaMemsetAsync(d_fill, 0, nt * 8ull, st));
    PTW_CUDA(cudaMemsetAsync(d_seg, 0, 8, st));
    // Pass 1: occupied entries per chunk and per table (+ histograms for top-k).
    if (k) {
        PTW_CUDA(db.alloc(&d_hist, (uint64_t)nt * kCountBins));
        PTW_CUDA(cudaMemsetAsync(d_hist, 0, (uint64_t)nt * kCountBins * 4, st));
        if (nch)
            k_tabs_count<true><<<(unsigned)nch, 256, 0, st>>>(d_slots, d_base, d_cap, d_dense, d_tch, nt, d_cnt, d_cc,
                                                             d_hc, d_hist);
    } else if (nch) {
        k_tabs_count<false><<<(unsigned)nch, 256, 0, st>>>(d_slots, d_base, d_cap, d_dense, d_tch, nt, d_cnt, d_cc,
                                                          d_hc, nullptr);
    }
    PTW_CUDA(cudaGetLastError());
    PTW_CUDA(cub_call([&](void *t, size_t &b) {
        return cub::DeviceScan::InclusiveSum(t, b, d_cnt, d_seg + 1, (int64_t)nt, st);
    }, st));
    PTW_CUDA(cudaMemcpyAsync(out->seg.data(), d_seg, (nt + 1) * 8ull, cudaMemcpyDeviceToHost, st));
    if (!k && nch) {
        // output position of every dense piece, sort-input position of every hash piece
        PTW_CUDA(db.alloc(&d_pos, npc));
        PTW_CUDA(db.alloc(&d_hpos, npc));
        PTW_CUDA(cub_call([&](void *t, size_t &b) {
            return cub::DeviceScan::ExclusiveSum(t, b, d_cc, d_pos, (int64_t)npc, st);
        }, st));
        PTW_CUDA(cub_call([&](void *t, size_t &b) {
            return cub::DeviceScan::ExclusiveSum(t, b, d_hc, d_hpos, (int64_t)npc, st);
        }, st));
    }
    ph->end(sp_count, st);
    PTW_CUDA(cudaStreamSynchronize(st));
    const uint64_t n_ent = out->seg[nt];
    // top-k: every table keeps its min(k, entries) largest counts
    std::vector<uint64_t> kseg;
    uint64_t n_out = n_ent;
    if (k && n_ent) {
        kseg.assign(nt + 1, 0);
        for (uint32_t i = 0; i < nt; ++i)
            kseg[i + 1] = kseg[i] + std::min<uint64_t>(k, out->seg[i + 1] - out->seg[i]);
        n_out = kseg[nt];
    }
    out->n = n_out;
    if (n_ent) {
        bool dst_pinned = false;  // the host lists are page-locked: copies run asynchronously
        if (out->device) {
            // the lists stay on the device: no host buffers, no copies
            if (out->pre_join) out->pre_join();
            out->pre_names.reset();
            out->pre_counts.reset();
        } else if (out->sink) {
            uint32_t *base = out->sink(n_out);
            if (!base) return fail(PTW_ENOMEM, "host staging of results failed");
            out->h_names = base;
            out->h_counts = base + n_out;
            dst_pinned = true;  // the sink hands out page-locked staging
        } else if (out->pre_names && n_out <= out->pre_cap) {
            // the buffers faulted in during the walk hold the lists
            const double tj = clk();
            out->pre_join();
            t_join = clk() - tj;
            out->names = std::move(out->pre_names);
            out->counts = std::move(out->pre_counts);
            out->h_names = out->names.get();
            out->h_counts = out->counts.get();
            out->cap = out->pre_cap;
            out->pinned = out->pre_pinned;
            dst_pinned = out->pinned;
            if (out->pinned) {
                out->touched = out->pre_cap;  // registered pages stay resident
            } else {
                release_tail(out->h_names, n_out * 4, out->pre_cap * 4);
                release_tail(out->h_counts, n_out * 4, out->pre_cap * 4);
                out->touched = n_out;  // the tail's pages were handed back
            }
        } else {
            if (out->pre_join) out->pre_join();
            out->pre_names.reset();
            out->pre_counts.reset();
            out->names.reset(new (std::nothrow) uint32_t[n_out]);  // no value-initialisation
            out->counts.reset(new (std::nothrow) uint32_t[n_out]);
            if (!out->names || !out->counts) return fail(PTW_ENOMEM, "host allocation of batch results failed");
            out->h_names = out->names.get();
            out->h_counts = out->counts.get();
            out->cap = out->touched = n_out;
            prefault.start({{out->h_names, n_out * 4}, {out->h_counts, n_out * 4}});
        }
        // The output lists: scratch of this call, or, for device-resident
        // results, arrays the results keep.
        auto alloc_out = [&](uint32_t **name, uint32_t **cnt, uint64_t count) -> cudaError_t {
            if (!out->device) {
                cudaError_t e = db.alloc(name, count);
                return e != cudaSuccess ? e : db.alloc(cnt, count);
            }
            cudaError_t e = out->d_names.alloc(count, st);
            if (e != cudaSuccess) return e;
            e = out->d_counts.alloc(count, st);
            *name = out->d_names.p;
            *cnt = out->d_counts.p;
            return e;
        };
        int name_bits = 1, q_bits = 1;
        while (name_bits < 32 && (1ull << name_bits) < g->dg.id_bound) ++name_bits;
        while ((1ull << q_bits) < nt) ++q_bits;
        uint32_t *o_name = nullptr, *o_cnt = nullptr;
        bool copied = false;  // the lists already reached the host (range copies)
        if (k) {
            // Top-k.  A histogram of each large table's counts (exact below
            // 256, 16 bins per octave above) gives the lowest bin that still
            // holds k entries; only entries in that bin or above are emitted
            // as keys, so the radix sort sees about k entries per table
            // instead of all of them.  The sort orders each table by count
            // (ties by name) and the first k are kept.
            uint32_t *d_thr;
            unsigned long long *d_sel, *d_sseg;
            const int sp_place = ph->begin(PhaseTimer::kPlace, st);
            PTW_CUDA(db.alloc(&d_thr, nt));
            PTW_CUDA(db.alloc(&d_sel, nt));
            PTW_CUDA(db.alloc(&d_sseg, nt + 1));
            PTW_CUDA(cudaMemsetAsync(d_sseg, 0, 8, st));
            k_tabs_thresh<<<(nt + 7) / 8, 256, 0, st>>>(d_cnt, d_hist, nt, k, d_thr, d_sel);
            PTW_CUDA(cudaGetLastError());
            PTW_CUDA(cub_call([&](void *t, size_t &b) {
                return cub::DeviceScan::InclusiveSum(t, b, d_sel, d_sseg + 1, (int64_t)nt, st);
            }, st));
            unsigned long long n_sel = 0;
            PTW_CUDA(cudaMemcpyAsync(&n_sel, d_sseg + nt, 8, cudaMemcpyDeviceToHost, st));
            PTW_CUDA(cudaStreamSynchronize(st));
            unsigned long long *e_key, *s_key;
            uint32_t *e_cnt, *s_cnt;
            PTW_CUDA(db.alloc(&e_key, n_sel));
            PTW_CUDA(db.alloc(&s_key, n_sel));
            PTW_CUDA(db.alloc(&e_cnt, n_sel));
            PTW_CUDA(db.alloc(&s_cnt, n_sel));
            // (table, ~count, name) in 64 bits: one sort, keys only
            const bool packed = q_bits + 32 + name_bits <= 64;
            k_tabs_place<true><<<(unsigned)nch, 256, 0, st>>>(d_slots, d_base, d_cap, d_dense, d_tch, nt, 0ull,
                                                             nullptr, nullptr, d_thr, d_sseg, d_fill, g->dg.int2name,
                                                             g->dg.names, name_bits, packed, nullptr, nullptr,
                                                             nullptr, nullptr, e_key, e_cnt);
            PTW_CUDA(cudaGetLastError());
            unsigned long long *d_kseg;
            PTW_CUDA(db.alloc(&d_kseg, nt + 1));
            PTW_CUDA(alloc_out(&o_name, &o_cnt, n_out));
            PTW_CUDA(cudaMemcpyAsync(d_kseg, kseg.data(), (nt + 1) * 8ull, cudaMemcpyHostToDevice, st));
            const unsigned sg = (unsigned)std::min<uint64_t>((n_sel + 255) / 256, (uint64_t)g->num_sms * 32);
            if (packed) {
                PTW_CUDA(cub_call([&](void *t, size_t &b) {
                    return cub::DeviceRadixSort::SortKeys(t, b, e_key, s_key, (int64_t)n_sel, 0,
                                                          q_bits + 32 + name_bits, st);
                }, st));
                k_topk_copy_packed<<<std::max(sg, 1u), 256, 0, st>>>(s_key, n_sel, name_bits, d_sseg, d_kseg, k,
                                                                     o_name, o_cnt);
            } else {
                // sort by (table, name), then stably by (table, ~count): equal
                // counts stay in name order
                PTW_CUDA(cub_call([&](void *t, size_t &b) {
                    return cub::DeviceRadixSort::SortPairs(t, b, e_key, s_key, e_cnt, s_cnt, (int64_t)n_sel, 0,
                                                           name_bits + q_bits, st);
                }, st));
                k_count_keys<<<std::max(sg, 1u), 256, 0, st>>>(s_key, s_cnt, n_sel, name_bits, e_key, e_cnt);
                PTW_CUDA(cudaGetLastError());
                PTW_CUDA(cub_call([&](void *t, size_t &b) {
                    return cub::DeviceRadixSort::SortPairs(t, b, e_key, s_key, e_cnt, s_cnt, (int64_t)n_sel, 0,
                                                           32 + q_bits, st);
                }, st));
                k_topk_copy<<<std::max(sg, 1u), 256, 0, st>>>(s_key, s_cnt, n_sel, d_sseg, d_kseg, k, o_name,
                                                              o_cnt);
            }
            PTW_CUDA(cudaGetLastError());
            ph->end(sp_place, st);
            out->seg = kseg;
        } else {
            // Full lists by name.  Dense tables are already in name order:
            // their nonzero counters go straight to the output.  Hash tables
            // put their entries into one range per table, each range is
            // sorted by name (a segmented sort of 32-bit names), and the
            // ranges are copied into their output segments.
            PTW_CUDA(alloc_out(&o_name, &o_cnt, n_ent));
            std::vector<uint64_t> hseg(nt + 1, 0);
            for (uint32_t i = 0; i < nt; ++i)
                hseg[i + 1] = hseg[i] + (dense_flags[i] ? 0 : out->seg[i + 1] - out->seg[i]);
            const uint64_t n_hash = hseg[nt];
            unsigned long long *d_hseg = nullptr;
            uint32_t *h_name = nullptr, *h_cnt = nullptr, *s_name = nullptr, *s_cnt = nullptr;
            if (n_hash) {
                PTW_CUDA(db.alloc(&h_name, n_hash));
                PTW_CUDA(db.alloc(&h_cnt, n_hash));
                PTW_CUDA(db.alloc(&s_name, n_hash));
                PTW_CUDA(db.alloc(&s_cnt, n_hash));
                PTW_CUDA(db.alloc(&d_hseg, nt + 1));
                PTW_CUDA(cudaMemcpyAsync(d_hseg, hseg.data(), (nt + 1) * 8ull, cudaMemcpyHostToDevice, st));
            }
            // Pass 2 and the hash sorts run over R ranges of consecutive tables
            // with about equal entries.  The lists of a range are final once
            // its kernels end, and they are a contiguous piece of the output
            // (tables are in output order), so with page-locked host lists
            // each range's copy to the host runs on a second stream while the
            // next range compacts.
            const uint32_t R = !out->device && dst_pinned && n_ent >= (16ull << 20) ? 4u : 1u;
            std::vector<uint32_t> tb(R + 1, nt);
            tb[0] = 0;
            for (uint32_t r = 1; r < R; ++r) {
                const uint64_t want = n_ent * r / R;
                tb[r] = (uint32_t)(std::upper_bound(out->seg.begin(), out->seg.begin() + nt + 1, want) -
                                   out->seg.begin() - 1);
                tb[r] = std::max(tb[r], tb[r - 1]);
            }
            cudaStream_t cs = st;
            if (R > 1) {
                if (!g->copy_stream) PTW_CUDA(cudaStreamCreateWithFlags(&g->copy_stream, cudaStreamNonBlocking));
                cs = g->copy_stream;
            }
            // On any return, copies still reading the device lists end before
            // those are freed (the frees are ordered on st, not on cs).
            struct CopyWait {
                cudaStream_t s;
                bool on;
                ~CopyWait()
                {
                    if (on) cudaStreamSynchronize(s);
                }
            } copy_wait{cs, R > 1};
            std::vector<cudaEvent_t> evs;
            struct EvFree {
                std::vector<cudaEvent_t> &e;
                ~EvFree()
                {
                    for (cudaEvent_t x : e) cudaEventDestroy(x);
                }
            } ev_free{evs};
            const int sp_place = ph->begin(PhaseTimer::kPlace, st);
            for (uint32_t r = 0; r < R; ++r) {
                const uint32_t t0 = tb[r], t1 = tb[r + 1];
                if (t0 >= t1) continue;
                const unsigned long long c0 = tch[t0], c1 = tch[t1];
                if (c1 > c0)
                    k_tabs_place<false><<<(unsigned)(c1 - c0), 256, 0, st>>>(
                        d_slots, d_base, d_cap, d_dense, d_tch, nt, c0, d_pos, d_hpos, nullptr, nullptr, nullptr,
                        g->dg.int2name, g->dg.names, name_bits, false, o_name, o_cnt, h_name, h_cnt, nullptr, nullptr);
                PTW_CUDA(cudaGetLastError());
                if (hseg[t1] > hseg[t0]) {
                    // segmented sorts over runs of whole tables of under 2^31 entries each
                    for (uint32_t u0 = t0; u0 < t1;) {
                        uint32_t u1 = u0 + 1;
                        while (u1 < t1 && hseg[u1 + 1] - hseg[u0] < (1ull << 31)) ++u1;
                        const uint64_t items = hseg[u1] - hseg[u0];
                        if (items) {
                            if (items >= (1ull << 31))
                                return fail(PTW_EINVAL, "a hash table holds 2^31 entries or more");
                            std::vector<unsigned long long> rel(u1 - u0 + 1);
                            for (uint32_t i = u0; i <= u1; ++i) rel[i - u0] = hseg[i] - hseg[u0];
                            unsigned long long *d_rel;
                            PTW_CUDA(db.alloc(&d_rel, rel.size()));
                            PTW_CUDA(cudaMemcpyAsync(d_rel, rel.data(), rel.size() * 8ull, cudaMemcpyHostToDevice,
                                                     st));
                            const uint64_t o = hseg[u0];
                            PTW_CUDA(cub_call([&](void *t, size_t &b) {
                                return cub::DeviceSegmentedSort::SortPairs(t, b, h_name + o, s_name + o, h_cnt + o,
                                                                           s_cnt + o, (int)items, (int)(u1 - u0),
                                                                           d_rel, d_rel + 1, st);
                            }, st));
                        }
                        u0 = u1;
                    }
                    const uint64_t nh = hseg[t1] - hseg[t0];
                    const unsigned hg = (unsigned)std::min<uint64_t>((nh + 255) / 256, (uint64_t)g->num_sms * 32);
                    k_place_hash<<<std::max(hg, 1u), 256, 0, st>>>(s_name, s_cnt, hseg[t0], hseg[t1], d_hseg, nt,
                                                                  d_seg, o_name, o_cnt);
                    PTW_CUDA(cudaGetLastError());
                }
                if (R > 1) {
                    const uint64_t e0 = out->seg[t0], e1 = out->seg[t1];
                    cudaEvent_t ev;
                    PTW_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
                    evs.push_back(ev);
                    PTW_CUDA(cudaEventRecord(ev, st));
                    PTW_CUDA(cudaStreamWaitEvent(cs, ev, 0));
                    if (e1 > e0) {
                        const int sp_copy = ph->begin(PhaseTimer::kCopy, cs);
                        PTW_CUDA(cudaMemcpyAsync(out->h_names + e0, o_name + e0, (e1 - e0) * 4,
                                                 cudaMemcpyDeviceToHost, cs));
                        PTW_CUDA(cudaMemcpyAsync(out->h_counts + e0, o_cnt + e0, (e1 - e0) * 4,
                                                 cudaMemcpyDeviceToHost, cs));
                        ph->end(sp_copy, cs);
                        ph->copy_bytes += (e1 - e0) * 8;
                    }
                }
            }
            ph->end(sp_place, st);
            if (R > 1) {
                // copies issued; wait for them here (the device buffers they read are freed below)
                PTW_CUDA(cudaStreamSynchronize(cs));
                copied = true;
            }
        }
        const double tj2 = clk();
        prefault.join();
        t_join += clk() - tj2;
        if (timing) {
            PTW_CUDA(cudaStreamSynchronize(st));
            t1 = clk();
        }
        if (!copied && !out->device) {
            const int sp_copy = ph->begin(PhaseTimer::kCopy, st);
            PTW_CUDA(cudaMemcpyAsync(out->h_names, o_name, n_out * 4, cudaMemcpyDeviceToHost, st));
            PTW_CUDA(cudaMemcpyAsync(out->h_counts, o_cnt, n_out * 4, cudaMemcpyDeviceToHost, st));
            ph->end(sp_copy, st);
            ph->copy_bytes += n_out * 8;
        }
        PTW_CUDA(cudaStreamSynchronize(st));
        if (timing) t2 = clk();
    }
    if (timing)
        std::fprintf(stderr,
                     "[ptw] compact %u tables (%zu dense), %llu entries: device %.1f ms (waiting for host pages "
                     "%.1f ms), d2h %.1f ms\n",
                     nt, (size_t)n_dense, (unsigned long long)n_ent, 1e3 * (t1 - t0), 1e3 * t_join, 1e3 * (t2 - t1));
    return PTW_OK;
}

uint64_t table_slots(double sp, uint32_t max_moves, int32_t app, double factor, uint64_t budget, uint32_t n);

TableSize dense_table(uint32_t n) { return TableSize{((uint64_t)n + 1) / 2, true}; }

TableSize count_table(double sp, uint32_t max_moves, int32_t app, double factor, uint64_t budget, uint32_t n,
                      uint32_t dense_ratio)
{
    const uint64_t hash = table_slots(sp, max_moves, app, factor, budget, n);
    const TableSize d = dense_table(n);
    if (d.slots <= dense_ratio * hash) return d;
    return TableSize{hash, false};
}

uint64_t table_slots(double sp, uint32_t max_moves, int32_t app, double factor, uint64_t budget, uint32_t n)
{
    const double len = max_moves ? std::min(1.0 / std::max(sp, 1e-12), (double)max_moves)
                                 : 1.0 / std::max(sp, 1e-12);
    const double per_walker = app == PTW_APP_VISITS ? len + 1.0 : 1.0;
    const double f = factor > 0 ? factor : 2.0;
    const double expect = std::ceil(f * per_walker * (double)budget) + 64.0;
    const uint64_t full_cap = next_pow2(2ull * n);
    return std::min(full_cap, std::max<uint64_t>(256, next_pow2((uint64_t)std::min(expect, 4e18))));
}


}  // namespace ptw

using namespace ptw;

namespace ptw {
namespace {

// ---- checkpoint file of a resumable batch ------------------------------------
//
// Header: magic "PTWBCK1\0", then a 64-bit key of everything the results
// depend on (graph: n, m, id bound and its names; configuration: sp, seed,
// app, max_moves, top_k; every query's source, id and budget).  Then one
// record per completed wave:
//   u32 'WAVE', u32 rerun (1 = dense rerun of overflowed queries),
//   u32 k_ok, u32 k_overflow, u64 moves (first-pass waves only), u64 entries,
//   u32 idx_ok[k_ok], u32 idx_overflow[k_overflow], u64 seg[k_ok + 1],
//   u32 names[entries], u32 counts[entries], u32 'DONE'.
// A record cut short (the process ended while writing it) is ignored and
// overwritten by the next append.
constexpr uint32_t kCkWave = 0x45564157u, kCkDone = 0x454E4F44u;
const char kCkMagic[8] = {'P', 'T', 'W', 'B', 'C', 'K', '1', '\0'};

struct Fnv {
    uint64_t h = 1469598103934665603ull;
    void add(const void *p, size_t n)
    {
        const unsigned char *c = (const unsigned char *)p;
        for (size_t i = 0; i < n; ++i) h = (h ^ c[i]) * 1099511628211ull;
    }
    template <typename T> void val(const T &x) { add(&x, sizeof x); }
};

uint64_t checkpoint_key(const ptw_graph *g, const ptw_query *q, uint32_t nq, const ptw_batch_cfg *cfg)
{
    Fnv f;
    f.val(g->dg.n);
    f.val(g->dg.m);
    f.val(g->dg.id_bound);
    f.add(g->h_names, (size_t)g->dg.n * 4);
    f.val(cfg->sp);
    f.val(cfg->seed);
    f.val(cfg->app);
    f.val(cfg->max_moves);
    f.val(cfg->top_k);
    f.val(nq);
    for (uint32_t i = 0; i < nq; ++i) {
        f.val(q[i].source);
        f.val(q[i].query_id);
        f.val(q[i].budget);
    }
    return f.h;
}

struct Checkpoint {
    FILE *f = nullptr;
    long good = 0;  // end of the last complete record
    ~Checkpoint()
    {
        if (f) std::fclose(f);
    }
};

template <typename T> bool rd(FILE *f, T *p, size_t n = 1) { return std::fread(p, sizeof(T), n, f) == n; }

// Opens (or creates) the checkpoint and loads its completed waves: their
// results become WaveResults, their queries are marked done, and queries
// that overflowed (and have no result yet) are marked for the dense rerun.
int checkpoint_open(const char *path, uint64_t key, uint32_t nq, Checkpoint &ck, std::vector<WaveResult> &waves,
                    std::vector<char> &done, std::vector<char> &dense_next, uint64_t *moves, uint32_t *n_waves)
{
    done.assign(nq, 0);
    dense_next.assign(nq, 0);
    ck.f = std::fopen(path, "r+b");
    if (!ck.f) {
        ck.f = std::fopen(path, "w+b");
        if (!ck.f) return fail(PTW_EIO, std::string("cannot create checkpoint ") + path);
        if (std::fwrite(kCkMagic, 1, 8, ck.f) != 8 || std::fwrite(&key, 8, 1, ck.f) != 1 || std::fflush(ck.f))
            return fail(PTW_EIO, std::string("cannot write checkpoint ") + path);
        ck.good = 16;
        return PTW_OK;
    }
    char magic[8];
    uint64_t k = 0;
    if (!rd(ck.f, magic, 8) || std::memcmp(magic, kCkMagic, 8) || !rd(ck.f, &k))
        return fail(PTW_EINVAL, std::string(path) + " is not a batch checkpoint");
    if (k != key)
        return fail(PTW_EINVAL, std::string(path) + " is the checkpoint of another batch (queries, "
                                                     "configuration or graph differ)");
    ck.good = 16;
    for (;;) {
        uint32_t hdr[4];
        uint64_t mv = 0, ne = 0;
        if (!rd(ck.f, hdr, 4) || hdr[0] != kCkWave || !rd(ck.f, &mv) || !rd(ck.f, &ne)) break;
        const uint32_t k_ok = hdr[2], k_ovf = hdr[3];
        if (k_ok > nq || k_ovf > nq) break;
        std::vector<uint32_t> ok(k_ok), ovf(k_ovf);
        WaveResult w;
        w.c.seg.resize(k_ok + 1ull);
        if (!rd(ck.f, ok.data(), k_ok) || !rd(ck.f, ovf.data(), k_ovf) || !rd(ck.f, w.c.seg.data(), k_ok + 1ull))
            break;
        if (w.c.seg[k_ok] != ne) break;
        w.c.names.reset(new uint32_t[std::max<uint64_t>(ne, 1)]);
        w.c.counts.reset(new uint32_t[std::max<uint64_t>(ne, 1)]);
        uint32_t tail = 0;
        if (!rd(ck.f, w.c.names.get(), ne) || !rd(ck.f, w.c.counts.get(), ne) || !rd(ck.f, &tail) ||
            tail != kCkDone)
            break;
        bool valid = true;
        for (uint32_t i : ok) valid = valid && i < nq;
        for (uint32_t i : ovf) valid = valid && i < nq;
        if (!valid) break;
        w.c.n = w.c.cap = w.c.touched = ne;
        w.c.h_names = w.c.names.get();
        w.c.h_counts = w.c.counts.get();
        w.idx = ok;
        w.overflow.assign(k_ok, 0);
        for (uint32_t i : ok) done[i] = 1;
        for (uint32_t i : ovf) dense_next[i] = 1;
        if (!hdr[1]) *moves += mv;
        ++*n_waves;
        waves.push_back(std::move(w));
        ck.good = std::ftell(ck.f);
    }
    for (uint32_t i = 0; i < nq; ++i)
        if (done[i]) dense_next[i] = 0;
    return PTW_OK;
}

// Appends the last wave of `waves` (its completed queries and those that
// overflowed) as one record, cutting off any partial record first.
int checkpoint_append(Checkpoint &ck, const WaveResult &w, bool rerun, uint64_t moves)
{
    std::vector<uint32_t> ok, ovf;
    std::vector<uint64_t> seg(1, 0);
    for (size_t k = 0; k < w.idx.size(); ++k) {
        if (w.overflow[k]) {
            ovf.push_back(w.idx[k]);
            continue;
        }
        ok.push_back(w.idx[k]);
        seg.push_back(seg.back() + (w.c.seg[k + 1] - w.c.seg[k]));
    }
    if (std::fflush(ck.f) || ftruncate(fileno(ck.f), ck.good) || std::fseek(ck.f, ck.good, SEEK_SET))
        return fail(PTW_EIO, "cannot position the batch checkpoint");
    const uint32_t hdr[4] = {kCkWave, rerun ? 1u : 0u, (uint32_t)ok.size(), (uint32_t)ovf.size()};
    const uint64_t ne = seg.back();
    bool good = std::fwrite(hdr, 4, 4, ck.f) == 4 && std::fwrite(&moves, 8, 1, ck.f) == 1 &&
                std::fwrite(&ne, 8, 1, ck.f) == 1 && std::fwrite(ok.data(), 4, ok.size(), ck.f) == ok.size() &&
                std::fwrite(ovf.data(), 4, ovf.size(), ck.f) == ovf.size() &&
                std::fwrite(seg.data(), 8, seg.size(), ck.f) == seg.size();
    for (int pass = 0; pass < 2 && good; ++pass) {
        const uint32_t *src = pass == 0 ? w.c.h_names : w.c.h_counts;
        for (size_t k = 0; k < w.idx.size() && good; ++k) {
            if (w.overflow[k]) continue;
            const uint64_t len = w.c.seg[k + 1] - w.c.seg[k];
            good = std::fwrite(src + w.c.seg[k], 4, len, ck.f) == len;
        }
    }
    good = good && std::fwrite(&kCkDone, 4, 1, ck.f) == 1 && std::fflush(ck.f) == 0 && fsync(fileno(ck.f)) == 0;
    if (!good) return fail(PTW_EIO, "cannot write the batch checkpoint");
    ck.good = std::ftell(ck.f);
    return PTW_OK;
}

// The batch, optionally resumable: with ckpt_path, completed waves are read
// from and appended to that file, and at most max_waves (0 = all) waves run
// in this call; *out stays null while queries remain.
int batch_impl(ptw_graph *g, const ptw_query *h_queries, uint32_t nq, const ptw_batch_cfg *cfg,
               const char *ckpt_path, uint32_t max_waves, ptw_batch **out)
{
    if (!cfg) return fail(PTW_EINVAL, "null argument");
    if (const int rc0 = check_stop(cfg->sp, cfg->max_moves)) return rc0;
    if (!g || !out) return fail(PTW_EINVAL, "null argument");
    *out = nullptr;
    if (nq && !h_queries) return fail(PTW_EINVAL, "null query table");
    if (cfg->app != PTW_APP_VISITS && cfg->app != PTW_APP_ENDPOINT) return fail(PTW_EINVAL, "unknown app");
    if (cfg->flags & ~PTW_BATCH_DEVICE_RESULTS) return fail(PTW_EINVAL, "unknown batch flags");
    PTW_CUDA(cudaSetDevice(g->device));
    const bool timing = std::getenv("PTW_TIMING") != nullptr;
    auto clk = [] { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); };
    const double t_enter = clk();
    double t_waves = 0, t_asm = 0;
    const uint32_t n = g->dg.n;
    const BatchTune bt = effective_tune(g);
    PhaseTimer ph;
    std::vector<WaveQuery> all(nq);
    for (uint32_t i = 0; i < nq; ++i) {
        const ptw_query &q = h_queries[i];
        if (q.budget < 1 || q.budget > kMaxBudget)
            return fail(PTW_EINVAL, "query " + std::to_string(i) + ": budget must be in [1, 2^28]");
        const uint32_t *p = std::lower_bound(g->h_names, g->h_names + n, q.source);
        if (p == g->h_names + n || *p != q.source)
            return fail(PTW_EINVAL, "query " + std::to_string(i) + ": source " + std::to_string(q.source) +
                                        " is not a vertex of the graph");
        all[i].index = i;
        all[i].src = g->h_idx2int[p - g->h_names];
        all[i].qid = q.query_id;
        all[i].budget = q.budget;
        // Dense when not larger than the hash table (a cut at twice its bytes
        // was 3% faster on the scale-22 batch but 7% slower in the serving
        // loop's top-k compaction).
        const TableSize ts = count_table(cfg->sp, cfg->max_moves, cfg->app, cfg->table_factor, q.budget, n,
                                         bt.dense_ratio);
        all[i].cap = ts.slots;
        all[i].dense = ts.dense;
    }
    uint64_t budget_bytes = cfg->table_bytes;
    if (budget_bytes == 0) {
        size_t fr = 0, tot = 0;
        PTW_CUDA(cudaMemGetInfo(&fr, &tot));
        budget_bytes = fr / 4;
    }
    ptw_batch *b = new (std::nothrow) ptw_batch();
    if (!b) return fail(PTW_ENOMEM, "host allocation failed");
    b->nq = nq;
    b->queries.assign(h_queries, h_queries + nq);
    b->device = (cfg->flags & PTW_BATCH_DEVICE_RESULTS) != 0;
    b->device_id = g->device;
    std::vector<WaveResult> waves;
    std::vector<uint32_t> overflow;
    const uint64_t thr = stop_threshold(cfg->sp);
    uint64_t moves = 0;
    float walk_ms = 0;
    // a resumable batch: completed waves come from its checkpoint
    Checkpoint ck;
    std::vector<char> done(nq, 0), dense_next(nq, 0);
    uint32_t waves_loaded = 0, waves_run = 0;
    if (ckpt_path) {
        const int rc0 = checkpoint_open(ckpt_path, checkpoint_key(g, h_queries, nq, cfg), nq, ck, waves, done,
                                        dense_next, &moves, &waves_loaded);
        if (rc0) {
            delete b;
            return rc0;
        }
    }
    auto budget_left = [&] { return max_waves == 0 || waves_run < max_waves; };
    PTW_CUDA(cudaEventRecord(g->ev[3], g->stream));
    int rc = PTW_OK;
    // Waves in query order, admitted while their tables fit the budget.
    uint32_t i = 0;
    auto skip_done = [&] {
        while (i < nq && (done[i] || dense_next[i])) ++i;
    };
    skip_done();
    while (i < nq && rc == PTW_OK && budget_left()) {
        std::vector<WaveQuery> wave;
        uint64_t bytes = 0;
        while (i < nq && (wave.empty() || bytes + all[i].cap * 8 <= budget_bytes) && wave.size() < (1u << 20)) {
            bytes += all[i].cap * 8;
            wave.push_back(all[i++]);
            skip_done();
        }
        uint64_t mv = 0;
        rc = run_wave(g, wave, cfg, thr, waves, overflow, &mv, &walk_ms, &ph);
        moves += mv;
        ++waves_run;
        if (rc == PTW_OK && ckpt_path) rc = checkpoint_append(ck, waves.back(), false, mv);
    }
    // Queries whose hash table filled run again with a dense array (which
    // cannot fill).
    std::vector<uint32_t> again;
    again.swap(overflow);
    for (uint32_t q = 0; q < nq; ++q)
        if (dense_next[q]) again.push_back(q);
    std::sort(again.begin(), again.end());
    size_t reran = 0;
    for (; reran < again.size() && rc == PTW_OK && budget_left(); ++reran) {
        WaveQuery w = all[again[reran]];
        const TableSize d = dense_table(n);
        w.cap = d.slots;
        w.dense = true;
        uint64_t m2 = 0;
        rc = run_wave(g, {w}, cfg, thr, waves, overflow, &m2, &walk_ms, &ph);
        ++waves_run;
        if (rc == PTW_OK && !overflow.empty()) rc = fail(PTW_EFULL, "count table overflow in a dense array");
        if (rc == PTW_OK && ckpt_path) rc = checkpoint_append(ck, waves.back(), true, 0);
    }
    if (rc == PTW_OK && (i < nq || reran < again.size())) {
        // the wave limit was reached with queries left: progress is in the checkpoint
        PTW_CUDA(cudaStreamSynchronize(g->stream));
        delete b;
        return PTW_OK;
    }
    t_waves = clk();
    if (rc == PTW_OK) rc = assemble(g, b, waves);
    t_asm = clk();
    if (rc != PTW_OK) {
        delete b;
        return rc;
    }
    PTW_CUDA(cudaEventRecord(g->ev[2], g->stream));
    PTW_CUDA(cudaEventSynchronize(g->ev[2]));
    uint64_t walkers = 0;
    for (uint32_t i = 0; i < nq; ++i) walkers += all[i].budget;
    b->top_k = cfg->top_k;
    b->stats.walkers = walkers;
    b->stats.moves = moves;
    b->stats.visits = cfg->app == PTW_APP_VISITS ? walkers + moves : walkers;
    float ms = 0;
    PTW_CUDA(cudaEventElapsedTime(&ms, g->ev[3], g->ev[2]));
    b->stats.total_ms = ms;
    b->stats.kernel_ms = walk_ms;  // walker kernels only; total_ms includes compaction and copies
    // the device arrays outlive this call and possibly the graph's stream:
    // everything on it has completed, so they are freed on the default stream
    b->d_names.st = b->d_counts.st = b->d_offsets.st = nullptr;
    double sums[PhaseTimer::kPhases], tail = 0;
    ph.sums(sums, &tail);
    ptw_batch_phases &P = b->phases;
    P.plan_ms = ph.plan_ms;
    P.device_ms = ms;
    P.upload_ms = sums[PhaseTimer::kUpload];
    P.walk_ms = sums[PhaseTimer::kWalk];
    P.count_ms = sums[PhaseTimer::kCount];
    P.place_ms = sums[PhaseTimer::kPlace];
    P.copy_ms = sums[PhaseTimer::kCopy];
    P.copy_tail_ms = tail;
    P.host_pages_ms = ph.host_pages_ms;
    P.copy_bytes = ph.copy_bytes;
    P.waves = (uint32_t)waves.size() - waves_loaded;
    P.reruns = (uint32_t)again.size();
    P.call_ms = 1e3 * (clk() - t_enter);
    if (timing)
        std::fprintf(stderr, "[ptw] batch of %u queries: %zu waves in %.1f ms, assemble %.1f ms, call %.1f ms\n", nq,
                     waves.size(), 1e3 * (t_waves - t_enter), 1e3 * (t_asm - t_waves), 1e3 * (clk() - t_enter));
    *out = b;
    return PTW_OK;
}

}  // namespace
}  // namespace ptw

extern "C" int ptw_ppr_batch(ptw_graph *g, const ptw_query *h_queries, uint32_t nq, const ptw_batch_cfg *cfg,
                             ptw_batch **out)
try {
    NvtxRange nvtx("ptw_ppr_batch");
    return batch_impl(g, h_queries, nq, cfg, nullptr, 0, out);
} catch (...) {
    return host_exception();
}

extern "C" int ptw_ppr_batch_resumable(ptw_graph *g, const ptw_query *h_queries, uint32_t nq,
                                       const ptw_batch_cfg *cfg, const char *checkpoint_path, uint32_t max_waves,
                                       ptw_batch **out)
try {
    NvtxRange nvtx("ptw_ppr_batch_resumable");
    if (out) *out = nullptr;
    if (!checkpoint_path) return fail(PTW_EINVAL, "null checkpoint path");
    if (cfg && (cfg->flags & PTW_BATCH_DEVICE_RESULTS))
        return fail(PTW_EINVAL, "a resumable batch keeps its results on the host (no PTW_BATCH_DEVICE_RESULTS)");
    return batch_impl(g, h_queries, nq, cfg, checkpoint_path, max_waves, out);
} catch (...) {
    return host_exception();
}

extern "C" int ptw_batch_info(const ptw_batch *b, uint32_t *nq, uint64_t *entries, ptw_walk_stats *stats)
try {
    if (!b) return fail(PTW_EINVAL, "null batch");
    if (nq) *nq = b->nq;
    if (entries) *entries = b->offsets.empty() ? 0 : b->offsets.back();
    if (stats) *stats = b->stats;
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_batch_export(const ptw_batch *b, uint64_t *h_offsets, uint32_t *h_names, uint32_t *h_counts)
try {
    if (!b) return fail(PTW_EINVAL, "null batch");
    const uint64_t n = b->offsets.empty() ? 0 : b->offsets.back();
    if (h_offsets) std::memcpy(h_offsets, b->offsets.data(), b->offsets.size() * 8);
    if (b->device) {
        if (!n || (!h_names && !h_counts)) return PTW_OK;
        PTW_CUDA(cudaSetDevice(b->device_id));
        if (h_names) PTW_CUDA(cudaMemcpy(h_names, b->d_names.p, n * 4, cudaMemcpyDeviceToHost));
        if (h_counts) PTW_CUDA(cudaMemcpy(h_counts, b->d_counts.p, n * 4, cudaMemcpyDeviceToHost));
        return PTW_OK;
    }
    if (h_names && n) std::memcpy(h_names, b->names.get(), n * 4);
    if (h_counts && n) std::memcpy(h_counts, b->counts.get(), n * 4);
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_batch_view(const ptw_batch *b, const uint64_t **offsets, const uint32_t **names,
                              const uint32_t **counts)
try {
    if (!b) return fail(PTW_EINVAL, "null batch");
    if (offsets) *offsets = b->offsets.data();
    if (names) *names = b->device ? nullptr : b->names.get();
    if (counts) *counts = b->device ? nullptr : b->counts.get();
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_batch_view_device(const ptw_batch *b, const uint64_t **d_offsets, const uint32_t **d_names,
                                     const uint32_t **d_counts)
try {
    if (!b) return fail(PTW_EINVAL, "null batch");
    if (!b->device) return fail(PTW_EINVAL, "the batch's results are in host memory (run without PTW_BATCH_DEVICE_RESULTS)");
    if (d_offsets) *d_offsets = reinterpret_cast<const uint64_t *>(b->d_offsets.p);
    if (d_names) *d_names = b->d_names.p;
    if (d_counts) *d_counts = b->d_counts.p;
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_batch_get_phases(const ptw_batch *b, ptw_batch_phases *out)
try {
    if (!b || !out) return fail(PTW_EINVAL, "null argument");
    *out = b->phases;
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" void ptw_batch_free(ptw_batch *b)
try {
    if (!b) return;
    if (b->device) {  // the pool memory goes back on the batch's device
        int prev = 0;
        const bool have_prev = cudaGetDevice(&prev) == cudaSuccess;
        cudaSetDevice(b->device_id);
        b->d_names.reset();
        b->d_counts.reset();
        b->d_offsets.reset();
        if (have_prev) cudaSetDevice(prev);
        cudaGetLastError();
    }
    delete b;
} catch (...) {
    delete b;
    host_exception();
}

extern "C" int ptw_graph_set_batch_tune(ptw_graph *g, const ptw_batch_tune *t)
try {
    if (!g || !t) return fail(PTW_EINVAL, "null argument");
    if (t->desc_walkers && (t->desc_walkers < 32 || t->desc_walkers > 65536))
        return fail(PTW_EINVAL, "batch tune: desc_walkers must be 0 or in [32, 65536]");
    if (t->blocks_per_sm > 64) return fail(PTW_EINVAL, "batch tune: blocks_per_sm must be in [0, 64]");
    if (t->dense_ratio > 64) return fail(PTW_EINVAL, "batch tune: dense_ratio must be in [0, 64]");
    if (t->ext_columns < 0 || t->ext_columns > 2) return fail(PTW_EINVAL, "batch tune: ext_columns must be 0, 1 or 2");
    g->btune = *t;
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_graph_get_batch_tune(const ptw_graph *g, ptw_batch_tune *t)
try {
    if (!g || !t) return fail(PTW_EINVAL, "null argument");
    *t = g->btune;
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_autotune_batch(ptw_graph *g, const ptw_query *q, uint32_t nq, const ptw_batch_cfg *cfg,
                                  ptw_batch_tune *best, double *best_ms)
try {
    NvtxRange nvtx("ptw_autotune_batch");
    if (!g || !cfg || (nq && !q)) return fail(PTW_EINVAL, "null argument");
    if (nq == 0) return fail(PTW_EINVAL, "the autotuner needs at least one query");
    ptw_batch_cfg c = *cfg;
    c.flags |= PTW_BATCH_DEVICE_RESULTS;  // results are discarded: no copies to the host
    const ptw_batch_tune saved = g->btune;
    // Device time of the whole batch under tune t: first upload to the end
    // of compaction (ev[3] -> ev[2] of the call).
    auto time_one = [&](const ptw_batch_tune &t, double *ms) -> int {
        int rc = ptw_graph_set_batch_tune(g, &t);
        if (rc) return rc;
        ptw_batch *b = nullptr;
        rc = ptw_ppr_batch(g, q, nq, &c, &b);
        if (rc) return rc;
        *ms = b->phases.device_ms;
        ptw_batch_free(b);
        return PTW_OK;
    };
    struct Cand {
        ptw_batch_tune t;
        double ms;
    };
    std::vector<Cand> all;
    double warm = 0;
    int rc = time_one(saved, &warm);  // maps the pool's memory, builds column copies
    if (rc) {
        g->btune = saved;
        return rc;
    }
    const ptw_batch_tune base = saved;
    auto run = [&](ptw_batch_tune t) -> int {
        double ms = 0;
        const int r = time_one(t, &ms);
        if (r == PTW_OK) all.push_back({t, ms});
        return r;
    };
    // Stage 1: descriptor size x group bytes.
    for (uint32_t dw : {128u, 256u, 512u, 1024u})
        for (uint64_t gbytes : {128ull << 20, 384ull << 20, 1024ull << 20, ~0ull}) {
            if (rc) break;
            ptw_batch_tune t = base;
            t.desc_walkers = dw;
            t.group_bytes = gbytes;
            t.blocks_per_sm = 0;
            t.dense_ratio = 1;
            t.ext_columns = 0;
            rc = run(t);
        }
    auto fastest = [&]() {
        return *std::min_element(all.begin(), all.end(), [](const Cand &a, const Cand &b) { return a.ms < b.ms; });
    };
    // Stage 2: blocks per SM x dense ratio x column layout around the best.
    if (rc == PTW_OK && !all.empty()) {
        const ptw_batch_tune b1 = fastest().t;
        for (uint32_t bps : {0u, 4u, 6u})
            for (uint32_t dr : {1u, 2u})
                for (int32_t ext : {1, 2}) {
                    if (rc) break;
                    ptw_batch_tune t = b1;
                    t.blocks_per_sm = bps;
                    t.dense_ratio = dr;
                    t.ext_columns = ext;
                    rc = run(t);
                }
    }
    if (rc != PTW_OK || all.empty()) {
        g->btune = saved;
        return rc ? rc : fail(PTW_EINVAL, "no batch tune could be timed");
    }
    // Stage 3: the three fastest again, three interleaved rounds; median.
    std::sort(all.begin(), all.end(), [](const Cand &a, const Cand &b) { return a.ms < b.ms; });
    const size_t top = std::min<size_t>(3, all.size());
    std::vector<std::vector<double>> again(top);
    for (int round = 0; round < 3 && rc == PTW_OK; ++round)
        for (size_t i = 0; i < top && rc == PTW_OK; ++i) {
            double ms = 0;
            rc = time_one(all[i].t, &ms);
            again[i].push_back(ms);
        }
    if (rc != PTW_OK) {
        g->btune = saved;
        return rc;
    }
    size_t pick = 0;
    double pick_ms = 0;
    for (size_t i = 0; i < top; ++i) {
        std::vector<double> v = again[i];
        v.push_back(all[i].ms);
        std::sort(v.begin(), v.end());
        const double med = v[v.size() / 2];
        if (i == 0 || med < pick_ms) {
            pick = i;
            pick_ms = med;
        }
    }
    g->btune = all[pick].t;
    if (best) *best = all[pick].t;
    if (best_ms) *best_ms = pick_ms;
    return PTW_OK;
} catch (...) {
    return host_exception();
}
