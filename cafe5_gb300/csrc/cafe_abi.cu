// C ABI and host runtime of the GB300 CAFE5 likelihood path.
//
// Mirrors what the reference does around its hot path, in one process on
// one GPU:
//   matrix_cache::precalculate_matrices / get_matrix / is_saturated
//     (src/matrix_cache.cpp:88-163)    -> device-resident matrix cache + K1
//   base_model / gamma_model ::infer_family_likelihoods
//     (src/base_model.cpp:53-100, src/gamma_core.cpp:168-237)
//                                        -> cafe_score: K1 + K3/K4 + finish
// and adds the batch-level boundary, S-binning and a serving loop.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <functional>
#include <numeric>
#include <random>
#include <unordered_set>

#include "runtime.h"

using namespace cafe;

namespace cafe {

const int kDefaultBins[] = {32, 64, 96, 128, 192, 256, 384, 512, 768, 1024};
const int kNumDefaultBins = sizeof(kDefaultBins) / sizeof(int);

// Stream that device buffers growing on this thread are ordered on (set
// while a request is enqueued): growth then neither synchronises the device
// nor waits for other requests' work.
thread_local cudaStream_t t_alloc_stream = nullptr;

AllocScope::AllocScope(cudaStream_t s) : prev(t_alloc_stream) { t_alloc_stream = s; }
AllocScope::~AllocScope() { t_alloc_stream = prev; }

// ---- MatCache
size_t MatCache::home(const MatKey& k) const {
    uint64_t h = (uint64_t)k.size * 0x9E3779B97F4A7C15ull ^ (uint64_t)k.lq * 0xC2B2AE3D27D4EB4Full ^
                 (uint64_t)k.tq * 0x165667B19E3779F9ull;
    h ^= h >> 33;   // 64-bit finaliser (xor-shift-multiply)
    h *= 0xFF51AFD7ED558CCDull;
    h ^= h >> 33;
    return (size_t)h & mask_;
}
void MatCache::grow(size_t cap) {
    std::vector<Slot> old_s;
    std::vector<MatEntry> old_v;
    old_s.swap(slots_);
    old_v.swap(vals_);
    slots_.assign(cap, Slot());
    vals_.assign(cap, MatEntry());
    mask_ = cap - 1;
    n_ = 0;
    for (size_t i = 0; i < old_s.size(); ++i)
        if (old_s[i].used) {
            auto r = try_emplace(old_s[i].key);
            *r.first = old_v[i];
        }
}
void MatCache::reserve(size_t n_entries) {
    // fourfold growth: a long search keeps adding keys, and every growth
    // rehashes the whole table
    size_t cap = slots_.empty() ? 1024 : slots_.size();
    while (cap < 2 * n_entries) cap *= 4;
    if (cap != slots_.size()) grow(cap);
}
void MatCache::prefetch(const MatKey& k) const {
    if (slots_.empty()) return;
    const size_t i = home(k);
    __builtin_prefetch(&slots_[i]);
    __builtin_prefetch(&vals_[i]);
}
MatEntry* MatCache::find(const MatKey& k) {
    if (slots_.empty()) return nullptr;
    for (size_t i = home(k);; i = (i + 1) & mask_) {
        if (!slots_[i].used) return nullptr;
        if (slots_[i].key == k) return &vals_[i];
    }
}
std::pair<MatEntry*, bool> MatCache::try_emplace(const MatKey& k) {
    if (2 * (n_ + 1) > slots_.size()) reserve(n_ + 1);
    for (size_t i = home(k);; i = (i + 1) & mask_) {
        if (!slots_[i].used) {
            slots_[i].used = true;
            slots_[i].key = k;
            vals_[i] = MatEntry();
            ++n_;
            return {&vals_[i], true};
        }
        if (slots_[i].key == k) return {&vals_[i], false};
    }
}
void MatCache::erase(const MatKey& k) {
    if (slots_.empty()) return;
    size_t i = home(k);
    for (;; i = (i + 1) & mask_) {
        if (!slots_[i].used) return;
        if (slots_[i].key == k) break;
    }
    // backward shift: pull later members of the probe run into the hole
    for (size_t j = (i + 1) & mask_; slots_[j].used; j = (j + 1) & mask_) {
        const size_t h = home(slots_[j].key);
        const bool movable = (i <= j) ? (h <= i || h > j) : (h <= i && h > j);
        if (movable) {
            slots_[i] = slots_[j];
            vals_[i] = vals_[j];
            i = j;
        }
    }
    slots_[i].used = false;
    --n_;
}
void MatCache::clear() {
    // keep the table's size (a reset cache refills to about the same size)
    for (Slot& sl : slots_) sl.used = false;
    n_ = 0;
}

DevBuf::~DevBuf() {
    if (p) cudaFree(p);
}
cudaError_t DevBuf::reserve(size_t n) {
    if (n <= bytes) return cudaSuccess;
    const cudaStream_t s = t_alloc_stream;
    if (p) {
        if (s) cudaFreeAsync(p, s);
        else cudaFree(p);
    }
    p = nullptr;
    // geometric growth: request sizes that creep up (merged batches) cost
    // O(log) reallocations
    size_t want = std::max<size_t>(std::max<size_t>(n, bytes + bytes / 2), 256);
    bytes = 0;
    cudaError_t e = s ? cudaMallocAsync(&p, want, s) : cudaMalloc(&p, want);
    if (e != cudaSuccess && want > n) {
        cudaGetLastError();
        want = n;
        e = s ? cudaMallocAsync(&p, want, s) : cudaMalloc(&p, want);
    }
    if (e != cudaSuccess) {
        p = nullptr;
        cudaGetLastError();
        return e;
    }
    bytes = want;
    return cudaSuccess;
}
PinnedBuf::~PinnedBuf() {
    if (p) cudaFreeHost(p);
}
cudaError_t PinnedBuf::reserve(size_t n) {
    if (n <= bytes) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
    size_t want = std::max<size_t>(n * 2, 4096);
    cudaError_t e = cudaMallocHost(&p, want);
    if (e != cudaSuccess) {
        p = nullptr;
        cudaGetLastError();
        return e;
    }
    bytes = want;
    return cudaSuccess;
}
Workspace::~Workspace() {
    for (auto& g : graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    if (stream_hi) cudaStreamDestroy(stream_hi);
    if (stream_lo) cudaStreamDestroy(stream_lo);
    if (ev_start) cudaEventDestroy(ev_start);
    if (ev_stop) cudaEventDestroy(ev_stop);
    if (ev_staged) cudaEventDestroy(ev_staged);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_jobs) cudaEventDestroy(ev_jobs);
    if (build) cudaStreamDestroy(build);
    for (int q = 0; q < kAux; ++q) {
        if (aux[q]) cudaStreamDestroy(aux[q]);
        if (ev_join[q]) cudaEventDestroy(ev_join[q]);
    }
}
int Workspace::init(int device) {
    (void)device;
    // pruning streams at the highest priority, K1 builds at the lowest: a
    // build overlapping an earlier request's pruning only fills what the
    // pruning CTAs leave free
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (cudaStreamCreateWithPriority(&stream_hi, cudaStreamNonBlocking, greatest) != cudaSuccess) return CAFE_ERR_CUDA;
    if (cudaStreamCreateWithPriority(&stream_lo, cudaStreamNonBlocking, std::min(least, greatest + 1)) != cudaSuccess)
        return CAFE_ERR_CUDA;
    stream = stream_hi;
    if (cudaEventCreate(&ev_start) != cudaSuccess) return CAFE_ERR_CUDA;
    if (cudaEventCreate(&ev_stop) != cudaSuccess) return CAFE_ERR_CUDA;
    if (cudaEventCreateWithFlags(&ev_staged, cudaEventDisableTiming) != cudaSuccess) return CAFE_ERR_CUDA;
    if (cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming) != cudaSuccess) return CAFE_ERR_CUDA;
    if (cudaEventCreateWithFlags(&ev_jobs, cudaEventDisableTiming) != cudaSuccess) return CAFE_ERR_CUDA;
    if (cudaStreamCreateWithPriority(&build, cudaStreamNonBlocking, least) != cudaSuccess) return CAFE_ERR_CUDA;
    for (int q = 0; q < kAux; ++q) {
        if (cudaStreamCreateWithPriority(&aux[q], cudaStreamNonBlocking, greatest) != cudaSuccess) return CAFE_ERR_CUDA;
        if (cudaEventCreateWithFlags(&ev_join[q], cudaEventDisableTiming) != cudaSuccess) return CAFE_ERR_CUDA;
    }
    return CAFE_OK;
}

cudaEvent_t Profiler::get() {
    if (!pool.empty()) {
        cudaEvent_t e = pool.back();
        pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}
void Profiler::begin(int kind, cudaStream_t s, cudaEvent_t* a) {
    (void)kind;
    *a = nullptr;
    if (!on) return;
    *a = get();
    cudaEventRecord(*a, s);
}
void Profiler::end(int kind, cudaStream_t s, cudaEvent_t a) {
    acc.launches++;
    if (!on || !a) return;
    cudaEvent_t b = get();
    cudaEventRecord(b, s);
    pending.push_back({kind, {a, b}});
}
void Profiler::collect() {
    for (auto& p : pending) {
        cudaEventSynchronize(p.second.second);
        float ms = 0;
        cudaEventElapsedTime(&ms, p.second.first, p.second.second);
        switch (p.first) {
            case 0: acc.matrix_ms += ms; break;
            case 1: acc.prune_ms += ms; acc.prune_launches++; break;
            case 2: acc.finish_ms += ms; break;
            default: acc.other_ms += ms; break;
        }
        pool.push_back(p.second.first);
        pool.push_back(p.second.second);
    }
    pending.clear();
}

cudaError_t launch_fill(double* p, int64_t n, double v, cudaStream_t s);
cudaError_t launch_fill_i32(int32_t* p, int64_t n, int32_t v, cudaStream_t s);

}  // namespace cafe

namespace {

int fail(cafe_ctx* C, int code, const char* fmt, ...) {
    if (C) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        C->last_error = buf;
    }
    return code;
}

int cuda_fail(cafe_ctx* C, cudaError_t e, const char* what) {
    if (e == cudaErrorMemoryAllocation) return fail(C, CAFE_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
    return fail(C, CAFE_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(expr, what)                                        \
    do {                                                      \
        cudaError_t _e = (expr);                              \
        if (_e != cudaSuccess) return cuda_fail(C, _e, what); \
    } while (0)

// Post-order of internal nodes, children with the larger slot need first
// (Sethi-Ullman), and greedy slot reuse.
void build_plan(TreeHost& T) {
    const int n = T.n_nodes;
    std::vector<int> need(n, 0);
    std::function<int(int)> rec_need = [&](int v) -> int {
        if (T.children[v].empty()) return need[v] = 0;
        std::vector<int> cn;
        for (int c : T.children[v]) cn.push_back(rec_need(c));
        std::sort(cn.begin(), cn.end(), std::greater<int>());
        int m = 0;
        for (size_t i = 0; i < cn.size(); ++i) m = std::max(m, cn[i] + (int)i);
        int held = 0;
        for (int c : T.children[v]) held += T.children[c].empty() ? 0 : 1;
        return need[v] = std::max(m, held + 1);
    };
    rec_need(T.root);
    std::vector<int> order;
    std::function<void(int)> visit = [&](int v) {
        if (T.children[v].empty()) return;
        std::vector<int> cs = T.children[v];
        std::stable_sort(cs.begin(), cs.end(), [&](int a, int b) { return need[a] > need[b]; });
        for (int c : cs) visit(c);
        order.push_back(v);
    };
    visit(T.root);
    T.internal.assign(order.begin(), order.end());
    T.cstart.assign(1, 0);
    T.child.clear();
    T.slot.assign(n, -1);
    T.max_children = 0;
    std::vector<int> free_slots;
    int n_slots = 0;
    for (int v : order) {
        for (int c : T.children[v]) T.child.push_back(c);   // product order: descendant order
        T.cstart.push_back((int)T.child.size());
        T.max_children = std::max<int>(T.max_children, (int)T.children[v].size());
        int s;
        if (!free_slots.empty()) {
            auto it = std::min_element(free_slots.begin(), free_slots.end());
            s = *it;
            free_slots.erase(it);
        } else {
            s = n_slots++;
        }
        T.slot[v] = s;
        for (int c : T.children[v])
            if (!T.children[c].empty()) free_slots.push_back(T.slot[c]);
    }
    T.n_slots = n_slots;
}

int upload_plan(cafe_ctx* C, TreeHost& T) {
    const int ni = (int)T.internal.size();
    std::vector<int32_t> blob;
    auto put = [&](const std::vector<int32_t>& v) {
        size_t off = blob.size();
        blob.insert(blob.end(), v.begin(), v.end());
        return off;
    };
    size_t o_int = put(T.internal), o_cs = put(T.cstart), o_ch = put(T.child), o_lc = put(T.leaf_col),
           o_sl = put(T.slot);
    CK(T.d_plan.reserve(blob.size() * sizeof(int32_t)), "tree plan");
    CK(cudaMemcpy(T.d_plan.p, blob.data(), blob.size() * sizeof(int32_t), cudaMemcpyHostToDevice), "tree plan");
    const int32_t* b = T.d_plan.as<int32_t>();
    T.plan.n_nodes = T.n_nodes;
    T.plan.n_internal = ni;
    T.plan.n_leaves = T.n_leaves;
    T.plan.root = T.root;
    T.plan.n_slots = T.n_slots;
    T.plan.max_children = T.max_children;
    T.plan.internal = b + o_int;
    T.plan.cstart = b + o_cs;
    T.plan.child = b + o_ch;
    T.plan.leaf_col = b + o_lc;
    T.plan.slot = b + o_sl;
    return CAFE_OK;
}

int compute_bins(cafe_ctx* C, FamSet& S) {
    BinPlan& B = S.bins;
    const int64_t F = S.F;
    std::vector<int> wf(F), rf(F);
    for (int64_t f = 0; f < F; ++f) {
        const int mx = S.max_count[f];
        const int need = (int)std::ceil(1.2 * mx) + 20 + 1;
        int w = kDefaultBins[kNumDefaultBins - 1];
        for (int i = 0; i < kNumDefaultBins; ++i)
            if (kDefaultBins[i] >= need) {
                w = kDefaultBins[i];
                break;
            }
        wf[f] = w;
        const int Sf = w - 1;
        rf[f] = std::min(Sf, std::max(30, (int)std::rint(mx * 1.25)));
    }
    std::vector<int64_t> perm(F);
    std::iota(perm.begin(), perm.end(), 0);
    std::stable_sort(perm.begin(), perm.end(), [&](int64_t a, int64_t b) { return wf[a] < wf[b]; });
    B.widths.clear();
    B.bin_first.clear();
    B.bin_count.clear();
    B.W_max = 0;
    for (int64_t i = 0; i < F; ++i) {
        const int w = wf[perm[i]];
        if (B.widths.empty() || B.widths.back() != w) {
            B.widths.push_back(w);
            B.bin_first.push_back(i);
            B.bin_count.push_back(0);
        }
        B.bin_count.back()++;
        B.W_max = std::max(B.W_max, w);
    }
    std::vector<int32_t> rf32(rf.begin(), rf.end());
    CK(B.d_perm.reserve(std::max<int64_t>(F, 1) * sizeof(int64_t)), "bins");
    CK(B.d_famR.reserve(std::max<int64_t>(F, 1) * sizeof(int32_t)), "bins");
    if (F) {
        CK(cudaMemcpy(B.d_perm.p, perm.data(), F * sizeof(int64_t), cudaMemcpyHostToDevice), "bins");
        CK(cudaMemcpy(B.d_famR.p, rf32.data(), F * sizeof(int32_t), cudaMemcpyHostToDevice), "bins");
    }
    return CAFE_OK;
}

int prepare_set(cafe_ctx* C, FamSet& S) {
    const int64_t F = S.F;
    const int nl = S.n_leaves;
    S.max_count.assign(F, 0);
    for (int64_t f = 0; f < F; ++f) {
        int m = 0;
        for (int c = 0; c < nl; ++c) m = std::max(m, S.h_counts[f * nl + c]);
        S.max_count[f] = m;
    }
    // dedupe (build_reference_list, src/base_model.cpp:27-51), hashed
    std::vector<int64_t> ref(F);
    std::unordered_map<uint64_t, std::vector<int64_t>> buckets;
    S.unique.clear();
    for (int64_t f = 0; f < F; ++f) {
        const int32_t* row = &S.h_counts[f * nl];
        uint64_t h = 1469598103934665603ull;
        for (int c = 0; c < nl; ++c) h = (h ^ (uint32_t)row[c]) * 1099511628211ull;
        auto& b = buckets[h];
        int64_t found = -1;
        for (int64_t g : b)
            if (std::memcmp(&S.h_counts[g * nl], row, sizeof(int32_t) * nl) == 0) {
                found = g;
                break;
            }
        if (found < 0) {
            b.push_back(f);
            S.unique.push_back(f);
            ref[f] = f;
        } else {
            ref[f] = found;
        }
    }
    std::vector<int64_t> ident(F);
    std::iota(ident.begin(), ident.end(), 0);
    const size_t nb = std::max<int64_t>(F, 1) * sizeof(int64_t);
    CK(S.d_ref.reserve(nb), "families");
    CK(S.d_identity.reserve(nb), "families");
    CK(S.d_unique.reserve(nb), "families");
    if (F) {
        CK(cudaMemcpy(S.d_ref.p, ref.data(), F * sizeof(int64_t), cudaMemcpyHostToDevice), "families");
        CK(cudaMemcpy(S.d_identity.p, ident.data(), F * sizeof(int64_t), cudaMemcpyHostToDevice), "families");
        CK(cudaMemcpy(S.d_unique.p, S.unique.data(), S.unique.size() * sizeof(int64_t), cudaMemcpyHostToDevice),
           "families");
    }
    return compute_bins(C, S);
}

// Matrix cache: look up or schedule (size, lambda, t). Caller holds C->mu.
// Matrices a request still has to build: their keys and the cache entries
// already inserted for them (filled by cache_build).
struct PendingJobs {
    std::vector<MatKey> keys;
    std::vector<MatEntry*> entries;
};

void cache_reset(cafe_ctx* C) {
    for (auto& g : C->gens) {
        for (auto& sl : g.slabs) {
            cudaFree(sl.p);
            if (sl.ev_alloc) cudaEventDestroy(sl.ev_alloc);
        }
        g.slabs.clear();
        g.cur = 0;
        g.n_marks = 0;
    }
    C->gen = 0;
    for (cudaEvent_t e : C->batch_events) cudaEventDestroy(e);
    C->batch_events.clear();
    C->cache.clear();
    C->cache_bytes = 0;
}

// Empties the cache and moves it to the other generation of slabs, without
// a device synchronisation: every stream that may still read a matrix of
// the generation being left (each workspace's two request streams;
// auxiliary streams join them before a request ends) or write one (the
// build streams) records that generation's marks, and builds into a
// generation wait for its marks (cache_build_impl) -- recorded a whole
// generation earlier, so normally long complete. Caller holds C->mu, so no
// request is between looking up its matrices and enqueueing the work that
// reads them.
cudaError_t cache_recycle(cafe_ctx* C) {
    std::vector<cudaStream_t> streams;
    auto add = [&](const Workspace* w) {
        if (!w) return;
        for (cudaStream_t s : {w->stream_hi, w->stream_lo, w->build})
            if (s) streams.push_back(s);
    };
    for (const auto& w : C->ws) add(w.get());
    add(C->ws_alt.get());
    cafe_ctx::SlabGen& old = C->gens[C->gen];
    while (old.marks.size() < streams.size()) {
        cudaEvent_t e;
        const cudaError_t err = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        if (err != cudaSuccess) return err;
        old.marks.push_back(e);
    }
    for (size_t i = 0; i < streams.size(); ++i) {
        const cudaError_t err = cudaEventRecord(old.marks[i], streams[i]);
        if (err != cudaSuccess) return err;
    }
    old.n_marks = (int)streams.size();
    C->gen ^= 1;
    cafe_ctx::SlabGen& g = C->gens[C->gen];
    for (auto& sl : g.slabs) sl.used = 0;
    g.cur = 0;
    // (waits enqueued on these events keep what they captured)
    for (cudaEvent_t e : C->batch_events) cudaEventDestroy(e);
    C->batch_events.clear();
    C->cache.clear();
    C->cache_bytes = 0;
    return cudaSuccess;
}

int cache_build_impl(cafe_ctx* C, Workspace& ws, PendingJobs& P);

// Allocate and enqueue K1 for the pending keys on `ws`. On failure the
// keys' placeholder entries leave the cache again.
int cache_build(cafe_ctx* C, Workspace& ws, PendingJobs& P) {
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = cache_build_impl(C, ws, P);
    if (C->prof.on && ws.sync)
        C->prof.acc.host_build_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (rc) {
        for (const MatKey& k : P.keys) C->cache.erase(k);
        P.keys.clear();
        P.entries.clear();
    }
    return rc;
}

int cache_build_impl(cafe_ctx* C, Workspace& ws, PendingJobs& P) {
    const size_t n = P.keys.size();
    if (!n) return CAFE_OK;
    size_t total = 0;
    int max_size = 0;
    for (auto& k : P.keys) {
        total += (size_t)k.size * k.size * sizeof(double);
        max_size = std::max(max_size, k.size);
    }
    // a build of up to 1 GB of matrices runs on the workspace's build
    // stream, so it fills the gaps the previous request's pruning leaves
    // (16-candidate config-1 steps: 3.43 -> 3.24 ms; 4-candidate config-2
    // steps, 0.5 GB of side-512 matrices beside the wide bins' walks: 4.0 ->
    // 3.5 ms); a larger one runs in line, since streaming gigabytes of
    // matrices beside the pruning evicts its working set from L2
    // (64-candidate K = 8 rounds: 116 -> 127 ms).
    // Synchronous calls build in line (nothing of theirs to hide behind), and
    // so do profiled calls, so each kernel is timed alone. Slab and
    // job-table growth follow the build's stream; every user of the
    // matrices waits on the ready event below.
    const bool beside = ws.build && !ws.build_inline && !(C->prof.on && ws.sync) && total <= ((size_t)1 << 30);
    const cudaStream_t bs = beside ? ws.build : ws.stream;
    AllocScope scope(bs);
    if (ws.jobs_pending) {   // the previous build has read h_jobs and ws.jobs
        CK(cudaEventSynchronize(ws.ev_jobs), "jobs");
        ws.jobs_pending = false;
    }
    // bump allocation from large slabs of the current generation (no
    // cudaMalloc per evaluation); each new slab is twice the last, up to
    // 4 GB, so a generation fills up with few allocations while a small
    // workload keeps a small footprint
    const size_t need = (total + 255) & ~(size_t)255;
    cafe_ctx::SlabGen& G = C->gens[C->gen];
    while (G.cur < G.slabs.size() && G.slabs[G.cur].used + need > G.slabs[G.cur].size) G.cur++;
    if (G.cur == G.slabs.size()) {
        Slab sl;
        const size_t grown = G.slabs.empty() ? ((size_t)256 << 20) : std::min(2 * G.slabs.back().size, (size_t)4 << 30);
        sl.size = std::max(need, grown);
        // stream-ordered when a request is being enqueued: requests on other
        // streams reach these matrices only through the build's ready event
        CK(t_alloc_stream ? cudaMallocAsync(&sl.p, sl.size, t_alloc_stream) : cudaMalloc(&sl.p, sl.size),
           "matrix cache");
        sl.used = 0;
        CK(cudaEventCreateWithFlags(&sl.ev_alloc, cudaEventDisableTiming), "event");
        CK(cudaEventRecord(sl.ev_alloc, bs), "event");
        G.slabs.push_back(sl);
    }
    Slab& slab = G.slabs[G.cur];
    // a slab another workspace allocated is written only after its allocation
    CK(cudaStreamWaitEvent(bs, slab.ev_alloc, 0), "event");
    // recycled memory is written only after everything that used it the
    // last time the cache held this generation
    for (int q = 0; q < G.n_marks; ++q) CK(cudaStreamWaitEvent(bs, G.marks[q], 0), "event");
    void* chunk = static_cast<char*>(slab.p) + slab.used;
    slab.used += need;
    C->cache_bytes += total;
    cudaEvent_t ready = nullptr;
    CK(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming), "event");
    C->batch_events.push_back(ready);
    const int batch = (int)C->batch_events.size() - 1;
    CK(ws.h_jobs.reserve(n * sizeof(MatrixJob)), "jobs");
    CK(ws.jobs.reserve(n * sizeof(MatrixJob)), "jobs");
    MatrixJob* J = ws.h_jobs.as<MatrixJob>();
    char* cur = static_cast<char*>(chunk);
    for (size_t i = 0; i < n; ++i) {
        const MatKey& k = P.keys[i];
        MatrixJob j{};
        j.lambda = (double)k.lq / 1000000000.0;
        j.t = (double)k.tq / 1000.0;
        j.dst = reinterpret_cast<double*>(cur);
        j.size = k.size;
        J[i] = j;
        P.entries[i]->d = j.dst;
        P.entries[i]->chunk = batch;
        cur += (size_t)k.size * k.size * sizeof(double);
    }
    CK(cudaMemcpyAsync(ws.jobs.p, J, n * sizeof(MatrixJob), cudaMemcpyHostToDevice, bs), "jobs");
    const bool prof = ws.sync;
    cudaEvent_t ev;
    if (prof) C->prof.begin(0, bs, &ev);
    CK(launch_matrix_build(ws.jobs.as<MatrixJob>(), (int)n, max_size, bs), "matrix build");
    if (prof) {
        C->prof.end(0, bs, ev);
        C->prof.acc.matrices_built += (int64_t)n;
    }
    // h_jobs and ws.jobs stay untouched until this build has read them (the
    // next build may run on the other stream, so stream order alone does
    // not protect a reallocation of ws.jobs)
    if (ws.ev_jobs) {
        CK(cudaEventRecord(ws.ev_jobs, bs), "event");
        ws.jobs_pending = true;
    }
    // every stream that reads these matrices orders itself after this build
    CK(cudaEventRecord(ready, bs), "event");
    P.keys.clear();
    P.entries.clear();
    return CAFE_OK;
}

MatKey make_key(int size, double lambda, double t) {
    MatKey k;
    k.size = size;
    k.lq = (long)(lambda * 1000000000);
    k.tq = (long)(t * 1000);
    return k;
}

// The cache entry of key k; a key seen for the first time gets an entry
// now and is queued for the next cache_build.
MatEntry* schedule(cafe_ctx* C, PendingJobs& P, const MatKey& k) {
    auto ins = C->cache.try_emplace(k);
    MatEntry* e = ins.first;
    if (ins.second) {
        P.keys.push_back(k);
        P.entries.push_back(e);
    }
    return e;
}

// Over the cap: start a fresh cache in the other generation of slabs before
// a request inserts its keys (the reference's cache lives for one
// evaluation; keeping matrices across calls is only a speed-up). `bytes`
// bounds what the request may add. Recycling keeps the memory bounded and
// spares the allocations (about 1 ms of host time per GB of new device
// memory).
void cache_make_room(cafe_ctx* C, size_t bytes) {
    if (!C->cache_cap || C->cache_bytes + bytes <= C->cache_cap || C->cache_bytes == 0) return;
    if (cache_recycle(C) != cudaSuccess) cudaGetLastError();
}

struct ScoreInfo {
    int64_t F = 0;
    int K = 1;
    int B = 1;                          // candidates scored together
    std::vector<char> cand_rejected;    // per candidate: +inf without pruning
    std::vector<int> cand_status;       // per candidate rejection status
    bool rejected = false;              // every candidate rejected
    int reject_status = CAFE_OK;
    bool scaled = false;
    size_t footprint = 0;
    int64_t n_fallback = 0;
    const int32_t* d_tail = nullptr;   // tensor-core pass: [status, fallback families, fallback tiles]
};

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// 2D FP32 tensor map [rows][cols] with boxes of box_rows x box_cols:
// box_cols = 16 uses the 64-byte swizzle, box_cols = 32 the 128-byte swizzle.
int encode_map(cafe_ctx* C, CUtensorMap* m, const float* base, int64_t rows, int cols, int box_cols, int box_rows,
               int64_t depth_stride = 0) {
    static EncodeTiledFn enc = nullptr;
    if (!enc) {
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", (void**)&enc, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            !enc) {
            enc = nullptr;
            return fail(C, CAFE_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
        }
    }
    // depth_stride > 0: a third dimension of 2 planes that many elements
    // apart (one box holds the same rows of both)
    cuuint64_t dims[3] = {(cuuint64_t)cols, (cuuint64_t)rows, 2};
    cuuint64_t strides[2] = {(cuuint64_t)cols * sizeof(float), (cuuint64_t)depth_stride * sizeof(float)};
    if (box_rows < 1 || box_rows > 256 || box_rows > rows) return fail(C, CAFE_ERR_INVALID, "tensor map box of %d rows", box_rows);
    if (depth_stride < 0 || (depth_stride * sizeof(float)) % 16) return fail(C, CAFE_ERR_INVALID, "tensor map plane stride");
    cuuint32_t box[3] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows, 2};
    cuuint32_t es[3] = {1, 1, 1};
    const CUtensorMapSwizzle sw = box_cols == 16 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B;
    const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, depth_stride > 0 ? 3 : 2, (void*)base, dims, strides, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(C, CAFE_ERR_CUDA, "tensor map encode failed (%d)", (int)r);
    return CAFE_OK;
}

int cached_map(cafe_ctx* C, Workspace& ws, int slot, CUtensorMap* out, const float* base, int64_t rows, int cols,
               int box_cols, int box_rows, int64_t depth_stride = 0) {
    Workspace::MapCache& mc = ws.map_cache[slot];
    if (mc.ptr != base || mc.rows != rows || mc.cols != cols || mc.box != box_cols || mc.box_rows != box_rows ||
        mc.depth != depth_stride) {
        int rc = encode_map(C, &mc.map, base, rows, cols, box_cols, box_rows, depth_stride);
        if (rc) {
            mc.ptr = nullptr;
            return rc;
        }
        mc.ptr = base;
        mc.rows = rows;
        mc.cols = cols;
        mc.box = box_cols;
        mc.box_rows = box_rows;
        mc.depth = depth_stride;
    }
    *out = mc.map;
    return CAFE_OK;
}

double host_ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// ---- op log: the stream operations of the pruning phase. In the dry mode
// they are only recorded (their parameters form the CUDA-graph signature),
// in the run and capture modes they are also issued.
template <class T>
void oplog(Workspace& ws, const T& v) {
    const uint8_t* p = reinterpret_cast<const uint8_t*>(&v);
    ws.oplog.insert(ws.oplog.end(), p, p + sizeof(T));
}
bool op_issue(const Workspace& ws) { return ws.op_mode != Workspace::kOpDry; }
cudaError_t op_h2d(Workspace& ws, void* dst, const void* src, size_t n, cudaStream_t s) {
    oplog(ws, 1); oplog(ws, dst); oplog(ws, src); oplog(ws, n); oplog(ws, s);
    return op_issue(ws) ? cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, s) : cudaSuccess;
}
cudaError_t op_memset(Workspace& ws, void* dst, int v, size_t n, cudaStream_t s) {
    oplog(ws, 2); oplog(ws, dst); oplog(ws, v); oplog(ws, n); oplog(ws, s);
    return op_issue(ws) ? cudaMemsetAsync(dst, v, n, s) : cudaSuccess;
}
cudaError_t op_record(Workspace& ws, cudaEvent_t e, cudaStream_t s) {
    oplog(ws, 3); oplog(ws, e); oplog(ws, s);
    return op_issue(ws) ? cudaEventRecord(e, s) : cudaSuccess;
}
cudaError_t op_wait(Workspace& ws, cudaStream_t s, cudaEvent_t e) {
    oplog(ws, 4); oplog(ws, s); oplog(ws, e);
    return op_issue(ws) ? cudaStreamWaitEvent(s, e, 0) : cudaSuccess;
}
// A kernel launch: `sig` are the launch's argument values (all of them).
template <class F, class... A>
cudaError_t op_launch(Workspace& ws, int tag, F&& launch, const A&... sig) {
    oplog(ws, 100 + tag);
    (oplog(ws, sig), ...);
    return op_issue(ws) ? launch() : cudaSuccess;
}

// Category probabilities of every (candidate, category) index, and the list
// of indices that are pruned (candidates not rejected), staged to the device.
int stage_cat_probs(cafe_ctx* C, Workspace& ws, const cafe_request* R, int K, int NB) {
    const int CT = NB * K;
    CK(ws.h_catp.reserve((size_t)CT * sizeof(double)), "cat probs");
    CK(ws.catp.reserve((size_t)CT * sizeof(double)), "cat probs");
    double* h = ws.h_catp.as<double>();
    for (int b = 0; b < NB; ++b)
        for (int k = 0; k < K; ++k) h[b * K + k] = R[b].model == CAFE_MODEL_GAMMA ? R[b].cat_probs[k] : 1.0;
    CK(op_h2d(ws, ws.catp.p, h, (size_t)CT * sizeof(double), ws.stream), "cat probs");
    return CAFE_OK;
}

// Per-family lnL and the total of every candidate, then +inf / NaN for
// the candidates rejected before pruning.
int finish_batch(cafe_ctx* C, Workspace& ws, const ScoreInfo* info, bool gamma, bool scaled, const int64_t* d_ref,
                 const int32_t* d_status, double* d_fam, double* d_total) {
    const int64_t F = info->F;
    const int NB = info->B;
    FinishArgs fa;
    std::memset(&fa, 0, sizeof fa);
    fa.F = F;
    fa.K = info->K;
    fa.n_cand = NB;
    fa.model = gamma ? 1 : 0;
    fa.scaled = scaled ? 1 : 0;
    fa.cat = ws.cat.as<double>();
    fa.ref = d_ref;
    fa.family_lnl = d_fam;
    fa.total = d_total;
    fa.n_failed = ws.nfail.as<int32_t>();
    const size_t parts = (size_t)finish_parts(F) * NB;
    CK(ws.parts.reserve(parts * 2 * (sizeof(double) + sizeof(int32_t))), "finish");
    fa.part_sum = ws.parts.as<double>();
    fa.part_cnt = reinterpret_cast<int32_t*>(fa.part_sum + 2 * parts);
    fa.status = d_status;
    const bool prof = ws.sync;
    cudaEvent_t ev;
    if (prof) C->prof.begin(2, ws.stream, &ev);
    CK(op_launch(ws, 1, [&] { return launch_finish(fa, ws.stream); }, fa, ws.stream), "finish");
    if (prof) C->prof.end(2, ws.stream, ev);
    for (int b = 0; b < NB; ++b) {
        if (!info->cand_rejected[b]) continue;
        double* pt = d_total ? d_total + b : nullptr;
        double* pf = (d_fam && F) ? d_fam + (size_t)b * F : nullptr;
        int32_t* pn = ws.nfail.as<int32_t>() + b;
        CK(op_launch(ws, 2, [&] {
               cudaError_t e = cudaSuccess;
               if (pt) e = launch_fill(pt, 1, INFINITY, ws.stream);
               if (e == cudaSuccess && pf) e = launch_fill(pf, F, NAN, ws.stream);
               if (e == cudaSuccess) e = launch_fill_i32(pn, 1, 0, ws.stream);
               return e;
           }, pt, pf, pn, F, ws.stream),
           "fill");
    }
    return CAFE_OK;
}

// Launch k_prune64 (per-node rescaled FP64) for the given 32-family tiles.
int launch_fp64_tiles(cafe_ctx* C, Workspace& ws, const cafe_request* R, TreeHost& T, FamSet& S, int K,
                      const std::vector<PruneTile>& tiles, DevBuf& d_tiles, PinnedBuf& h_tiles, const int64_t* d_perm,
                      int W, int msize, double* out, int prof_kind) {
    if (tiles.empty()) return CAFE_OK;
    const int n = (int)tiles.size();
    CK(h_tiles.reserve(n * sizeof(PruneTile)), "tiles");
    CK(d_tiles.reserve(n * sizeof(PruneTile)), "tiles");
    std::memcpy(h_tiles.p, tiles.data(), n * sizeof(PruneTile));
    CK(op_h2d(ws, d_tiles.p, h_tiles.p, n * sizeof(PruneTile), ws.stream), "tiles");
    const int n_ctas = std::max(1, std::min(n, C->n_ctas));
    const int64_t per_cta = (int64_t)T.n_slots * W * 32;
    CK(ws.scratch.reserve((size_t)n_ctas * per_cta * sizeof(double)), "scratch");
    Prune64Args a;
    std::memset(&a, 0, sizeof a);
    a.plan = T.plan;
    a.tiles = d_tiles.as<PruneTile>();
    a.n_tiles = n;
    a.counts = S.d_counts.as<int32_t>();
    a.perm = d_perm;
    a.mats = ws.mats.as<const double*>();
    a.ld_mat = msize;
    a.prior = C->d_prior.as<double>();
    a.n_prior = (int)C->prior.size();
    a.err = R->use_error_model ? C->d_err.as<double>() : nullptr;
    a.err_rows = C->err_rows;
    a.err_ndev = C->err_ndev;
    a.fam_R = S.bins.d_famR.as<int32_t>();
    a.scratch = ws.scratch.as<double>();
    a.scratch_per_cta = per_cta;
    a.scaled = 1;
    a.model = R->model == CAFE_MODEL_GAMMA ? 1 : 0;
    a.out = out;
    a.K = K;
    a.cat_probs = ws.catp.as<double>();
    a.tile_families = 32;
    a.W = W;
    const bool prof = ws.sync;
    cudaEvent_t ev;
    if (prof) C->prof.begin(prof_kind, ws.stream, &ev);
    CK(op_launch(ws, 3, [&] { return launch_prune64(a, n_ctas, ws.stream); }, a, n_ctas, ws.stream), "prune fp64");
    if (prof) C->prof.end(prof_kind, ws.stream, ev);
    return CAFE_OK;
}

// Bins walked one family per thread-block cluster (k_prune64_cl): those whose
// 32-family tiles of one candidate would occupy less than half of the SMs.
// The choice depends on the family set and the category count only, so a
// candidate gets the same bits alone and in a batch. The cluster gives each
// CTA at least 64 rows of the bin.
int fp64_cluster_size(int w) { return w >= 512 ? 8 : w >= 256 ? 4 : w >= 128 ? 2 : 1; }

bool fp64_cluster_bin(const cafe_ctx* C, const TreeHost& T, int64_t count, int K, int w) {
    return count > 0 && ((count + 31) / 32) * (int64_t)K * 2 < C->sm_count &&
           prune64_cluster_smem(T.n_slots, w) <= prune64_cluster_max_smem();
}

// One tile per family of bin b for every category index in `active`.
void add_cluster_tiles(std::vector<PruneTile>& out, const BinPlan& B, size_t b, const std::vector<int32_t>& active) {
    const int w = B.widths[b];
    for (int k : active)
        for (int64_t i = 0; i < B.bin_count[b]; ++i) {
            PruneTile t{};
            t.first = (int)(B.bin_first[b] + i);
            t.count = 1;
            t.k = k;
            t.S = w - 1;
            t.R = w - 1;
            out.push_back(t);
        }
}

// Launch the one-family-per-cluster FP64 walk over `tiles` (grouped by bin,
// bins ascending): one launch per bin, sized by the bin's width.
int launch_fp64_cluster(cafe_ctx* C, Workspace& ws, const cafe_request* R, TreeHost& T, FamSet& S, int K,
                        const std::vector<PruneTile>& tiles, const int64_t* d_perm, const int32_t* d_famR, int msize,
                        bool scaled, double* out, cudaStream_t st, int prof_kind) {
    if (tiles.empty()) return CAFE_OK;
    const size_t n = tiles.size();
    CK(ws.h_tiles_cl.reserve(n * sizeof(PruneTile)), "tiles");
    CK(ws.tiles_cl.reserve(n * sizeof(PruneTile)), "tiles");
    std::memcpy(ws.h_tiles_cl.p, tiles.data(), n * sizeof(PruneTile));
    CK(op_h2d(ws, ws.tiles_cl.p, ws.h_tiles_cl.p, n * sizeof(PruneTile), st), "tiles");
    Prune64Args a;
    std::memset(&a, 0, sizeof a);
    a.plan = T.plan;
    a.counts = S.d_counts.as<int32_t>();
    a.perm = d_perm;
    a.mats = ws.mats.as<const double*>();
    a.ld_mat = msize;
    a.prior = C->d_prior.as<double>();
    a.n_prior = (int)C->prior.size();
    a.err = R->use_error_model ? C->d_err.as<double>() : nullptr;
    a.err_rows = C->err_rows;
    a.err_ndev = C->err_ndev;
    a.fam_R = d_famR;
    a.scaled = scaled ? 1 : 0;
    a.model = R->model == CAFE_MODEL_GAMMA ? 1 : 0;
    a.out = out;
    a.K = K;
    a.cat_probs = ws.catp.as<double>();
    a.tile_families = 1;
    const bool prof = ws.sync;
    cudaEvent_t ev;
    if (prof) C->prof.begin(prof_kind, st, &ev);
    for (size_t i = 0; i < n;) {
        size_t j = i;
        while (j < n && tiles[j].S == tiles[i].S) ++j;
        Prune64Args b;
        std::memcpy(&b, &a, sizeof b);   // padding included: the bytes are a graph signature
        b.tiles = ws.tiles_cl.as<PruneTile>() + i;
        b.n_tiles = (int)(j - i);
        b.W = std::max(tiles[i].S + 1, tiles[i].R);
        const int cl = fp64_cluster_size(b.W);
        const int n_cl = (int)std::min<int64_t>((int64_t)(j - i), (int64_t)C->sm_count * 8);
        CK(op_launch(ws, 8, [&] { return launch_prune64_cluster(b, cl, n_cl, st); }, b, cl, n_cl, st),
           "prune fp64 (cluster)");
        i = j;
    }
    if (prof) C->prof.end(prof_kind, st, ev);
    return CAFE_OK;
}

// Algorithmic flops of one family of a tile (the roofline basis), by the
// tile's (S, R) and error-model use.
double family_flops(const TreeHost& T, int S, int R, bool err) {
    double per = 0;
    for (size_t ii = 0; ii < T.internal.size(); ++ii) {
        const int v = T.internal[ii];
        const int rows = (v == T.root) ? R : S + 1;
        const int nch = T.cstart[ii + 1] - T.cstart[ii];
        for (int ci = T.cstart[ii]; ci < T.cstart[ii + 1]; ++ci)
            if (!T.children[T.child[ci]].empty()) per += 2.0 * rows * (S + 1);
            else if (err) per += 6.0 * rows;
        per += (double)(nch - 1) * rows;
    }
    return per;
}

double tiles_flops(const TreeHost& T, const std::vector<PruneTile>& tiles, bool err) {
    double fl = 0;
    int last_S = -1, last_R = -1;
    double per = 0;
    for (const PruneTile& t : tiles) {
        if (t.S != last_S || t.R != last_R) {
            per = family_flops(T, t.S, t.R, err);
            last_S = t.S;
            last_R = t.R;
        }
        fl += per * t.count;
    }
    return fl;
}

// Launch shape of the tensor-core kernel for bin width W: TMEM columns per
// CTA, CTAs per SM and pipeline stages. By default the most CTAs per SM that
// TMEM and shared memory allow, then the deepest pipeline that keeps them;
// cafe_autotune may have measured a better pair for this width.
struct TcShape {
    int tmem_cols = 0, per_sm = 0, stages = 0;
    size_t smem = 0;
};

int tc_by_smem(const TreeHost& T, int W, int stages, size_t* smem, int nsplit = 1) {
    *smem = prune_tc_smem_bytes(W, T.n_slots, stages, (int)T.internal.size());
    if (*smem > (size_t)prune_tc_max_smem(nsplit)) return 0;
    return (int)((227 * 1024) / (*smem + 1024));
}

TcShape tc_shape(cafe_ctx* C, const TreeHost& T, int W) {
    TcShape sh;
    sh.tmem_cols = 32;
    while (sh.tmem_cols < 2 * W) sh.tmem_cols *= 2;
    const int by_tmem = 512 / sh.tmem_cols;
    auto it = C->tuned.find(W);
    if (it != C->tuned.end()) {
        size_t sm;
        const int per = it->second.first, st = it->second.second;
        if (per >= 1 && per <= by_tmem && st >= 1 && st <= 4 && tc_by_smem(T, W, st, &sm) >= per) {
            sh.per_sm = per;
            sh.stages = st;
            sh.smem = sm;
            return sh;
        }
    }
    for (int st = 4; st >= 1; --st) {
        size_t sm;
        const int per = std::min(by_tmem, tc_by_smem(T, W, st, &sm));
        if (per > sh.per_sm) {
            sh.per_sm = per;
            sh.stages = st;
            sh.smem = sm;
        }
    }
    return sh;
}

// Share of the 1e-6 per-family budget (|dlnL| / |lnL|) left to FP32 range
// loss; TF32x3 rounding takes the rest.
constexpr double kRangeTau = 1e-7;

// Widest bin on the tensor cores: one CTA per tile up to 256 states (both
// children's factors in 2 W <= 512 TMEM columns), a pair of CTAs (half the
// states each) for 384 and 512.
constexpr int kTcMaxW = 512;

// MIXED_TF32X3: tensor-core tiles for bins <= 512 states, FP64 tiles for
// wider bins and for families the tensor-core pass flags. Caller holds C->mu;
// hm holds the FP64 matrix of every (category, node).
int enqueue_mixed(cafe_ctx* C, Workspace& ws, const cafe_request* R, TreeHost& T, FamSet& S, int K, int CT,
                  const std::vector<int32_t>& active, double** hm, double* d_fam, double* d_total, ScoreInfo* info) {
    const bool gamma = R->model == CAFE_MODEL_GAMMA;
    const int KC = K;    // categories per candidate
    K = CT;              // below, K counts the combined (candidate, category) indices
    const int64_t F = S.F;
    const BinPlan& B = S.bins;
    const int msize = B.W_max;
    int Wm = 0;
    for (int w : B.widths)
        if (w <= kTcMaxW) Wm = std::max(Wm, w);
    info->scaled = true;

    // request-local matrix list and conversion to TF32 operands (a cache
    // entry stamped with this request already has its conversion slot)
    std::vector<int32_t> mat_index((size_t)K * T.n_nodes, -1);
    std::vector<ConvertJob> jobs;
    const uint64_t stamp = ++C->request_stamp;
    for (int k = 0; k < K; ++k)
        for (int v = 0; v < T.n_nodes; ++v) {
            MatEntry* e = ws.entry_vec[(size_t)k * T.n_nodes + v];
            if (!e) continue;
            if (e->stamp != stamp) {
                e->stamp = stamp;
                e->conv = (int)jobs.size();
                jobs.push_back(ConvertJob{e->d, msize, e->conv, 0});
            }
            // a leaf's branch is read as transposed rows, an internal child's
            // as the GEMM's hi and lo operands
            jobs[(size_t)e->conv].what |= T.leaf_col[v] >= 0 ? 2 : 1;
            mat_index[(size_t)k * T.n_nodes + v] = e->conv | (ws.sat_vec[(size_t)k * T.n_nodes + v] ? (1 << 30) : 0);
        }
    const int n_mat = (int)jobs.size();

    // category probabilities (device) for both kernels
    int rc0 = stage_cat_probs(C, ws, R, KC, CT / KC);
    if (rc0) return rc0;
    CK(ws.mats.reserve((size_t)K * T.n_nodes * sizeof(double*)), "mats");
    CK(op_h2d(ws, ws.mats.p, hm, (size_t)K * T.n_nodes * sizeof(double*), ws.stream), "mats");
    CK(ws.cat.reserve((size_t)std::max<int64_t>(F, 1) * K * sizeof(double)), "category buffer");
    CK(ws.nfail.reserve(sizeof(int32_t)), "fail counter");
    CK(ws.flags.reserve((size_t)std::max<int64_t>(F, 1) * sizeof(int32_t) + 64), "flags");
    int32_t* d_flags = ws.flags.as<int32_t>();
    int32_t* d_status = d_flags + std::max<int64_t>(F, 1);
    CK(op_memset(ws, ws.flags.p, 0, (size_t)std::max<int64_t>(F, 1) * sizeof(int32_t) + 64, ws.stream), "flags");
    // which category terms the FP64 pass recomputes, [F][K]
    CK(ws.term_flags.reserve((size_t)std::max<int64_t>(F, 1) * K), "term flags");
    uint8_t* d_term = ws.term_flags.as<uint8_t>();
    CK(op_memset(ws, ws.term_flags.p, 0, (size_t)std::max<int64_t>(F, 1) * K, ws.stream), "term flags");

    // tiles: 128 families (tensor cores) or 32 families (FP64, wide bins)
    // grouped by bin (bins ascend in width), so each bin's tiles are contiguous
    std::vector<PruneTile> tc_tiles, wide_tiles;
    std::vector<PruneTile>& cl_tiles = ws.cl_tile_vec;
    cl_tiles.clear();
    for (size_t b = 0; b < B.widths.size(); ++b) {
        if (B.widths[b] > kTcMaxW && fp64_cluster_bin(C, T, B.bin_count[b], KC, B.widths[b])) {
            add_cluster_tiles(cl_tiles, B, b, active);
            continue;
        }
        for (int k : active) {
            const int w = B.widths[b];
            const int step = w <= kTcMaxW ? 128 : 32;
            for (int64_t i = 0; i < B.bin_count[b]; i += step) {
                PruneTile t{};
                t.first = (int)(B.bin_first[b] + i);
                t.count = (int)std::min<int64_t>(step, B.bin_count[b] - i);
                t.k = k;
                t.S = w - 1;
                t.R = w - 1;
                (w <= kTcMaxW ? tc_tiles : wide_tiles).push_back(t);
            }
        }
    }
    const bool prof = ws.sync;
    cudaEvent_t ev;
    // FP64 bins (wider than the tensor-core tiles): 32-family tiles, or one
    // family per cluster where a bin is sparse; beside the tensor-core bins
    // when those fork onto the auxiliary streams (profiled calls: after them)
    bool wide_done = false;
    auto launch_wide = [&]() -> int {
        wide_done = true;
        int rc = launch_fp64_tiles(C, ws, R, T, S, K, wide_tiles, ws.tiles64, ws.h_tiles64, B.d_perm.as<int64_t>(),
                                   msize, msize, ws.cat.as<double>(), 3);
        if (!rc)
            rc = launch_fp64_cluster(C, ws, R, T, S, K, cl_tiles, B.d_perm.as<int64_t>(), B.d_famR.as<int32_t>(),
                                     msize, true, ws.cat.as<double>(), ws.stream, 3);
        return rc;
    };
    if (!tc_tiles.empty()) {
        const size_t fl = (size_t)n_mat * Wm * Wm;
        CK(ws.tc_hi.reserve(2 * fl * sizeof(float)), "tc matrices");     // hi, then lo
        CK(ws.tc_tr.reserve(fl * sizeof(float)), "tc matrices");
        CK(ws.h_conv.reserve(jobs.size() * sizeof(ConvertJob)), "convert jobs");
        CK(ws.conv.reserve(jobs.size() * sizeof(ConvertJob)), "convert jobs");
        std::memcpy(ws.h_conv.p, jobs.data(), jobs.size() * sizeof(ConvertJob));
        CK(op_h2d(ws, ws.conv.p, ws.h_conv.p, jobs.size() * sizeof(ConvertJob), ws.stream), "convert jobs");
        CK(ws.tc_mi.reserve(mat_index.size() * sizeof(int32_t)), "mat index");
        CK(ws.h_mi.reserve(mat_index.size() * sizeof(int32_t)), "mat index");
        std::memcpy(ws.h_mi.p, mat_index.data(), mat_index.size() * sizeof(int32_t));
        CK(op_h2d(ws, ws.tc_mi.p, ws.h_mi.p, mat_index.size() * sizeof(int32_t), ws.stream), "mat index");
        TcBuffers tb;
        std::memset(&tb, 0, sizeof tb);
        tb.hi = ws.tc_hi.as<float>();
        tb.lo = ws.tc_hi.as<float>() + fl;
        tb.tr = ws.tc_tr.as<float>();
        tb.Wm = Wm;
        if (R->use_error_model) {
            tb.err = C->d_err.as<double>();
            tb.err_rows = C->err_rows;
            tb.err_ndev = C->err_ndev;
        }
        if (prof) C->prof.begin(3, ws.stream, &ev);
        const ConvertJob* cj = ws.conv.as<ConvertJob>();
        CK(op_launch(ws, 4, [&] { return launch_convert_tc(cj, n_mat, tb, ws.stream); }, cj, n_mat, tb, ws.stream),
           "convert");
        if (prof) C->prof.end(3, ws.stream, ev);

        // one launch per S-bin, each sized for its own width, run
        // concurrently: TMEM (512 columns per SM) and shared memory set how
        // many tiles of a bin share an SM
        struct BinLaunch {
            int W, tmem_cols, stages, per_sm, n_ctas, nsplit;
            size_t smem;
            int64_t first_tile, n_tiles, vrow_base;
        };
        // Bins of 128 states or more split each tile over a cluster of
        // nsplit CTAs (4 or 2; W / nsplit a multiple of 32 and at least 64)
        // when the bin is sparse enough that every tile still gets SMs of
        // its own: a lone tile's walk is bound by what one SM can stream.
        // Bins over 256 states always split (both children's factors, 2 W
        // columns, would not fit one CTA's TMEM).
        auto pick_split = [&](int W, int64_t n_tiles) {
            for (int ns : {4, 2}) {
                const int wn = W / ns;
                if (W % ns || wn % 32 || wn < 64 || wn > 256) continue;
                if (n_tiles * ns <= (int64_t)C->sm_count) return ns;
            }
            return W > 256 ? 2 : 1;
        };
        std::vector<BinLaunch> launches;
        int64_t vrows = 0;
        for (size_t i = 0; i < tc_tiles.size();) {
            size_t j = i;
            while (j < tc_tiles.size() && tc_tiles[j].S == tc_tiles[i].S) ++j;
            BinLaunch L{};
            L.W = tc_tiles[i].S + 1;
            L.first_tile = (int64_t)i;
            L.n_tiles = (int64_t)(j - i);
            L.nsplit = pick_split(L.W, L.n_tiles);
            if (L.nsplit > 1) {
                // the deepest pipeline of W / nsplit B rows that fits
                const int wn = L.W / L.nsplit;
                L.tmem_cols = 32;
                while (L.tmem_cols < 2 * wn) L.tmem_cols *= 2;
                L.per_sm = 1;
                for (int st = 4; st >= 1 && !L.stages; --st)
                    if (tc_by_smem(T, wn, st, &L.smem, L.nsplit) >= 1) L.stages = st;
                if (!L.stages) return fail(C, CAFE_ERR_INVALID, "tensor-core tile does not fit shared memory");
                // over half an SM's shared memory: two cluster CTAs (of this or
                // another cluster launch) never share an SM, so no CTA holding
                // TMEM waits on a peer that waits for that SM's TMEM
                L.smem = std::min(std::max(L.smem, (size_t)120 * 1024), (size_t)prune_tc_max_smem(L.nsplit));
                const int64_t clusters =
                    std::max<int64_t>(1, std::min<int64_t>(L.n_tiles, (int64_t)C->sm_count / L.nsplit));
                L.n_ctas = (int)(L.nsplit * clusters);
                L.vrow_base = vrows;
                vrows += clusters * T.n_slots * 128;
                launches.push_back(L);
                i = j;
                continue;
            }
            L.nsplit = 1;
            const TcShape shape = tc_shape(C, T, L.W);
            if (shape.per_sm < 1) return fail(C, CAFE_ERR_INVALID, "tensor-core tile does not fit shared memory");
            L.tmem_cols = shape.tmem_cols;
            L.stages = shape.stages;
            L.smem = shape.smem;
            L.per_sm = shape.per_sm;
            // pad shared memory so no more CTAs of this launch than TMEM allows share an SM
            L.smem = std::max(L.smem, (size_t)((227 * 1024) / L.per_sm) - 2048);
            L.smem = std::min(L.smem, (size_t)prune_tc_max_smem());
            L.n_ctas = (int)std::max<int64_t>(1, std::min<int64_t>(L.n_tiles, (int64_t)C->sm_count * L.per_sm));
            L.vrow_base = vrows;
            vrows += (int64_t)L.n_ctas * T.n_slots * 128;
            launches.push_back(L);
            i = j;
        }
        CK(ws.tc_vec.reserve((size_t)vrows * Wm * sizeof(float)), "tc vectors");
        // node vectors move in boxes of one tile's 128 rows; each launch's
        // matrix maps have boxes of its Ws rows (one TMA instruction per
        // operand and chunk)
        TcMaps maps;
        const int kbox = prune_tc_kchunk();
        int rc = cached_map(C, ws, 2, &maps.vec, ws.tc_vec.as<float>(), vrows, Wm, kbox, 128);
        if (!rc) rc = cached_map(C, ws, 3, &maps.vst, ws.tc_vec.as<float>(), vrows, Wm, 32, 128);
        if (rc) return rc;
        auto launch_maps = [&](int Ws, TcMaps* m) {
            *m = maps;
            const int q = 4 + (Ws / 32 - 1);      // Ws: a multiple of 32 up to 256
            const int64_t fl = (int64_t)n_mat * Wm * Wm;
            int r = cached_map(C, ws, q, &m->mat, ws.tc_hi.as<float>(), (int64_t)n_mat * Wm, Wm, kbox, Ws, fl);
            // leaf blocks: W x W (read only where W <= 64, one CTA per tile)
            if (!r) r = cached_map(C, ws, 12 + (Ws / 32 - 1), &m->tr, ws.tc_tr.as<float>(), (int64_t)n_mat * Wm, Wm, 32, Ws);
            return r;
        };
        const int n_tc = (int)tc_tiles.size();
        CK(ws.tiles.reserve(n_tc * sizeof(PruneTile)), "tiles");
        CK(ws.h_tiles.reserve(n_tc * sizeof(PruneTile)), "tiles");
        std::memcpy(ws.h_tiles.p, tc_tiles.data(), n_tc * sizeof(PruneTile));
        CK(op_h2d(ws, ws.tiles.p, ws.h_tiles.p, n_tc * sizeof(PruneTile), ws.stream), "tiles");
        PruneTcArgs a;
        std::memset(&a, 0, sizeof a);
        a.plan = T.plan;
        a.counts = S.d_counts.as<int32_t>();
        a.perm = B.d_perm.as<int64_t>();
        a.mat_index = ws.tc_mi.as<int32_t>();
        a.Wm = Wm;
        a.mat_tr = ws.tc_tr.as<float>();
        a.vec = ws.tc_vec.as<float>();
        a.n_slots = T.n_slots;
        a.prior = C->d_prior.as<double>();
        a.n_prior = (int)C->prior.size();
        a.err = R->use_error_model ? C->d_err.as<double>() : nullptr;
        a.err_rows = C->err_rows;
        a.err_ndev = C->err_ndev;
        a.fam_R = B.d_famR.as<int32_t>();
        a.out = ws.cat.as<double>();
        a.K = K;
        a.model = gamma ? 1 : 0;
        a.cat_probs = ws.catp.as<double>();
        a.flags = d_flags;
        a.term_flags = d_term;
        a.status = d_status;
        a.debug_wait_limit = C->debug_wait_limit;
        // range-error bounds of the category terms: zero for every term the
        // tensor cores do not write (FP64 bins, candidates not pruned)
        CK(ws.cerr.reserve((size_t)std::max<int64_t>(F, 1) * K * sizeof(float)), "range bounds");
        CK(op_memset(ws, ws.cerr.p, 0, (size_t)std::max<int64_t>(F, 1) * K * sizeof(float), ws.stream), "range bounds");
        a.out_err = ws.cerr.as<float>();
        a.phase_clocks = nullptr;
        static const bool phase_env = getenv("CAFE_TC_PHASES") != nullptr;
        if (phase_env) {
            CK(ws.phase.reserve(kPhases * sizeof(unsigned long long)), "phase clocks");
            CK(cudaMemsetAsync(ws.phase.p, 0, kPhases * sizeof(unsigned long long), ws.stream), "phase clocks");
            a.phase_clocks = ws.phase.as<unsigned long long>();
        }
        if (prof) {
            C->prof.begin(1, ws.stream, &ev);
            C->prof.acc.prune_flops += tiles_flops(T, tc_tiles, R->use_error_model);
        }
        // tile counters of the one-CTA-per-tile launches, zeroed before the fork
        CK(ws.tile_ctr.reserve(std::max<size_t>(launches.size(), 1) * sizeof(int)), "tile counters");
        CK(op_memset(ws, ws.tile_ctr.p, 0, std::max<size_t>(launches.size(), 1) * sizeof(int), ws.stream), "tile counters");
        // fork: bins run on the auxiliary streams after everything queued so far
        const bool fork = launches.size() > 1;
        if (fork) {
            CK(op_record(ws, ws.ev_fork, ws.stream), "fork");
            for (int q = 0; q < Workspace::kAux; ++q) CK(op_wait(ws, ws.aux[q], ws.ev_fork), "fork");
        }
        // widest bins (the longest walks) first, each on its own stream
        for (size_t q = 0; q < launches.size(); ++q) {
            const size_t li = launches.size() - 1 - q;
            const BinLaunch& L = launches[li];
            PruneTcArgs b;
            std::memcpy(&b, &a, sizeof b);     // padding included: the bytes are a graph signature
            b.tiles = ws.tiles.as<PruneTile>() + L.first_tile;
            b.n_tiles = (int)L.n_tiles;
            b.tmem_cols = L.tmem_cols;
            b.nsplit = L.nsplit;
            b.Ws = L.W / L.nsplit;
            b.stages = L.stages;
            b.vrow_base = L.vrow_base;
            b.tile_counter = L.nsplit == 1 ? ws.tile_ctr.as<int>() + li : nullptr;
            cudaStream_t st = fork ? ws.aux[q % Workspace::kAux] : ws.stream;
            if (b.Ws % 32 || b.Ws < 32 || b.Ws > 256) return fail(C, CAFE_ERR_INVALID, "tensor-core tile of %d rows", b.Ws);
            TcMaps lm;
            const int rcm = launch_maps(b.Ws, &lm);
            if (rcm) return rcm;
            CK(op_launch(ws, 5, [&] { return launch_prune_tc(lm, b, L.n_ctas, L.smem, st); }, lm, b, L.n_ctas, L.smem,
                         st),
               "prune tc");
        }
        if (fork && !prof) {
            const int rcw = launch_wide();
            if (rcw) return rcw;
        }
        if (fork) {
            for (int q = 0; q < Workspace::kAux; ++q) {
                CK(op_record(ws, ws.ev_join[q], ws.aux[q]), "join");
                CK(op_wait(ws, ws.stream, ws.ev_join[q]), "join");
            }
        }

        if (phase_env) {
            unsigned long long h[kPhases];
            CK(cudaMemcpyAsync(h, ws.phase.p, sizeof(h), cudaMemcpyDeviceToHost, ws.stream), "phase clocks");
            CK(cudaStreamSynchronize(ws.stream), "phase clocks");
            const double n = (double)h[5] + 1e-9;
            fprintf(stderr, "k_prune_tc clocks per tile-node: setup %.0f gemm %.0f epilogue %.0f root %.0f sync %.0f (%llu tile-nodes)\n",
                    h[0] / n, h[1] / n, h[2] / n, h[3] / n, h[4] / n, h[5]);
            fprintf(stderr, "  per tile-node: store wait %.0f leaf gather %.0f; per chunk (%.2f per tile-node): stage wait %.0f "
                    "TMA wait %.0f split %.0f MMA issue %.0f (of which the stage's wait %.0f); last-MMA wait per tile-node %.0f\n",
                    h[12] / n, h[13] / n, h[11] / n, h[6] / (h[11] + 1e-9), h[7] / (h[11] + 1e-9), h[8] / (h[11] + 1e-9),
                    h[9] / (h[11] + 1e-9), h[14] / (h[11] + 1e-9), h[10] / n);
            fprintf(stderr, "  TMA issue per chunk %.0f; barriers per tile-node: after the chunks %.0f, after the last MMAs %.0f\n",
                    h[15] / (h[11] + 1e-9), h[16] / n, h[17] / n);
        }

        if (prof) C->prof.end(1, ws.stream, ev);
    }
    if (!wide_done) {
        const int rc = launch_wide();
        if (rc) return rc;
    }

    // families the tensor-core pass could not represent, or whose result FP32's
    // range may have cost accuracy: planned on the device and recomputed in
    // FP64 without a host round trip
    if (!tc_tiles.empty()) {
        RangeFlagArgs rf;
        std::memset(&rf, 0, sizeof rf);
        rf.cat = ws.cat.as<double>();
        rf.err = ws.cerr.as<float>();
        rf.F = F;
        rf.K = K;
        rf.KC = KC;
        rf.tau = kRangeTau;
        rf.flags = d_flags;
        rf.term_flags = d_term;
        rf.any_flag = d_status + 3;
        CK(op_launch(ws, 9, [&] { return launch_range_flags(rf, ws.stream); }, rf, ws.stream), "range flags");
        static const bool flag_env = getenv("CAFE_DEBUG_FLAGS") != nullptr;
        if (flag_env && op_issue(ws)) {
            // diagnostics: which families the FP64 pass will recompute, and why
            // (bit 1: the tensor-core walk could not represent a category term;
            // bit 2: the weighted FP32 range bound), and which category terms
            // the walk left unwritten
            std::vector<int32_t> hf((size_t)F);
            std::vector<double> hc((size_t)F * K);
            CK(cudaMemcpyAsync(hf.data(), d_flags, (size_t)F * sizeof(int32_t), cudaMemcpyDeviceToHost, ws.stream), "flags");
            CK(cudaMemcpyAsync(hc.data(), ws.cat.p, (size_t)F * K * sizeof(double), cudaMemcpyDeviceToHost, ws.stream), "flags");
            CK(cudaStreamSynchronize(ws.stream), "flags");
            int64_t n1 = 0, n2 = 0, n12 = 0, terms = 0;
            std::vector<int64_t> by_cat((size_t)KC, 0);
            for (int64_t f = 0; f < F; ++f) {
                const int v = hf[(size_t)f];
                n1 += (v & 1) != 0;
                n2 += (v & 2) != 0;
                n12 += (v & 3) == 3;
                if (v & 1)
                    for (int k = 0; k < K; ++k)
                        if (std::isnan(hc[(size_t)f * K + k])) {
                            terms++;
                            by_cat[(size_t)(k % KC)]++;
                        }
            }
            fprintf(stderr, "flags: %lld families (walk %lld, range %lld, both %lld); unwritten terms %lld of %lld; by category:",
                    (long long)(n1 + n2 - n12), (long long)n1, (long long)n2, (long long)n12, (long long)terms,
                    (long long)(F * K));
            for (int k = 0; k < KC; ++k) fprintf(stderr, " %lld", (long long)by_cat[(size_t)k]);
            fprintf(stderr, "\n");
        }
        FallbackPlanArgs fp;
        std::memset(&fp, 0, sizeof fp);
        fp.flags = d_flags;
        fp.term_flags = d_term;
        fp.K = K;
        fp.perm = B.d_perm.as<int64_t>();
        fp.n_bins = 0;
        for (size_t b = 0; b < B.widths.size() && fp.n_bins < 16; ++b) {
            if (B.widths[b] > kTcMaxW) continue;
            fp.bin_width[fp.n_bins] = B.widths[b];
            fp.bin_first[fp.n_bins] = B.bin_first[b];
            fp.bin_count[fp.n_bins] = B.bin_count[b];
            fp.n_bins++;
        }
        fp.cats = ws.catids.as<int32_t>();
        fp.n_cats = (int)active.size();
        const int64_t max_tiles = (int64_t)active.size() * (F / 32 + fp.n_bins + 1);
        CK(ws.fb_perm.reserve((size_t)std::max<int64_t>(F, 1) * sizeof(int64_t)), "fallback");
        CK(ws.tiles_fb.reserve((size_t)max_tiles * sizeof(PruneTile)), "fallback");
        CK(ws.fb_bins.reserve(32 * sizeof(int64_t)), "fallback");
        fp.fb_perm = ws.fb_perm.as<int64_t>();
        fp.fb_bins = ws.fb_bins.as<int64_t>();
        fp.fb_tiles = ws.tiles_fb.as<PruneTile>();
        fp.out_counts = d_status + 1;     // [families, tiles]
        fp.any_flag = d_status + 3;
        if (prof) C->prof.begin(3, ws.stream, &ev);
        CK(op_launch(ws, 6, [&] { return launch_fallback_plan(fp, ws.stream); }, fp, ws.stream), "fallback plan");
        if (prof) C->prof.end(3, ws.stream, ev);
        const int n_ctas = C->sm_count;
        const int64_t per_cta = (int64_t)T.n_slots * msize * 32;
        CK(ws.scratch.reserve((size_t)n_ctas * per_cta * sizeof(double)), "scratch");
        Prune64Args a;
        std::memset(&a, 0, sizeof a);
        a.plan = T.plan;
        a.tiles = fp.fb_tiles;
        a.n_tiles = 0;
        a.n_tiles_dev = d_status + 2;
        a.counts = S.d_counts.as<int32_t>();
        a.perm = fp.fb_perm;
        a.mats = ws.mats.as<const double*>();
        a.ld_mat = msize;
        a.prior = C->d_prior.as<double>();
        a.n_prior = (int)C->prior.size();
        a.err = R->use_error_model ? C->d_err.as<double>() : nullptr;
        a.err_rows = C->err_rows;
        a.err_ndev = C->err_ndev;
        a.fam_R = B.d_famR.as<int32_t>();
        a.scratch = ws.scratch.as<double>();
        a.scratch_per_cta = per_cta;
        a.scaled = 1;
        a.model = gamma ? 1 : 0;
        a.out = ws.cat.as<double>();
        a.K = K;
        a.cat_probs = ws.catp.as<double>();
        a.tile_families = 32;
        a.W = msize;
        a.term_mask = d_term;     // only the flagged terms of each tile are written
        if (prof) C->prof.begin(3, ws.stream, &ev);
        CK(op_launch(ws, 7, [&] { return launch_prune64(a, n_ctas, ws.stream); }, a, n_ctas, ws.stream),
           "fallback prune");
        if (prof) C->prof.end(3, ws.stream, ev);
        info->d_tail = d_status;     // [status, fallback families, fallback tiles]
    }

    return finish_batch(C, ws, info, gamma, true, nullptr, tc_tiles.empty() ? nullptr : d_status, d_fam, d_total);
}

// The pruning phase of a mixed-precision request as a CUDA graph. A dry
// pass runs the host planning (it fills the pinned tables the graph's copy
// nodes read) and records every stream op; if the record matches a graph
// this workspace captured before, that graph is launched; otherwise the
// phase is captured (thread-local stream capture, the auxiliary streams
// joined by events) and instantiated. Profiled calls issue directly.
int enqueue_mixed_graph(cafe_ctx* C, Workspace& ws, const cafe_request* R, TreeHost& T, FamSet& S, int K, int CT,
                        const std::vector<int32_t>& active, double** hm, double* d_fam, double* d_total,
                        ScoreInfo* info) {
    static const bool phase_env = getenv("CAFE_TC_PHASES") != nullptr || getenv("CAFE_DEBUG_FLAGS") != nullptr;
    ws.oplog.clear();
    if (C->prof.on || phase_env) {
        ws.op_mode = Workspace::kOpRun;
        return enqueue_mixed(C, ws, R, T, S, K, CT, active, hm, d_fam, d_total, info);
    }
    ws.op_mode = Workspace::kOpDry;
    int rc = enqueue_mixed(C, ws, R, T, S, K, CT, active, hm, d_fam, d_total, info);
    ws.op_mode = Workspace::kOpRun;
    if (rc) return rc;
    for (auto& g : ws.graphs)
        if (g.exec && g.sig == ws.oplog) {
            g.used = ++ws.graph_clock;
            CK(cudaGraphLaunch(g.exec, ws.stream), "graph launch");
            return CAFE_OK;
        }
    std::vector<uint8_t> sig;
    sig.swap(ws.oplog);
    auto issue_directly = [&]() {
        cudaGetLastError();
        ws.oplog.clear();
        ws.op_mode = Workspace::kOpRun;
        return enqueue_mixed(C, ws, R, T, S, K, CT, active, hm, d_fam, d_total, info);
    };
    // capture into a free slot at once; evict a cached graph only for a
    // signature seen before (FNV-1a over the op record), so a stream of
    // one-off requests does not pay a capture each
    uint64_t h = 1469598103934665603ull;
    for (uint8_t b : sig) h = (h ^ b) * 1099511628211ull;
    h |= 1;
    bool seen = false, free_slot = false;
    for (uint64_t x : ws.seen) seen |= (x == h);
    for (const auto& g : ws.graphs) free_slot |= g.exec == nullptr;
    if (!seen && !free_slot) {
        ws.seen[ws.seen_next] = h;
        ws.seen_next = (ws.seen_next + 1) % (int)(sizeof(ws.seen) / sizeof(ws.seen[0]));
        return issue_directly();
    }
    if (cudaStreamBeginCapture(ws.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return issue_directly();
    ws.op_mode = Workspace::kOpCapture;
    rc = enqueue_mixed(C, ws, R, T, S, K, CT, active, hm, d_fam, d_total, info);
    ws.op_mode = Workspace::kOpRun;
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(ws.stream, &graph);
    cudaGraphExec_t exec = nullptr;
    const bool same = ws.oplog == sig;
    if (rc || ec != cudaSuccess || !graph || !same || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        if (rc) return rc;
        return issue_directly();
    }
    cudaGraphDestroy(graph);
    Workspace::GraphEntry* slot = &ws.graphs[0];
    for (auto& g : ws.graphs)
        if (!g.exec || g.used < slot->used) slot = &g;
    if (slot->exec) cudaGraphExecDestroy(slot->exec);
    slot->sig.swap(sig);
    slot->exec = exec;
    slot->used = ++ws.graph_clock;
    CK(cudaGraphLaunch(exec, ws.stream), "graph launch");
    return CAFE_OK;
}

// Enqueue the evaluation of NB candidate requests (same tree, family set,
// model, categories and precision; own lambdas, multipliers and category
// probabilities) on ws.stream. Candidate b, category k is pruned as the
// combined category b * K + k. d_fam is [NB][F], d_total [NB]. Caller
// holds C->mu.
int enqueue_score(cafe_ctx* C, Workspace& ws, const cafe_request* Rs, int NB, double* d_fam, double* d_total,
                  ScoreInfo* info) {
    if (!Rs || NB < 1) return fail(C, CAFE_ERR_INVALID, "null request");
    const cafe_request* R = Rs;
    // pinned staging buffers of this workspace are rewritten below: the
    // previous request's copies out of them must have run
    if (ws.staged) {
        CK(cudaEventSynchronize(ws.ev_staged), "staging");
        ws.staged = false;
    }
    auto ti = C->trees.find(R->tree_id);
    if (ti == C->trees.end()) return fail(C, CAFE_ERR_NOT_FOUND, "unknown tree id %d", R->tree_id);
    auto si = C->sets.find(R->set_id);
    if (si == C->sets.end()) return fail(C, CAFE_ERR_NOT_FOUND, "unknown family set id %d", R->set_id);
    TreeHost& T = *ti->second;
    FamSet& S = *si->second;
    if (S.tree_id != R->tree_id) return fail(C, CAFE_ERR_INVALID, "family set %d belongs to tree %d", R->set_id, S.tree_id);
    const bool gamma = R->model == CAFE_MODEL_GAMMA;
    if (R->model != CAFE_MODEL_BASE && !gamma) return fail(C, CAFE_ERR_INVALID, "bad model %d", R->model);
    const int K = gamma ? R->n_categories : 1;
    if (C->prior.empty()) return fail(C, CAFE_ERR_INVALID, "no prior set (cafe_prior_set)");
    if (R->use_error_model && C->err_rows == 0) return fail(C, CAFE_ERR_INVALID, "no error model set");
    if (R->precision != CAFE_PREC_FP64_REF && R->precision != CAFE_PREC_FP64_BINNED &&
        R->precision != CAFE_PREC_MIXED_TF32X3)
        return fail(C, CAFE_ERR_INVALID, "bad precision %d", R->precision);
    for (int b = 0; b < NB; ++b) {
        const cafe_request& Q = Rs[b];
        if (Q.tree_id != R->tree_id || Q.set_id != R->set_id || Q.model != R->model ||
            Q.precision != R->precision || Q.use_error_model != R->use_error_model ||
            Q.lambda_kind != R->lambda_kind || Q.dedupe != R->dedupe ||
            (R->precision == CAFE_PREC_FP64_REF &&
             (Q.max_family_size != R->max_family_size || Q.max_root_family_size != R->max_root_family_size)) ||
            (gamma && Q.n_categories != K))
            return fail(C, CAFE_ERR_INVALID, "batched request %d differs from request 0 in more than its parameters", b);
        if (Q.n_lambdas < 1 || !Q.lambdas) return fail(C, CAFE_ERR_INVALID, "request %d has no lambdas", b);
        for (int v = 0; v < T.n_nodes; ++v)
            if (T.parent[v] >= 0 && (T.lambda_index[v] < 0 || T.lambda_index[v] >= Q.n_lambdas))
                return fail(C, CAFE_ERR_INVALID, "lambda index %d out of range at node %d", T.lambda_index[v], v);
        if (gamma && (K < 1 || !Q.multipliers || !Q.cat_probs))
            return fail(C, CAFE_ERR_INVALID, "gamma needs K >= 1 with multipliers and probabilities");
    }
    const int64_t F = S.F;
    info->F = F;
    info->K = K;
    info->B = NB;
    info->cand_rejected.assign(NB, 0);
    info->cand_status.assign(NB, CAFE_OK);

    // lambda::is_valid (src/lambda.h:58-60, src/lambda.cpp:172-175) and
    // gamma_model::can_infer (src/gamma_core.cpp:123-141), per candidate
    int n_rej = 0;
    for (int b = 0; b < NB; ++b) {
        const cafe_request& Q = Rs[b];
        bool valid = true;
        double largest = Q.lambdas[0];
        for (int i = 0; i < Q.n_lambdas; ++i) {
            const double l = Q.lambdas[i];
            if (Q.lambda_kind == CAFE_LAMBDA_SINGLE ? !(l > 0) : (l < 0)) valid = false;
            largest = std::max(largest, l);
        }
        bool reject = !valid;
        if (!reject && gamma && T.longest_branch > 0) {
            const double al = largest * T.longest_branch / (1 + largest * T.longest_branch);
            if ((1 - 2 * al) < 0) reject = true;
        }
        if (reject) {
            info->cand_rejected[b] = 1;
            info->cand_status[b] = valid ? CAFE_ERR_SATURATED : CAFE_OK;
            n_rej++;
        }
    }
    CK(ws.nfail.reserve((size_t)NB * sizeof(int32_t)), "fail counter");
    if (n_rej == NB) {
        info->rejected = true;
        info->reject_status = info->cand_status[0];
        if (d_total) CK(launch_fill(d_total, NB, INFINITY, ws.stream), "fill");
        if (d_fam && F) CK(launch_fill(d_fam, (int64_t)NB * F, NAN, ws.stream), "fill");
        CK(launch_fill_i32(ws.nfail.as<int32_t>(), NB, 0, ws.stream), "fill");
        return CAFE_OK;
    }
    const int CT = NB * K;
    std::vector<int32_t> active;
    for (int b = 0; b < NB; ++b)
        if (!info->cand_rejected[b])
            for (int k = 0; k < K; ++k) active.push_back(b * K + k);

    const bool ref_mode = R->precision == CAFE_PREC_FP64_REF;
    const bool scaled = !ref_mode;
    info->scaled = scaled;
    int Sg = 0, Rg = 0, msize, W;
    int maxc = 0;
    for (int64_t f = 0; f < F; ++f) maxc = std::max(maxc, S.max_count[f]);
    if (ref_mode) {
        Sg = R->max_family_size;
        Rg = R->max_root_family_size;
        if (Sg < 1 || Rg < 1) return fail(C, CAFE_ERR_INVALID, "FP64_REF needs max_family_size and max_root_family_size");
        if (maxc > Sg) return fail(C, CAFE_ERR_INVALID, "a count (%d) exceeds max_family_size (%d)", maxc, Sg);
        msize = std::max(Rg, Sg) + 1;   // base_model.cpp:65
        W = std::max(Sg + 1, Rg);
    } else {
        msize = S.bins.W_max;
        W = S.bins.W_max;
    }

    // matrices for every (candidate, category, non-root node)
    const auto t_keys = std::chrono::steady_clock::now();
    cache_make_room(C, active.size() * (size_t)T.n_nodes * msize * msize * sizeof(double));
    C->cache.reserve(C->cache.size() + active.size() * (size_t)T.n_nodes);   // entry pointers stay valid
    PendingJobs P;
    std::vector<MatEntry*>& node_entry = ws.entry_vec;
    node_entry.assign((size_t)CT * T.n_nodes, nullptr);
    ws.sat_vec.assign((size_t)CT * T.n_nodes, 0);
    // the request's keys first, with their table slots prefetched (a large
    // cache misses in the CPU caches on every probe), then one
    // find-or-insert per key
    std::vector<MatKey>& keys = ws.key_vec;
    keys.clear();
    for (int c : active) {
        const cafe_request& Q = Rs[c / K];
        const double m = gamma ? Q.multipliers[c % K] : 1.0;
        for (int v = 0; v < T.n_nodes; ++v) {
            if (T.parent[v] < 0) continue;
            keys.push_back(make_key(msize, Q.lambdas[T.lambda_index[v]] * m, T.branch_length[v]));
            C->cache.prefetch(keys.back());
        }
    }
    size_t q = 0;
    for (int c : active)
        for (int v = 0; v < T.n_nodes; ++v) {
            if (T.parent[v] < 0) continue;
            const MatKey& key = keys[q++];
            node_entry[(size_t)c * T.n_nodes + v] = schedule(C, P, key);
            const double lq = (double)key.lq / 1000000000.0, tq = (double)key.tq / 1000.0;
            const double al = lq * tq / (1 + lq * tq), co = 1 - 2 * al;
            if (!(co > 0 && co != 1)) ws.sat_vec[(size_t)c * T.n_nodes + v] = 1;   // zero rows below row 0
        }
    int rc = cache_build(C, ws, P);
    if (rc) return rc;
    // one pass over the entries: matrix pointers, and the builds to wait for
    CK(ws.h_mats.reserve((size_t)CT * T.n_nodes * sizeof(double*)), "mats");
    CK(ws.mats.reserve((size_t)CT * T.n_nodes * sizeof(double*)), "mats");
    double** hm = ws.h_mats.as<double*>();
    std::fill(hm, hm + (size_t)CT * T.n_nodes, nullptr);
    std::vector<int> wait_chunks;
    for (int c : active)
        for (int v = 0; v < T.n_nodes; ++v) {
            const MatEntry* e = node_entry[(size_t)c * T.n_nodes + v];
            if (!e) continue;
            if (!e->d) return fail(C, CAFE_ERR_MISSING_MATRIX, "matrix not built");
            hm[(size_t)c * T.n_nodes + v] = e->d;
            if (std::find(wait_chunks.begin(), wait_chunks.end(), e->chunk) == wait_chunks.end())
                wait_chunks.push_back(e->chunk);
        }
    for (int b : wait_chunks) CK(cudaStreamWaitEvent(ws.stream, C->batch_events[b], 0), "event");
    if (C->prof.on) C->prof.acc.host_keys_ms += host_ms_since(t_keys);
    CK(ws.cat.reserve((size_t)std::max<int64_t>(F, 1) * CT * sizeof(double)), "category buffer");
    if (R->precision == CAFE_PREC_MIXED_TF32X3) {
        // polytomies stay on the FP64 path, and so do error models wider than
        // the +-kMaxErrHalf deviations the transposed leaf rows fold in;
        // saturated keys (1 - 2a < 0) run on the tensor cores (a family that
        // is exactly zero through one ends there)
        const bool to_fp64 = T.max_children > 2 || (R->use_error_model && C->err_ndev > 2 * kMaxErrHalf + 1);
        if (!to_fp64) {
            CK(ws.catids.reserve(active.size() * sizeof(int32_t)), "categories");
            CK(ws.h_catids.reserve(active.size() * sizeof(int32_t)), "categories");
            std::memcpy(ws.h_catids.p, active.data(), active.size() * sizeof(int32_t));
            CK(cudaMemcpyAsync(ws.catids.p, ws.h_catids.p, active.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                               ws.stream),
               "categories");
            const auto t_plan = std::chrono::steady_clock::now();
            const int rcm = enqueue_mixed_graph(C, ws, Rs, T, S, K, CT, active, hm, d_fam, d_total, info);
            if (C->prof.on) C->prof.acc.host_plan_ms += host_ms_since(t_plan);
            return rcm;
        }
        info->n_fallback = F;
    }

    // tiles
    std::vector<PruneTile>& tiles = ws.tile_vec;
    tiles.clear();
    std::vector<PruneTile>& cl_tiles = ws.cl_tile_vec;
    cl_tiles.clear();
    const int TFm = 32;
    const int64_t* d_perm;
    const int32_t* d_famR = nullptr;
    const bool dedupe = R->dedupe && !gamma && ref_mode;
    if (ref_mode) {
        const int64_t nf = dedupe ? (int64_t)S.unique.size() : F;
        d_perm = dedupe ? S.d_unique.as<int64_t>() : S.d_identity.as<int64_t>();
        // few families: one per cluster (the same bits as the tile walk)
        const bool cl = fp64_cluster_bin(C, T, nf, K, W);
        for (int c : active)
            for (int64_t i = 0; i < nf; i += cl ? 1 : TFm) {
                PruneTile t{};
                t.first = (int)i;
                t.count = cl ? 1 : (int)std::min<int64_t>(TFm, nf - i);
                t.k = c;
                t.S = Sg;
                t.R = Rg;
                (cl ? cl_tiles : tiles).push_back(t);
            }
    } else {
        d_perm = S.bins.d_perm.as<int64_t>();
        d_famR = S.bins.d_famR.as<int32_t>();
        for (size_t b = 0; b < S.bins.widths.size(); ++b)
            if (fp64_cluster_bin(C, T, S.bins.bin_count[b], K, S.bins.widths[b]))
                add_cluster_tiles(cl_tiles, S.bins, b, active);
        for (int c : active)
            for (size_t b = 0; b < S.bins.widths.size(); ++b) {
                if (fp64_cluster_bin(C, T, S.bins.bin_count[b], K, S.bins.widths[b])) continue;
                for (int64_t i = 0; i < S.bins.bin_count[b]; i += TFm) {
                    PruneTile t{};
                    t.first = (int)(S.bins.bin_first[b] + i);
                    t.count = (int)std::min<int64_t>(TFm, S.bins.bin_count[b] - i);
                    t.k = c;
                    t.S = S.bins.widths[b] - 1;
                    t.R = S.bins.widths[b] - 1;
                    tiles.push_back(t);
                }
            }
    }
    const int n_tiles = (int)tiles.size();
    CK(ws.h_tiles.reserve(std::max(n_tiles, 1) * sizeof(PruneTile)), "tiles");
    CK(ws.tiles.reserve(std::max(n_tiles, 1) * sizeof(PruneTile)), "tiles");
    std::memcpy(ws.h_tiles.p, tiles.data(), n_tiles * sizeof(PruneTile));

    const int n_ctas = std::max(1, std::min(n_tiles, C->n_ctas));
    const int64_t per_cta = (int64_t)T.n_slots * W * TFm;
    CK(ws.scratch.reserve((size_t)n_ctas * per_cta * sizeof(double)), "scratch");
    info->footprint = (size_t)n_ctas * per_cta * sizeof(double) + (size_t)F * CT * sizeof(double);

    CK(cudaMemcpyAsync(ws.tiles.p, ws.h_tiles.p, n_tiles * sizeof(PruneTile), cudaMemcpyHostToDevice, ws.stream),
       "tiles");
    CK(cudaMemcpyAsync(ws.mats.p, hm, (size_t)CT * T.n_nodes * sizeof(double*), cudaMemcpyHostToDevice, ws.stream),
       "mats");
    if (gamma && !scaled) CK(launch_fill(ws.cat.as<double>(), F * CT, 0.0, ws.stream), "fill");
    rc = stage_cat_probs(C, ws, Rs, K, NB);
    if (rc) return rc;

    Prune64Args a{};
    a.plan = T.plan;
    a.tiles = ws.tiles.as<PruneTile>();
    a.n_tiles = n_tiles;
    a.counts = S.d_counts.as<int32_t>();
    a.perm = d_perm;
    a.mats = ws.mats.as<const double*>();
    a.ld_mat = msize;
    a.prior = C->d_prior.as<double>();
    a.n_prior = (int)C->prior.size();
    a.err = R->use_error_model ? C->d_err.as<double>() : nullptr;
    a.err_rows = C->err_rows;
    a.err_ndev = C->err_ndev;
    a.fam_R = d_famR;
    a.scratch = ws.scratch.as<double>();
    a.scratch_per_cta = per_cta;
    a.scaled = scaled ? 1 : 0;
    a.model = gamma ? 1 : 0;
    a.out = ws.cat.as<double>();
    a.K = CT;
    a.cat_probs = ws.catp.as<double>();
    a.tile_families = TFm;
    a.W = W;
    const bool prof = ws.sync;
    cudaEvent_t ev;
    if (prof) {
        C->prof.begin(1, ws.stream, &ev);
        C->prof.acc.prune_flops += tiles_flops(T, tiles, R->use_error_model);
    }
    CK(launch_prune64(a, n_ctas, ws.stream), "prune");
    if (prof) C->prof.end(1, ws.stream, ev);
    if (prof) C->prof.acc.prune_flops += tiles_flops(T, cl_tiles, R->use_error_model);
    rc = launch_fp64_cluster(C, ws, R, T, S, CT, cl_tiles, d_perm, d_famR, msize, scaled, ws.cat.as<double>(),
                             ws.stream, 1);
    if (rc) return rc;
    return finish_batch(C, ws, info, gamma, scaled, dedupe ? S.d_ref.as<int64_t>() : nullptr, nullptr, d_fam, d_total);
}

bool small_request(const cafe_ctx* C, const cafe_request* R, int NB, int64_t F) {
    const int K = R->model == CAFE_MODEL_GAMMA ? std::max(1, R->n_categories) : 1;
    return F * NB * K < (int64_t)C->sm_count * 128;
}

// Direct calls on the context's own workspaces (cafe_score_batch_device)
// keep their device timelines in call order: each waits for the previous
// call's last launch. Serving batches do not: their work overlaps on the
// device (the matrix cache is append-only while anything is in flight, and
// every other buffer a batch writes belongs to its workspace). Caller
// holds C->mu.
cudaError_t gate_enter(cafe_ctx* C, Workspace& ws) {
    return C->gate_set ? cudaStreamWaitEvent(ws.stream, C->gate, 0) : cudaSuccess;
}
cudaError_t gate_leave(cafe_ctx* C, Workspace& ws) {
    const cudaError_t e = cudaEventRecord(C->gate, ws.stream);
    if (e == cudaSuccess) C->gate_set = true;
    return e;
}

// Phase 1 of a host-visible score of NB batched candidates: enqueue the
// evaluation and the copies back into pinned staging (caller holds C->mu).
// Host staging: totals [NB], fail counts [NB], family lnL [NB][F], then
// category values [F][NB * K] when any result asks for them.
int score_enqueue(cafe_ctx* C, Workspace& ws, const cafe_request* R, int NB, cafe_result* res, ScoreInfo* info) {
    AllocScope scope(ws.stream);
    auto si = C->sets.find(R ? R->set_id : -1);
    if (si == C->sets.end()) return fail(C, CAFE_ERR_NOT_FOUND, "unknown family set");
    if (NB < 1) return fail(C, CAFE_ERR_INVALID, "empty batch");
    const int64_t F = si->second->F;
    CK(ws.fam_lnl.reserve((size_t)std::max<int64_t>(F, 1) * NB * sizeof(double)), "family buffer");
    CK(ws.total.reserve((size_t)NB * sizeof(double)), "total");
    CK(cudaEventRecord(ws.ev_start, ws.stream), "event");
    const auto t_host = std::chrono::steady_clock::now();
    int rc = enqueue_score(C, ws, R, NB, ws.fam_lnl.as<double>(), ws.total.as<double>(), info);
    if (rc) return rc;
    if (C->prof.on && ws.sync) C->prof.acc.host_total_ms += host_ms_since(t_host);
    CK(cudaEventRecord(ws.ev_staged, ws.stream), "event");
    ws.staged = true;
    CK(cudaEventRecord(ws.ev_stop, ws.stream), "event");
    const int K = info->K;
    bool any_cat = false;
    for (int b = 0; b < NB && res; ++b) any_cat |= res[b].category_lnl != nullptr;
    const size_t head = (size_t)NB * (sizeof(double) + sizeof(int32_t));
    const size_t head8 = (head + 7) & ~(size_t)7;
    const size_t out_bytes = head8 + (size_t)NB * F * sizeof(double) + (any_cat ? (size_t)F * NB * K * sizeof(double) : 0);
    CK(ws.h_out.reserve(out_bytes + 64), "host staging");
    CK(ws.h_tail.reserve(64), "host staging");
    if (info->d_tail)
        CK(cudaMemcpyAsync(ws.h_tail.p, info->d_tail, 3 * sizeof(int32_t), cudaMemcpyDeviceToHost, ws.stream), "d2h");
    char* h = static_cast<char*>(ws.h_out.p);
    double* h_total = reinterpret_cast<double*>(h);
    int32_t* h_fail = reinterpret_cast<int32_t*>(h + (size_t)NB * sizeof(double));
    double* h_fam = reinterpret_cast<double*>(h + head8);
    double* h_cat = h_fam + (size_t)NB * F;
    CK(cudaMemcpyAsync(h_total, ws.total.p, (size_t)NB * sizeof(double), cudaMemcpyDeviceToHost, ws.stream), "d2h");
    CK(cudaMemcpyAsync(h_fail, ws.nfail.p, (size_t)NB * sizeof(int32_t), cudaMemcpyDeviceToHost, ws.stream), "d2h");
    if (F) CK(cudaMemcpyAsync(h_fam, ws.fam_lnl.p, (size_t)NB * F * sizeof(double), cudaMemcpyDeviceToHost, ws.stream), "d2h");
    if (any_cat && F && !info->rejected)
        CK(cudaMemcpyAsync(h_cat, ws.cat.p, (size_t)F * NB * K * sizeof(double), cudaMemcpyDeviceToHost, ws.stream), "d2h");
    return CAFE_OK;
}

// Phase 2: wait for the stream and fill the results (no context lock
// needed: the workspace belongs to the caller).
int score_complete(cafe_ctx* C, Workspace& ws, const cafe_request* R, int NB, cafe_result* res, const ScoreInfo& info) {
    CK(cudaStreamSynchronize(ws.stream), "score");
    if (!res) return CAFE_OK;
    const int64_t F = info.F;
    const int K = info.K;
    const size_t head = (size_t)NB * (sizeof(double) + sizeof(int32_t));
    const size_t head8 = (head + 7) & ~(size_t)7;
    char* h = static_cast<char*>(ws.h_out.p);
    const double* h_total = reinterpret_cast<const double*>(h);
    const int32_t* h_fail = reinterpret_cast<const int32_t*>(h + (size_t)NB * sizeof(double));
    const double* h_fam = reinterpret_cast<const double*>(h + head8);
    const double* h_cat = h_fam + (size_t)NB * F;
    float ms = 0;
    cudaEventElapsedTime(&ms, ws.ev_start, ws.ev_stop);
    int64_t n_fb = info.n_fallback;
    if (info.d_tail) {
        const int32_t* tail = ws.h_tail.as<int32_t>();
        if (tail[0]) return fail(C, CAFE_ERR_TIMEOUT, "tensor-core pruning gave up waiting (status %d)", tail[0]);
        n_fb = tail[1];
    }
    const bool gamma = R->model == CAFE_MODEL_GAMMA;
    for (int b = 0; b < NB; ++b) {
        cafe_result& r = res[b];
        const bool rej = info.cand_rejected.empty() ? info.rejected : info.cand_rejected[b] != 0;
        r.device_ms = ms;
        r.total_neg_lnl = h_total[b];
        r.n_failed = rej ? 0 : h_fail[b];
        r.n_fallback = n_fb;
        if (r.family_lnl && F) std::memcpy(r.family_lnl, h_fam + (size_t)b * F, F * sizeof(double));
        if (r.category_lnl && F) {
            const bool want_cat = !rej;
            for (int64_t f = 0; f < F; ++f)
                for (int k = 0; k < K; ++k) {
                    double v = NAN;
                    if (want_cat && gamma) {
                        const double c = h_cat[(size_t)f * NB * K + (size_t)b * K + k];
                        v = info.scaled ? c : (c < 0 ? NAN : std::log(c));
                    } else if (want_cat) {
                        v = h_fam[(size_t)b * F + f];
                    }
                    r.category_lnl[f * K + k] = v;
                }
        }
        if (rej) r.status = info.cand_status.empty() ? info.reject_status : info.cand_status[b];
        else if (r.n_failed) r.status = CAFE_ERR_SATURATED;
        else if (std::isinf(r.total_neg_lnl)) r.status = CAFE_ERR_UNDERFLOW;
        else r.status = CAFE_OK;
    }
    return CAFE_OK;
}

int score_sync(cafe_ctx* C, Workspace& ws, const cafe_request* R, int NB, cafe_result* res) {
    ScoreInfo info;
    // nothing of this workspace is in flight for a build to hide behind
    struct Inline {
        Workspace& w;
        explicit Inline(Workspace& x) : w(x) { w.build_inline = true; }
        ~Inline() { w.build_inline = false; }
    } in_line(ws);
    int rc = score_enqueue(C, ws, R, NB, res, &info);
    if (rc) return rc;
    return score_complete(C, ws, R, NB, res, info);
}

// ---- ancestral reconstruction

// Shared checks of cafe_reconstruct / cafe_branch_probabilities: tree, set,
// lambdas, bounds; the FP64 matrix of every (category, non-root node) at
// side max(S, R) + 1 (the reference's cache side plus 100 holds the same
// entries), pointers staged into ws.mats with the builds waited for.
struct ReconSetup {
    TreeHost* T = nullptr;
    FamSet* S = nullptr;
    int K = 1, Smax = 0, Rmax = 0, msize = 0;
    bool gamma = false;
};

int recon_setup(cafe_ctx* C, Workspace& ws, const cafe_request* R, bool categories, ReconSetup* o) {
    if (!R) return fail(C, CAFE_ERR_INVALID, "null request");
    auto ti = C->trees.find(R->tree_id);
    if (ti == C->trees.end()) return fail(C, CAFE_ERR_NOT_FOUND, "unknown tree id %d", R->tree_id);
    auto si = C->sets.find(R->set_id);
    if (si == C->sets.end()) return fail(C, CAFE_ERR_NOT_FOUND, "unknown family set id %d", R->set_id);
    TreeHost& T = *ti->second;
    FamSet& S = *si->second;
    if (S.tree_id != R->tree_id) return fail(C, CAFE_ERR_INVALID, "family set %d belongs to tree %d", R->set_id, S.tree_id);
    const bool gamma = categories && R->model == CAFE_MODEL_GAMMA;
    if (R->model != CAFE_MODEL_BASE && R->model != CAFE_MODEL_GAMMA) return fail(C, CAFE_ERR_INVALID, "bad model %d", R->model);
    const int K = gamma ? R->n_categories : 1;
    if (gamma && (K < 1 || !R->multipliers || !R->cat_probs))
        return fail(C, CAFE_ERR_INVALID, "gamma needs K >= 1 with multipliers and probabilities");
    if (R->n_lambdas < 1 || !R->lambdas) return fail(C, CAFE_ERR_INVALID, "no lambdas");
    for (int v = 0; v < T.n_nodes; ++v)
        if (T.parent[v] >= 0 && (T.lambda_index[v] < 0 || T.lambda_index[v] >= R->n_lambdas))
            return fail(C, CAFE_ERR_INVALID, "lambda index %d out of range at node %d", T.lambda_index[v], v);
    const int Sg = R->max_family_size, Rg = R->max_root_family_size;
    if (Sg < 1 || Rg < 1) return fail(C, CAFE_ERR_INVALID, "reconstruction needs max_family_size and max_root_family_size");
    int maxc = 0;
    for (int64_t f = 0; f < S.F; ++f) maxc = std::max(maxc, S.max_count[f]);
    if (maxc > Sg) return fail(C, CAFE_ERR_INVALID, "a count (%d) exceeds max_family_size (%d)", maxc, Sg);
    const int msize = std::max(Sg, Rg) + 1;
    cache_make_room(C, (size_t)K * T.n_nodes * msize * msize * sizeof(double));
    C->cache.reserve(C->cache.size() + (size_t)K * T.n_nodes);
    PendingJobs P;
    std::vector<MatEntry*>& ent = ws.entry_vec;
    ent.assign((size_t)K * T.n_nodes, nullptr);
    for (int k = 0; k < K; ++k) {
        const double m = gamma ? R->multipliers[k] : 1.0;
        for (int v = 0; v < T.n_nodes; ++v) {
            if (T.parent[v] < 0) continue;
            const double lam = R->lambdas[T.lambda_index[v]] * m;   // lambda::multiply, then get_value_for_clade
            ent[(size_t)k * T.n_nodes + v] = schedule(C, P, make_key(msize, lam, T.branch_length[v]));
        }
    }
    int rc = cache_build(C, ws, P);
    if (rc) return rc;
    CK(ws.h_mats.reserve((size_t)K * T.n_nodes * sizeof(double*)), "mats");
    CK(ws.mats.reserve((size_t)K * T.n_nodes * sizeof(double*)), "mats");
    double** hm = ws.h_mats.as<double*>();
    std::vector<int> wait_chunks;
    for (size_t i = 0; i < (size_t)K * T.n_nodes; ++i) {
        const MatEntry* e = ent[i];
        hm[i] = e ? e->d : nullptr;
        if (!e) continue;
        if (!e->d) return fail(C, CAFE_ERR_MISSING_MATRIX, "matrix not built");
        if (std::find(wait_chunks.begin(), wait_chunks.end(), e->chunk) == wait_chunks.end())
            wait_chunks.push_back(e->chunk);
    }
    for (int b : wait_chunks) CK(cudaStreamWaitEvent(ws.stream, C->batch_events[b], 0), "event");
    CK(cudaMemcpyAsync(ws.mats.p, hm, (size_t)K * T.n_nodes * sizeof(double*), cudaMemcpyHostToDevice, ws.stream),
       "mats");
    o->T = &T;
    o->S = &S;
    o->K = K;
    o->Smax = Sg;
    o->Rmax = Rg;
    o->msize = msize;
    o->gamma = gamma;
    return CAFE_OK;
}

int reconstruct_sync(cafe_ctx* C, Workspace& ws, const cafe_request* R, cafe_reconstruction* out) {
    AllocScope scope(ws.stream);
    if (ws.staged) {   // the previous request's copies out of the pinned staging buffers
        CK(cudaEventSynchronize(ws.ev_staged), "staging");
        ws.staged = false;
    }
    if (!out) return fail(C, CAFE_ERR_INVALID, "null output");
    if (C->prior.empty()) return fail(C, CAFE_ERR_INVALID, "no prior set (cafe_prior_set)");
    CK(cudaEventRecord(ws.ev_start, ws.stream), "event");
    ReconSetup Z;
    int rc = recon_setup(C, ws, R, true, &Z);
    if (rc) return rc;
    TreeHost& T = *Z.T;
    const int64_t F = Z.S->F;
    const int K = Z.K, n = T.n_nodes;
    std::vector<PruneTile>& tiles = ws.tile_vec;
    tiles.clear();
    for (int k = 0; k < K; ++k)
        for (int64_t f = 0; f < F; f += 32) {
            PruneTile t{};
            t.first = (int)f;
            t.count = (int)std::min<int64_t>(32, F - f);
            t.k = k;
            tiles.push_back(t);
        }
    const int n_tiles = (int)tiles.size();
    const int n_ctas = std::max(1, std::min(n_tiles, C->n_ctas));
    const size_t per_cta = pupko_scratch_doubles(T.plan, Z.Smax);
    const size_t c_per_cta = pupko_c_entries(T.plan, Z.Smax);
    CK(ws.h_tiles.reserve(std::max(n_tiles, 1) * sizeof(PruneTile)), "tiles");
    CK(ws.tiles.reserve(std::max(n_tiles, 1) * sizeof(PruneTile)), "tiles");
    CK(ws.scratch.reserve((size_t)n_ctas * per_cta * sizeof(double)), "scratch");
    CK(ws.rc_c.reserve(std::max<size_t>((size_t)n_ctas * c_per_cta, 1) * sizeof(int32_t)), "argmax tables");
    const size_t n_state = (size_t)K * F * n, n_fam = (size_t)F * n;
    CK(ws.rc_state.reserve(std::max<size_t>(n_state, 1) * sizeof(int32_t)), "states");
    CK(ws.rc_rmax.reserve(std::max<size_t>((size_t)K * F, 1) * sizeof(double)), "root max");
    CK(ws.rc_mean.reserve(std::max<size_t>(n_fam, 1) * sizeof(double)), "means");
    CK(ws.rc_count.reserve(std::max<size_t>(n_fam, 1) * sizeof(int32_t)), "counts");
    CK(ws.rc_nfail.reserve(sizeof(int32_t)), "failed");
    std::memcpy(ws.h_tiles.p, tiles.data(), n_tiles * sizeof(PruneTile));
    CK(cudaMemcpyAsync(ws.tiles.p, ws.h_tiles.p, n_tiles * sizeof(PruneTile), cudaMemcpyHostToDevice, ws.stream),
       "tiles");
    CK(cudaMemsetAsync(ws.rc_nfail.p, 0, sizeof(int32_t), ws.stream), "failed");
    if (Z.gamma) {
        rc = stage_cat_probs(C, ws, R, K, 1);
        if (rc) return rc;
    }
    // transposed log2 of every internal non-root node's matrix (pass 1 of k_pupko)
    const int nstate = Z.Smax + 1;
    std::vector<const void*> lsrc, ldst;
    std::vector<const float*> lmats((size_t)K * n, nullptr);
    {
        int n_int = 0;
        for (int v = 0; v < n; ++v) n_int += (T.parent[v] >= 0 && T.leaf_col[v] < 0);
        const size_t per = (size_t)nstate * nstate;
        CK(ws.rc_lm.reserve(std::max<size_t>((size_t)K * n_int * per, 1) * sizeof(float)), "log2 matrices");
        const double* const* hmats = ws.h_mats.as<const double*>();
        size_t slot = 0;
        for (int k = 0; k < K; ++k)
            for (int v = 0; v < n; ++v) {
                if (T.parent[v] < 0 || T.leaf_col[v] >= 0) continue;
                float* d = ws.rc_lm.as<float>() + slot++ * per;
                lmats[(size_t)k * n + v] = d;
                lsrc.push_back(hmats[(size_t)k * n + v]);
                ldst.push_back(d);
            }
        const size_t np = lmats.size() + 2 * lsrc.size();
        CK(ws.rc_lptr.reserve(std::max<size_t>(np, 1) * sizeof(void*)), "log2 matrices");
        std::vector<const void*> all;
        all.reserve(np);
        for (const float* p : lmats) all.push_back(p);
        all.insert(all.end(), lsrc.begin(), lsrc.end());
        all.insert(all.end(), ldst.begin(), ldst.end());
        CK(cudaMemcpyAsync(ws.rc_lptr.p, all.data(), np * sizeof(void*), cudaMemcpyHostToDevice, ws.stream), "h2d");
    }
    const void* const* dptr = ws.rc_lptr.as<const void*>();
    PupkoArgs a{};
    a.lmats = reinterpret_cast<const float* const*>(dptr);
    a.plan = T.plan;
    a.tiles = ws.tiles.as<PruneTile>();
    a.n_tiles = n_tiles;
    a.counts = Z.S->d_counts.as<int32_t>();
    a.F = F;
    a.mats = ws.mats.as<const double*>();
    a.ld_mat = Z.msize;
    a.prior = C->d_prior.as<double>();
    a.n_prior = (int)C->prior.size();
    a.S = Z.Smax;
    a.root_len = std::min(Z.Smax, Z.Rmax) + 1;
    a.scratch = ws.scratch.as<double>();
    a.scratch_per_cta = (int64_t)per_cta;
    a.cscratch = ws.rc_c.as<int32_t>();
    a.c_per_cta = (int64_t)c_per_cta;
    a.state = ws.rc_state.as<int32_t>();
    a.root_max = ws.rc_rmax.as<double>();
    a.n_failed = ws.rc_nfail.as<int32_t>();
    a.exhaustive = out->exhaustive ? 1 : 0;
    if (F > 0) {
        CK(launch_log2_matrices(reinterpret_cast<const double* const*>(dptr + lmats.size()),
                                reinterpret_cast<float* const*>(const_cast<void**>(dptr + lmats.size() + lsrc.size())),
                                (int)lsrc.size(), nstate, Z.msize, ws.stream),
           "log2 matrices");
        CK(launch_pupko(a, n_ctas, ws.stream), "reconstruct");
        CK(launch_recon_counts(ws.rc_state.as<int32_t>(), F, n, K, Z.gamma ? ws.catp.as<double>() : nullptr,
                               Z.gamma ? 1 : 0, T.plan.leaf_col, ws.rc_mean.as<double>(), ws.rc_count.as<int32_t>(),
                               ws.stream),
           "node counts");
    }
    CK(cudaEventRecord(ws.ev_stop, ws.stream), "event");
    int32_t nf = 0;
    CK(cudaMemcpyAsync(&nf, ws.rc_nfail.p, sizeof(int32_t), cudaMemcpyDeviceToHost, ws.stream), "d2h");
    if (F > 0) {
        if (out->node_count)
            CK(cudaMemcpyAsync(out->node_count, ws.rc_count.p, n_fam * sizeof(int32_t), cudaMemcpyDeviceToHost, ws.stream),
               "d2h");
        if (out->node_mean)
            CK(cudaMemcpyAsync(out->node_mean, ws.rc_mean.p, n_fam * sizeof(double), cudaMemcpyDeviceToHost, ws.stream),
               "d2h");
        if (out->category_state)
            CK(cudaMemcpyAsync(out->category_state, ws.rc_state.p, n_state * sizeof(int32_t), cudaMemcpyDeviceToHost,
                               ws.stream),
               "d2h");
        if (out->root_max)
            CK(cudaMemcpyAsync(out->root_max, ws.rc_rmax.p, (size_t)K * F * sizeof(double), cudaMemcpyDeviceToHost,
                               ws.stream),
               "d2h");
    }
    CK(cudaStreamSynchronize(ws.stream), "reconstruct");
    float ms = 0;
    cudaEventElapsedTime(&ms, ws.ev_start, ws.ev_stop);
    out->device_ms = ms;
    out->n_failed = nf;
    return CAFE_OK;
}

// ---- host row sampling (p-values, simulation)

// Prefix order (clade::apply_prefix_order, src/clade.cpp:275-291): a node,
// then its children's subtrees in descendant order.
std::vector<int> prefix_order(const TreeHost& T) {
    std::vector<int> prefix, st{T.root};
    while (!st.empty()) {
        const int v = st.back();
        st.pop_back();
        prefix.push_back(v);
        for (auto it = T.children[v].rbegin(); it != T.children[v].rend(); ++it) st.push_back(*it);
    }
    return prefix;
}

// Samples a child size from the parent's matrix row with the reference's
// draws (matrix::select_random_y, src/matrix_cache.cpp:60-66:
// std::discrete_distribution over the first S entries of the row; on a
// saturated branch set_weighted_random_family_size, src/probability.cpp:
// 458-468, first draws and discards a uniform size). The matrices are the
// context cache's (built on the GPU), copied to the host; distributions are
// built once per (matrix, parent size) instead of once per draw.
struct HostSampler {
    int msize = 0, S = 0, n = 0, n_ps = 0;
    std::vector<std::vector<double>> mats;   // distinct matrices
    std::vector<int> node_mi;                // [K][n] matrix of (category, node), -1 at the root
    std::vector<char> saturated;             // [K][n]
    std::vector<std::unique_ptr<std::discrete_distribution<int>>> dists;   // [matrix][parent size]

    int draw(int k, int v, int ps, std::mt19937& eng) {
        const size_t kv = (size_t)k * n + v;
        if (saturated[kv]) {
            std::uniform_int_distribution<int> d(0, S - 1);
            d(eng);
        }
        std::unique_ptr<std::discrete_distribution<int>>& d = dists[(size_t)node_mi[kv] * n_ps + ps];
        if (!d) {
            const double* row = mats[node_mi[kv]].data() + (size_t)ps * msize;
            d.reset(new std::discrete_distribution<int>(row, row + S));
        }
        return (*d)(eng);
    }
};

// ws.h_mats holds the K x n matrix pointers recon_setup staged; parent sizes
// reach max(R, S).
int host_sampler_init(cafe_ctx* C, Workspace& ws, const cafe_request* R, const TreeHost& T, const ReconSetup& Z,
                      int K, const double* multipliers, HostSampler* hs) {
    const int n = T.n_nodes;
    hs->msize = Z.msize;
    hs->S = Z.Smax;
    hs->n = n;
    hs->n_ps = std::max(Z.Rmax, Z.Smax) + 1;
    hs->node_mi.assign((size_t)K * n, -1);
    hs->saturated.assign((size_t)K * n, 0);
    const double* const* hm = ws.h_mats.as<const double*>();
    std::map<const double*, int> ids;
    for (int k = 0; k < K; ++k) {
        const double mult = multipliers ? multipliers[k] : 1.0;
        for (int v = 0; v < n; ++v) {
            if (T.parent[v] < 0) continue;
            const double* d = hm[(size_t)k * n + v];
            auto ins = ids.emplace(d, (int)hs->mats.size());
            if (ins.second) {
                hs->mats.emplace_back((size_t)Z.msize * Z.msize);
                CK(cudaMemcpyAsync(hs->mats.back().data(), d, hs->mats.back().size() * sizeof(double),
                                   cudaMemcpyDeviceToHost, ws.stream),
                   "d2h");
            }
            hs->node_mi[(size_t)k * n + v] = ins.first->second;
            const double lam = R->lambdas[T.lambda_index[v]] * mult, t = T.branch_length[v];
            hs->saturated[(size_t)k * n + v] = (1 - 2 * (lam * t / (1 + lam * t))) < 0;   // matrix_cache::is_saturated
        }
    }
    CK(cudaStreamSynchronize(ws.stream), "matrices");
    hs->dists.clear();
    hs->dists.resize(hs->mats.size() * (size_t)hs->n_ps);
    return CAFE_OK;
}

// ---- p-values

// compute_pvalues with the simulated families drawn on the GPU (k_pvalue.cu:
// a counter-based generator, one thread per family; the same distributions
// as the reference's draws, not its stream). Every step runs on the device:
// the row CDFs, the draws, the grouping of the simulated families into
// 32-family tiles of equal (root size, state bound), their pruning with the
// root fixed, the per-root-size sort and the p-value search; the host only
// copies the results back.
int pvalues_device(cafe_ctx* C, Workspace& ws, const cafe_request* R, cafe_pvalues_out* out) {
    const auto t_host0 = std::chrono::steady_clock::now();
    ReconSetup Z;
    int rc = recon_setup(C, ws, R, false, &Z);
    if (rc) return rc;
    TreeHost& T = *Z.T;
    FamSet& FS = *Z.S;
    const int S = Z.Smax, RR = Z.Rmax, msize = Z.msize, nsim = out->n_simulations, n = T.n_nodes;
    if (nsim > kSortRowsMaxP)
        return fail(C, CAFE_ERR_INVALID, "device sampling takes at most %d simulations per root size", kSortRowsMaxP);
    const int n_ps = std::max(RR, S) + 1;
    if (n_ps > msize) return fail(C, CAFE_ERR_INVALID, "parent sizes beyond the matrices");
    const int64_t F = FS.F;
    const int L = T.n_leaves;
    const int64_t NS = (int64_t)RR * nsim;
    const int n_keys = RR * (S + 1);
    const int64_t max_tiles = NS / 32 + n_keys + 1;
    const int Wmax = std::max(S + 1, RR);
    DevBuf d_cdf, d_sizes, d_sim, d_keys, d_hist, d_cursor, d_perm, d_tiles, d_ntiles, d_simL, d_obsL, d_pv, d_tree,
        d_otiles;
    CK(d_cdf.reserve((size_t)n * n_ps * S * sizeof(double)), "row cdfs");
    CK(d_sizes.reserve((size_t)NS * n * sizeof(int32_t)), "simulated families");
    CK(d_sim.reserve(std::max<size_t>((size_t)NS * L, 1) * sizeof(int32_t)), "simulated families");
    CK(d_keys.reserve((size_t)NS * sizeof(int32_t)), "simulated families");
    CK(d_hist.reserve((size_t)n_keys * sizeof(int32_t)), "simulation plan");
    CK(d_cursor.reserve((size_t)n_keys * sizeof(int32_t)), "simulation plan");
    CK(d_perm.reserve((size_t)NS * sizeof(int64_t)), "simulation plan");
    CK(d_tiles.reserve((size_t)max_tiles * sizeof(PruneTile)), "tiles");
    CK(d_ntiles.reserve(16), "tiles");
    CK(d_simL.reserve((size_t)NS * sizeof(double)), "simulated likelihoods");
    CK(d_obsL.reserve(std::max<size_t>((size_t)F * RR, 1) * sizeof(double)), "root vectors");
    CK(d_pv.reserve(std::max<size_t>((size_t)F, 1) * sizeof(double)), "p-values");
    // prefix order, parents and leaf columns of the tree
    const std::vector<int> prefix = prefix_order(T);
    std::vector<int32_t> tree_tab(3 * (size_t)n);
    for (int i = 0; i < n; ++i) {
        tree_tab[i] = prefix[i];
        tree_tab[n + i] = T.parent[i];
        tree_tab[2 * n + i] = T.leaf_col[i];
    }
    CK(d_tree.reserve(tree_tab.size() * sizeof(int32_t)), "tree");
    CK(cudaMemcpy(d_tree.p, tree_tab.data(), tree_tab.size() * sizeof(int32_t), cudaMemcpyHostToDevice), "tree");
    // observed families: states 0..S, root sizes 1..R
    std::vector<PruneTile> otiles;
    for (int64_t f = 0; f < F; f += 32) {
        PruneTile t{};
        t.first = (int)f;
        t.count = (int)std::min<int64_t>(32, F - f);
        t.S = S;
        t.R = RR;
        t.root_lo = 1;
        otiles.push_back(t);
    }
    if (!otiles.empty()) {
        CK(d_otiles.reserve(otiles.size() * sizeof(PruneTile)), "tiles");
        CK(cudaMemcpy(d_otiles.p, otiles.data(), otiles.size() * sizeof(PruneTile), cudaMemcpyHostToDevice), "tiles");
    }
    const int n_ctas_max = C->n_ctas;
    CK(ws.scratch.reserve((size_t)n_ctas_max * T.n_slots * Wmax * 32 * sizeof(double)), "scratch");
    double host_ms = host_ms_since(t_host0);

    Prune64Args a{};
    a.plan = T.plan;
    a.mats = ws.mats.as<const double*>();
    a.ld_mat = msize;
    a.scratch = ws.scratch.as<double>();
    a.scratch_per_cta = (int64_t)T.n_slots * Wmax * 32;
    a.K = 1;
    a.tile_families = 32;
    a.W = Wmax;
    CK(cudaEventRecord(ws.ev_start, ws.stream), "event");
    if (!otiles.empty()) {
        Prune64Args o = a;
        o.tiles = d_otiles.as<PruneTile>();
        o.n_tiles = (int)otiles.size();
        o.counts = FS.d_counts.as<int32_t>();
        o.perm = FS.d_identity.as<int64_t>();
        o.root_out = d_obsL.as<double>();
        o.root_ld = RR;
        CK(launch_prune64(o, std::max(1, std::min((int)otiles.size(), n_ctas_max)), ws.stream), "prune root vectors");
    }
    CK(launch_cdf_build(ws.mats.as<const double*>(), n, msize, S, n_ps, d_cdf.as<double>(), ws.stream), "row cdfs");
    CK(cudaMemsetAsync(d_hist.p, 0, (size_t)n_keys * sizeof(int32_t), ws.stream), "simulation plan");
    SimDrawArgs sd{};
    sd.cdf = d_cdf.as<double>();
    sd.prefix = d_tree.as<int32_t>();
    sd.parent = d_tree.as<int32_t>() + n;
    sd.leaf_col = d_tree.as<int32_t>() + 2 * n;
    sd.n_nodes = n;
    sd.n_leaves = L;
    sd.root = T.root;
    sd.n_ps = n_ps;
    sd.S = S;
    sd.n_sim = nsim;
    sd.n_families = NS;
    sd.key = sim_seed_key(out->seed);
    sd.sizes = d_sizes.as<int32_t>();
    sd.counts = d_sim.as<int32_t>();
    sd.keys = d_keys.as<int32_t>();
    sd.hist = d_hist.as<int32_t>();
    CK(launch_sim_draw(sd, ws.stream), "simulation draws");
    SimPlanArgs sp{};
    sp.hist = d_hist.as<int32_t>();
    sp.n_keys = n_keys;
    sp.S = S;
    sp.cursor = d_cursor.as<int32_t>();
    sp.tiles = d_tiles.as<PruneTile>();
    sp.max_tiles = max_tiles;
    sp.n_tiles = d_ntiles.as<int32_t>();
    CK(launch_sim_plan(sp, ws.stream), "simulation plan");
    CK(launch_sim_scatter(d_keys.as<int32_t>(), NS, d_cursor.as<int32_t>(), d_perm.as<int64_t>(), ws.stream),
       "simulation plan");
    Prune64Args p = a;
    p.tiles = d_tiles.as<PruneTile>();
    p.n_tiles = 0;
    p.n_tiles_dev = d_ntiles.as<int32_t>();
    p.counts = d_sim.as<int32_t>();
    p.perm = d_perm.as<int64_t>();
    p.root_out = d_simL.as<double>();
    p.root_ld = 1;
    CK(launch_prune64(p, (int)std::max<int64_t>(1, std::min<int64_t>(max_tiles, n_ctas_max)), ws.stream),
       "prune simulated families");
    CK(launch_sort_rows(d_simL.as<double>(), RR, nsim, ws.stream), "sort");
    PvalueSearchArgs ps{};
    ps.counts = FS.d_counts.as<int32_t>();
    ps.F = F;
    ps.n_leaves = L;
    ps.obs = d_obsL.as<double>();
    ps.sorted = d_simL.as<double>();
    ps.R = RR;
    ps.n_sim = nsim;
    ps.out = d_pv.as<double>();
    CK(launch_pvalue_search(ps, ws.stream), "p-values");
    CK(cudaEventRecord(ws.ev_stop, ws.stream), "event");
    if (F) CK(cudaMemcpyAsync(out->pvalues, d_pv.p, (size_t)F * sizeof(double), cudaMemcpyDeviceToHost, ws.stream), "d2h");
    if (out->conditional)
        CK(cudaMemcpyAsync(out->conditional, d_simL.p, (size_t)NS * sizeof(double), cudaMemcpyDeviceToHost, ws.stream),
           "d2h");
    if (out->root_likelihood && F)
        CK(cudaMemcpyAsync(out->root_likelihood, d_obsL.p, (size_t)F * RR * sizeof(double), cudaMemcpyDeviceToHost,
                           ws.stream),
           "d2h");
    CK(cudaStreamSynchronize(ws.stream), "p-values");
    float ms = 0;
    cudaEventElapsedTime(&ms, ws.ev_start, ws.ev_stop);
    out->device_ms = ms;
    out->host_ms = host_ms;     // the host only plans and copies; it draws nothing
    return CAFE_OK;
}

// compute_pvalues (src/probability.cpp:376-570). The simulation runs on the
// host because its random stream is the reference's: one std::mt19937
// seeded by the caller, drawing in the reference's order (create_family,
// :351-373, set_weighted_random_family_size, :449-476) through
// std::discrete_distribution over the parent's matrix row
// (matrix::select_random_y, src/matrix_cache.cpp:60-66) -- identical draws
// for identical rows. The distributions are built once per (matrix, row)
// instead of once per draw. Both prunings (R x n_sim simulated families
// with the root fixed, and the observed families) run on the GPU.
int pvalues_sync(cafe_ctx* C, Workspace& ws, const cafe_request* R, cafe_pvalues_out* out) {
    AllocScope scope(ws.stream);
    if (ws.staged) {
        CK(cudaEventSynchronize(ws.ev_staged), "staging");
        ws.staged = false;
    }
    if (!out || !out->pvalues || out->n_simulations < 1) return fail(C, CAFE_ERR_INVALID, "bad p-value arguments");
    if (out->device_sampling) return pvalues_device(C, ws, R, out);
    const auto t_host0 = std::chrono::steady_clock::now();
    double host_ms = 0.0;
    ReconSetup Z;
    int rc = recon_setup(C, ws, R, false, &Z);
    if (rc) return rc;
    TreeHost& T = *Z.T;
    FamSet& FS = *Z.S;
    const int S = Z.Smax, RR = Z.Rmax, msize = Z.msize, nsim = out->n_simulations, n = T.n_nodes;
    const int64_t F = FS.F;
    HostSampler hs;
    rc = host_sampler_init(C, ws, R, T, Z, 1, nullptr, &hs);
    if (rc) return rc;
    host_ms += host_ms_since(t_host0);
    const auto t_sim = std::chrono::steady_clock::now();
    const std::vector<int> prefix = prefix_order(T);
    std::mt19937 engine(out->seed);
    const int64_t NS = (int64_t)RR * nsim;
    const int L = T.n_leaves;
    // device buffers: simulated counts, their order, tiles, the root values
    const int Wmax = std::max(S + 1, RR);
    const int64_t max_tiles = NS / 32 + (int64_t)RR * (S + 2) + F / 32 + 2;
    DevBuf d_sim, d_perm, d_simL, d_obsL, d_tiles;
    CK(d_sim.reserve(std::max<size_t>((size_t)NS * L, 1) * sizeof(int32_t)), "simulated families");
    CK(d_perm.reserve(std::max<int64_t>(NS, 1) * sizeof(int64_t)), "simulated families");
    CK(d_simL.reserve(std::max<int64_t>(NS, 1) * sizeof(double)), "simulated likelihoods");
    CK(d_obsL.reserve(std::max<int64_t>(F * RR, 1) * sizeof(double)), "root vectors");
    CK(d_tiles.reserve((size_t)max_tiles * sizeof(PruneTile)), "tiles");
    const int n_ctas_max = C->n_ctas;
    const int64_t per_cta = (int64_t)T.n_slots * Wmax * 32;
    CK(ws.scratch.reserve((size_t)n_ctas_max * per_cta * sizeof(double)), "scratch");
    // host staging in pinned memory, so the copies stay asynchronous
    CK(ws.h_tiles.reserve((size_t)max_tiles * sizeof(PruneTile)), "tiles");
    CK(ws.h_sim.reserve(std::max<size_t>((size_t)NS * L, 1) * sizeof(int32_t)), "simulated families");
    CK(ws.h_simperm.reserve(std::max<int64_t>(NS, 1) * sizeof(int64_t)), "simulated families");
    PruneTile* tiles = ws.h_tiles.as<PruneTile>();
    size_t n_tiles = 0;
    // k_prune64 with the root vectors as output over tiles[t0, t1), on the
    // stream (the host goes on simulating meanwhile)
    auto launch_tiles = [&](size_t t0, size_t t1, const int32_t* counts, const int64_t* perm, int W, double* d_out,
                            int root_ld) -> int {
        const int n_t = (int)(t1 - t0);
        if (n_t <= 0) return CAFE_OK;
        CK(cudaMemcpyAsync(d_tiles.as<PruneTile>() + t0, tiles + t0, n_t * sizeof(PruneTile),
                           cudaMemcpyHostToDevice, ws.stream),
           "tiles");
        Prune64Args a{};
        a.plan = T.plan;
        a.tiles = d_tiles.as<PruneTile>() + t0;
        a.n_tiles = n_t;
        a.counts = counts;
        a.perm = perm;
        a.mats = ws.mats.as<const double*>();
        a.ld_mat = msize;
        a.scratch = ws.scratch.as<double>();
        a.scratch_per_cta = (int64_t)T.n_slots * W * 32;
        a.K = 1;
        a.tile_families = 32;
        a.W = W;
        a.root_out = d_out;
        a.root_ld = root_ld;
        CK(launch_prune64(a, std::max(1, std::min(n_t, n_ctas_max)), ws.stream), "prune root vectors");
        return CAFE_OK;
    };
    host_ms += host_ms_since(t_sim);
    CK(cudaEventRecord(ws.ev_start, ws.stream), "event");
    // observed families first: states 0..S, root sizes 1..R
    for (int64_t f = 0; f < F; f += 32) {
        PruneTile t{};
        t.first = (int)f;
        t.count = (int)std::min<int64_t>(32, F - f);
        t.S = S;
        t.R = RR;
        t.root_lo = 1;
        tiles[n_tiles++] = t;
    }
    rc = launch_tiles(0, n_tiles, FS.d_counts.as<int32_t>(), FS.d_identity.as<int64_t>(), Wmax,
                      d_obsL.as<double>(), RR);
    if (rc) return rc;
    // simulated families, a group of root sizes at a time: the device prunes
    // a group while the host draws the next
    const auto t_sim2 = std::chrono::steady_clock::now();
    int32_t* sim_counts = ws.h_sim.as<int32_t>();
    int64_t* perm = ws.h_simperm.as<int64_t>();
    std::vector<int32_t> sim_m(NS);
    std::vector<int> sizes(n);
    const int group = std::max(1, (RR + 7) / 8);
    for (int g0 = 0; g0 < RR; g0 += group) {
        const int g1 = std::min(RR, g0 + group);
        for (int i = g0; i < g1; ++i)
            for (int k = 0; k < nsim; ++k) {
                const int64_t fi = (int64_t)i * nsim + k;
                sizes[T.root] = i + 1;
                int mx = i + 1;
                for (int v : prefix) {
                    if (v == T.root) continue;
                    const int ps = sizes[T.parent[v]];
                    int c = 0;
                    if (ps > 0) c = hs.draw(0, v, ps, engine);
                    sizes[v] = c;
                    mx = std::max(mx, c);
                }
                for (int v = 0; v < n; ++v)
                    if (T.leaf_col[v] >= 0) sim_counts[(size_t)fi * L + T.leaf_col[v]] = sizes[v];
                sim_m[fi] = std::min(S, mx + std::max(50, mx / 5));   // compute_family_probabilities bound
            }
        // tiles of the group: families grouped by (root size, bound)
        const int64_t a0 = (int64_t)g0 * nsim, a1 = (int64_t)g1 * nsim;
        std::iota(perm + a0, perm + a1, a0);
        std::stable_sort(perm + a0, perm + a1, [&](int64_t a, int64_t b) {
            const int ra = (int)(a / nsim), rb = (int)(b / nsim);
            return ra != rb ? ra < rb : sim_m[a] < sim_m[b];
        });
        const size_t t0 = n_tiles;
        int Wg = 1;
        for (int64_t i = a0; i < a1;) {
            const int64_t f0 = perm[i];
            const int r = (int)(f0 / nsim), m = sim_m[f0];
            int64_t j = i;
            while (j < a1 && j - i < 32 && perm[j] / nsim == r && sim_m[perm[j]] == m) ++j;
            PruneTile t{};
            t.first = (int)i;
            t.count = (int)(j - i);
            t.S = m;
            t.R = 1;
            t.root_lo = r + 1;
            tiles[n_tiles++] = t;
            Wg = std::max(Wg, m + 1);
            i = j;
        }
        CK(cudaMemcpyAsync(d_sim.as<int32_t>() + (size_t)a0 * L, sim_counts + (size_t)a0 * L,
                           (size_t)(a1 - a0) * L * sizeof(int32_t), cudaMemcpyHostToDevice, ws.stream),
           "h2d");
        CK(cudaMemcpyAsync(d_perm.as<int64_t>() + a0, perm + a0, (size_t)(a1 - a0) * sizeof(int64_t),
                           cudaMemcpyHostToDevice, ws.stream),
           "h2d");
        rc = launch_tiles(t0, n_tiles, d_sim.as<int32_t>(), d_perm.as<int64_t>(), Wg, d_simL.as<double>(), 1);
        if (rc) return rc;
    }
    host_ms += host_ms_since(t_sim2);
    CK(cudaEventRecord(ws.ev_stop, ws.stream), "event");
    std::vector<double> simL(NS), obsL((size_t)F * RR);
    CK(cudaMemcpyAsync(simL.data(), d_simL.p, NS * sizeof(double), cudaMemcpyDeviceToHost, ws.stream), "d2h");
    if (F) CK(cudaMemcpyAsync(obsL.data(), d_obsL.p, obsL.size() * sizeof(double), cudaMemcpyDeviceToHost, ws.stream),
              "d2h");
    CK(cudaStreamSynchronize(ws.stream), "p-values");
    float ms = 0;
    cudaEventElapsedTime(&ms, ws.ev_start, ws.ev_stop);
    const auto t_pv = std::chrono::steady_clock::now();
    // sorted conditional distributions (get_random_probabilities)
    for (int i = 0; i < RR; ++i) std::sort(simL.begin() + (size_t)i * nsim, simL.begin() + (size_t)(i + 1) * nsim);
    if (out->conditional) std::memcpy(out->conditional, simL.data(), NS * sizeof(double));
    if (out->root_likelihood && F) std::memcpy(out->root_likelihood, obsL.data(), obsL.size() * sizeof(double));
    // find_best_pvalue / pvalue (:503-528)
    const std::vector<int32_t>& hc = FS.h_counts;
    std::vector<double> pv(RR);
    for (int64_t f = 0; f < F; ++f) {
        int fmax = 0;
        for (int c = 0; c < L; ++c) fmax = std::max(fmax, hc[(size_t)f * L + c]);
        std::fill(pv.begin(), pv.end(), 0.0);
        const int check = std::min(RR, (int)std::rint(fmax * 1.25));
        for (int j = 0; j < check; ++j) {
            const double* d = simL.data() + (size_t)j * nsim;
            const double v = obsL[(size_t)f * RR + j];
            int idx = nsim - 1;
            const double* b = std::upper_bound(d, d + nsim, v);
            if (b != d + nsim) idx = (int)(b - d);
            pv[j] = idx / (double)nsim;
        }
        out->pvalues[f] = *std::max_element(pv.begin(), pv.end());
    }
    host_ms += host_ms_since(t_pv);
    out->device_ms = ms;
    out->host_ms = host_ms;
    return CAFE_OK;
}

// The simulator action (src/simulator.cpp:29-91) on the host sampler: per
// family the gamma model draws its rate category
// (gamma_model::get_simulation_lambda, src/gamma_core.cpp:91-95), then up
// to 50 attempts (simulator::create_trial) fill the tree in prefix order
// from the family's root size, leaves through the error model
// (adjust_for_error_model, src/probability.cpp:478-500), until the family
// exists at the root (gene_family::exists_at_root, src/gene_family.cpp:62-91).
int simulate_sync(cafe_ctx* C, Workspace& ws, const cafe_request* R, cafe_simulation* io) {
    AllocScope scope(ws.stream);
    if (ws.staged) {
        CK(cudaEventSynchronize(ws.ev_staged), "staging");
        ws.staged = false;
    }
    if (!io || io->n_families < 0 || (io->n_families && (!io->root_sizes || !io->sizes)))
        return fail(C, CAFE_ERR_INVALID, "bad simulation arguments");
    if (R && R->use_error_model && (C->err_rows == 0 || C->err_ndev != 3))
        return fail(C, CAFE_ERR_INVALID, "the simulation's error model needs deviations -1, 0, +1");
    ReconSetup Z;
    int rc = recon_setup(C, ws, R, true, &Z);
    if (rc) return rc;
    TreeHost& T = *Z.T;
    const int n = T.n_nodes, K = Z.K;
    HostSampler hs;
    rc = host_sampler_init(C, ws, R, T, Z, K, Z.gamma ? R->multipliers : nullptr, &hs);
    if (rc) return rc;
    const std::vector<int> prefix = prefix_order(T);
    std::vector<int> post(prefix.rbegin(), prefix.rend());
    std::mt19937 engine(io->seed);
    std::vector<int> z(n);
    std::vector<char> reg(n);
    const double* err = R->use_error_model ? C->err.data() : nullptr;
    for (int f = 0; f < io->n_families; ++f) {
        const int root = io->root_sizes[f];
        if (root < 0 || root >= hs.n_ps) return fail(C, CAFE_ERR_INVALID, "root size %d outside 0..%d", root, hs.n_ps - 1);
        int k = 0;
        if (Z.gamma) {
            std::discrete_distribution<int> pick(R->cat_probs, R->cat_probs + K);
            k = pick(engine);
        }
        if (io->lambdas) io->lambdas[f] = R->lambdas[0] * (Z.gamma ? R->multipliers[k] : 1.0);
        for (int attempt = 0; attempt < 50; ++attempt) {
            z[T.root] = root;
            for (int v : prefix) {
                if (v == T.root) continue;
                const int ps = z[T.parent[v]];
                int c = ps > 0 ? hs.draw(k, v, ps, engine) : 0;
                if (err && T.leaf_col[v] >= 0) {
                    if (c >= C->err_rows)
                        return fail(C, CAFE_ERR_INVALID,
                                    "Trying to simulate leaf family size that was not included in error model");
                    const double* p = err + (size_t)c * 3;
                    std::uniform_real_distribution<double> u(0.0, 1.0);
                    const double rnd = u(engine);
                    if (rnd < p[0]) c--;
                    else if (rnd > (1 - p[2])) c++;
                }
                z[v] = c;
            }
            std::fill(reg.begin(), reg.end(), 0);
            for (int v : post)
                if (T.leaf_col[v] >= 0 && z[v] > 0)
                    for (int p = v; p >= 0 && !reg[p]; p = T.parent[p]) reg[p] = 1;
            bool all = true;
            for (int ch : T.children[T.root]) all &= reg[ch] != 0;
            if (all) break;
        }
        std::memcpy(io->sizes + (size_t)f * n, z.data(), sizeof(int32_t) * n);
    }
    return CAFE_OK;
}

int branch_prob_sync(cafe_ctx* C, Workspace& ws, const cafe_request* R, const int32_t* node_count, double* out) {
    AllocScope scope(ws.stream);
    if (ws.staged) {   // the previous request's copies out of the pinned staging buffers
        CK(cudaEventSynchronize(ws.ev_staged), "staging");
        ws.staged = false;
    }
    if (!node_count || !out) return fail(C, CAFE_ERR_INVALID, "null buffers");
    ReconSetup Z;
    int rc = recon_setup(C, ws, R, false, &Z);
    if (rc) return rc;
    TreeHost& T = *Z.T;
    const int64_t F = Z.S->F;
    const size_t n_fam = (size_t)F * T.n_nodes;
    if (!n_fam) return CAFE_OK;
    CK(ws.rc_count.reserve(n_fam * sizeof(int32_t)), "counts");
    CK(ws.rc_bp.reserve(n_fam * sizeof(double)), "branch probabilities");
    CK(ws.rc_parent.reserve((size_t)T.n_nodes * sizeof(int32_t)), "parents");
    CK(ws.rc_nfail.reserve(sizeof(int32_t)), "bad");
    CK(cudaMemcpyAsync(ws.rc_count.p, node_count, n_fam * sizeof(int32_t), cudaMemcpyHostToDevice, ws.stream), "h2d");
    CK(cudaMemcpyAsync(ws.rc_parent.p, T.parent.data(), (size_t)T.n_nodes * sizeof(int32_t), cudaMemcpyHostToDevice,
                       ws.stream),
       "h2d");
    CK(cudaMemsetAsync(ws.rc_nfail.p, 0, sizeof(int32_t), ws.stream), "bad");
    BranchProbArgs a{};
    a.parent = ws.rc_parent.as<int32_t>();
    a.n_nodes = T.n_nodes;
    a.F = F;
    a.node_count = ws.rc_count.as<int32_t>();
    a.mats = ws.mats.as<const double*>();
    a.ld_mat = Z.msize;
    a.S = Z.Smax;
    a.out = ws.rc_bp.as<double>();
    a.n_bad = ws.rc_nfail.as<int32_t>();
    CK(launch_branch_prob(a, ws.stream), "branch probabilities");
    int32_t bad = 0;
    CK(cudaMemcpyAsync(out, ws.rc_bp.p, n_fam * sizeof(double), cudaMemcpyDeviceToHost, ws.stream), "d2h");
    CK(cudaMemcpyAsync(&bad, ws.rc_nfail.p, sizeof(int32_t), cudaMemcpyDeviceToHost, ws.stream), "d2h");
    CK(cudaStreamSynchronize(ws.stream), "branch probabilities");
    if (bad) return fail(C, CAFE_ERR_INVALID, "%d node counts lie outside the transition matrices", bad);
    return CAFE_OK;
}

}  // namespace

// ===================================================================== ABI

extern "C" {

int cafe_version(void) { return 1; }

int cafe_debug_set(cafe_ctx* C, int knob, int64_t value) {
    if (!C) return CAFE_ERR_INVALID;
    std::lock_guard<std::mutex> lk(C->mu);
    if (knob == CAFE_DEBUG_TC_WAIT_LIMIT) {
        if (value < 0 || value > ((int64_t)1 << 30)) return fail(C, CAFE_ERR_INVALID, "wait limit out of range");
        C->debug_wait_limit = (int)value;
        return CAFE_OK;
    }
    return fail(C, CAFE_ERR_INVALID, "unknown debug knob %d", knob);
}

const char* cafe_status_string(int s) {
    switch (s) {
        case CAFE_OK: return "ok";
        case CAFE_ERR_OOM: return "out of device memory";
        case CAFE_ERR_MISSING_MATRIX: return "missing matrix";
        case CAFE_ERR_SATURATED: return "saturated";
        case CAFE_ERR_UNDERFLOW: return "underflow";
        case CAFE_ERR_TIMEOUT: return "timeout";
        case CAFE_ERR_INVALID: return "invalid argument";
        case CAFE_ERR_CUDA: return "CUDA error";
        case CAFE_ERR_BUSY: return "busy";
        case CAFE_ERR_NOT_FOUND: return "not found";
        default: return "unknown status";
    }
}

const char* cafe_last_error(const cafe_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

int cafe_is_saturated(double branch_length, double lambda) {
    const double alpha = lambda * branch_length / (1 + lambda * branch_length);
    return (1 - 2 * alpha) < 0;
}

int cafe_ctx_create(const cafe_config* cfg, cafe_ctx** out) {
    if (!out) return CAFE_ERR_INVALID;
    *out = nullptr;
    int dev = cfg ? cfg->device : 0;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return CAFE_ERR_CUDA;
    }
    if (dev < 0 || dev >= n) return CAFE_ERR_INVALID;
    if (cudaSetDevice(dev) != cudaSuccess) return CAFE_ERR_CUDA;
    auto* C = new cafe_ctx();
    C->device = dev;
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, dev);
    C->sm_count = prop.multiProcessorCount;
    if (tc_kernels_init() != cudaSuccess || prune64_cluster_init() != cudaSuccess || pvalue_kernels_init() != cudaSuccess ||
        cudaEventCreateWithFlags(&C->gate, cudaEventDisableTiming) != cudaSuccess) {
        delete C;
        return CAFE_ERR_CUDA;
    }
    C->n_ctas = prop.multiProcessorCount * 4;
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    // 4 GB of matrices per generation by default (a 16-candidate step of 24
    // taxa and side 96 adds 0.2 GB; a 64-candidate K = 8 round of 48 taxa,
    // 3.5 GB)
    C->cache_cap = (cfg && cfg->matrix_cache_bytes) ? cfg->matrix_cache_bytes : std::min(fr / 8, (size_t)4 << 30);
    {
        // stream-ordered buffer growth draws on the device's default pool;
        // keep what it frees instead of returning it at every synchronisation
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        cudaGetLastError();
    }
    C->serve_budget = fr / 4;
    C->cache.reserve(1 << 17);   // 262,144 slots (16 MB of host memory): no rehash in a typical search
    const int n_streams = (cfg && cfg->n_streams > 0) ? cfg->n_streams : 4;
    for (int i = 0; i <= n_streams; ++i) {
        auto w = std::make_unique<Workspace>();
        if (w->init(dev) != CAFE_OK) {
            delete C;
            return CAFE_ERR_CUDA;
        }
        w->sync = (i == 0);
        C->ws.push_back(std::move(w));
    }
    C->ws_alt = std::make_unique<Workspace>();
    if (C->ws_alt->init(dev) != CAFE_OK) {
        delete C;
        return CAFE_ERR_CUDA;
    }
    C->ws_alt->sync = true;
    *out = C;
    return CAFE_OK;
}

void cafe_serving_stop(cafe_ctx* C);

int cafe_ctx_destroy(cafe_ctx* C) {
    if (!C) return CAFE_ERR_INVALID;
    cudaSetDevice(C->device);
    cafe_serving_stop(C);
    cudaDeviceSynchronize();
    cache_reset(C);
    for (auto& g : C->gens)
        for (cudaEvent_t e : g.marks) cudaEventDestroy(e);
    if (C->gate) cudaEventDestroy(C->gate);
    if (C->serve_epoch) cudaEventDestroy(C->serve_epoch);
    delete C;
    return CAFE_OK;
}

int cafe_tree_upload(cafe_ctx* C, int n_nodes, const int32_t* parent, const double* branch_length,
                     const int32_t* lambda_index, int* tree_id) {
    if (!C || !parent || !branch_length || !tree_id || n_nodes < 2 || n_nodes > kMaxNodes)
        return fail(C, CAFE_ERR_INVALID, "bad tree arguments (n_nodes %d)", n_nodes);
    std::lock_guard<std::mutex> lk(C->mu);
    cudaSetDevice(C->device);
    auto T = std::make_unique<TreeHost>();
    T->n_nodes = n_nodes;
    T->parent.assign(parent, parent + n_nodes);
    T->branch_length.assign(branch_length, branch_length + n_nodes);
    T->lambda_index.assign(n_nodes, 0);
    if (lambda_index) T->lambda_index.assign(lambda_index, lambda_index + n_nodes);
    T->children.assign(n_nodes, {});
    int roots = 0;
    for (int i = 0; i < n_nodes; ++i) {
        const int p = parent[i];
        if (p < 0) {
            roots++;
            T->root = i;
        } else if (p >= n_nodes || p == i) {
            return fail(C, CAFE_ERR_INVALID, "bad parent %d of node %d", p, i);
        } else {
            T->children[p].push_back(i);
        }
    }
    if (roots != 1) return fail(C, CAFE_ERR_INVALID, "tree needs exactly one root (got %d)", roots);
    // reject cycles: every node must reach the root
    for (int i = 0; i < n_nodes; ++i) {
        int v = i, steps = 0;
        while (parent[v] >= 0 && steps <= n_nodes) {
            v = parent[v];
            steps++;
        }
        if (steps > n_nodes) return fail(C, CAFE_ERR_INVALID, "cycle through node %d", i);
    }
    T->leaf_col.assign(n_nodes, -1);
    for (int i = 0; i < n_nodes; ++i)
        if (T->children[i].empty()) T->leaf_col[i] = T->n_leaves++;
    for (int i = 0; i < n_nodes; ++i) {
        if (i != T->root && !(branch_length[i] > 0))
            return fail(C, CAFE_ERR_INVALID, "branch length of node %d must be > 0", i);
        if (branch_length[i] > 0) {
            T->longest_branch = std::max(T->longest_branch, branch_length[i]);
            T->distinct_lengths.push_back(branch_length[i]);
        }
    }
    std::sort(T->distinct_lengths.begin(), T->distinct_lengths.end());
    T->distinct_lengths.erase(std::unique(T->distinct_lengths.begin(), T->distinct_lengths.end()),
                              T->distinct_lengths.end());
    if (T->n_leaves == n_nodes || T->root < 0) return fail(C, CAFE_ERR_INVALID, "tree has no internal node");
    build_plan(*T);
    int rc = upload_plan(C, *T);
    if (rc) return rc;
    *tree_id = C->next_tree++;
    C->trees[*tree_id] = std::move(T);
    return CAFE_OK;
}

int cafe_families_upload(cafe_ctx* C, int tree_id, const int32_t* counts, int64_t n_families, int n_leaves,
                         int* set_id) {
    if (!C || !set_id || n_families < 0 || (n_families > 0 && !counts)) return fail(C, CAFE_ERR_INVALID, "bad family arguments");
    std::lock_guard<std::mutex> lk(C->mu);
    cudaSetDevice(C->device);
    auto ti = C->trees.find(tree_id);
    if (ti == C->trees.end()) return fail(C, CAFE_ERR_NOT_FOUND, "unknown tree id %d", tree_id);
    if (n_leaves != ti->second->n_leaves)
        return fail(C, CAFE_ERR_INVALID, "tree has %d leaves, counts have %d columns", ti->second->n_leaves, n_leaves);
    for (int64_t i = 0; i < n_families * n_leaves; ++i)
        if (counts[i] < 0) return fail(C, CAFE_ERR_INVALID, "negative count at %lld", (long long)i);
    auto S = std::make_unique<FamSet>();
    S->tree_id = tree_id;
    S->F = n_families;
    S->n_leaves = n_leaves;
    S->h_counts.assign(counts, counts + n_families * n_leaves);
    const size_t bytes = std::max<size_t>((size_t)n_families * n_leaves * sizeof(int32_t), 4);
    CK(S->d_counts.reserve(bytes), "counts");
    if (n_families) CK(cudaMemcpy(S->d_counts.p, counts, (size_t)n_families * n_leaves * sizeof(int32_t), cudaMemcpyHostToDevice), "counts");
    int rc = prepare_set(C, *S);
    if (rc) return rc;
    *set_id = C->next_set++;
    C->sets[*set_id] = std::move(S);
    return CAFE_OK;
}

int cafe_families_update(cafe_ctx* C, int set_id, const int32_t* counts) {
    if (!C) return CAFE_ERR_INVALID;
    std::lock_guard<std::mutex> lk(C->mu);
    cudaSetDevice(C->device);
    auto si = C->sets.find(set_id);
    if (si == C->sets.end()) return fail(C, CAFE_ERR_NOT_FOUND, "unknown family set id %d", set_id);
    FamSet& S = *si->second;
    const size_t n = (size_t)S.F * S.n_leaves;
    if (!counts && n) return fail(C, CAFE_ERR_INVALID, "null counts");
    // unchanged counts keep their derived tables (maxima, duplicates, bins)
    const bool same = S.h_counts.size() == n && (n == 0 || std::memcmp(S.h_counts.data(), counts, n * sizeof(int32_t)) == 0);
    if (!same) {
        for (size_t i = 0; i < n; ++i)
            if (counts[i] < 0) return fail(C, CAFE_ERR_INVALID, "negative count");
        S.h_counts.assign(counts, counts + n);
    }
    Workspace& ws = *C->ws[0];
    CK(cudaMemcpyAsync(S.d_counts.p, counts, n * sizeof(int32_t), cudaMemcpyHostToDevice, ws.stream), "counts");
    CK(cudaStreamSynchronize(ws.stream), "counts");
    return same ? CAFE_OK : prepare_set(C, S);
}

int cafe_families_free(cafe_ctx* C, int set_id) {
    if (!C) return CAFE_ERR_INVALID;
    std::lock_guard<std::mutex> lk(C->mu);
    cudaSetDevice(C->device);
    cudaDeviceSynchronize();
    if (!C->sets.erase(set_id)) return fail(C, CAFE_ERR_NOT_FOUND, "unknown family set id %d", set_id);
    return CAFE_OK;
}

int cafe_prior_set(cafe_ctx* C, const double* prior, int n) {
    if (!C || n < 1 || !prior) return fail(C, CAFE_ERR_INVALID, "bad prior");
    std::lock_guard<std::mutex> lk(C->mu);
    cudaSetDevice(C->device);
    cudaDeviceSynchronize();
    C->prior.assign(prior, prior + n);
    CK(C->d_prior.reserve(n * sizeof(double)), "prior");
    CK(cudaMemcpy(C->d_prior.p, prior, n * sizeof(double), cudaMemcpyHostToDevice), "prior");
    return CAFE_OK;
}

int cafe_error_model_set(cafe_ctx* C, const double* rows, int n_rows, int n_dev) {
    if (!C || n_rows < 0 || (n_rows > 0 && (!rows || n_dev < 1 || n_dev % 2 == 0)))
        return fail(C, CAFE_ERR_INVALID, "bad error model (n_dev must be odd)");
    std::lock_guard<std::mutex> lk(C->mu);
    cudaSetDevice(C->device);
    cudaDeviceSynchronize();
    C->err.assign(rows, rows + (size_t)n_rows * n_dev);
    C->err_rows = n_rows;
    C->err_ndev = n_rows ? n_dev : 0;
    if (n_rows) {
        CK(C->d_err.reserve((size_t)n_rows * n_dev * sizeof(double)), "error model");
        CK(cudaMemcpy(C->d_err.p, rows, (size_t)n_rows * n_dev * sizeof(double), cudaMemcpyHostToDevice), "error model");
    }
    return CAFE_OK;
}

int cafe_matrices_build(cafe_ctx* C, const double* lambdas, int n_lambdas, const double* branch_lengths,
                        int n_t, int matrix_size) {
    if (!C || n_lambdas < 0 || n_t < 0 || matrix_size < 1 || (n_lambdas && !lambdas) || (n_t && !branch_lengths))
        return fail(C, CAFE_ERR_INVALID, "bad matrix build arguments");
    std::lock_guard<std::mutex> lk(C->mu);
    cudaSetDevice(C->device);
    cache_make_room(C, (size_t)n_lambdas * n_t * matrix_size * matrix_size * sizeof(double));
    C->cache.reserve(C->cache.size() + (size_t)n_lambdas * n_t);
    PendingJobs P;
    for (int i = 0; i < n_lambdas; ++i)
        for (int j = 0; j < n_t; ++j) schedule(C, P, make_key(matrix_size, lambdas[i], branch_lengths[j]));
    Workspace& ws = *C->ws[0];
    int rc = cache_build(C, ws, P);
    if (rc) return rc;
    if (!C->batch_events.empty()) CK(cudaEventSynchronize(C->batch_events.back()), "matrix build");
    return CAFE_OK;
}

int cafe_matrix_get(cafe_ctx* C, double lambda, double branch_length, int matrix_size, double* out) {
    if (!C || !out || matrix_size < 1) return fail(C, CAFE_ERR_INVALID, "bad matrix_get arguments");
    std::lock_guard<std::mutex> lk(C->mu);
    cudaSetDevice(C->device);
    const MatEntry* e = C->cache.find(make_key(matrix_size, lambda, branch_length));
    if (!e || !e->d)
        return fail(C, CAFE_ERR_MISSING_MATRIX, "Failed to find matrix for %d,%g,%g", matrix_size, branch_length, lambda);
    CK(cudaEventSynchronize(C->batch_events[e->chunk]), "matrix_get");   // its build has run
    CK(cudaMemcpy(out, e->d, (size_t)matrix_size * matrix_size * sizeof(double), cudaMemcpyDeviceToHost), "matrix_get");
    return CAFE_OK;
}

int cafe_matrix_cache_size(cafe_ctx* C, int64_t* n) {
    if (!C || !n) return CAFE_ERR_INVALID;
    std::lock_guard<std::mutex> lk(C->mu);
    *n = (int64_t)C->cache.size();
    return CAFE_OK;
}

int cafe_matrix_cache_clear(cafe_ctx* C) {
    if (!C) return CAFE_ERR_INVALID;
    std::lock_guard<std::mutex> lk(C->mu);
    cudaSetDevice(C->device);
    cudaDeviceSynchronize();
    cache_reset(C);
    return CAFE_OK;
}

int cafe_score(cafe_ctx* C, const cafe_request* req, cafe_result* res) {
    if (!C) return CAFE_ERR_INVALID;
    std::lock_guard<std::mutex> lk(C->mu);
    cudaSetDevice(C->device);
    return score_sync(C, *C->ws[0], req, 1, res);
}

int cafe_reconstruct(cafe_ctx* C, const cafe_request* req, cafe_reconstruction* out) {
    if (!C) return CAFE_ERR_INVALID;
    std::lock_guard<std::mutex> lk(C->mu);
    cudaSetDevice(C->device);
    return reconstruct_sync(C, *C->ws[0], req, out);
}

int cafe_pvalues(cafe_ctx* C, const cafe_request* req, cafe_pvalues_out* out) {
    if (!C) return CAFE_ERR_INVALID;
    std::lock_guard<std::mutex> lk(C->mu);
    cudaSetDevice(C->device);
    return pvalues_sync(C, *C->ws[0], req, out);
}

int cafe_simulate(cafe_ctx* C, const cafe_request* req, cafe_simulation* io) {
    if (!C) return CAFE_ERR_INVALID;
    std::lock_guard<std::mutex> lk(C->mu);
    cudaSetDevice(C->device);
    return simulate_sync(C, *C->ws[0], req, io);
}

int cafe_branch_probabilities(cafe_ctx* C, const cafe_request* req, const int32_t* node_count, double* out) {
    if (!C) return CAFE_ERR_INVALID;
    std::lock_guard<std::mutex> lk(C->mu);
    cudaSetDevice(C->device);
    return branch_prob_sync(C, *C->ws[0], req, node_count, out);
}

int cafe_autotune(cafe_ctx* C, const cafe_request* reqs, int n, int reps, cafe_tune_result* out, int max_out,
                  int* n_out) {
    if (!C || !reqs || n < 1 || (max_out > 0 && !out)) return CAFE_ERR_INVALID;
    if (reqs[0].precision != CAFE_PREC_MIXED_TF32X3) return fail(C, CAFE_ERR_INVALID, "autotune needs MIXED_TF32X3");
    std::lock_guard<std::mutex> lk(C->mu);
    cudaSetDevice(C->device);
    auto si = C->sets.find(reqs[0].set_id);
    auto ti = C->trees.find(reqs[0].tree_id);
    if (si == C->sets.end() || ti == C->trees.end()) return fail(C, CAFE_ERR_NOT_FOUND, "unknown tree or family set");
    const TreeHost& T = *ti->second;
    reps = std::max(1, reps);
    std::vector<cafe_result> res(n);
    // mean device time of the request with the current shapes (one untimed run first)
    auto timed = [&](double* ms) -> int {
        *ms = 0;
        for (int r = 0; r <= reps; ++r) {
            for (auto& x : res) x = cafe_result{};
            const int rc = score_sync(C, *C->ws[0], reqs, n, res.data());
            if (rc) return rc;
            if (r > 0) *ms += res[0].device_ms / reps;
        }
        return CAFE_OK;
    };
    std::vector<int> widths;
    const BinPlan& B = si->second->bins;
    for (size_t b = 0; b < B.widths.size(); ++b)
        if (B.widths[b] <= 256 && B.bin_count[b] > 0) widths.push_back(B.widths[b]);
    int k = 0;
    for (int W : widths) {
        // candidates: the three largest feasible CTA counts per SM, each with every stage count that fits
        C->tuned.erase(W);
        const TcShape def = tc_shape(C, T, W);
        double best_ms;
        int rc = timed(&best_ms);
        if (rc) return rc;
        std::pair<int, int> best{def.per_sm, def.stages};
        const int by_tmem = 512 / def.tmem_cols;
        for (int per = by_tmem; per >= 1 && per > by_tmem - 3; --per)
            for (int st = 1; st <= 4; ++st) {
                size_t sm;
                if (tc_by_smem(T, W, st, &sm) < per || (per == def.per_sm && st == def.stages)) continue;
                C->tuned[W] = {per, st};
                double ms;
                rc = timed(&ms);
                if (rc) {
                    C->tuned.erase(W);
                    return rc;
                }
                if (ms < best_ms) {
                    best_ms = ms;
                    best = {per, st};
                }
            }
        C->tuned[W] = best;
        if (k < max_out) out[k] = cafe_tune_result{W, best.first, best.second, best_ms};
        ++k;
    }
    if (n_out) *n_out = k;
    return CAFE_OK;
}

int cafe_score_batch(cafe_ctx* C, const cafe_request* reqs, int n, cafe_result* results) {
    if (!C || !reqs || n < 1 || !results) return CAFE_ERR_INVALID;
    std::lock_guard<std::mutex> lk(C->mu);
    cudaSetDevice(C->device);
    return score_sync(C, *C->ws[0], reqs, n, results);
}

int cafe_profile_enable(cafe_ctx* C, int enable) {
    if (!C) return CAFE_ERR_INVALID;
    std::lock_guard<std::mutex> lk(C->mu);
    C->prof.on = enable != 0;
    return CAFE_OK;
}

int cafe_profile_read(cafe_ctx* C, cafe_timings* out) {
    if (!C || !out) return CAFE_ERR_INVALID;
    std::lock_guard<std::mutex> lk(C->mu);
    cudaSetDevice(C->device);
    C->prof.collect();
    *out = C->prof.acc;
    C->prof.acc = cafe_timings{};
    return CAFE_OK;
}

int cafe_score_device(cafe_ctx* C, const cafe_request* req, double* d_family_lnl, double* d_total, void* stream) {
    return cafe_score_batch_device(C, req, 1, d_family_lnl, d_total, stream);
}

int cafe_score_batch_device(cafe_ctx* C, const cafe_request* req, int n, double* d_family_lnl, double* d_total,
                            void* stream) {
    if (!C || n < 1) return CAFE_ERR_INVALID;
    std::lock_guard<std::mutex> lk(C->mu);
    cudaSetDevice(C->device);
    // consecutive calls alternate between two workspaces: the host prepares
    // a call (refilling that workspace's pinned staging buffers) while the
    // device still runs the previous one
    C->dev_flip ^= 1;
    Workspace& ws = C->dev_flip ? *C->ws_alt : *C->ws[0];
    AllocScope scope(ws.stream);
    cudaStream_t user = static_cast<cudaStream_t>(stream);
    ScoreInfo info;
    auto si = C->sets.find(req ? req->set_id : -1);
    if (si == C->sets.end()) return fail(C, CAFE_ERR_NOT_FOUND, "unknown family set");
    const int64_t F = si->second->F;
    CK(ws.fam_lnl.reserve((size_t)std::max<int64_t>(F, 1) * n * sizeof(double)), "family buffer");
    CK(ws.total.reserve((size_t)n * sizeof(double)), "total");
    if (user) {
        // order the workspace stream after the caller's stream, and back
        CK(cudaEventRecord(ws.ev_start, user), "event");
        CK(cudaStreamWaitEvent(ws.stream, ws.ev_start, 0), "event");
    }
    CK(gate_enter(C, ws), "gate");
    const auto t_host = std::chrono::steady_clock::now();
    int rc = enqueue_score(C, ws, req, n, d_family_lnl ? d_family_lnl : ws.fam_lnl.as<double>(),
                           d_total ? d_total : ws.total.as<double>(), &info);
    if (rc) return rc;
    if (C->prof.on) C->prof.acc.host_total_ms += host_ms_since(t_host);
    CK(gate_leave(C, ws), "gate");
    CK(cudaEventRecord(ws.ev_staged, ws.stream), "event");
    ws.staged = true;
    if (user) {
        CK(cudaEventRecord(ws.ev_stop, ws.stream), "event");
        CK(cudaStreamWaitEvent(user, ws.ev_stop, 0), "event");
    }
    return CAFE_OK;
}

}  // extern "C"

// ------------------------------------------------------- serving loop

namespace cafe {
struct Request {
    cafe_request req{};
    std::vector<double> lambdas, mult, probs;
    cafe_result* res = nullptr;
    size_t bytes = 0;          // admission footprint
    bool small = false;        // too small to fill the device alone (runs beside others)
    int rc = CAFE_OK;
    bool done = false;
    std::chrono::steady_clock::time_point t_submit;
    std::mutex m;
    std::condition_variable cv;
};
}  // namespace cafe

namespace {

// Requests that can share one batched launch: same tree, family set,
// model, category count, precision and error-model use (and FP64_REF
// bounds); each keeps its own lambdas, multipliers and probabilities.
bool batchable(const cafe_request& a, const cafe_request& b) {
    if (a.tree_id != b.tree_id || a.set_id != b.set_id || a.model != b.model || a.precision != b.precision ||
        a.use_error_model != b.use_error_model || a.lambda_kind != b.lambda_kind || a.dedupe != b.dedupe ||
        a.n_lambdas != b.n_lambdas)
        return false;
    if (a.model == CAFE_MODEL_GAMMA && a.n_categories != b.n_categories) return false;
    if (a.precision == CAFE_PREC_FP64_REF &&
        (a.max_family_size != b.max_family_size || a.max_root_family_size != b.max_root_family_size))
        return false;
    return true;
}

// Device bytes a request holds while admitted: per-family category terms,
// results and flags (the workspaces' fixed buffers are not counted).
size_t request_footprint(cafe_ctx* C, const cafe_request& r) {
    auto it = C->sets.find(r.set_id);
    const int64_t F = it == C->sets.end() ? 0 : it->second->F;
    const int K = r.model == CAFE_MODEL_GAMMA ? std::max(r.n_categories, 1) : 1;
    return (size_t)F * ((size_t)K * 8 + 8 + 4) + 4096;
}

constexpr int kMaxMerge = 32;           // candidates merged into one batched launch
constexpr int kMaxBatchesInFlight = 2;  // one on the device, one being enqueued

void server_loop(cafe_ctx* C, int wi) {
    cudaSetDevice(C->device);
    Workspace& ws = *C->ws[wi];
    for (;;) {
        std::vector<std::shared_ptr<Request>> batch;
        size_t bytes = 0;
        bool behind = false;     // another batch is in flight: this one runs at the lower priority
        {
            std::unique_lock<std::mutex> lk(C->qmu);
            // admit when the queue has work and the footprint fits (an idle
            // loop always admits one request, however large)
            // (and while at most one other batch is in flight, so requests that
            // arrive meanwhile queue up and share the next launch)
            C->qcv.wait(lk, [&] {
                if (C->stop) return true;
                if (C->queue.empty()) return false;
                // small requests run side by side on every server stream
                const bool small = C->queue.front()->small;
                if (C->batches_in_flight >= (small ? (int)C->servers.size() : kMaxBatchesInFlight)) return false;
                return C->in_flight == 0 || C->in_flight_bytes + C->queue.front()->bytes <= C->serve_budget;
            });
            if (C->stop && C->queue.empty()) return;
            batch.push_back(C->queue.front());
            C->queue.pop_front();
            bytes = batch[0]->bytes;
            // continuous batching: compatible requests queued behind it join
            // the same launch
            for (auto it = C->queue.begin(); it != C->queue.end() && (int)batch.size() < kMaxMerge;) {
                if (batchable(batch[0]->req, (*it)->req) && C->in_flight_bytes + bytes + (*it)->bytes <= C->serve_budget) {
                    bytes += (*it)->bytes;
                    batch.push_back(*it);
                    it = C->queue.erase(it);
                } else {
                    ++it;
                }
            }
            C->in_flight += (int)batch.size();
            C->in_flight_bytes += bytes;
            C->batches_in_flight++;
            behind = C->batches_in_flight > 1;
        }
        const int n = (int)batch.size();
        std::vector<cafe_request> reqs(n);
        std::vector<cafe_result> res(n);
        for (int i = 0; i < n; ++i) {
            reqs[i] = batch[i]->req;
            res[i] = batch[i]->res ? *batch[i]->res : cafe_result{};
        }
        int rc;
        ScoreInfo info;
        const auto t0 = std::chrono::steady_clock::now();
        {
            // enqueue under the context lock; the GPU work of this batch then
            // overlaps with batches running on the other streams (this
            // workspace's previous batch has completed, so it may switch
            // streams)
            std::unique_lock<std::mutex> lk(C->mu);
            ws.stream = behind ? ws.stream_lo : ws.stream_hi;
            rc = score_enqueue(C, ws, reqs.data(), n, res.data(), &info);
        }
        const auto t1 = std::chrono::steady_clock::now();
        if (rc == CAFE_OK) rc = score_complete(C, ws, reqs.data(), n, res.data(), info);
        const auto t2 = std::chrono::steady_clock::now();
        std::vector<int> rcs(n, rc);
        {
            std::lock_guard<std::mutex> lk(C->qmu);
            cafe_serving_info& si = C->serving;
            si.batches++;
            si.merged += n > 1 ? n : 0;
            si.retried += (rc != CAFE_OK && n > 1) ? n : 0;
            si.enqueue_ms += std::chrono::duration<double, std::milli>(t1 - t0).count();
            si.wait_ms += std::chrono::duration<double, std::milli>(t2 - t1).count();
            if (rc == CAFE_OK) si.device_ms += res[0].device_ms;
            // this batch's device interval against the recent ones: the time
            // they ran side by side
            float s0 = 0.0f, s1 = 0.0f;
            if (rc == CAFE_OK && C->serve_epoch && cudaEventElapsedTime(&s0, C->serve_epoch, ws.ev_start) == cudaSuccess &&
                cudaEventElapsedTime(&s1, C->serve_epoch, ws.ev_stop) == cudaSuccess) {
                for (const auto& iv : C->serve_intervals) {
                    const float lo = std::max(iv.first, s0), hi = std::min(iv.second, s1);
                    if (hi > lo) si.overlap_ms += hi - lo;
                }
                C->serve_intervals.emplace_back(s0, s1);
                if (C->serve_intervals.size() > 32) C->serve_intervals.pop_front();
            }
            cudaGetLastError();
        }
        if (rc != CAFE_OK && n > 1) {
            // one bad request must not fail the others: run them one by one
            for (int i = 0; i < n; ++i) {
                ScoreInfo one;
                res[i] = batch[i]->res ? *batch[i]->res : cafe_result{};
                {
                    std::unique_lock<std::mutex> lk(C->mu);
                    rcs[i] = score_enqueue(C, ws, &reqs[i], 1, &res[i], &one);
                }
                if (rcs[i] == CAFE_OK) rcs[i] = score_complete(C, ws, &reqs[i], 1, &res[i], one);
            }
        }
        const auto now = std::chrono::steady_clock::now();
        {
            std::lock_guard<std::mutex> lk(C->qmu);
            C->in_flight -= n;
            C->in_flight_bytes -= bytes;
            C->batches_in_flight--;
            C->completed += n;
            for (auto& r : batch)
                C->latencies_ms.push_back(std::chrono::duration<double, std::milli>(now - r->t_submit).count());
        }
        C->qcv.notify_all();     // freed footprint may admit queued requests
        for (int i = 0; i < n; ++i) {
            auto& r = batch[i];
            {
                std::lock_guard<std::mutex> lk(r->m);
                if (r->res) *r->res = res[i];
                r->rc = rcs[i];
                r->done = true;
            }
            r->cv.notify_all();
        }
    }
}

}  // namespace

void cafe_serving_stop(cafe_ctx* C) {
    {
        std::lock_guard<std::mutex> lk(C->qmu);
        C->stop = true;
    }
    C->qcv.notify_all();
    for (auto& t : C->servers)
        if (t.joinable()) t.join();
    C->servers.clear();
}

extern "C" {

int cafe_submit(cafe_ctx* C, const cafe_request* req, cafe_result* res, uint64_t* ticket) {
    if (!C || !req || !ticket) return CAFE_ERR_INVALID;
    auto r = std::make_shared<Request>();
    r->req = *req;
    r->lambdas.assign(req->lambdas, req->lambdas + std::max(req->n_lambdas, 0));
    r->req.lambdas = r->lambdas.data();
    if (req->model == CAFE_MODEL_GAMMA && req->n_categories > 0) {
        r->mult.assign(req->multipliers, req->multipliers + req->n_categories);
        r->probs.assign(req->cat_probs, req->cat_probs + req->n_categories);
        r->req.multipliers = r->mult.data();
        r->req.cat_probs = r->probs.data();
    }
    r->res = res;
    r->t_submit = std::chrono::steady_clock::now();
    {
        std::lock_guard<std::mutex> lk(C->mu);
        r->bytes = request_footprint(C, r->req);
        auto si = C->sets.find(r->req.set_id);
        r->small = si != C->sets.end() && small_request(C, &r->req, 1, si->second->F);
    }
    std::lock_guard<std::mutex> lk(C->qmu);
    if (C->servers.empty()) {
        C->stop = false;
        // the epoch of the batches' device intervals, on a serving stream
        // with nothing queued
        C->serve_intervals.clear();
        if (!C->serve_epoch && cudaEventCreate(&C->serve_epoch) != cudaSuccess) C->serve_epoch = nullptr;
        if (C->serve_epoch && C->ws.size() > 1) cudaEventRecord(C->serve_epoch, C->ws[1]->stream);
        for (size_t i = 1; i < C->ws.size(); ++i) C->servers.emplace_back(server_loop, C, (int)i);
    }
    *ticket = C->next_ticket++;
    C->tickets[*ticket] = r;
    C->queue.push_back(r);
    C->qcv.notify_one();
    return CAFE_OK;
}

int cafe_poll(cafe_ctx* C, uint64_t ticket, int wait_ms) {
    if (!C) return CAFE_ERR_INVALID;
    std::shared_ptr<Request> r;
    {
        std::lock_guard<std::mutex> lk(C->qmu);
        auto it = C->tickets.find(ticket);
        if (it == C->tickets.end()) return CAFE_ERR_NOT_FOUND;
        r = it->second;
    }
    std::unique_lock<std::mutex> lk(r->m);
    if (!r->done) {
        if (wait_ms < 0) r->cv.wait(lk, [&] { return r->done; });
        else if (wait_ms > 0) r->cv.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return r->done; });
    }
    if (!r->done) return CAFE_ERR_BUSY;
    const int rc = r->rc;
    lk.unlock();
    std::lock_guard<std::mutex> lk2(C->qmu);
    C->tickets.erase(ticket);
    return rc;
}

int cafe_serving_counters(cafe_ctx* C, cafe_serving_info* out) {
    if (!C || !out) return CAFE_ERR_INVALID;
    std::lock_guard<std::mutex> lk(C->qmu);
    *out = C->serving;
    return CAFE_OK;
}

int cafe_serving_stats(cafe_ctx* C, int64_t* completed, double* p50, double* p99, int* in_flight) {
    if (!C) return CAFE_ERR_INVALID;
    std::lock_guard<std::mutex> lk(C->qmu);
    std::vector<double> v = C->latencies_ms;
    std::sort(v.begin(), v.end());
    auto pct = [&](double q) { return v.empty() ? 0.0 : v[std::min(v.size() - 1, (size_t)(q * (v.size() - 1) + 0.5))]; };
    if (completed) *completed = C->completed;
    if (p50) *p50 = pct(0.50);
    if (p99) *p99 = pct(0.99);
    if (in_flight) *in_flight = C->in_flight + (int)C->queue.size();
    return CAFE_OK;
}

}  // extern "C"
