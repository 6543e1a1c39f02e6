// Host runtime of the GB300 CAFE5 likelihood path (internal).
#pragma once

#include <condition_variable>
#include <cstdint>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "../../include/cafe_gb300.h"
#include "common.cuh"

namespace cafe {

// Default S-bin widths (vector length = states 0..W-1).
extern const int kDefaultBins[];
extern const int kNumDefaultBins;

// While alive, device buffers that grow on this thread are freed and
// allocated stream-ordered on `s`.
struct AllocScope {
    cudaStream_t prev;
    explicit AllocScope(cudaStream_t s);
    ~AllocScope();
};

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    ~DevBuf();
    cudaError_t reserve(size_t n);
    template <class T> T* as() const { return static_cast<T*>(p); }
};

struct PinnedBuf {
    void* p = nullptr;
    size_t bytes = 0;
    ~PinnedBuf();
    cudaError_t reserve(size_t n);
    template <class T> T* as() const { return static_cast<T*>(p); }
};

struct TreeHost {
    int n_nodes = 0, n_leaves = 0, root = -1;
    std::vector<int32_t> parent, lambda_index, leaf_col;
    std::vector<double> branch_length;
    std::vector<std::vector<int>> children;
    // plan (internal nodes in post-order) and its device copy
    std::vector<int32_t> internal, cstart, child, slot;
    int n_slots = 0, max_children = 0;
    DevBuf d_plan;
    TreePlan plan{};
    double longest_branch = 0.0;
    std::vector<double> distinct_lengths;   // positive, sorted (root branch included)
};

struct BinPlan {
    // families grouped by bin; perm holds family indices bin by bin
    std::vector<int> widths;                 // bin widths used
    std::vector<int64_t> bin_first, bin_count;
    DevBuf d_perm, d_famR;
    int W_max = 0;
};

struct FamSet {
    int tree_id = 0;
    int64_t F = 0;
    int n_leaves = 0;
    DevBuf d_counts;
    std::vector<int32_t> h_counts;
    std::vector<int32_t> max_count;
    // dedupe: unique families and reference per family
    std::vector<int64_t> unique;
    DevBuf d_unique, d_ref, d_identity;
    BinPlan bins;
};

struct MatKey {
    int size;
    long lq, tq;
    bool operator==(const MatKey& o) const { return size == o.size && lq == o.lq && tq == o.tq; }
};
struct MatKeyHash {
    size_t operator()(const MatKey& k) const {
        return std::hash<long>()(k.lq * 1000003L ^ k.tq) ^ std::hash<int>()(k.size);
    }
};

struct MatEntry {
    double* d = nullptr;       // FP64 row-major size x size (null until its build is enqueued)
    int chunk = -1;            // build batch (index of its ready event)
    uint64_t stamp = 0;        // request that last gave it a conversion slot
    int conv = -1;             // that request's converted-matrix index
};

// Open-addressing hash table of the matrix cache: keys and entries inline
// (one cache line per probe instead of a node chase), linear probing,
// backward-shift deletion. Entry pointers stay valid until the table grows;
// callers reserve() for a request's keys before taking pointers.
class MatCache {
   public:
    MatEntry* find(const MatKey& k);
    void prefetch(const MatKey& k) const;   // bring k's home slot into the CPU caches
    // (entry, inserted)
    std::pair<MatEntry*, bool> try_emplace(const MatKey& k);
    void erase(const MatKey& k);
    void reserve(size_t n_entries);
    void clear();
    size_t size() const { return n_; }

   private:
    struct Slot {
        MatKey key;
        bool used = false;
    };
    std::vector<Slot> slots_;
    std::vector<MatEntry> vals_;
    size_t n_ = 0, mask_ = 0;
    size_t home(const MatKey& k) const;
    void grow(size_t cap);
};

struct Slab {
    void* p = nullptr;
    size_t size = 0, used = 0;
    cudaEvent_t ev_alloc = nullptr;   // after its stream-ordered allocation
};

// Per-request device workspace (one per stream).
struct Workspace {
    cudaStream_t stream = nullptr;     // the stream of the current request: stream_hi or stream_lo
    // Serving batches admitted while another batch runs go to stream_lo (one
    // priority step lower): their blocks fill the SMs the earlier batch
    // leaves idle instead of competing with it.
    cudaStream_t stream_hi = nullptr, stream_lo = nullptr;
    bool sync = false;                 // a synchronous-call workspace (profiled when profiling is on)
    cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
    cudaEvent_t ev_staged = nullptr;   // after the last request's host->device staging copies
    bool staged = false;
    cudaStream_t build = nullptr;      // K1 builds (overlap the previous request's pruning)
    bool build_inline = false;         // this call builds on `stream` (synchronous calls)
    cudaEvent_t ev_jobs = nullptr;     // after the last build (its job table read)
    bool jobs_pending = false;
    static constexpr int kAux = 8;     // streams for concurrent per-bin launches (one per bin)
    cudaStream_t aux[kAux] = {};
    cudaEvent_t ev_fork = nullptr;
    cudaEvent_t ev_join[kAux] = {};
    struct MapCache {
        const void* ptr = nullptr;
        int64_t rows = 0;
        int cols = 0;
        int box = 0;
        int box_rows = 0;
        int64_t depth = 0;
        CUtensorMap map;
    } map_cache[20];   // [2] vector loads, [3] vector stores, [4 + Ws/32 - 1] matrices (hi and lo planes),
                       // [12 + Ws/32 - 1] transposed matrices
    DevBuf scratch, tiles, mats, cat, fam_lnl, total, nfail, jobs, catp;
    PinnedBuf h_tiles, h_mats, h_jobs, h_out, h_catp;
    // tensor-core path
    DevBuf term_flags, fb_bins, tile_ctr, tc_hi, tc_tr, tc_mi, tc_vec, conv, flags, fb_perm, tiles64, tiles_fb, parts, fb_count, phase,
        catids, cerr;
    PinnedBuf h_conv, h_mi, h_flags, h_tiles64, h_tiles_fb, h_tail, h_catids;
    // FP64 bins walked one family per cluster
    DevBuf tiles_cl;
    PinnedBuf h_tiles_cl;
    std::vector<PruneTile> cl_tile_vec;
    // reconstruction
    DevBuf rc_c, rc_state, rc_rmax, rc_mean, rc_count, rc_nfail, rc_parent, rc_bp, rc_lm, rc_lptr;
    PinnedBuf h_sim, h_simperm;        // p-values: simulated families staged for the device
    std::vector<PruneTile> tile_vec;
    std::vector<MatEntry*> entry_vec;   // cache entry of every (combined category, node)
    std::vector<MatKey> key_vec;        // the request's matrix keys
    std::vector<uint8_t> sat_vec;       // its key is saturated (1 - 2a outside (0, 1))
    // CUDA graphs of the pruning phase: stream ops go through an op log;
    // a dry pass records their parameters as the graph's signature
    enum OpMode { kOpRun = 0, kOpDry = 1, kOpCapture = 2 };
    int op_mode = kOpRun;
    std::vector<uint8_t> oplog;
    struct GraphEntry {
        std::vector<uint8_t> sig;
        cudaGraphExec_t exec = nullptr;
        uint64_t used = 0;
    } graphs[16];
    uint64_t graph_clock = 0;
    // hashes of recently issued signatures: once every slot holds a graph,
    // a phase is captured only when its signature comes back
    uint64_t seen[64] = {};
    int seen_next = 0;
    ~Workspace();
    int init(int device);
};

struct Request;   // serving-loop request record

// Event pairs recorded around launches when profiling is on.
struct Profiler {
    bool on = false;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;   // (kind, events)
    std::vector<cudaEvent_t> pool;
    cafe_timings acc{};
    cudaEvent_t get();
    void begin(int kind, cudaStream_t s, cudaEvent_t* a);
    void end(int kind, cudaStream_t s, cudaEvent_t a);
    void collect();
};

}  // namespace cafe

struct cafe_ctx {
    int device = 0;
    std::string last_error;
    std::mutex mu;
    std::map<int, std::unique_ptr<cafe::TreeHost>> trees;
    std::map<int, std::unique_ptr<cafe::FamSet>> sets;
    int next_tree = 1, next_set = 1;
    std::vector<double> prior;
    cafe::DevBuf d_prior;
    std::vector<double> err;
    int err_rows = 0, err_ndev = 0;
    cafe::DevBuf d_err;
    // matrix cache
    cafe::MatCache cache;
    // two generations of slabs, used in turn: the cache fills one; past the
    // cap it starts over in the other (whose users were issued a whole
    // generation earlier)
    struct SlabGen {
        std::vector<cafe::Slab> slabs;
        size_t cur = 0;                         // the slab builds draw from (slabs before it are full)
        std::vector<cudaEvent_t> marks;         // recorded on every stream when the cache left this generation
        int n_marks = 0;                        // builds into this generation wait for them
    } gens[2];
    int gen = 0;
    std::vector<cudaEvent_t> batch_events;
    size_t cache_bytes = 0, cache_cap = 0;      // bytes of the current generation, cap of one
    uint64_t request_stamp = 0;
    std::map<int, std::pair<int, int>> tuned;   // bin width -> (CTAs per SM, stages) chosen by cafe_autotune
    int debug_wait_limit = 0;    // cafe_debug_set: polls before the tensor-core wait for a node's GEMMs gives up
    // workspaces: [0] for synchronous calls, [1..] for the serving loop
    std::vector<std::unique_ptr<cafe::Workspace>> ws;
    std::unique_ptr<cafe::Workspace> ws_alt;   // second workspace of the device-pointer calls
    int dev_flip = 0;
    int n_ctas = 0;
    int sm_count = 0;
    // serving loop
    std::mutex qmu;
    std::condition_variable qcv;
    std::deque<std::shared_ptr<cafe::Request>> queue;
    std::map<uint64_t, std::shared_ptr<cafe::Request>> tickets;
    std::vector<std::thread> servers;
    bool stop = false;
    uint64_t next_ticket = 1;
    int in_flight = 0;
    size_t in_flight_bytes = 0;       // estimated device footprint of admitted requests
    size_t serve_budget = 0;          // admission limit for that footprint
    std::vector<double> latencies_ms;
    int batches_in_flight = 0;
    cafe_serving_info serving{};     // serving counters
    cudaEvent_t serve_epoch = nullptr;                    // recorded when the server threads start
    std::deque<std::pair<float, float>> serve_intervals;  // recent batches' device [start, end] (ms from the epoch)
    // last launch of the most recent request: the next request's device work
    // starts after it
    cudaEvent_t gate = nullptr;
    bool gate_set = false;
    int64_t completed = 0;
    cafe::Profiler prof;
};
