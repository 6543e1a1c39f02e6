// cafe_prune_fp64_noalloc: the FP64 pruning kernel (k_prune64) with all of
// its scratch in one file-scope static device array, for callers that must
// not allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is off limits -- a host
// framework that owns every device allocation through its own pool and
// forbids hidden ones, a latency-critical serving loop that must not
// allocate per request, or a plug-in loaded into a process whose allocator
// is not CUDA's. Such a caller brings its own device buffers for inputs and
// outputs and gets the working space from this library's static array.
//
// The array below is reserved on every GPU that loads the library and stays
// reserved until the process exits. Its size is fixed: 40 MiB, of which the
// first 8 MiB hold per-call metadata (work tiles, the family order, the tree
// plan, the per-node matrix table) and the remaining 32 MiB hold node
// vectors. Every call shares it and it keeps the previous call's contents;
// nothing in it has to start at zero because the kernel writes every node
// vector before reading it. Two calls whose GPU work overlaps (for example
// on two streams) race on the array: serialise them.
//
// Host code may not use the array's name as a device address (in host code
// it names a host-side stand-in); its device address is obtained once per
// device with cudaGetSymbolAddress, with that device current. The first call
// on each device performs that set-up, so make the first call before any
// stream capture.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/cafe_gb300.h"
#include "common.cuh"

namespace cafe {
namespace {

constexpr size_t kNoAllocBytes = size_t(40) << 20;           // whole static array
constexpr size_t kMetaBytes = size_t(8) << 20;               // metadata region
constexpr size_t kVectorBytes = kNoAllocBytes - kMetaBytes;  // node-vector region
constexpr int64_t kMaxFamilies = int64_t(1) << 18;           // 262,144
constexpr int kMaxTiles = (int)(kMaxFamilies / 32);
constexpr int kMaxDevices = 64;
constexpr int kTileFamilies = 32;                             // k_prune64's tile width

// metadata layout (byte offsets inside the array)
constexpr size_t kOffTiles = 0;                                           // PruneTile[kMaxTiles]
constexpr size_t kOffPerm = kOffTiles + sizeof(PruneTile) * kMaxTiles;     // int64[kMaxFamilies]
constexpr size_t kOffPlan = kOffPerm + sizeof(int64_t) * kMaxFamilies;     // int32[5 * kMaxNodes + 1]
constexpr size_t kOffMats = kOffPlan + 65536;                              // const double*[kMaxNodes]
static_assert(kOffMats + sizeof(double*) * kMaxNodes <= kMetaBytes, "metadata region too small");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_setup_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Once per device, with that device current: the array's device address.
int scratch_address(int dev, unsigned char** out) {
    if (dev < 0 || dev >= kMaxDevices) return CAFE_ERR_INVALID;
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return CAFE_ERR_CUDA;
        }
        g_scratch_addr[dev] = p;
    }
    *out = static_cast<unsigned char*>(g_scratch_addr[dev]);
    return CAFE_OK;
}

__global__ void k_iota64(int64_t* p, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = i;
}

}  // namespace
}  // namespace cafe

using namespace cafe;

extern "C" int cafe_prune_fp64_noalloc(int n_nodes, const int32_t* parent, const double* const* node_matrix,
                                       int matrix_size, const int32_t* d_counts, int64_t n_families, int n_leaves,
                                       int max_family_size, int max_root_family_size, const double* d_prior,
                                       int n_prior, int scaled, double* d_family_lnl, void* stream) {
    // ---- argument checks (nothing is launched on failure) ----
    if (n_nodes < 2 || n_nodes > kMaxNodes || !parent || !node_matrix || !d_counts || !d_prior || !d_family_lnl)
        return CAFE_ERR_INVALID;
    if (n_families < 0 || n_families > kMaxFamilies || n_prior < 1) return CAFE_ERR_INVALID;
    const int S = max_family_size, R = max_root_family_size;
    if (S < 1 || R < 1 || matrix_size < std::max(R, S) + 1) return CAFE_ERR_INVALID;
    if (n_families == 0) return CAFE_OK;

    // ---- tree plan on the host: post-order of internal nodes, greedy slots ----
    std::vector<std::vector<int>> children(n_nodes);
    int root = -1, roots = 0;
    for (int i = 0; i < n_nodes; ++i) {
        const int p = parent[i];
        if (p < 0) {
            root = i;
            roots++;
        } else if (p >= n_nodes || p == i) {
            return CAFE_ERR_INVALID;
        } else {
            children[p].push_back(i);
        }
    }
    if (roots != 1 || children[root].empty()) return CAFE_ERR_INVALID;
    std::vector<int32_t> leaf_col(n_nodes, -1);
    int leaves = 0;
    for (int i = 0; i < n_nodes; ++i)
        if (children[i].empty()) leaf_col[i] = leaves++;
    if (leaves != n_leaves) return CAFE_ERR_INVALID;
    std::vector<int32_t> order;
    {
        std::vector<std::pair<int, size_t>> st{{root, 0}};
        std::vector<char> seen(n_nodes, 0);
        while (!st.empty()) {
            auto& top = st.back();
            const int v = top.first;
            if (top.second < children[v].size()) {
                const int c = children[v][top.second++];
                if (seen[c]++) return CAFE_ERR_INVALID;   // not a tree
                if (!children[c].empty()) st.push_back({c, 0});
            } else {
                order.push_back(v);
                st.pop_back();
            }
        }
    }
    std::vector<int32_t> cstart{0}, child, slot(n_nodes, -1);
    std::vector<int> free_slots;
    int n_slots = 0, max_children = 0;
    for (int v : order) {
        for (int c : children[v]) {
            child.push_back(c);
            if (c != root && !node_matrix[c]) return CAFE_ERR_INVALID;
        }
        cstart.push_back((int32_t)child.size());
        max_children = std::max<int>(max_children, (int)children[v].size());
        int s;
        if (!free_slots.empty()) {
            auto it = std::min_element(free_slots.begin(), free_slots.end());
            s = *it;
            free_slots.erase(it);
        } else {
            s = n_slots++;
        }
        slot[v] = s;
        for (int c : children[v])
            if (!children[c].empty()) free_slots.push_back(slot[c]);
    }

    // ---- fit the work into the static array ----
    const int W = std::max(S + 1, R);
    const int64_t per_cta = (int64_t)n_slots * W * kTileFamilies;   // doubles
    const int64_t fit = (int64_t)(kVectorBytes / sizeof(double)) / per_cta;
    if (fit < 1) return CAFE_ERR_INVALID;
    const int n_tiles = (int)((n_families + kTileFamilies - 1) / kTileFamilies);
    if (n_tiles > kMaxTiles) return CAFE_ERR_INVALID;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return CAFE_ERR_CUDA;
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int n_ctas = (int)std::max<int64_t>(1, std::min<int64_t>({(int64_t)n_tiles, fit, (int64_t)std::max(sms, 1) * 4}));

    unsigned char* base = nullptr;
    const int rc = scratch_address(dev, &base);
    if (rc != CAFE_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    std::vector<PruneTile> tiles(n_tiles);
    for (int t = 0; t < n_tiles; ++t) {
        PruneTile tl{};
        tl.first = t * kTileFamilies;
        tl.count = (int)std::min<int64_t>(kTileFamilies, n_families - tl.first);
        tl.k = 0;
        tl.S = S;
        tl.R = R;
        tiles[t] = tl;
    }
    const size_t ni = order.size();
    std::vector<int32_t> plan;
    plan.insert(plan.end(), order.begin(), order.end());
    plan.insert(plan.end(), cstart.begin(), cstart.end());
    plan.insert(plan.end(), child.begin(), child.end());
    plan.insert(plan.end(), leaf_col.begin(), leaf_col.end());
    plan.insert(plan.end(), slot.begin(), slot.end());
    std::vector<const double*> mats(node_matrix, node_matrix + n_nodes);
    mats[root] = nullptr;

    PruneTile* d_tiles = reinterpret_cast<PruneTile*>(base + kOffTiles);
    int64_t* d_perm = reinterpret_cast<int64_t*>(base + kOffPerm);
    int32_t* d_plan = reinterpret_cast<int32_t*>(base + kOffPlan);
    const double** d_mats = reinterpret_cast<const double**>(base + kOffMats);
    double* d_vec = reinterpret_cast<double*>(base + kMetaBytes);

    cudaError_t e = cudaMemcpyAsync(d_tiles, tiles.data(), tiles.size() * sizeof(PruneTile), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_plan, plan.data(), plan.size() * sizeof(int32_t), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_mats, mats.data(), mats.size() * sizeof(const double*), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        const int blocks = (int)std::min<int64_t>((n_families + 255) / 256, 1024);
        k_iota64<<<blocks, 256, 0, s>>>(d_perm, n_families);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return CAFE_ERR_CUDA;

    Prune64Args a{};
    a.plan.n_nodes = n_nodes;
    a.plan.n_internal = (int)ni;
    a.plan.n_leaves = n_leaves;
    a.plan.root = root;
    a.plan.n_slots = n_slots;
    a.plan.max_children = max_children;
    a.plan.internal = d_plan;
    a.plan.cstart = d_plan + ni;
    a.plan.child = d_plan + ni + cstart.size();
    a.plan.leaf_col = d_plan + ni + cstart.size() + child.size();
    a.plan.slot = d_plan + ni + cstart.size() + child.size() + n_nodes;
    a.tiles = d_tiles;
    a.n_tiles = n_tiles;
    a.counts = d_counts;
    a.perm = d_perm;
    a.mats = d_mats;
    a.ld_mat = matrix_size;
    a.prior = d_prior;
    a.n_prior = n_prior;
    a.err = nullptr;
    a.err_rows = 0;
    a.err_ndev = 0;
    a.fam_R = nullptr;
    a.scratch = d_vec;
    a.scratch_per_cta = per_cta;
    a.scaled = scaled ? 1 : 0;
    a.model = 0;
    a.out = d_family_lnl;
    a.K = 1;
    a.cat_probs = nullptr;
    a.tile_families = kTileFamilies;
    a.W = W;
    e = launch_prune64(a, n_ctas, s);
    return e == cudaSuccess ? CAFE_OK : CAFE_ERR_CUDA;
}
