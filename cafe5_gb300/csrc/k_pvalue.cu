// K7 (opt-in): the simulations of compute_pvalues drawn on the GPU.
//
// compute_pvalues (src/probability.cpp:376-570) simulates n_sim families
// per root size r = 1..R down the tree (create_family, :351-373, over
// set_weighted_random_family_size, :449-476): every child's size is drawn
// from its parent's matrix row restricted to sizes 0..S-1
// (matrix::select_random_y, src/matrix_cache.cpp:60-66, a
// std::discrete_distribution over the row's first S entries). The
// reference draws from one std::mt19937 in a fixed order, which is serial
// by construction; this mode draws from a counter-based generator instead
// (the SplitMix64 sequence of Steele, Lea and Flood, OOPSLA 2014, indexed
// by (family, node)), so every simulated family is one thread. The draws
// follow the same distributions but are not the reference's stream: the
// p-values agree in distribution, not bit for bit.
//
//  * k_cdf_build: cumulative weights of every (node, parent size) row.
//  * k_sim_draw: one thread per simulated family: sizes in prefix order by
//    inverse-CDF search, the leaf counts, the family's state bound
//    m = min(S, largest + max(50, largest / 5)) (compute_family_probabilities)
//    and its (root size, bound) key.
//  * k_sim_plan (one block): families per key -> offsets, and 32-family
//    tiles of equal (root size, bound) with the tile count on the device.
//  * k_sim_scatter: the family order the tiles read.
//  * (k_prune64 over the device tile count writes each family's root value.)
//  * k_sort_rows: each root size's n_sim likelihoods sorted (bitonic sort
//    in shared memory), the conditional distributions.
//  * k_pvalue_search: per observed family, the largest share of simulated
//    likelihoods not above its own over root sizes up to 1.25 x its largest
//    count (find_best_pvalue / pvalue, :503-528).
#include "common.cuh"

#include <algorithm>

namespace cafe {
namespace {

constexpr uint64_t kGolden = 0x9E3779B97F4A7C15ull;

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Output c + 1 of the SplitMix64 sequence started at `key`, as a double in
// [0, 1) with 53 random bits.
__device__ __forceinline__ double uniform01(uint64_t key, uint64_t c) {
    return (double)(mix64(key + (c + 1) * kGolden) >> 11) * 0x1.0p-53;
}

__global__ void __launch_bounds__(128) k_cdf_build(const double* const* __restrict__ mats, int n_nodes, int msize,
                                                   int S, int n_ps, double* __restrict__ cdf) {
    const int v = blockIdx.x;
    const int ps = blockIdx.y * blockDim.x + threadIdx.x;
    if (v >= n_nodes || ps >= n_ps) return;
    const double* M = mats[v];
    if (!M) return;   // the root
    const double* row = M + (size_t)ps * msize;
    double* out = cdf + ((size_t)v * n_ps + ps) * S;
    double acc = 0.0;
    for (int c = 0; c < S; ++c) {
        acc += row[c];
        out[c] = acc;
    }
}

__global__ void __launch_bounds__(128) k_sim_draw(SimDrawArgs a) {
    const int64_t fi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (fi >= a.n_families) return;
    const int r = (int)(fi / a.n_sim);     // root size r + 1
    int32_t* sz = a.sizes + (size_t)fi * a.n_nodes;
    sz[a.root] = r + 1;
    int mx = r + 1;
    const int S = a.S;
    for (int i = 0; i < a.n_nodes; ++i) {
        const int v = a.prefix[i];
        if (v == a.root) continue;
        const int ps = sz[a.parent[v]];
        int c = 0;
        if (ps > 0) {
            const double* cd = a.cdf + ((size_t)v * a.n_ps + ps) * S;
            const double total = cd[S - 1];
            if (total > 0.0) {
                // first size whose cumulative weight exceeds u * total
                double target = uniform01(a.key, (uint64_t)fi * a.n_nodes + v) * total;
                if (target >= total) target = nextafter(total, 0.0);
                int lo = 0, hi = S - 1;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (cd[mid] > target) hi = mid;
                    else lo = mid + 1;
                }
                c = lo;
            }
        }
        sz[v] = c;
        mx = max(mx, c);
        if (a.leaf_col[v] >= 0) a.counts[(size_t)fi * a.n_leaves + a.leaf_col[v]] = c;
    }
    const int m = min(S, mx + max(50, mx / 5));
    const int key = r * (S + 1) + m;
    a.keys[fi] = key;
    atomicAdd(&a.hist[key], 1);
}

// Block-wide inclusive sum of one value per thread (1024 threads).
__device__ __forceinline__ int64_t block_scan(int64_t x, int64_t* sh, int64_t* total) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int64_t w = sh[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        sh[lane] = w;
    }
    __syncthreads();
    if (warp > 0) x += sh[warp - 1];
    *total = sh[31];
    __syncthreads();
    return x;
}

__global__ void __launch_bounds__(1024) k_sim_plan(SimPlanArgs a) {
    __shared__ int64_t sh[32];
    int64_t fam_base = 0, tile_base = 0;
    for (int k0 = 0; k0 < a.n_keys; k0 += 1024) {
        const int key = k0 + threadIdx.x;
        const int64_t cnt = key < a.n_keys ? a.hist[key] : 0;
        const int64_t nt = (cnt + 31) / 32;
        int64_t tf, tt;
        const int64_t fam_inc = block_scan(cnt, sh, &tf);
        const int64_t tile_inc = block_scan(nt, sh, &tt);
        if (key < a.n_keys) {
            const int64_t f0 = fam_base + fam_inc - cnt, t0 = tile_base + tile_inc - nt;
            a.cursor[key] = (int32_t)f0;
            const int r = key / (a.S + 1), m = key % (a.S + 1);
            for (int64_t i = 0; i < nt && t0 + i < a.max_tiles; ++i) {
                PruneTile t{};
                t.first = (int)(f0 + 32 * i);
                t.count = (int)(cnt - 32 * i < 32 ? cnt - 32 * i : 32);
                t.k = 0;
                t.S = m;
                t.R = 1;
                t.root_lo = r + 1;
                a.tiles[t0 + i] = t;
            }
        }
        fam_base += tf;
        tile_base += tt;
    }
    if (threadIdx.x == 0) *a.n_tiles = (int32_t)(tile_base < a.max_tiles ? tile_base : a.max_tiles);
}

__global__ void __launch_bounds__(256) k_sim_scatter(const int32_t* __restrict__ keys, int64_t n,
                                                     int32_t* __restrict__ cursor, int64_t* __restrict__ perm) {
    const int64_t fi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (fi >= n) return;
    const int pos = atomicAdd(&cursor[keys[fi]], 1);
    perm[pos] = fi;
}

// One block per row of n values: ascending bitonic sort of the row padded
// with +inf to P = a power of two (dynamic shared memory, P doubles).
__global__ void __launch_bounds__(512) k_sort_rows(double* __restrict__ v, int n, int P) {
    extern __shared__ double s[];
    double* row = v + (size_t)blockIdx.x * n;
    for (int i = threadIdx.x; i < P; i += blockDim.x) s[i] = i < n ? row[i] : INFINITY;
    __syncthreads();
    for (int k = 2; k <= P; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const bool up = (i & k) == 0;
                    const double x = s[i], y = s[l];
                    if (up ? (x > y) : (x < y)) {
                        s[i] = y;
                        s[l] = x;
                    }
                }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < n; i += blockDim.x) row[i] = s[i];
}

__global__ void __launch_bounds__(128) k_pvalue_search(PvalueSearchArgs a) {
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= a.F) return;
    int largest = 0;
    for (int c = 0; c < a.n_leaves; ++c) largest = max(largest, a.counts[(size_t)f * a.n_leaves + c]);
    const int check = min(a.R, (int)rint(largest * 1.25));
    double best = 0.0;
    for (int j = 0; j < check; ++j) {
        const double v = a.obs[(size_t)f * a.R + j];
        const double* d = a.sorted + (size_t)j * a.n_sim;
        // first simulated value above v (the reference's upper_bound; past
        // the end it counts n_sim - 1)
        int lo = 0, hi = a.n_sim;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (d[mid] > v) hi = mid;
            else lo = mid + 1;
        }
        const int idx = lo == a.n_sim ? a.n_sim - 1 : lo;
        best = fmax(best, idx / (double)a.n_sim);
    }
    a.out[f] = best;
}

}  // namespace

uint64_t sim_seed_key(uint32_t seed) {
    uint64_t z = (uint64_t)seed + kGolden;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

cudaError_t pvalue_kernels_init() {
    return cudaFuncSetAttribute(k_sort_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, kSortRowsMaxP * 8);
}

cudaError_t launch_cdf_build(const double* const* mats, int n_nodes, int msize, int S, int n_ps, double* cdf,
                             cudaStream_t s) {
    if (n_nodes <= 0 || n_ps <= 0 || S <= 0) return cudaSuccess;
    k_cdf_build<<<dim3((unsigned)n_nodes, (unsigned)((n_ps + 127) / 128)), 128, 0, s>>>(mats, n_nodes, msize, S, n_ps,
                                                                                        cdf);
    return cudaGetLastError();
}

cudaError_t launch_sim_draw(const SimDrawArgs& a, cudaStream_t s) {
    if (a.n_families <= 0) return cudaSuccess;
    k_sim_draw<<<(unsigned)((a.n_families + 127) / 128), 128, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_sim_plan(const SimPlanArgs& a, cudaStream_t s) {
    k_sim_plan<<<1, 1024, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_sim_scatter(const int32_t* keys, int64_t n, int32_t* cursor, int64_t* perm, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_sim_scatter<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(keys, n, cursor, perm);
    return cudaGetLastError();
}

cudaError_t launch_sort_rows(double* v, int rows, int n, cudaStream_t s) {
    if (rows <= 0 || n <= 0) return cudaSuccess;
    int P = 1;
    while (P < n) P <<= 1;
    if (P > kSortRowsMaxP) return cudaErrorInvalidValue;
    k_sort_rows<<<(unsigned)rows, 512, (size_t)P * sizeof(double), s>>>(v, n, P);
    return cudaGetLastError();
}

cudaError_t launch_pvalue_search(const PvalueSearchArgs& a, cudaStream_t s) {
    if (a.F <= 0) return cudaSuccess;
    k_pvalue_search<<<(unsigned)((a.F + 127) / 128), 128, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace cafe
