// K5: Pupko joint ancestral reconstruction and branch probabilities.
//
// Replaces pupko_reconstructor::reconstruct_gene_family
// (src/gene_family_reconstructor.cpp:161-190) with its leaf, internal and
// root steps (:30-116), as driven by base_model / gamma_model
// ::reconstruct_ancestral_states (src/base_model.cpp:133-170,
// src/gamma_core.cpp:290-339), the weighted category average of the gamma
// model (get_weighted_averages, src/gamma_core.cpp:268-287) and
// compute_viterbi_sum (src/gene_family_reconstructor.cpp:390-430).
//
// Per internal non-root node v, parent state i and family f the reference
// scans every child state j in ascending order:
//     u[j]    = prod over children c (descendant order) of L_c[j]
//     L_v[i]  = max_j u[j] * M_v[i][j],   C_v[i] = first j attaining it
// in FP64: (S+1)^2 products per node and family. GB300's FP64 pipe issues
// about two such products per clock and SM (and a divergent one costs a
// whole warp's issue), so k_pupko ranks the products in FP32 logarithms:
//   p_j = log2 u[j] + log2 M[i][j]   (FP32; log2 M precomputed once per
//                                     request, transposed, by k_log2_matrices)
// One pass keeps the largest p (b1, at j1) and the second largest (b2).
// Every log2 carries an absolute error <= 6.3e-5 (FP32 rounding of a value
// of magnitude <= 1075 plus log2f's 1 ulp) and the sum <= 1.3e-4 more, so a
// j whose exact product equals the FP64 row maximum has p_j >= b1 - 5e-4.
// With delta = 2^-8 (8x margin):
//   b1 < -1075 - delta          every product rounds to 0 in FP64: L = 0,
//                               C = 0 (the reference's result for such rows)
//   b1 >= -1022 + delta and     only j1 can reach the FP64 maximum: C = j1,
//   b2 < b1 - delta             L = u[j1] * M[i][j1] in FP64 (one product)
//   otherwise                   the (row, family) joins a per-block list
//                               that all threads then scan in FP64 over the
//                               j with p_j >= b1 - delta (every j when b1 is
//                               near the subnormal range), ascending, with
//                               the reference's strict '>'
// `exhaustive` sends every (row, family) through the FP64 scan of every j:
// the plain reference arithmetic, used to check the ranking.
#include "common.cuh"

#include <math.h>

#include <algorithm>

namespace cafe {
namespace {

constexpr int TF = 32;       // families per tile (one per lane)
constexpr int NT = 256;      // threads: 8 warps
constexpr int RW = 4;        // parent states per warp and block
constexpr int RB = 8 * RW;   // parent states per block
constexpr int JC = 64;       // child states per staged chunk
constexpr float kDelta = 0.00390625f;   // 2^-8, in log2 units

// log2 of x >= 0 in FP32 (-inf for 0) from the bits of x, without FP64
// arithmetic on normal numbers: exponent exact, the top 23 mantissa bits
// (truncation: relative error < 2^-23, i.e. < 1.8e-7 in log2) through
// log2f (1 ulp), then the FP32 sum (<= 2^-14 for |result| < 2048).
__device__ __forceinline__ float flog2(double x) {
    long long b = __double_as_longlong(x);
    if (b <= 0) return -INFINITY;   // +0 (and negative values, which never occur)
    int e = (int)((b >> 52) & 0x7ff);
    int bias = 1023;
    if (e == 0) {                   // subnormal: scale into the normal range
        b = __double_as_longlong(x * 0x1p64);
        e = (int)((b >> 52) & 0x7ff);
        bias += 64;
    }
    const float m = __int_as_float(0x3f800000 | (int)((b >> 29) & 0x7fffff));
    return (float)(e - bias) + log2f(m);
}

struct Staging {
    float lm[JC][RB];       // log2 M tile, child-state major
    float lu[JC][TF];       // log2 u chunk
};

constexpr int kSlowCap = RB * TF;   // (row, family) pairs of one block of rows

// Factor of child `ci` at child state j for family `fam` (tile lane f): a
// column of the leaf's matrix at the observed count, or the child's L.
__device__ __forceinline__ double child_value(const PupkoArgs& a, const double* const* mats, int ci, int j,
                                              int64_t fam, int f, const double* Lbase, int n) {
    const TreePlan& P = a.plan;
    const int ch = P.child[ci];
    const int lc = P.leaf_col[ch];
    if (lc >= 0) {
        const int cnt = a.counts[(size_t)fam * P.n_leaves + lc];
        return mats[ch][(size_t)j * a.ld_mat + cnt];
    }
    return Lbase[((size_t)P.slot[ch] * n + j) * TF + f];
}

// Stage the log2 tile (parent states i0.., child states j0..) from the
// transposed log2 matrix LMt[j][i] (pitch n) and the log2 u chunk.
__device__ __forceinline__ void stage(Staging& s, const float* LMt, int n, int i0, int j0, const float* LU) {
    const int tid = threadIdx.x;
    for (int e = tid; e < RB * JC; e += NT) {
        const int jj = e / RB, r = e % RB;
        const int i = i0 + r, j = j0 + jj;
        s.lm[jj][r] = (i < n && j < n) ? LMt[(size_t)j * n + i] : -INFINITY;
    }
    for (int e = tid; e < JC * TF; e += NT) {
        const int jj = e / TF, f = e % TF;
        const int j = j0 + jj;
        s.lu[jj][f] = j < n ? LU[(size_t)j * TF + f] : -INFINITY;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(NT, 4) k_pupko(PupkoArgs a) {
    __shared__ __align__(16) Staging s;
    __shared__ int node_ii[kMaxNodes];
    __shared__ int slow_pair[kSlowCap];      // (row - i0) * TF + family
    __shared__ float slow_best[kSlowCap];    // b1 of the pair (-inf: scan every j)
    __shared__ int n_slow;
    __shared__ int root_arg[TF];
    __shared__ double root_val[TF];

    const TreePlan& P = a.plan;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n = a.S + 1;
    double* Lbase = a.scratch + (size_t)blockIdx.x * a.scratch_per_cta;   // [n_slots][n][TF]
    double* U = Lbase + (size_t)P.n_slots * n * TF;                        // [n][TF]
    float* LU = reinterpret_cast<float*>(U + (size_t)n * TF);              // [n][TF]
    int32_t* Cbase = a.cscratch + (size_t)blockIdx.x * a.c_per_cta;        // [n_internal][n][TF]

    for (int v = tid; v < P.n_nodes; v += NT) node_ii[v] = -1;
    __syncthreads();
    for (int ii = tid; ii < P.n_internal; ii += NT) node_ii[P.internal[ii]] = ii;
    __syncthreads();

    for (int t = blockIdx.x; t < a.n_tiles; t += gridDim.x) {
        const PruneTile tile = a.tiles[t];
        const int cnt = tile.count, k = tile.k;
        const double* const* mats = a.mats + (size_t)k * P.n_nodes;

        for (int ii = 0; ii < P.n_internal; ++ii) {
            const int v = P.internal[ii];
            const int c0 = P.cstart[ii], c1 = P.cstart[ii + 1];
            if (v == P.root) {
                // reconstruct_root_node (:47-78): max over root sizes
                // j in [1, root_len) of prod_children L[j] * prior(j)
                if (tid < TF) {
                    double best = -1.0;
                    int arg = 0;
                    if (tid < cnt) {
                        const int64_t fam = tile.first + tid;
                        for (int j = 1; j < a.root_len; ++j) {
                            double value = 1.0;
                            for (int ci = c0; ci < c1; ++ci)
                                value *= child_value(a, mats, ci, j, fam, tid, Lbase, n);
                            const double val = value * (j < a.n_prior ? a.prior[j] : 0.0);
                            if (val > best) {
                                best = val;
                                arg = j;
                            }
                        }
                    }
                    root_val[tid] = a.root_len > 1 ? best : 0.0;
                    root_arg[tid] = arg;
                }
                continue;
            }
            // u[j] and log2 u[j] of every family of the tile
            for (int idx = tid; idx < n * TF; idx += NT) {
                const int j = idx / TF, f = idx % TF;
                double value = 0.0;
                if (f < cnt) {
                    value = 1.0;
                    for (int ci = c0; ci < c1; ++ci)
                        value *= child_value(a, mats, ci, j, tile.first + f, f, Lbase, n);
                }
                U[idx] = value;
                LU[idx] = flog2(value);
            }
            __syncthreads();
            double* Lv = Lbase + (size_t)P.slot[v] * n * TF;
            int32_t* Cv = Cbase + (size_t)ii * n * TF;
            const double* M = mats[v];
            const float* LMt = a.lmats[(size_t)k * P.n_nodes + v];
            for (int i0 = 0; i0 < n; i0 += RB) {
                float b1[RW], b2[RW];
                int j1[RW];
#pragma unroll
                for (int r = 0; r < RW; ++r) {
                    b1[r] = -INFINITY;
                    b2[r] = -INFINITY;
                    j1[r] = 0;
                }
                if (tid == 0) n_slow = 0;
                if (!a.exhaustive) {
                    for (int j0 = 0; j0 < n; j0 += JC) {
                        stage(s, LMt, n, i0, j0, LU);
                        const int jn = min(JC, n - j0);
                        for (int jj = 0; jj < jn; ++jj) {
                            const float lu = s.lu[jj][lane];
                            float lm[RW];
#pragma unroll
                            for (int q = 0; q < RW / 4; ++q) {
                                const float4 lm4 = *reinterpret_cast<const float4*>(&s.lm[jj][warp * RW + 4 * q]);
                                lm[4 * q + 0] = lm4.x;
                                lm[4 * q + 1] = lm4.y;
                                lm[4 * q + 2] = lm4.z;
                                lm[4 * q + 3] = lm4.w;
                            }
#pragma unroll
                            for (int r = 0; r < RW; ++r) {
                                const float p = lu + lm[r];
                                j1[r] = p > b1[r] ? j0 + jj : j1[r];
                                b2[r] = fmaxf(b2[r], fminf(b1[r], p));
                                b1[r] = fmaxf(b1[r], p);
                            }
                        }
                        __syncthreads();
                    }
                } else {
                    __syncthreads();
                }
#pragma unroll
                for (int r = 0; r < RW; ++r) {
                    const int i = i0 + warp * RW + r;
                    const bool valid = i < n && lane < cnt;
                    const bool zero = !a.exhaustive && !(b1[r] >= -1075.0f - kDelta);
                    const bool near_sub = b1[r] < -1022.0f + kDelta;
                    const bool fast = !a.exhaustive && !near_sub && b2[r] < b1[r] - kDelta;
                    if (valid && (zero || fast)) {
                        double L = 0.0;
                        int Cj = 0;
                        if (fast) {
                            L = U[(size_t)j1[r] * TF + lane] * M[(size_t)i * a.ld_mat + j1[r]];
                            Cj = j1[r];
                        }
                        Lv[(size_t)i * TF + lane] = L;
                        Cv[(size_t)i * TF + lane] = Cj;
                    } else if (valid) {
                        const int q = atomicAdd(&n_slow, 1);
                        slow_pair[q] = (i - i0) * TF + lane;
                        slow_best[q] = (a.exhaustive || near_sub) ? -INFINITY : b1[r];
                    }
                }
                __syncthreads();
                // near-ties and rows near the subnormal range: FP64 over the
                // candidate child states, one (row, family) per thread
                for (int q = tid; q < n_slow; q += NT) {
                    const int i = i0 + slow_pair[q] / TF, f = slow_pair[q] % TF;
                    const float best = slow_best[q];
                    const bool all = !(best > -INFINITY);
                    const float thr = best - kDelta;
                    const double* Mi = M + (size_t)i * a.ld_mat;
                    double mx = -1.0;
                    int arg = 0;
                    for (int j = 0; j < n; ++j) {
                        if (all || LU[(size_t)j * TF + f] + LMt[(size_t)j * n + i] >= thr) {
                            const double val = U[(size_t)j * TF + f] * Mi[j];
                            if (val > mx) {
                                mx = val;
                                arg = j;
                            }
                        }
                    }
                    Lv[(size_t)i * TF + f] = mx;
                    Cv[(size_t)i * TF + f] = arg;
                }
                __syncthreads();
            }
            __syncthreads();   // L_v complete; U / LU free for the next node
        }
        __syncthreads();

        // backtrack (:177-188) from the root's state: parents before
        // children (reverse post-order); leaves keep their observed count
        if (tid < cnt) {
            const int64_t fam = tile.first + tid;
            int32_t* out = a.state + ((size_t)k * a.F + fam) * P.n_nodes;
            out[P.root] = root_arg[tid];
            for (int ii = P.n_internal - 1; ii >= 0; --ii) {
                const int v = P.internal[ii];
                const int sv = out[v];
                for (int ci = P.cstart[ii]; ci < P.cstart[ii + 1]; ++ci) {
                    const int ch = P.child[ci];
                    const int lc = P.leaf_col[ch];
                    if (lc >= 0) out[ch] = a.counts[(size_t)fam * P.n_leaves + lc];
                    else out[ch] = Cbase[((size_t)node_ii[ch] * n + sv) * TF + tid];
                }
            }
            a.root_max[(size_t)k * a.F + fam] = root_val[tid];
            if (!(root_val[tid] > 0.0)) atomicAdd(a.n_failed, 1);
        }
        __syncthreads();
    }
}

// Node counts: gamma get_weighted_averages (sum_k p_k * state_k in category
// order, no contraction) rounded half away from zero by get_node_count
// (src/gamma_core.cpp:396-402); base: the state itself. Leaves report their
// observed count in both models (get_node_count's leaf branch).
__global__ void k_recon_counts(const int32_t* __restrict__ state, int64_t F, int n_nodes, int K,
                               const double* __restrict__ cat_probs, int gamma, const int32_t* __restrict__ leaf_col,
                               double* __restrict__ mean, int32_t* __restrict__ node_count) {
    const int64_t total = F * n_nodes;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        double val;
        if (gamma && leaf_col[e % n_nodes] < 0) {
            val = 0.0;
            for (int k = 0; k < K; ++k) val = __dadd_rn(val, __dmul_rn(cat_probs[k], (double)state[(size_t)k * total + e]));
        } else {
            val = (double)state[e];
        }
        if (mean) mean[e] = val;
        if (node_count) node_count[e] = (int32_t)round(val);
    }
}

// compute_viterbi_sum for one (family, non-root node) per thread: the
// matrix row of the parent's count, summed over child sizes m < S in
// order, ties counting half.
__global__ void k_branch_prob(BranchProbArgs a) {
    const int64_t total = a.F * a.n_nodes;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int v = (int)(e % a.n_nodes);
        const int p = a.parent[v];
        if (p < 0) {
            a.out[e] = NAN;
            continue;
        }
        const int64_t f = e / a.n_nodes;
        const int ps = a.node_count[f * a.n_nodes + p], cs = a.node_count[f * a.n_nodes + v];
        if (ps < 0 || cs < 0 || ps >= a.ld_mat || cs >= a.ld_mat) {
            a.out[e] = NAN;
            atomicAdd(a.n_bad, 1);
            continue;
        }
        const double* row = a.mats[v] + (size_t)ps * a.ld_mat;
        const double calc = row[cs];
        double result = 0.0;
        for (int m = 0; m < a.S; ++m) {
            const double pm = row[m];
            if (pm == calc) result = __dadd_rn(result, __dmul_rn(pm, 0.5));
            else if (pm < calc) result = __dadd_rn(result, pm);
        }
        a.out[e] = result;
    }
}

// Transposed log2 of the first n x n block of each matrix:
// out[j * n + i] = log2 M[i][j] (one conversion per entry and request
// instead of one per entry, tile and pass).
__global__ void k_log2_matrices(const double* const* __restrict__ src, float* const* __restrict__ dst, int n,
                                int ld) {
    const double* M = src[blockIdx.y];
    float* out = dst[blockIdx.y];
    const int64_t total = (int64_t)n * n;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(e / n), i = (int)(e % n);
        out[e] = flog2(M[(size_t)i * ld + j]);
    }
}

}  // namespace

cudaError_t launch_log2_matrices(const double* const* src, float* const* dst, int n_mats, int n, int ld,
                                 cudaStream_t s) {
    if (n_mats <= 0 || n <= 0) return cudaSuccess;
    const int bx = (int)std::min<int64_t>(((int64_t)n * n + 255) / 256, 64);
    k_log2_matrices<<<dim3(bx, n_mats), 256, 0, s>>>(src, dst, n, ld);
    return cudaGetLastError();
}

cudaError_t launch_pupko(const PupkoArgs& a, int n_ctas, cudaStream_t s) {
    if (a.n_tiles <= 0) return cudaSuccess;
    k_pupko<<<n_ctas, NT, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_recon_counts(const int32_t* state, int64_t F, int n_nodes, int K, const double* cat_probs,
                                int gamma, const int32_t* leaf_col, double* mean, int32_t* node_count, cudaStream_t s) {
    const int64_t total = F * n_nodes;
    if (total <= 0) return cudaSuccess;
    const int blocks = (int)std::min<int64_t>((total + 255) / 256, 4096);
    k_recon_counts<<<blocks, 256, 0, s>>>(state, F, n_nodes, K, cat_probs, gamma, leaf_col, mean, node_count);
    return cudaGetLastError();
}

cudaError_t launch_branch_prob(const BranchProbArgs& a, cudaStream_t s) {
    const int64_t total = a.F * a.n_nodes;
    if (total <= 0) return cudaSuccess;
    const int blocks = (int)std::min<int64_t>((total + 127) / 128, 8192);
    k_branch_prob<<<blocks, 128, 0, s>>>(a);
    return cudaGetLastError();
}

size_t pupko_scratch_doubles(const TreePlan& P, int S) {
    const size_t n = (size_t)S + 1;
    // L slots + u (doubles) + log2 u (floats, rounded up to doubles)
    return (size_t)P.n_slots * n * TF + n * TF + (n * TF + 1) / 2;
}

size_t pupko_c_entries(const TreePlan& P, int S) { return (size_t)P.n_internal * ((size_t)S + 1) * TF; }

}  // namespace cafe
