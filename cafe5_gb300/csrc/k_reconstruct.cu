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
// about two such products per clock and SM, so k_pupko finds the argmax in
// two passes instead:
//   pass 1  p_j = log2 u[j] + log2 M[i][j] in FP32 (FP32 pipes, ~60x the
//           FP64 rate); best = max_j p_j
//   pass 2  the exact FP64 product u[j] * M[i][j] only for the j with
//           p_j >= best - delta, scanned in ascending j with the
//           reference's strict '>' rule
// Every log2 carries an absolute error <= 6.3e-5 (FP32 rounding of a value
// of magnitude <= 1075 plus log2f's 1 ulp) and the sum <= 1.3e-4 more, so a
// j whose exact product equals the FP64 maximum has p_j >= best - 5e-4;
// delta = 2^-8 leaves an 8x margin. When the maximum cannot be a normal
// FP64 number the filter is not used: best below -1075 - delta means every
// product rounds to 0 (the reference then returns L = 0, C = 0), and best
// within delta of the subnormal range makes the row scan every j exactly.
// `exhaustive` turns the filter off everywhere (the plain FP64 scan).
#include "common.cuh"

#include <math.h>

#include <algorithm>

namespace cafe {
namespace {

constexpr int TF = 32;       // families per tile (one per lane)
constexpr int NT = 256;      // threads: 8 warps
constexpr int RW = 4;        // parent states per warp and block
constexpr int RB = 8 * RW;   // parent states per block
constexpr int JC = 32;       // child states per staged chunk
constexpr float kDelta = 0.00390625f;   // 2^-8, in log2 units

// log2 of x >= 0 in FP32 (-inf for 0): exponent exact, mantissa through
// log2f; absolute error <= 2^-14 + 1 ulp of log2f for |result| < 2048.
__device__ __forceinline__ float flog2(double x) {
    if (!(x > 0.0)) return -INFINITY;
    int e = 0;
    const double m = frexp(x, &e);   // x = m * 2^e, m in [0.5, 1), exact
    return (float)(e - 1) + log2f((float)(m * 2.0));
}

struct Staging {
    double m[RB][JC + 1];   // M tile: parent states i0.., child states j0..
    double u[JC][TF];       // u chunk
    float lm[JC][RB];       // log2 of the M tile, child-state major
    float lu[JC][TF];
};

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

// Stage the M tile (rows i0.., columns j0..) and the u / log2 u chunk.
__device__ __forceinline__ void stage(Staging& s, const double* M, int ld, int n, int i0, int j0, const double* U,
                                      const float* LU, bool with_u) {
    const int tid = threadIdx.x;
    for (int e = tid; e < RB * JC; e += NT) {
        const int r = e / JC, jj = e % JC;
        const int i = i0 + r, j = j0 + jj;
        s.m[r][jj] = (i < n && j < n) ? M[(size_t)i * ld + j] : 0.0;
    }
    for (int e = tid; e < JC * TF; e += NT) {
        const int jj = e / TF, f = e % TF;
        const int j = j0 + jj;
        s.lu[jj][f] = j < n ? LU[(size_t)j * TF + f] : -INFINITY;
        if (with_u) s.u[jj][f] = j < n ? U[(size_t)j * TF + f] : 0.0;
    }
    __syncthreads();
    for (int e = tid; e < RB * JC; e += NT) {
        const int r = e % RB, jj = e / RB;
        s.lm[jj][r] = flog2(s.m[r][jj]);
    }
    __syncthreads();
}

__global__ void __launch_bounds__(NT) k_pupko(PupkoArgs a) {
    __shared__ __align__(16) Staging s;
    __shared__ int node_ii[kMaxNodes];
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
            for (int i0 = 0; i0 < n; i0 += RB) {
                float best[RW];
#pragma unroll
                for (int r = 0; r < RW; ++r) best[r] = -INFINITY;
                if (!a.exhaustive) {
                    for (int j0 = 0; j0 < n; j0 += JC) {
                        stage(s, M, a.ld_mat, n, i0, j0, U, LU, false);
                        const int jn = min(JC, n - j0);
                        for (int jj = 0; jj < jn; ++jj) {
                            const float lu = s.lu[jj][lane];
                            const float4 lm = *reinterpret_cast<const float4*>(&s.lm[jj][warp * RW]);
                            best[0] = fmaxf(best[0], lu + lm.x);
                            best[1] = fmaxf(best[1], lu + lm.y);
                            best[2] = fmaxf(best[2], lu + lm.z);
                            best[3] = fmaxf(best[3], lu + lm.w);
                        }
                        __syncthreads();
                    }
                }
                bool zero[RW], exh[RW];
                float thr[RW];
                double mx[RW];
                int arg[RW];
                bool need = false;
#pragma unroll
                for (int r = 0; r < RW; ++r) {
                    const int i = i0 + warp * RW + r;
                    zero[r] = !a.exhaustive && !(best[r] >= -1075.0f - kDelta);
                    exh[r] = a.exhaustive || best[r] < -1022.0f + kDelta;
                    thr[r] = best[r] - kDelta;
                    mx[r] = -1.0;
                    arg[r] = 0;
                    need |= (i < n && lane < cnt && !zero[r]);
                }
                if (__syncthreads_or(need)) {
                    for (int j0 = 0; j0 < n; j0 += JC) {
                        stage(s, M, a.ld_mat, n, i0, j0, U, LU, true);
                        const int jn = min(JC, n - j0);
                        for (int jj = 0; jj < jn; ++jj) {
                            const float lu = s.lu[jj][lane];
                            const float4 lm4 = *reinterpret_cast<const float4*>(&s.lm[jj][warp * RW]);
                            const float lm[RW] = {lm4.x, lm4.y, lm4.z, lm4.w};
#pragma unroll
                            for (int r = 0; r < RW; ++r) {
                                if (!zero[r] && (exh[r] || lu + lm[r] >= thr[r])) {
                                    const double val = s.u[jj][lane] * s.m[warp * RW + r][jj];
                                    if (val > mx[r]) {
                                        mx[r] = val;
                                        arg[r] = j0 + jj;
                                    }
                                }
                            }
                        }
                        __syncthreads();
                    }
                }
#pragma unroll
                for (int r = 0; r < RW; ++r) {
                    const int i = i0 + warp * RW + r;
                    if (i < n) {
                        Lv[(size_t)i * TF + lane] = zero[r] ? 0.0 : mx[r];
                        Cv[(size_t)i * TF + lane] = zero[r] ? 0 : arg[r];
                    }
                }
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

}  // namespace

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
