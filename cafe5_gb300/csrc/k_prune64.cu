// K3/K4 (FP64): Felsenstein pruning of family tiles up the species tree,
// with the root weighting fused into the last node.
//
// Replaces inference_prune (src/core.cpp:134-145) ->
// compute_node_probability (src/probability.cpp:175-234) ->
// lambda::calculate_child_factor (src/lambda.cpp:13-40) ->
// matrix::multiply (src/matrix_cache.cpp:32-58), and the per-family root
// reductions of base_model::infer_family_likelihoods
// (src/base_model.cpp:77-95) and gamma_model::prune
// (src/gamma_core.cpp:143-165).
//
// One CTA walks one tile of up to 32 families of one gamma category through
// the tree in post-order. Node vectors live in a per-CTA scratch area
// (L2-resident), state-major: V[state][family]. For every internal node the
// product over children is formed in descendant order starting from the
// first child's factor (= 1 * factor, as the reference does):
//   leaf child      factor[s] = M[s][n]              (a column gather; the
//                   reference's dense product with a one-hot vector adds only
//                   exact zeros), or the error-model row sum over n-1, n, n+1
//   internal child  factor[s] = sum_j M[s][j] L[j]   (an FP64 GEMM tile,
//                   64 states x 32 families, K staged through shared memory;
//                   each sum as four FMA chains over j = 0, 1, 2, 3 mod 4 in
//                   ascending j, combined as (s0 + s1) + (s2 + s3))
// Internal nodes use states 0..S; the root uses rows 1..R (root index j is
// root size j + 1, src/probability.cpp:206-219). With `scaled`, each node
// vector is renormalised per family by a power of two and the exponents are
// carried as integers, which keeps families finite where unscaled FP64
// underflows.
#include "common.cuh"

#include <math.h>

#include <algorithm>
#include <cstring>

namespace cafe {
namespace {

constexpr int TF = 32;      // families per tile
constexpr int RT = 64;      // GEMM rows per pass
constexpr int KT = 32;      // GEMM K chunk
constexpr int NT = 256;     // threads

__device__ __forceinline__ double* slot_ptr(double* base, int slot, int W) {
    return base + (size_t)slot * W * TF;
}

__global__ void __launch_bounds__(NT) k_prune64(Prune64Args a) {
    __shared__ double Ms[RT][KT + 1];
    __shared__ double Ls[KT][TF + 1];
    __shared__ int64_t fam[TF];
    __shared__ double red[NT / 32][TF];
    __shared__ int redi[NT / 32][TF];
    extern __shared__ int s_exp[];   // [n_slots][TF] power-of-two exponents

    const TreePlan& P = a.plan;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    double* base = a.scratch + (size_t)blockIdx.x * a.scratch_per_cta;
    const int W = a.W;

    const int n_tiles = a.n_tiles_dev ? *a.n_tiles_dev : a.n_tiles;
    for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
        const PruneTile tile = a.tiles[t];
        const int cnt = tile.count, S = tile.S, R = tile.R, k = tile.k;
        if (tid < TF) fam[tid] = tid < cnt ? a.perm[tile.first + tid] : -1;
        __syncthreads();
        const double* const* mats = a.mats + (size_t)k * P.n_nodes;

        for (int ii = 0; ii < P.n_internal; ++ii) {
            const int v = P.internal[ii];
            const bool is_root = (v == P.root);
            const int rows = is_root ? R : S + 1;
            const int row0 = is_root ? (tile.root_lo > 0 ? tile.root_lo : 1) : 0;
            const int vs = P.slot[v];
            double* dst = slot_ptr(base, vs, W);
            if (tid < TF) s_exp[vs * TF + tid] = 0;
            __syncthreads();
            for (int ci = P.cstart[ii]; ci < P.cstart[ii + 1]; ++ci) {
                const int ch = P.child[ci];
                const bool first = (ci == P.cstart[ii]);
                const double* __restrict__ M = mats[ch];
                const int ld = a.ld_mat;
                const int lc = P.leaf_col[ch];
                if (lc >= 0) {
                    // leaf: column gather (or the 3-term error-model sum)
                    for (int idx = tid; idx < rows * TF; idx += NT) {
                        const int r = idx / TF, i = idx % TF;
                        if (i >= cnt) continue;
                        const int s = row0 + r;
                        const int n = a.counts[(size_t)fam[i] * P.n_leaves + lc];
                        double val = 0.0;
                        const double* Mr = M + (size_t)s * ld;
                        if (a.err) {
                            const double* pr = a.err + (size_t)(n < a.err_rows ? n : a.err_rows - 1) * a.err_ndev;
                            const int off = n - (a.err_ndev - 1) / 2;
                            for (int d = 0; d < a.err_ndev; ++d) {
                                const int c = off + d;
                                if (c < 0 || c > S) continue;
                                val = fma(Mr[c], pr[d], val);
                            }
                        } else if (n >= 0 && n <= S) {
                            val = Mr[n];
                        }
                        double* o = dst + (size_t)r * TF + i;
                        *o = first ? val : *o * val;
                    }
                } else {
                    // internal child: dst[r][i] (*)= sum_j M[row0 + r][j] * L[j][i]
                    const double* L = slot_ptr(base, P.slot[ch], W);
                    const int ty = tid >> 4, tx = tid & 15;   // 16 x 16 threads: 4 rows x 2 families each
                    for (int r0 = 0; r0 < rows; r0 += RT) {
                        // four partial sums per output, over j = 0, 1, 2, 3 (mod 4)
                        double acc[4][2][4];
#pragma unroll
                        for (int q = 0; q < 4; ++q)
#pragma unroll
                            for (int p = 0; p < 2; ++p)
#pragma unroll
                                for (int m = 0; m < 4; ++m) acc[q][p][m] = 0.0;
                        for (int j0 = 0; j0 <= S; j0 += KT) {
                            for (int e = tid; e < RT * KT; e += NT) {
                                const int rr = e / KT, jj = e % KT;
                                const int r = r0 + rr, j = j0 + jj;
                                Ms[rr][jj] = (r < rows && j <= S) ? M[(size_t)(row0 + r) * ld + j] : 0.0;
                            }
                            for (int e = tid; e < KT * TF; e += NT) {
                                const int jj = e / TF, i = e % TF;
                                const int j = j0 + jj;
                                Ls[jj][i] = (j <= S && i < cnt) ? L[(size_t)j * TF + i] : 0.0;
                            }
                            __syncthreads();
#pragma unroll 2
                            for (int jj = 0; jj < KT; jj += 4) {
#pragma unroll
                                for (int m = 0; m < 4; ++m) {
                                    const double b0 = Ls[jj + m][tx * 2], b1 = Ls[jj + m][tx * 2 + 1];
#pragma unroll
                                    for (int q = 0; q < 4; ++q) {
                                        const double av = Ms[ty * 4 + q][jj + m];
                                        acc[q][0][m] = fma(av, b0, acc[q][0][m]);
                                        acc[q][1][m] = fma(av, b1, acc[q][1][m]);
                                    }
                                }
                            }
                            __syncthreads();
                        }
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const int r = r0 + ty * 4 + q;
                            if (r >= rows) continue;
#pragma unroll
                            for (int p = 0; p < 2; ++p) {
                                const int i = tx * 2 + p;
                                if (i >= cnt) continue;
                                const double sum = (acc[q][p][0] + acc[q][p][1]) + (acc[q][p][2] + acc[q][p][3]);
                                double* o = dst + (size_t)r * TF + i;
                                *o = first ? sum : *o * sum;
                            }
                        }
                    }
                    if (tid < TF) s_exp[vs * TF + tid] += s_exp[P.slot[ch] * TF + tid];
                }
                __syncthreads();
            }
            if (a.scaled) {
                // per-family max over states -> power-of-two renormalisation
                double mx = 0.0;
                for (int r = warp; r < rows; r += NT / 32) {
                    const double x = dst[(size_t)r * TF + lane];
                    mx = x > mx ? x : mx;
                }
                red[warp][lane] = mx;
                __syncthreads();
                if (warp == 0) {
                    double m = 0.0;
                    for (int w = 0; w < NT / 32; ++w) m = red[w][lane] > m ? red[w][lane] : m;
                    int e = 0;
                    if (m > 0.0 && isfinite(m)) frexp(m, &e);
                    redi[0][lane] = e;
                    s_exp[vs * TF + lane] += e;
                }
                __syncthreads();
                const int e = redi[0][lane];
                if (e != 0)
                    for (int r = warp; r < rows; r += NT / 32) {
                        double* o = dst + (size_t)r * TF + lane;
                        *o = scalbn(*o, -e);
                    }
                __syncthreads();
            }
        }

        // ---- root weighting (K4) ----
        const int rs = P.slot[P.root];
        const double* root = slot_ptr(base, rs, W);
        if (a.root_out) {
            // the root vectors themselves (p-values: compute_family_probabilities
            // and the observed families of compute_pvalues)
            for (int idx = tid; idx < R * TF; idx += NT) {
                const int j = idx / TF, ii = idx % TF;
                if (ii < cnt) a.root_out[(size_t)fam[ii] * a.root_ld + j] = root[(size_t)j * TF + ii];
            }
            __syncthreads();
            continue;
        }
        const int i = lane;
        const int64_t f = i < cnt ? fam[i] : -1;
        const int Rf = (f >= 0 && a.fam_R) ? a.fam_R[f] : R;
        if (a.model == 0) {
            double best = -INFINITY;
            bool any = false;
            for (int j = warp; j < Rf; j += NT / 32) {
                const double eq = j < a.n_prior ? a.prior[j] : 0.0;
                const double vv = log(root[(size_t)j * TF + i]) + log(eq);
                if (!any || vv > best) best = vv;
                any = true;
            }
            red[warp][lane] = any ? best : NAN;
            __syncthreads();
            if (warp == 0 && f >= 0 && (!a.term_mask || a.term_mask[(size_t)f * a.K + k])) {
                double b = -INFINITY;
                bool got = false;
                for (int w = 0; w < NT / 32; ++w) {
                    const double x = red[w][lane];
                    if (isnan(x)) continue;
                    if (!got || x > b) b = x;
                    got = true;
                }
                a.out[(size_t)f * a.K + k] = b + (double)s_exp[rs * TF + i] * 0.69314718055994530942;
            }
        } else {
            double mx = 0.0;
            int nz = 0;
            for (int j = warp; j < Rf; j += NT / 32) {
                const double x = root[(size_t)j * TF + i];
                const double eq = j < a.n_prior ? a.prior[j] : 0.0;
                const double vv = x * eq;
                mx = vv > mx ? vv : mx;
                nz |= (x != 0.0);
            }
            red[warp][lane] = mx;
            redi[warp][lane] = nz;
            __syncthreads();
            if (warp == 0 && f >= 0 && (!a.term_mask || a.term_mask[(size_t)f * a.K + k])) {
                double m = 0.0;
                int z = 0;
                for (int w = 0; w < NT / 32; ++w) {
                    m = red[w][lane] > m ? red[w][lane] : m;
                    z |= redi[w][lane];
                }
                const double cat = m * a.cat_probs[k];
                double o;
                if (!z) o = a.scaled ? NAN : -1.0;   // all-zero root vector: family fails
                else if (a.scaled) o = log(cat) + (double)s_exp[rs * TF + i] * 0.69314718055994530942;
                else o = cat;
                a.out[(size_t)f * a.K + k] = o;
            }
        }
        __syncthreads();
    }
}

// ---- the same walk for sparse bins: one family of one category per cluster ----
//
// A bin with few families leaves most SMs idle under 32-family tiles (one CTA
// walks the whole tree per tile, and FP64 issue is the bound). Here a
// thread-block cluster of CL CTAs walks one family: every CTA keeps a full
// copy of the family's node vectors in shared memory and forms its own slice
// of each node's rows (four lanes per row over column chunks of the matrix
// staged in shared memory). After each node the CTAs exchange their slice
// maxima (the power-of-two rescale, identical in every CTA) and then their
// rows through distributed shared memory, each exchange closed by a cluster
// barrier. Factors, products (the same four FMA chains per row), rescale
// and root weighting are those of k_prune64, so a family gets the same bits
// from either kernel; the walk's latency is spread over up to 8 SMs.
constexpr int kClThreads = 256;
constexpr int kClWarps = kClThreads / 32;
constexpr int kClRows = kClThreads / 4;           // rows per pass (four lanes per row)
constexpr int kClK = 32;                          // matrix columns staged per step
constexpr int kClStage = kClRows * kClK / kClThreads;   // staged values per thread
constexpr int kClMax = 8;

__device__ __forceinline__ unsigned cl_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cl_size() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cl_id() {
    unsigned r;
    asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cl_count() {
    unsigned r;
    asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
    return r;
}
// every thread of every CTA of the cluster; orders shared-memory stores
// (local and remote) before the loads that follow it
__device__ __forceinline__ void cl_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// store v at CTA `rank`'s copy of the shared-memory location p
__device__ __forceinline__ void st_peer(double* p, unsigned rank, double v) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    unsigned ra;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
    asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(ra), "d"(v) : "memory");
}

__global__ void __launch_bounds__(kClThreads) k_prune64_cl(Prune64Args a) {
    extern __shared__ double s_vec[];   // [n_slots][W] node vectors of the family (full copy)
    int* s_exp = reinterpret_cast<int*>(s_vec + (size_t)a.plan.n_slots * a.W);   // [n_slots]
    __shared__ double Ms[kClRows][kClK + 4];   // matrix rows of this pass, one column chunk
    __shared__ double s_part[kClMax];   // slice maxima, one per CTA of the cluster
    __shared__ double s_red[kClWarps];
    __shared__ int s_redi[kClWarps];

    const TreePlan& P = a.plan;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const unsigned rank = cl_rank(), CL = cl_size();
    const int W = a.W, ld = a.ld_mat;
    cl_sync();   // every CTA of the cluster runs before the first remote store

    for (int t = (int)cl_id(); t < a.n_tiles; t += (int)cl_count()) {
        const PruneTile tile = a.tiles[t];
        const int S = tile.S, R = tile.R, k = tile.k;
        const int64_t f = a.perm[tile.first];
        const double* const* mats = a.mats + (size_t)k * P.n_nodes;

        for (int ii = 0; ii < P.n_internal; ++ii) {
            const int v = P.internal[ii];
            const bool is_root = (v == P.root);
            const int rows = is_root ? R : S + 1;
            const int row0 = is_root ? (tile.root_lo > 0 ? tile.root_lo : 1) : 0;
            const int chunk = (rows + (int)CL - 1) / (int)CL;
            const int r_lo = min(rows, (int)rank * chunk), r_hi = min(rows, r_lo + chunk);
            const int vs = P.slot[v];
            double* dst = s_vec + (size_t)vs * W;
            int e_sum = 0;
            for (int ci = P.cstart[ii]; ci < P.cstart[ii + 1]; ++ci) {
                const int ch = P.child[ci];
                const bool first = (ci == P.cstart[ii]);
                const double* __restrict__ M = mats[ch];
                const int lc = P.leaf_col[ch];
                if (lc >= 0) {
                    const int n = a.counts[(size_t)f * P.n_leaves + lc];
                    for (int r = r_lo + tid; r < r_hi; r += kClThreads) {
                        const double* Mr = M + (size_t)(row0 + r) * ld;
                        double val = 0.0;
                        if (a.err) {
                            const double* pr = a.err + (size_t)(n < a.err_rows ? n : a.err_rows - 1) * a.err_ndev;
                            const int off = n - (a.err_ndev - 1) / 2;
                            for (int d = 0; d < a.err_ndev; ++d) {
                                const int c = off + d;
                                if (c < 0 || c > S) continue;
                                val = fma(Mr[c], pr[d], val);
                            }
                        } else if (n >= 0 && n <= S) {
                            val = Mr[n];
                        }
                        dst[r] = first ? val : dst[r] * val;
                    }
                } else {
                    // dst[r] (*)= sum_j M[row0 + r][j] * L[j]: four lanes per row,
                    // lane q the FMA chain over j = q (mod 4) in ascending j, then
                    // (s0 + s1) + (s2 + s3), the sums of k_prune64 bit for bit.
                    // Matrix chunks are staged coalesced, the next one loaded
                    // into registers while the current one is used.
                    const double* L = s_vec + (size_t)P.slot[ch] * W;
                    const int rp = tid >> 2, q = tid & 3;
                    for (int rb = r_lo; rb < r_hi; rb += kClRows) {
                        const int nr = min(kClRows, r_hi - rb);
                        double pre[kClStage];
                        auto load_chunk = [&](int j0) {
#pragma unroll
                            for (int i = 0; i < kClStage; ++i) {
                                const int rr = warp + kClWarps * i, j = j0 + lane;
                                pre[i] = (rr < nr && j <= S) ? M[(size_t)(row0 + rb + rr) * ld + j] : 0.0;
                            }
                        };
                        load_chunk(0);
                        double acc = 0.0;
                        for (int j0 = 0; j0 <= S; j0 += kClK) {
#pragma unroll
                            for (int i = 0; i < kClStage; ++i) Ms[warp + kClWarps * i][lane] = pre[i];
                            __syncthreads();
                            if (j0 + kClK <= S) load_chunk(j0 + kClK);
#pragma unroll
                            for (int i = 0; i < kClK / 4; ++i) {
                                const int jj = q + 4 * i, j = j0 + jj;
                                const double lv = j <= S ? L[j] : 0.0;
                                acc = fma(Ms[rp][jj], lv, acc);
                            }
                            __syncthreads();
                        }
                        acc += __shfl_xor_sync(0xffffffffu, acc, 1);
                        acc += __shfl_xor_sync(0xffffffffu, acc, 2);
                        if (q == 0 && rp < nr) dst[rb + rp] = first ? acc : dst[rb + rp] * acc;
                    }
                    e_sum += s_exp[P.slot[ch]];
                }
                __syncthreads();
            }
            int e = 0;
            if (a.scaled) {
                // the node's maximum over all rows -> one power-of-two scale
                double mx = 0.0;
                for (int r = r_lo + tid; r < r_hi; r += kClThreads) {
                    const double x = dst[r];
                    mx = x > mx ? x : mx;
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const double y = __shfl_xor_sync(0xffffffffu, mx, o);
                    mx = y > mx ? y : mx;
                }
                if (lane == 0) s_red[warp] = mx;
                __syncthreads();
                if (tid < (int)CL) {
                    double m = 0.0;
                    for (int w = 0; w < kClWarps; ++w) m = s_red[w] > m ? s_red[w] : m;
                    st_peer(&s_part[rank], (unsigned)tid, m);
                }
                cl_sync();
                double m = 0.0;
                for (unsigned q = 0; q < CL; ++q) m = s_part[q] > m ? s_part[q] : m;
                if (m > 0.0 && isfinite(m)) frexp(m, &e);
            }
            // rescale this CTA's rows and send them to every other CTA
            for (int r = r_lo + tid; r < r_hi; r += kClThreads) {
                double x = dst[r];
                if (e != 0) {
                    x = scalbn(x, -e);
                    dst[r] = x;
                }
                for (unsigned q = 0; q < CL; ++q)
                    if (q != rank) st_peer(dst + r, q, x);
            }
            if (tid == 0) s_exp[vs] = e_sum + e;
            cl_sync();
        }

        // ---- root weighting (K4), by the cluster's first CTA ----
        const int rs = P.slot[P.root];
        const double* root = s_vec + (size_t)rs * W;
        if (rank == 0) {
            if (a.root_out) {
                for (int j = tid; j < R; j += kClThreads) a.root_out[(size_t)f * a.root_ld + j] = root[j];
            } else {
                const int Rf = a.fam_R ? a.fam_R[f] : R;
                if (a.model == 0) {
                    double best = -INFINITY;
                    for (int j = tid; j < Rf; j += kClThreads) {
                        const double eq = j < a.n_prior ? a.prior[j] : 0.0;
                        const double vv = log(root[j]) + log(eq);
                        best = vv > best ? vv : best;
                    }
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        const double y = __shfl_xor_sync(0xffffffffu, best, o);
                        best = y > best ? y : best;
                    }
                    if (lane == 0) s_red[warp] = best;
                    __syncthreads();
                    if (tid == 0) {
                        double b = -INFINITY;
                        for (int w = 0; w < kClWarps; ++w) b = s_red[w] > b ? s_red[w] : b;
                        a.out[(size_t)f * a.K + k] = b + (double)s_exp[rs] * 0.69314718055994530942;
                    }
                } else {
                    double mx = 0.0;
                    int nz = 0;
                    for (int j = tid; j < Rf; j += kClThreads) {
                        const double x = root[j];
                        const double eq = j < a.n_prior ? a.prior[j] : 0.0;
                        const double vv = x * eq;
                        mx = vv > mx ? vv : mx;
                        nz |= (x != 0.0);
                    }
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        const double y = __shfl_xor_sync(0xffffffffu, mx, o);
                        mx = y > mx ? y : mx;
                        nz |= __shfl_xor_sync(0xffffffffu, nz, o);
                    }
                    if (lane == 0) {
                        s_red[warp] = mx;
                        s_redi[warp] = nz;
                    }
                    __syncthreads();
                    if (tid == 0) {
                        double m = 0.0;
                        int z = 0;
                        for (int w = 0; w < kClWarps; ++w) {
                            m = s_red[w] > m ? s_red[w] : m;
                            z |= s_redi[w];
                        }
                        const double cat = m * a.cat_probs[k];
                        double o;
                        if (!z) o = a.scaled ? NAN : -1.0;   // all-zero root vector: family fails
                        else if (a.scaled) o = log(cat) + (double)s_exp[rs] * 0.69314718055994530942;
                        else o = cat;
                        a.out[(size_t)f * a.K + k] = o;
                    }
                }
            }
        }
        cl_sync();   // the root is read before the next family's rows arrive
    }
}

// Per-family lnL from category values (many blocks), then -sum lnL with a
// deterministic compensated reduction: Neumaier sums per thread, combined
// in a fixed order per block and then across blocks.
__device__ __forceinline__ void neumaier_add(double& sum, double& comp, double x) {
    const double tt = sum + x;
    if (fabs(sum) >= fabs(x)) comp += (sum - tt) + x;
    else comp += (x - tt) + sum;
    sum = tt;
}

constexpr int kFinishThreads = 64;

// Pairwise tree over the block's (sum, compensation, fail, -inf) partials in
// a fixed order: log2(N) dependent steps instead of N (FP64 latency is long
// on this part). Deterministic for a given N. Leaves the result in slot 0.
template <int N>
__device__ __forceinline__ void block_combine(double* ssum, double* scomp, int* sfail, int* sinf) {
    __syncthreads();
#pragma unroll
    for (int h = N / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            const int o = threadIdx.x + h;
            double s = ssum[threadIdx.x], c = scomp[threadIdx.x] + scomp[o];
            neumaier_add(s, c, ssum[o]);
            ssum[threadIdx.x] = s;
            scomp[threadIdx.x] = c;
            sfail[threadIdx.x] += sfail[o];
            sinf[threadIdx.x] += sinf[o];
        }
        __syncthreads();
    }
}

// Candidate b (blockIdx.y here, blockIdx.x in k_finish_total) reads
// category k of family row r at cat[r * K * n_cand + b * K + k] and writes
// family_lnl[b * F + f], total[b], n_failed[b].
__global__ void __launch_bounds__(kFinishThreads) k_finish_fam(FinishArgs a) {
    __shared__ double ssum[kFinishThreads], scomp[kFinishThreads];
    __shared__ int sfail[kFinishThreads], sinf[kFinishThreads];
    const int b = blockIdx.y;
    const size_t stride = (size_t)a.K * a.n_cand;
    const double* cat = a.cat + (size_t)b * a.K;
    double* fam_out = a.family_lnl ? a.family_lnl + (size_t)b * a.F : nullptr;
    double sum = 0.0, comp = 0.0;
    int fail = 0, ninf = 0;   // ninf: families with lnL = -inf (log of an underflowed 0)
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < a.F; f += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = a.ref ? a.ref[f] : f;
        const double* c_r = cat + (size_t)r * stride;
        double lnl;
        if (a.model == 0) {
            lnl = c_r[0];
        } else if (!a.scaled) {
            // gamma_core.cpp:196-207: family likelihood = sum_k category terms
            double lh = 0.0;
            bool bad = false;
            for (int k = 0; k < a.K; ++k) {
                const double c = c_r[k];
                if (c < 0) bad = true;
                lh += c;
            }
            lnl = bad ? NAN : log(lh);
            fail += bad;
        } else {
            double mx = -INFINITY;
            bool bad = false;
            for (int k = 0; k < a.K; ++k) {
                const double c = c_r[k];
                if (isnan(c)) bad = true;
                else mx = c > mx ? c : mx;
            }
            double acc = 0.0;
            if (!bad && mx > -INFINITY)
                for (int k = 0; k < a.K; ++k) acc += exp(c_r[k] - mx);
            lnl = bad ? NAN : (mx > -INFINITY ? mx + log(acc) : -INFINITY);
            fail += bad;
        }
        if (fam_out) fam_out[f] = lnl;
        if (isinf(lnl)) ninf++;
        else if (!isnan(lnl)) neumaier_add(sum, comp, lnl);
    }
    ssum[threadIdx.x] = sum;
    scomp[threadIdx.x] = comp;
    sfail[threadIdx.x] = fail;
    sinf[threadIdx.x] = ninf;
    block_combine<kFinishThreads>(ssum, scomp, sfail, sinf);
    if (threadIdx.x == 0) {
        const size_t p = (size_t)b * gridDim.x + blockIdx.x;
        a.part_sum[2 * p] = ssum[0];
        a.part_sum[2 * p + 1] = scomp[0];
        a.part_cnt[2 * p] = sfail[0];
        a.part_cnt[2 * p + 1] = sinf[0];
    }
}

__global__ void __launch_bounds__(256) k_finish_total(FinishArgs a, int n_parts) {
    // fixed partition (thread i takes parts i, i + 256, ...), then a fixed
    // sequential combine: deterministic for a given family count
    __shared__ double ssum[256], scomp[256];
    __shared__ int sfail[256], sinf[256];
    const int b = blockIdx.x;
    const double* ps = a.part_sum + (size_t)2 * b * n_parts;
    const int32_t* pc = a.part_cnt + (size_t)2 * b * n_parts;
    double s = 0.0, c = 0.0;
    int fl = 0, ni = 0;
    for (int i = threadIdx.x; i < n_parts; i += blockDim.x) {
        neumaier_add(s, c, ps[2 * i]);
        c += ps[2 * i + 1];
        fl += pc[2 * i];
        ni += pc[2 * i + 1];
    }
    ssum[threadIdx.x] = s;
    scomp[threadIdx.x] = c;
    sfail[threadIdx.x] = fl;
    sinf[threadIdx.x] = ni;
    block_combine<256>(ssum, scomp, sfail, sinf);
    if (threadIdx.x != 0) return;
    s = ssum[0];
    c = scomp[0];
    fl = sfail[0];
    ni = sinf[0];
    a.n_failed[b] = fl;
    // -sum lnL: +inf on gamma failure or when any family's lnL is -inf;
    // NaN if the tensor-core pass reported a time-out
    double t = (fl || ni) ? INFINITY : -(s + c);
    if (a.status && *a.status) t = NAN;
    if (a.total) a.total[b] = t;
}

__global__ void k_fill(double* p, int64_t n, double v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}
__global__ void k_fill_i32(int32_t* p, int64_t n, int32_t v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

}  // namespace

cudaError_t launch_fill(double* p, int64_t n, double v, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, 4096);
    k_fill<<<blocks, 256, 0, s>>>(p, n, v);
    return cudaGetLastError();
}

cudaError_t launch_fill_i32(int32_t* p, int64_t n, int32_t v, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, 4096);
    k_fill_i32<<<blocks, 256, 0, s>>>(p, n, v);
    return cudaGetLastError();
}

cudaError_t launch_prune64(const Prune64Args& a, int n_ctas, cudaStream_t s) {
    if (a.n_tiles <= 0 && !a.n_tiles_dev) return cudaSuccess;
    size_t smem = sizeof(int) * (size_t)a.plan.n_slots * TF;
    k_prune64<<<n_ctas, NT, smem, s>>>(a);
    return cudaGetLastError();
}

size_t prune64_cluster_smem(int n_slots, int W) {
    return (size_t)n_slots * W * sizeof(double) + (size_t)n_slots * sizeof(int);
}

// (the kernel also holds 19 KB of static shared memory; the opt-in limit is 227 KB)
size_t prune64_cluster_max_smem() { return 160 * 1024; }

cudaError_t prune64_cluster_init() {
    return cudaFuncSetAttribute(k_prune64_cl, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)prune64_cluster_max_smem());
}

cudaError_t launch_prune64_cluster(const Prune64Args& a, int cl, int n_clusters, cudaStream_t s) {
    if (a.n_tiles <= 0) return cudaSuccess;
    if (cl < 1 || cl > kClMax || n_clusters < 1) return cudaErrorInvalidValue;
    const size_t smem = prune64_cluster_smem(a.plan.n_slots, a.W);
    if (smem > prune64_cluster_max_smem()) return cudaErrorInvalidValue;
    cudaLaunchConfig_t cfg;
    std::memset(&cfg, 0, sizeof cfg);
    cfg.gridDim = dim3((unsigned)(n_clusters * cl), 1, 1);
    cfg.blockDim = dim3(kClThreads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)cl;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_prune64_cl, a);
}

int finish_parts(int64_t F) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((F + kFinishThreads - 1) / kFinishThreads, 2048));
}

cudaError_t launch_finish(const FinishArgs& a, cudaStream_t s) {
    const int parts = finish_parts(a.F);
    const int nc = a.n_cand > 0 ? a.n_cand : 1;
    FinishArgs b = a;
    b.n_cand = nc;
    k_finish_fam<<<dim3(parts, nc), kFinishThreads, 0, s>>>(b);
    k_finish_total<<<nc, 256, 0, s>>>(b, parts);
    return cudaGetLastError();
}

}  // namespace cafe
