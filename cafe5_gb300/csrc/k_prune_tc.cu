// K3/K4 on the tensor cores: split-TF32 (TF32x3) pruning of 128-family tiles
// with FP32 accumulation in TMEM and integer-exponent rescaling.
//
// Same algorithm as k_prune64 (inference_prune, src/core.cpp:134-145 ->
// compute_node_probability, src/probability.cpp:175-234 -> matrix::multiply,
// src/matrix_cache.cpp:32-58; root weighting src/gamma_core.cpp:143-165),
// mapped onto tcgen05:
//
//  * One CTA (4 warps) owns a tile of 128 families of one gamma category and
//    one S-bin of width W (<= 256) and walks the tree in post-order.
//  * Internal child c: D[f][s] = sum_j L_c[f][j] M_c[s][j] is one
//    M=128 x N=W x K=W GEMM: A = node vectors (128 families x W states,
//    K-major), B = the transition matrix (W x W, K-major: row s, column j).
//    Operands are FP32 pairs hi + lo, each rounded to TF32, and
//    D = A_hi B_hi + A_hi B_lo + A_lo B_hi (the lo*lo term is below the
//    TF32x3 error). Tiles of 32 K-columns (one 128-byte swizzle row) are
//    staged by TMA into two shared-memory stages; one thread issues TMA and
//    tcgen05.mma; the accumulators of up to two children sit side by side in
//    TMEM.
//  * Leaf child: its factor is the matrix column of the observed count,
//    read from an FP32 column-normalised transposed copy (with the column's
//    power-of-two exponent), or the three-column error-model sum.
//  * Epilogue (thread f owns family f = TMEM lane f): the product over
//    children is rescaled by the largest per-state sum of the factors'
//    binary exponents, so the product's maximum is ~1 and nothing
//    underflows unless the factors are >2^250 apart; the exponent goes into
//    the family's integer exponent. The node vector is stored as TF32 hi/lo
//    for the parent's GEMM. At the root the vector is weighted by the prior
//    in FP64 (root index j = state j + 1) and the category term's natural
//    log is written.
//  * A family whose factors are too far apart, or whose root vector is all
//    zero, is flagged; the host recomputes flagged families in FP64.
//
// Every mbarrier wait is bounded; on time-out the kernel records a status,
// waits (bounded) for its own copies, frees TMEM and returns.
#include "common.cuh"
#include "tc_ptx.cuh"

#include <math.h>

namespace cafe {
namespace {

constexpr int TM = 128;   // families per tile = MMA M = TMEM lanes
constexpr int KC = 32;    // K per stage: 32 fp32 = one 128-byte swizzle row
constexpr int NTHREADS = 128;

__host__ __device__ inline size_t stage_bytes(int Wm) { return (size_t)(2 * TM + 2 * Wm) * KC * sizeof(float); }

__device__ __forceinline__ int bexp(float y) {
    // binary exponent e with y = m 2^e, m in [0.5, 1); zero -> very negative
    const uint32_t b = __float_as_uint(y);
    const int be = (int)((b >> 23) & 0xFF);
    if (!(y > 0.0f)) return -100000;
    return be ? be - 126 : -149;
}
__device__ __forceinline__ float pow2f(int a) {
    a = a < -126 ? -126 : (a > 127 ? 127 : a);
    return __uint_as_float((uint32_t)(a + 127) << 23);
}

struct ChildInfo {
    int node;
    int leaf_col;   // >= 0: leaf
    int mat;
    int tcol;       // TMEM column base for internal children
};

__global__ void __launch_bounds__(NTHREADS, 1)
    k_prune_tc(const __grid_constant__ CUtensorMap map_mhi, const __grid_constant__ CUtensorMap map_mlo,
               const __grid_constant__ CUtensorMap map_vhi, const __grid_constant__ CUtensorMap map_vlo,
               const PruneTcArgs a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    __shared__ __align__(8) uint64_t bar_full[2], bar_empty[2], bar_done;
    __shared__ uint32_t tmem_sh;
    __shared__ int abort_sh;
    __shared__ ChildInfo ch_sh[8];

    const int tid = threadIdx.x, warp = tid >> 5;
    const int Wm = a.Wm;
    const TreePlan& P = a.plan;
    const size_t sbytes = stage_bytes(Wm);
    int* Esh = reinterpret_cast<int*>(smem + 2 * sbytes);   // [n_slots][TM]

    if (warp == 0) tc::tmem_alloc(&tmem_sh, (uint32_t)a.tmem_cols);
    if (tid == 0) {
        tc::mbar_init(&bar_full[0], 1);
        tc::mbar_init(&bar_full[1], 1);
        tc::mbar_init(&bar_empty[0], 1);
        tc::mbar_init(&bar_empty[1], 1);
        tc::mbar_init(&bar_done, 1);
        tc::mbar_init_fence();
        abort_sh = 0;
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmem_sh;
    const uint32_t lane_base = (uint32_t)(32 * warp) << 16;

    uint32_t g = 0;          // chunks issued so far (thread 0)
    uint32_t dn = 0;         // completions of bar_done observed (all threads)
    int last_full = -1;      // stage of the last issued TMA (thread 0)
    uint32_t last_full_parity = 0;
    const int64_t vrow_cta = (int64_t)blockIdx.x * a.n_slots * TM;

    for (int t = blockIdx.x; t < a.n_tiles; t += gridDim.x) {
        const PruneTile tile = a.tiles[t];
        const int cnt = tile.count, k = tile.k, S = tile.S, W = tile.S + 1;
        const int64_t fam = tid < cnt ? a.perm[tile.first + tid] : -1;
        const int Rf = (fam >= 0 && a.fam_R) ? a.fam_R[fam] : tile.R;
        const int32_t* mi = a.mat_index + (size_t)k * P.n_nodes;
        const uint32_t idesc = tc::idesc_tf32(TM, W);
        bool flag = false;

        for (int ii = 0; ii < P.n_internal; ++ii) {
            const int v = P.internal[ii];
            const bool is_root = (v == P.root);
            const int vs = P.slot[v];
            const int c0 = P.cstart[ii], c1 = P.cstart[ii + 1];
            const int nch = c1 - c0;
            if (tid == 0) {
                int nint = 0;
                for (int c = c0; c < c1; ++c) {
                    ChildInfo ci;
                    ci.node = P.child[c];
                    ci.leaf_col = P.leaf_col[ci.node];
                    ci.mat = mi[ci.node];
                    ci.tcol = ci.leaf_col < 0 ? (nint++) * W : -1;
                    ch_sh[c - c0] = ci;
                }
            }
            __syncthreads();
            int nint = 0;
            for (int c = 0; c < nch; ++c) nint += ch_sh[c].leaf_col < 0;

            // ---------------- GEMMs of the internal children ----------------
            if (nint > 0) {
                if (tid == 0 && !abort_sh) {
                    const int kpc = W / KC;             // K chunks per child
                    const int total = nint * kpc;
                    auto child_of = [&](int j) -> const ChildInfo& {
                        int seen = 0;
                        for (int c = 0; c < nch; ++c)
                            if (ch_sh[c].leaf_col < 0) {
                                if (seen == j) return ch_sh[c];
                                ++seen;
                            }
                        return ch_sh[0];
                    };
                    auto issue = [&](int i) -> bool {
                        const uint32_t ci = g + (uint32_t)i;
                        const int st = ci & 1;
                        const uint32_t u = ci >> 1;
                        if (u >= 1 && !tc::mbar_wait(&bar_empty[st], (u - 1) & 1)) return false;
                        const ChildInfo& c = child_of(i / kpc);
                        const int kc = i % kpc;
                        uint8_t* base = smem + st * sbytes;
                        float* Ahi = reinterpret_cast<float*>(base);
                        float* Alo = Ahi + TM * KC;
                        float* Bhi = Alo + TM * KC;
                        float* Blo = Bhi + Wm * KC;
                        tc::mbar_expect_tx(&bar_full[st], (uint32_t)((2 * TM + 2 * W) * KC * sizeof(float)));
                        const int vrow = (int)(vrow_cta + (int64_t)P.slot[c.node] * TM);
                        for (int r = 0; r < TM / 32; ++r) {
                            tc::tma_load_2d(Ahi + r * 32 * KC, &map_vhi, kc * KC, vrow + 32 * r, &bar_full[st]);
                            tc::tma_load_2d(Alo + r * 32 * KC, &map_vlo, kc * KC, vrow + 32 * r, &bar_full[st]);
                        }
                        const int mrow = c.mat * Wm;
                        for (int r = 0; r < W / 32; ++r) {
                            tc::tma_load_2d(Bhi + r * 32 * KC, &map_mhi, kc * KC, mrow + 32 * r, &bar_full[st]);
                            tc::tma_load_2d(Blo + r * 32 * KC, &map_mlo, kc * KC, mrow + 32 * r, &bar_full[st]);
                        }
                        last_full = st;
                        last_full_parity = u & 1;
                        return true;
                    };
                    bool ok = issue(0);
                    for (int i = 0; i < total && ok; ++i) {
                        if (i + 1 < total) ok = issue(i + 1);
                        const uint32_t ci = g + (uint32_t)i;
                        const int st = ci & 1;
                        if (ok) ok = tc::mbar_wait(&bar_full[st], (ci >> 1) & 1);
                        if (!ok) break;
                        tc::fence_after();
                        const ChildInfo& c = child_of(i / kpc);
                        const int kc = i % kpc;
                        uint8_t* base = smem + st * sbytes;
                        const float* Ahi = reinterpret_cast<const float*>(base);
                        const float* Alo = Ahi + TM * KC;
                        const float* Bhi = Alo + TM * KC;
                        const float* Blo = Bhi + Wm * KC;
                        const uint32_t d = tmem + (uint32_t)c.tcol;
#pragma unroll
                        for (int ks = 0; ks < KC / 8; ++ks) {
                            const uint64_t ah = tc::desc_sw128(Ahi + ks * 8), al = tc::desc_sw128(Alo + ks * 8);
                            const uint64_t bh = tc::desc_sw128(Bhi + ks * 8), bl = tc::desc_sw128(Blo + ks * 8);
                            tc::mma_tf32(d, ah, bh, idesc, (kc | ks) != 0);
                            tc::mma_tf32(d, ah, bl, idesc, 1);
                            tc::mma_tf32(d, al, bh, idesc, 1);
                        }
                        tc::mma_commit(&bar_empty[st]);
                    }
                    if (ok) {
                        tc::mma_commit(&bar_done);
                        g += (uint32_t)total;
                    } else {
                        atomicExch(a.status, 1);
                        abort_sh = 1;
                    }
                }
                __syncthreads();
                if (!abort_sh) {
                    if (!tc::mbar_wait(&bar_done, dn & 1)) {
                        atomicExch(a.status, 2);
                        abort_sh = 1;
                    }
                }
                dn++;
                tc::fence_after();
            }
            __syncthreads();
            if (abort_sh) break;

            // ---------------- epilogue: product over children ----------------
            int Eacc = 0;
            int lcol[8];
            float lw[8][3];
            int lrow[8][3];
            for (int c = 0; c < nch; ++c) {
                const ChildInfo& ci = ch_sh[c];
                if (ci.leaf_col >= 0) {
                    const int n = fam >= 0 ? a.counts[(size_t)fam * P.n_leaves + ci.leaf_col] : 0;
                    const int32_t* ce = a.ce + (size_t)ci.mat * Wm;
                    if (a.err) {
                        // error-model leaf: weights p_d 2^(ce_d - ce_max) over columns n-1, n, n+1
                        const double* pr = a.err + (size_t)(n < a.err_rows ? n : a.err_rows - 1) * a.err_ndev;
                        const int off = n - (a.err_ndev - 1) / 2;
                        int cmax = -100000;
                        for (int d = 0; d < 3 && d < a.err_ndev; ++d) {
                            const int col = off + d;
                            if (col >= 0 && col <= S && pr[d] > 0) cmax = max(cmax, ce[col]);
                        }
                        for (int d = 0; d < 3; ++d) {
                            const int col = off + d;
                            const bool use = d < a.err_ndev && col >= 0 && col <= S && pr[d] > 0;
                            lrow[c][d] = use ? col : -1;
                            lw[c][d] = use ? (float)(pr[d] * exp2((double)(ce[col] - cmax))) : 0.0f;
                        }
                        Eacc += cmax > -100000 ? cmax : 0;
                        if (cmax == -100000) flag = true;
                    } else {
                        const bool use = n >= 0 && n <= S;
                        lrow[c][0] = use ? n : -1;
                        lw[c][0] = 1.0f;
                        lrow[c][1] = lrow[c][2] = -1;
                        lw[c][1] = lw[c][2] = 0.0f;
                        Eacc += use ? ce[n] : 0;
                        if (!use) flag = true;
                    }
                    lcol[c] = 0;
                } else {
                    Eacc += Esh[P.slot[ci.node] * TM + tid];
                    lcol[c] = ci.tcol;
                }
            }
            const int s_lo = is_root ? 1 : 0;
            const int s_hi = is_root ? Rf + 1 : W;   // exclusive

            auto load_factor = [&](int c, int col0, float (&y)[32]) {
                const ChildInfo& ci = ch_sh[c];
                if (ci.leaf_col < 0) {
                    tc::tmem_ld32(tmem + lane_base + (uint32_t)(lcol[c] + col0), y);
                } else {
                    const float* ct = a.ct + (size_t)ci.mat * Wm * Wm;
#pragma unroll
                    for (int j = 0; j < 32; ++j) y[j] = 0.0f;
                    for (int d = 0; d < 3; ++d) {
                        if (lrow[c][d] < 0) continue;
                        const float4* src = reinterpret_cast<const float4*>(ct + (size_t)lrow[c][d] * Wm + col0);
                        const float w = lw[c][d];
#pragma unroll
                        for (int q = 0; q < 8; ++q) {
                            const float4 x = __ldg(src + q);
                            y[4 * q + 0] = fmaf(w, x.x, y[4 * q + 0]);
                            y[4 * q + 1] = fmaf(w, x.y, y[4 * q + 1]);
                            y[4 * q + 2] = fmaf(w, x.z, y[4 * q + 2]);
                            y[4 * q + 3] = fmaf(w, x.w, y[4 * q + 3]);
                        }
                    }
                }
            };

            // pass A: largest per-state sum of binary exponents
            int maxe = -100000;
            for (int col0 = 0; col0 < W; col0 += 32) {
                int ex[32];
#pragma unroll
                for (int j = 0; j < 32; ++j) ex[j] = 0;
                for (int c = 0; c < nch; ++c) {
                    float y[32];
                    load_factor(c, col0, y);
#pragma unroll
                    for (int j = 0; j < 32; ++j) ex[j] += bexp(y[j]);
                }
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const int s = col0 + j;
                    if (s >= s_lo && s < s_hi && ex[j] > maxe) maxe = ex[j];
                }
            }
            if (maxe < -250) {
                flag = true;     // factors too far apart (or all zero): FP64 recomputes this family
                maxe = 0;
            }
            // split the rescale over the children so no factor overflows
            int shift[8];
            {
                const int sh = -maxe;
                const int part = sh / nch;
                for (int c = 0; c < nch; ++c) shift[c] = part;
                shift[0] += sh - part * nch;
            }

            // pass B: product, then store (internal node) or weight by the prior (root)
            double best = 0.0;
            float* rowhi = a.vec_hi + (size_t)(vrow_cta + (int64_t)vs * TM + tid) * Wm;
            float* rowlo = a.vec_lo + (size_t)(vrow_cta + (int64_t)vs * TM + tid) * Wm;
            for (int col0 = 0; col0 < W; col0 += 32) {
                float p[32];
#pragma unroll
                for (int j = 0; j < 32; ++j) p[j] = 1.0f;
                for (int c = 0; c < nch; ++c) {
                    float y[32];
                    load_factor(c, col0, y);
                    const float sc = pow2f(shift[c]);
#pragma unroll
                    for (int j = 0; j < 32; ++j) p[j] *= y[j] * sc;
                }
                if (!is_root) {
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        float4 h, l;
                        h.x = tc::round_tf32(p[4 * q + 0]);
                        h.y = tc::round_tf32(p[4 * q + 1]);
                        h.z = tc::round_tf32(p[4 * q + 2]);
                        h.w = tc::round_tf32(p[4 * q + 3]);
                        l.x = tc::round_tf32(p[4 * q + 0] - h.x);
                        l.y = tc::round_tf32(p[4 * q + 1] - h.y);
                        l.z = tc::round_tf32(p[4 * q + 2] - h.z);
                        l.w = tc::round_tf32(p[4 * q + 3] - h.w);
                        reinterpret_cast<float4*>(rowhi + col0)[q] = h;
                        reinterpret_cast<float4*>(rowlo + col0)[q] = l;
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 32; ++j) {
                        const int s = col0 + j;
                        if (s >= 1 && s <= Rf) {
                            const int jr = s - 1;
                            const double eq = jr < a.n_prior ? a.prior[jr] : 0.0;
                            const double vv = (double)p[j] * eq;
                            best = vv > best ? vv : best;
                        }
                    }
                }
            }
            const int E = Eacc + maxe;
            if (!is_root) {
                Esh[vs * TM + tid] = E;
            } else if (fam >= 0) {
                double o = NAN;
                if (best > 0.0 && !flag) o = log(best * a.cat_probs[k]) + (double)E * 0.69314718055994530942;
                else flag = true;
                a.out[(size_t)fam * a.K + k] = o;
            }
            // node vectors are read back by TMA (async proxy) for the parent
            tc::fence_proxy_async_global();
            tc::fence_before();
            __syncthreads();
            tc::fence_after();
        }
        if (flag && fam >= 0) atomicOr(&a.flags[fam], 1);
        __syncthreads();
        if (abort_sh) break;
    }

    // teardown: no copy of ours may still be landing when TMEM goes away
    tc::fence_before();
    __syncthreads();
    if (abort_sh && tid == 0 && last_full >= 0) tc::mbar_wait(&bar_full[last_full], last_full_parity, 1 << 20);
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, (uint32_t)a.tmem_cols);
}

// FP64 matrix -> TF32 hi/lo operands (row-major) and the FP32
// column-normalised transposed copy used for leaf columns.
__global__ void __launch_bounds__(256) k_convert_tc(const ConvertJob* __restrict__ jobs, TcBuffers b) {
    const ConvertJob J = jobs[blockIdx.x];
    const int Wm = b.Wm;
    const size_t base = (size_t)J.mat * Wm * Wm;
    for (int idx = threadIdx.x; idx < Wm * Wm; idx += blockDim.x) {
        const int s = idx / Wm, c = idx % Wm;
        const float x = (float)J.src[(size_t)s * J.ld + c];
        const float h = tc::round_tf32(x);
        b.hi[base + idx] = h;
        b.lo[base + idx] = tc::round_tf32(x - h);
    }
    for (int c = threadIdx.x; c < Wm; c += blockDim.x) {
        double mx = 0.0;
        for (int s = 0; s < Wm; ++s) {
            const double x = J.src[(size_t)s * J.ld + c];
            mx = x > mx ? x : mx;
        }
        int e = 0;
        if (mx > 0.0) frexp(mx, &e);
        b.ce[(size_t)J.mat * Wm + c] = e;
        float* row = b.ct + base + (size_t)c * Wm;
        for (int s = 0; s < Wm; ++s) row[s] = (float)scalbn(J.src[(size_t)s * J.ld + c], -e);
    }
}

}  // namespace

size_t prune_tc_smem_bytes(int Wm, int n_slots) { return 2 * stage_bytes(Wm) + (size_t)n_slots * TM * sizeof(int) + 1024; }

cudaError_t launch_convert_tc(const ConvertJob* d_jobs, int n_jobs, TcBuffers b, cudaStream_t s) {
    if (n_jobs <= 0) return cudaSuccess;
    k_convert_tc<<<n_jobs, 256, 0, s>>>(d_jobs, b);
    return cudaGetLastError();
}

cudaError_t launch_prune_tc(const TcMaps& m, const PruneTcArgs& a, int n_ctas, size_t smem, cudaStream_t s) {
    if (a.n_tiles <= 0) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(k_prune_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_prune_tc<<<n_ctas, NTHREADS, smem, s>>>(m.mat_hi, m.mat_lo, m.vec_hi, m.vec_lo, a);
    return cudaGetLastError();
}

}  // namespace cafe
