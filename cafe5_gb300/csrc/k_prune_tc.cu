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
constexpr int CW = 16;    // epilogue columns per TMEM load

__host__ __device__ inline size_t stage_bytes(int Ws) { return (size_t)(2 * TM + 2 * Ws) * KC * sizeof(float); }

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

// Per-child source of the factor: TMEM columns (internal child) or up to
// three weighted rows of the column-normalised matrix copy (leaf).
struct Src {
    bool leaf;      // also true for the unit factor of an absent second child
    bool unit;
    uint32_t taddr;
    const float* row[3];
    float w[3];
};

template <int NC>
struct NodeSrc {
    Src s[NC];
    int Eacc;     // sum of the children's power-of-two exponents
    bool flag;
};

// Child sources of one node for this thread's family; issued before the
// GEMM wait so the count / exponent loads overlap the tensor-core work.
template <int NC>
__device__ __forceinline__ void setup_src(const PruneTcArgs& a, const ChildInfo* ch, int nch, const int* Esh,
                                          uint32_t tmem_lane, int64_t fam, int tid, int S, int Wm,
                                          NodeSrc<NC>& ns) {
    ns.Eacc = 0;
    ns.flag = false;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        Src& sc = ns.s[c];
        sc.unit = c >= nch;
        if (sc.unit) {
            sc.leaf = true;
            sc.taddr = 0;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                sc.row[d] = nullptr;
                sc.w[d] = 0.0f;
            }
            continue;
        }
        const ChildInfo ci = ch[c];
        sc.leaf = ci.leaf_col >= 0;
        sc.taddr = tmem_lane + (uint32_t)(ci.tcol > 0 ? ci.tcol : 0);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            sc.row[d] = nullptr;
            sc.w[d] = 0.0f;
        }
        if (ci.leaf_col >= 0) {
            const int n = fam >= 0 ? __ldg(a.counts + (size_t)fam * a.plan.n_leaves + ci.leaf_col) : 0;
            const int32_t* ce = a.ce + (size_t)ci.mat * Wm;
            const float* ct = a.ct + (size_t)ci.mat * Wm * Wm;
            if (a.err) {
                // error-model leaf: weights p_d 2^(ce_d - ce_max) over columns n-1, n, n+1
                const double* pr = a.err + (size_t)(n < a.err_rows ? n : a.err_rows - 1) * a.err_ndev;
                const int off = n - (a.err_ndev - 1) / 2;
                int cmax = -100000;
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const int col = off + d;
                    if (d < a.err_ndev && col >= 0 && col <= S && pr[d] > 0) cmax = max(cmax, __ldg(ce + col));
                }
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const int col = off + d;
                    if (d < a.err_ndev && col >= 0 && col <= S && pr[d] > 0) {
                        sc.row[d] = ct + (size_t)col * Wm;
                        sc.w[d] = (float)pr[d] * pow2f(__ldg(ce + col) - cmax);
                    }
                }
                if (cmax == -100000) ns.flag = true;
                else ns.Eacc += cmax;
            } else if (n >= 0 && n <= S) {
                sc.row[0] = ct + (size_t)n * Wm;
                sc.w[0] = 1.0f;
                ns.Eacc += __ldg(ce + n);
            } else {
                ns.flag = true;
            }
        } else {
            ns.Eacc += Esh[a.plan.slot[ci.node] * TM + tid];
        }
    }
}

// 16 values of a leaf factor starting at column col0.
__device__ __forceinline__ void load_leaf(const Src& c, int col0, uint32_t (&out)[CW]) {
    if (c.unit) {
#pragma unroll
        for (int j = 0; j < CW; ++j) out[j] = __float_as_uint(1.0f);
        return;
    }
    float y[CW];
#pragma unroll
    for (int j = 0; j < CW; ++j) y[j] = 0.0f;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (!c.row[d]) continue;
        const float4* src = reinterpret_cast<const float4*>(c.row[d] + col0);
        const float w = c.w[d];
#pragma unroll
        for (int q = 0; q < CW / 4; ++q) {
            const float4 x = __ldg(src + q);
            y[4 * q + 0] = fmaf(w, x.x, y[4 * q + 0]);
            y[4 * q + 1] = fmaf(w, x.y, y[4 * q + 1]);
            y[4 * q + 2] = fmaf(w, x.z, y[4 * q + 2]);
            y[4 * q + 3] = fmaf(w, x.w, y[4 * q + 3]);
        }
    }
#pragma unroll
    for (int j = 0; j < CW; ++j) out[j] = __float_as_uint(y[j]);
}

struct EpiOut {
    int E;
    bool flag;
    double best;            // root: max_j L[j] prior[j] (in units of 2^E)
};

__device__ __forceinline__ void store_tf32x2(float* __restrict__ hi, float* __restrict__ lo, int col0,
                                             const float (&p)[CW]) {
#pragma unroll
    for (int q = 0; q < CW / 4; ++q) {
        float4 h, l;
        h.x = tc::round_tf32(p[4 * q + 0]);
        h.y = tc::round_tf32(p[4 * q + 1]);
        h.z = tc::round_tf32(p[4 * q + 2]);
        h.w = tc::round_tf32(p[4 * q + 3]);
        l.x = tc::round_tf32(p[4 * q + 0] - h.x);
        l.y = tc::round_tf32(p[4 * q + 1] - h.y);
        l.z = tc::round_tf32(p[4 * q + 2] - h.z);
        l.w = tc::round_tf32(p[4 * q + 3] - h.w);
        reinterpret_cast<float4*>(hi + col0)[q] = h;
        reinterpret_cast<float4*>(lo + col0)[q] = l;
    }
}

// Fast epilogue: one pass. Every factor is <= 1 (rows of M sum to <= 1,
// node vectors and normalised leaf columns are <= 1), so the plain product
// cannot overflow; its maximum is tracked and the stored row is rescaled
// only if it drifts below 2^-32. Leaf loads run one chunk ahead.
// `need_exact` is set when the product underflowed (max < 2^-120, or an
// all-zero weighted root) so the exact two-pass epilogue must redo it.
template <int NC>
__device__ __forceinline__ void epi_fast(const NodeSrc<NC>& ns, int W, bool is_root, int Rf, const float* prior_f,
                                         float* __restrict__ rowhi, float* __restrict__ rowlo, EpiOut& out,
                                         bool& need_exact) {
    float maxp = 0.0f;
    float best_f = 0.0f, best_p = 0.0f, best_q = 0.0f;
    uint32_t lf[NC][CW];
#pragma unroll
    for (int c = 0; c < NC; ++c)
        if (ns.s[c].leaf) load_leaf(ns.s[c], 0, lf[c]);
    for (int col0 = 0; col0 < W; col0 += CW) {
        uint32_t r[NC][CW];
        bool any_tmem = false;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            if (!ns.s[c].leaf) {
                tc::tmem_ld16_issue(ns.s[c].taddr + (uint32_t)col0, r[c]);
                any_tmem = true;
            } else {
#pragma unroll
                for (int j = 0; j < CW; ++j) r[c][j] = lf[c][j];
                if (col0 + CW < W) load_leaf(ns.s[c], col0 + CW, lf[c]);   // next chunk, in flight
            }
        }
        if (any_tmem) tc::tmem_wait();
        float p[CW];
#pragma unroll
        for (int j = 0; j < CW; ++j) p[j] = 1.0f;
#pragma unroll
        for (int c = 0; c < NC; ++c)
#pragma unroll
            for (int j = 0; j < CW; ++j) p[j] *= __uint_as_float(r[c][j]);
        if (!is_root) {
#pragma unroll
            for (int j = 0; j < CW; ++j) maxp = fmaxf(maxp, p[j]);
            store_tf32x2(rowhi, rowlo, col0, p);
        } else {
#pragma unroll
            for (int j = 0; j < CW; ++j) {
                const int s = col0 + j;
                if (s >= 1 && s <= Rf) {
                    const float q = prior_f[s - 1];
                    const float v = p[j] * q;
                    if (v > best_f) {
                        best_f = v;
                        best_p = p[j];
                        best_q = q;
                    }
                }
            }
        }
    }
    int E = ns.Eacc;
    need_exact = false;
    if (!is_root && maxp < 0x1p-32f) {
        if (!(maxp >= 0x1p-120f)) {
            need_exact = true;
        } else {
            // bring this row's maximum back to [0.5, 1)
            const int k = -bexp(maxp);
            const float sc = pow2f(k);
            for (int col0 = 0; col0 < W; col0 += 4) {
                float4 h = *reinterpret_cast<const float4*>(rowhi + col0);
                float4 l = *reinterpret_cast<const float4*>(rowlo + col0);
                float v[4] = {(h.x + l.x) * sc, (h.y + l.y) * sc, (h.z + l.z) * sc, (h.w + l.w) * sc};
                h.x = tc::round_tf32(v[0]);
                h.y = tc::round_tf32(v[1]);
                h.z = tc::round_tf32(v[2]);
                h.w = tc::round_tf32(v[3]);
                l.x = tc::round_tf32(v[0] - h.x);
                l.y = tc::round_tf32(v[1] - h.y);
                l.z = tc::round_tf32(v[2] - h.z);
                l.w = tc::round_tf32(v[3] - h.w);
                *reinterpret_cast<float4*>(rowhi + col0) = h;
                *reinterpret_cast<float4*>(rowlo + col0) = l;
            }
            E -= k;
        }
    }
    if (is_root && !(best_f > 0.0f)) need_exact = true;
    out.E = E;
    out.flag = ns.flag;
    out.best = (double)best_p * (double)best_q;
}

// Exact epilogue (warp-collective: every lane runs it when any lane needs
// it): pass A finds the largest per-state sum of the factors' binary
// exponents, pass B forms the product rescaled by it, so the product's
// maximum is in [2^-NC, 1) and nothing underflows unless the factors are
// more than 2^250 apart. Results are stored only where `write` is set.
template <int NC>
__device__ __noinline__ void epi_exact(const NodeSrc<NC>& ns, int W, bool is_root, int Rf, const float* prior_f,
                                       float* __restrict__ rowhi, float* __restrict__ rowlo, bool write,
                                       EpiOut& out) {
    const int s_lo = is_root ? 1 : 0;
    const int s_hi = is_root ? Rf + 1 : W;
    int maxe = -100000;
    for (int col0 = 0; col0 < W; col0 += CW) {
        int ex[CW];
#pragma unroll
        for (int j = 0; j < CW; ++j) ex[j] = 0;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            uint32_t r[CW];
            if (!ns.s[c].leaf) {
                tc::tmem_ld16_issue(ns.s[c].taddr + (uint32_t)col0, r);
                tc::tmem_wait();
            } else {
                load_leaf(ns.s[c], col0, r);
            }
#pragma unroll
            for (int j = 0; j < CW; ++j) ex[j] += bexp(__uint_as_float(r[j]));
        }
#pragma unroll
        for (int j = 0; j < CW; ++j) {
            const int s = col0 + j;
            if (s >= s_lo && s < s_hi && ex[j] > maxe) maxe = ex[j];
        }
    }
    bool flag = ns.flag;
    if (maxe < -250) {
        flag = true;     // factors too far apart (or all zero): FP64 recomputes this family
        maxe = 0;
    }
    float scl[NC];
    {
        const int sh = -maxe;
        const int part = sh / NC;
#pragma unroll
        for (int c = 0; c < NC; ++c) scl[c] = pow2f(part + (c == 0 ? sh - part * NC : 0));
    }
    float best_f = 0.0f, best_p = 0.0f, best_q = 0.0f;
    for (int col0 = 0; col0 < W; col0 += CW) {
        float p[CW];
#pragma unroll
        for (int j = 0; j < CW; ++j) p[j] = 1.0f;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            uint32_t r[CW];
            if (!ns.s[c].leaf) {
                tc::tmem_ld16_issue(ns.s[c].taddr + (uint32_t)col0, r);
                tc::tmem_wait();
            } else {
                load_leaf(ns.s[c], col0, r);
            }
#pragma unroll
            for (int j = 0; j < CW; ++j) p[j] *= __uint_as_float(r[j]) * scl[c];
        }
        if (!is_root) {
            if (write) store_tf32x2(rowhi, rowlo, col0, p);
        } else {
#pragma unroll
            for (int j = 0; j < CW; ++j) {
                const int s = col0 + j;
                if (s >= 1 && s <= Rf) {
                    const float q = prior_f[s - 1];
                    const float v = p[j] * q;
                    if (v > best_f) {
                        best_f = v;
                        best_p = p[j];
                        best_q = q;
                    }
                }
            }
        }
    }
    if (write) {
        out.E = ns.Eacc + maxe;
        out.flag = flag;
        out.best = (double)best_p * (double)best_q;
    }
}

__global__ void __launch_bounds__(NTHREADS, 4)
    k_prune_tc(const __grid_constant__ CUtensorMap map_mhi, const __grid_constant__ CUtensorMap map_mlo,
               const __grid_constant__ CUtensorMap map_vhi, const __grid_constant__ CUtensorMap map_vlo,
               const PruneTcArgs a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    __shared__ __align__(8) uint64_t bar_full[2], bar_empty[2], bar_done;
    __shared__ uint32_t tmem_sh;
    __shared__ int abort_sh;
    __shared__ ChildInfo ch_sh[8];
    __shared__ float prior_f[256];

    const int tid = threadIdx.x, warp = tid >> 5;
    const int Wm = a.Wm;
    const int NS = a.stages;
    const TreePlan& P = a.plan;
    const size_t sbytes = stage_bytes(a.Ws);
    int* Esh = reinterpret_cast<int*>(smem + NS * sbytes);   // [n_slots][TM]

    for (int j = tid; j < 256; j += NTHREADS) prior_f[j] = j < a.n_prior ? (float)a.prior[j] : 0.0f;
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
    const int64_t vrow_cta = a.vrow_base + (int64_t)blockIdx.x * a.n_slots * TM;
    unsigned long long ph[4] = {0, 0, 0, 0};
    const bool timing = a.phase_clocks != nullptr && tid == 0;

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
            // child sources (count / exponent loads) overlap the GEMM below
            NodeSrc<2> ns2;
            setup_src<2>(a, ch_sh, nch, Esh, tmem + lane_base, fam, tid, S, Wm, ns2);

            // ---------------- GEMMs of the internal children ----------------
            long long t0 = timing ? clock64() : 0;
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
                        const int st = (int)(ci % (uint32_t)NS);
                        const uint32_t u = ci / (uint32_t)NS;
                        if (u >= 1 && !tc::mbar_wait(&bar_empty[st], (u - 1) & 1)) return false;
                        const ChildInfo& c = child_of(i / kpc);
                        const int kc = i % kpc;
                        uint8_t* base = smem + st * sbytes;
                        float* Ahi = reinterpret_cast<float*>(base);
                        float* Alo = Ahi + TM * KC;
                        float* Bhi = Alo + TM * KC;
                        float* Blo = Bhi + a.Ws * KC;
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
                        // with two stages the next chunk's TMA overlaps this chunk's MMAs
                        if (NS > 1 && i + 1 < total) ok = issue(i + 1);
                        const uint32_t ci = g + (uint32_t)i;
                        const int st = (int)(ci % (uint32_t)NS);
                        if (ok) ok = tc::mbar_wait(&bar_full[st], (ci / (uint32_t)NS) & 1);
                        if (!ok) break;
                        tc::fence_after();
                        const ChildInfo& c = child_of(i / kpc);
                        const int kc = i % kpc;
                        uint8_t* base = smem + st * sbytes;
                        const float* Ahi = reinterpret_cast<const float*>(base);
                        const float* Alo = Ahi + TM * KC;
                        const float* Bhi = Alo + TM * KC;
                        const float* Blo = Bhi + a.Ws * KC;
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
                        if (NS == 1 && i + 1 < total) ok = issue(i + 1);
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
            long long t1 = timing ? clock64() : 0;

            // ---------------- epilogue: product over children ----------------
            EpiOut eo;
            float* rowhi = a.vec_hi + (size_t)(vrow_cta + (int64_t)vs * TM + tid) * Wm;
            float* rowlo = a.vec_lo + (size_t)(vrow_cta + (int64_t)vs * TM + tid) * Wm;
            bool need;
            epi_fast<2>(ns2, W, is_root, Rf, prior_f, rowhi, rowlo, eo, need);
            if (__any_sync(0xffffffffu, need)) epi_exact<2>(ns2, W, is_root, Rf, prior_f, rowhi, rowlo, need, eo);
            long long t2 = timing ? clock64() : 0;
            flag |= eo.flag;
            if (!is_root) {
                Esh[vs * TM + tid] = eo.E;
            } else if (fam >= 0) {
                double o = NAN;
                if (eo.best > 0.0 && !flag)
                    o = log(eo.best * a.cat_probs[k]) + (double)eo.E * 0.69314718055994530942;
                else flag = true;
                a.out[(size_t)fam * a.K + k] = o;
            }
            // node vectors are read back by TMA (async proxy) for the parent
            long long t3 = timing ? clock64() : 0;
            if (timing) t2 = t3;
            tc::fence_proxy_async_global();
            tc::fence_before();
            __syncthreads();
            tc::fence_after();
            if (timing) {
                const long long t4 = clock64();
                ph[0] += t1 - t0;
                ph[1] += t2 - t1;
                ph[2] += t3 - t2;
                ph[3] += t4 - t3;
            }
        }
        if (flag && fam >= 0) {
            atomicOr(&a.flags[fam], 1);
            atomicOr(a.status + 3, 1);     // "some family is flagged"
        }
        __syncthreads();
        if (abort_sh) break;
    }

    if (timing)
        for (int q = 0; q < 4; ++q) atomicAdd(&a.phase_clocks[q], ph[q]);
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

// One block: flagged families of each bin, compacted in permutation order
// (a block-wide prefix sum per 256-family chunk), then tiles bin by bin.
__global__ void __launch_bounds__(256) k_fallback_plan(FallbackPlanArgs a) {
    __shared__ int scan[256];
    __shared__ int64_t base_sh;
    __shared__ int n_tiles_sh;
    if (a.any_flag && *a.any_flag == 0) {     // nothing flagged: no work
        if (threadIdx.x == 0) {
            a.out_counts[0] = 0;
            a.out_counts[1] = 0;
        }
        return;
    }
    if (threadIdx.x == 0) {
        base_sh = 0;
        n_tiles_sh = 0;
    }
    __syncthreads();
    for (int b = 0; b < a.n_bins; ++b) {
        const int64_t start = base_sh;
        for (int64_t i0 = 0; i0 < a.bin_count[b]; i0 += 256) {
            const int64_t i = i0 + threadIdx.x;
            int64_t fam = -1;
            int f = 0;
            if (i < a.bin_count[b]) {
                fam = a.perm[a.bin_first[b] + i];
                f = a.flags[fam] != 0;
            }
            scan[threadIdx.x] = f;
            __syncthreads();
            for (int off = 1; off < 256; off <<= 1) {
                const int add = threadIdx.x >= off ? scan[threadIdx.x - off] : 0;
                __syncthreads();
                scan[threadIdx.x] += add;
                __syncthreads();
            }
            if (f) a.fb_perm[base_sh + scan[threadIdx.x] - 1] = fam;
            const int total = scan[255];
            __syncthreads();
            if (threadIdx.x == 0) base_sh += total;
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            const int64_t cnt = base_sh - start;
            for (int q = 0; q < a.n_cats; ++q)
                for (int64_t i = 0; i < cnt; i += 32) {
                    const int k = a.cats[q];
                    PruneTile t;
                    t.first = (int)(start + i);
                    t.count = (int)(cnt - i < 32 ? cnt - i : 32);
                    t.k = k;
                    t.S = a.bin_width[b] - 1;
                    t.R = a.bin_width[b] - 1;
                    t.pad[0] = t.pad[1] = t.pad[2] = 0;
                    a.fb_tiles[n_tiles_sh++] = t;
                }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.out_counts[0] = (int32_t)base_sh;
        a.out_counts[1] = n_tiles_sh;
    }
}

}  // namespace

cudaError_t launch_fallback_plan(const FallbackPlanArgs& a, cudaStream_t s) {
    k_fallback_plan<<<1, 256, 0, s>>>(a);
    return cudaGetLastError();
}

size_t prune_tc_smem_bytes(int Ws, int n_slots, int stages) {
    return (size_t)stages * stage_bytes(Ws) + (size_t)n_slots * TM * sizeof(int) + 1024;
}

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
