// K3/K4 on the tensor cores, warp-specialised: split-TF32 (TF32x3) pruning of
// 128-family tiles with FP32 accumulation in TMEM and integer-exponent
// rescaling, several tiles in flight per CTA.
//
// Algorithm: inference_prune (src/core.cpp:134-145) -> compute_node_probability
// (src/probability.cpp:175-234) -> matrix::multiply (src/matrix_cache.cpp:32-58),
// with the root weighting of base_model (src/base_model.cpp:77-95) and
// gamma_model::prune (src/gamma_core.cpp:143-165) -- the same arithmetic as
// k_prune_tc, laid out so that one tile's epilogue overlaps other tiles'
// GEMMs:
//
//  * One persistent CTA per SM holds NCTX family tiles ("contexts"), each
//    walking the tree in post-order. Warp roles:
//      warp 0       producer: for whichever context's next node may start,
//                   TMA loads of the GEMM operand chunks into a ring of
//                   stages -- per child and 32-state K chunk the matrix's TF32
//                   hi/lo rows and, for an internal child, its FP32 node
//                   vector (128 families x 32 states);
//      warp 1       MMA issuer (owns TMEM): D_c[f][s] += A_hi B_hi + A_hi B_lo
//                   (+ A_lo B_hi), tcgen05.mma kind::tf32, into the context's
//                   accumulator of child c;
//      warps 2..    one warpgroup per context (thread = family = TMEM lane),
//                   which first builds its node's A operands -- an internal
//                   child's landed chunk split in place into TF32 hi and lo
//                   (hi = tf32(v), lo = tf32(v - hi)), a leaf child's chunk
//                   written as the one-hot row of the family's count (with
//                   the error model, the weights of counts n-1, n, n+1 as
//                   hi/lo), so the GEMM gathers the column M[.][n] into TMEM
//                   -- then runs the epilogue: product over the children's
//                   factors, power-of-two rescale, the node vector written
//                   to its slot (FP32), root weighting and the category term.
//  * Only the K chunks of a leaf child that hold a count of the tile are
//    issued (the producer warp ORs the tile's counts into a chunk mask).
//  * Hand-offs: stage ring full / built / empty mbarriers and a per-stage
//    descriptor (context, child, chunk, first / last) from the producer to
//    the context and the MMA warp; per context the node's chunk range
//    (producer -> context), an accumulator-ready mbarrier (MMA -> context,
//    once per node), and monotonic counts of finished nodes and staged
//    tiles (context -> producer). A context's node is issued only when its
//    tile's counts are staged and every earlier node of the tile is
//    finished (children's vectors written, accumulators read). One lead
//    thread per context polls (with back-off); the others wait in a named
//    barrier, so waiting costs no issue slots.
//  * FP32 range: every node vector carries an absolute error bound E (its own
//    normalised units): an internal child's factor is off by at most
//    E_child + 8 W 2^-126 (flushed matrix entries, lo parts and products;
//    matrix rows sum to <= 1), a leaf factor by a few 2^-126 where it is below
//    2^-100; the node's bound is u_A (max f_B + u_B) + u_B max f_A, scaled
//    like the product (a leaf's u counted only if it fell below 2^-100). The
//    root writes the category term's relative bound per state (out_err);
//    families over tau |lnL| are recomputed in FP64.
//  * Every wait is bounded and gives up when another role aborted; on time-
//    out the kernel records a status, drains its own MMAs and copies (bounded
//    waits), frees TMEM and returns.
#include "common.cuh"
#include "tc_ptx.cuh"

#include <math.h>

#include <algorithm>

namespace cafe {
namespace {

constexpr int TM = 128;        // families per tile = MMA M = TMEM lanes
constexpr int KC = 32;         // K columns per chunk (one 128-byte swizzle row of FP32)
constexpr int CW = 16;         // columns per TMEM load in the epilogue
constexpr int MAXST = 4;       // ring stages at most
constexpr int MAXCTX = 3;      // contexts per CTA at most
constexpr int kRoleThreads = 64;    // producer and MMA warps
constexpr float kTiny = 0x1p-126f;
constexpr int32_t kSatBit = 1 << 30;
constexpr int kLimit = 1 << 24;     // polls before a wait gives up
constexpr uint8_t kNoCount = 255;   // padding row

__host__ __device__ inline size_t ws_stage_bytes(int W) { return (size_t)(2 * TM + 2 * W) * KC * sizeof(float); }

// Tile-independent node table (the tree's structure), built once per CTA.
struct WsNode {
    int slot;
    int is_root;
    int nch;
    int node[2];      // child node ids
    int leaf_col[2];  // >= 0: leaf
    int cslot[2];     // slot of an internal child
};

// Stage descriptor, producer -> context and MMA warp.
struct StageDesc {
    int ctx, acc, kc, first, last, end, leaf;   // leaf: the child's leaf column, or -1
};

__device__ __forceinline__ int bexp(float y) {
    const uint32_t b = __float_as_uint(y);
    const int be = (int)((b >> 23) & 0xFF);
    if (!(y > 0.0f)) return -100000;
    return be ? be - 126 : -149;
}
__device__ __forceinline__ float pow2f(int a) {
    a = a < -126 ? -126 : (a > 127 ? 127 : a);
    return __uint_as_float((uint32_t)(a + 127) << 23);
}

// Polls an mbarrier phase with back-off; gives up after `limit` polls or
// when *stop is set.
__device__ __forceinline__ bool poll_wait(uint64_t* b, uint32_t parity, const volatile int* stop, int limit) {
    for (int i = 0; i < limit; ++i) {
        if (tc::mbar_try_wait(b, parity)) return true;
        if (*stop) return false;
        if (i > 8) __nanosleep(i < 64 ? 20 : 100);
    }
    return false;
}
// Polls `*p >= target` (acquire) with back-off.
__device__ __forceinline__ bool poll_count(const int* p, int target, const volatile int* stop, int limit) {
    for (int i = 0; i < limit; ++i) {
        if (tc::ld_acquire_shared(p) >= target) return true;
        if (*stop) return false;
        if (i > 8) __nanosleep(i < 64 ? 20 : 100);
    }
    return false;
}

// A child's factor for this thread's family.
struct Fac {
    int unit;           // no such child: the factor is 1
    uint32_t taddr;     // TMEM columns of the child's accumulator (this warp's lanes)
    bool leaf;
    float ue;           // absolute error bound (unscaled units): internal child at every
                        // state, leaf where its value is below 2^-100
};

__device__ __forceinline__ float fac_err(const Fac& f, float raw) {
    return f.leaf ? (raw < 0x1p-100f ? f.ue : 0.0f) : f.ue;
}

// CW columns of both factors (bit patterns; valid after the wait).
__device__ __forceinline__ void load_facs(const Fac (&F)[2], int col0, uint32_t (&r)[2][CW]) {
    bool tm = false;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        if (!F[c].unit) {
            tc::tmem_ld_issue(F[c].taddr + (uint32_t)col0, r[c]);
            tm = true;
        } else {
#pragma unroll
            for (int j = 0; j < CW; ++j) r[c][j] = 0x3f800000u;   // 1.0f
        }
    }
    // tcgen05.ld is warp-collective; the sources are the same for the whole
    // tile, so every lane of the warp reaches the wait
    if (tm) tc::tmem_wait();
}

// Pass 1: the product's maximum (inner node) or the best prior-weighted row
// of root sizes 1..Rf with its range-error bound (root); the factors'
// maxima and minima (for the node's bound).
__device__ __forceinline__ void ws_scan(const Fac (&F)[2], int W, bool is_root, int Rf, const float* prior_f,
                                        const float (&scl)[2], float& maxp, float& best_f, float& best_p,
                                        float& best_q, float& best_err, float (&fmx)[2], float (&fmn)[2]) {
    maxp = 0.0f;
    best_f = best_p = best_q = best_err = 0.0f;
    fmx[0] = fmx[1] = 0.0f;
    fmn[0] = fmn[1] = 1.0f;
    for (int col0 = 0; col0 < W; col0 += CW) {
        uint32_t r[2][CW];
        load_facs(F, col0, r);
#pragma unroll
        for (int j = 0; j < CW; ++j) {
            const float r0 = __uint_as_float(r[0][j]), r1 = __uint_as_float(r[1][j]);
            const float f0 = r0 * scl[0], f1 = r1 * scl[1];
            const float p = f0 * f1;
            if (!is_root) {
                maxp = fmaxf(maxp, p);
                fmx[0] = fmaxf(fmx[0], r0);
                fmx[1] = fmaxf(fmx[1], r1);
                fmn[0] = fminf(fmn[0], r0);
                fmn[1] = fminf(fmn[1], r1);
            } else {
                const int s = col0 + j;
                if (s >= 1 && s <= Rf) {
                    maxp = fmaxf(maxp, p);
                    const float q = prior_f[s - 1];
                    const float v = p * q;
                    if (v > best_f) {
                        best_f = v;
                        best_p = p;
                        best_q = q;
                    }
                    const float u0 = fac_err(F[0], r0) * scl[0], u1 = fac_err(F[1], r1) * scl[1];
                    best_err = fmaxf(best_err, (u0 * (f1 + u1) + u1 * f0) * q);
                }
            }
        }
    }
}

// The exact rescale: the largest per-state sum of the factors' binary
// exponents over states [s_lo, s_hi).
__device__ __noinline__ int ws_maxexp(const Fac F0, const Fac F1, int W, int s_lo, int s_hi) {
    const Fac F[2] = {F0, F1};
    int maxe = -100000;
    for (int col0 = 0; col0 < W; col0 += CW) {
        uint32_t r[2][CW];
        load_facs(F, col0, r);
#pragma unroll
        for (int j = 0; j < CW; ++j) {
            const int s = col0 + j;
            const int e = bexp(__uint_as_float(r[0][j])) + bexp(__uint_as_float(r[1][j]));
            if (s >= s_lo && s < s_hi && e > maxe) maxe = e;
        }
    }
    return maxe;
}

// Optional per-role SM clocks (a.phase_clocks, 16 counters), added once per
// role at the end: where each role of the CTA spends its time.
enum {
    kPhPick = 0, kPhEmpty, kPhProdAll, kPhFull, kPhBuild, kPhBuilt, kPhIssue, kPhAcc, kPhScan, kPhStore,
    kPhEnd, kPhSetup, kPhNodes, kPhChunks, kPhKernel, kPhCount
};

template <int NCTX>
__global__ void __launch_bounds__(kRoleThreads + 128 * NCTX, 1)
    k_prune_ws(const __grid_constant__ CUtensorMap map_mhi, const __grid_constant__ CUtensorMap map_mlo,
               const __grid_constant__ CUtensorMap map_vec, const PruneTcArgs a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    __shared__ __align__(8) uint64_t bar_full[MAXST], bar_built[MAXST], bar_empty[MAXST], bar_acc[MAXCTX],
        bar_drain;
    __shared__ StageDesc sdesc[MAXST];
    __shared__ int done_sh[MAXCTX], ready_sh[MAXCTX], issued_sh[MAXCTX], node_g0[MAXCTX], node_nc[MAXCTX];
    __shared__ int abort_sh;
    __shared__ uint32_t tmem_sh;
    __shared__ float prior_f[256];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int NS = a.stages;
    const int W = a.Ws;                     // the launch's bin width (S + 1)
    const int S = W - 1;
    const int Wm = a.Wm;
    const TreePlan& P = a.plan;
    const int ni = P.n_internal;
    const int nl = P.n_leaves;
    const size_t sbytes = ws_stage_bytes(W);
    uint8_t* cnt8 = smem + (size_t)NS * sbytes;                                         // [NCTX][n_leaves][TM]
    int* mi_sh = reinterpret_cast<int*>(cnt8 + (((size_t)NCTX * nl * TM + 15) & ~(size_t)15));   // [NCTX][n_nodes]
    int* Esh = mi_sh + (((size_t)NCTX * P.n_nodes + 3) & ~(size_t)3);                   // [NCTX][slots][TM]
    float* Erh = reinterpret_cast<float*>(Esh + (size_t)NCTX * a.n_slots * TM);        // [NCTX][slots][TM]
    WsNode* nodes = reinterpret_cast<WsNode*>(Erh + (size_t)NCTX * a.n_slots * TM);    // [n_internal]
    // error-model weights of counts 0..255, hi and lo (with an error model only)
    float* errw_hi = reinterpret_cast<float*>(nodes + ni);
    float* errw_lo = errw_hi + 256 * 3;
    const volatile int* stop = &abort_sh;

    // ---- set-up: node table, prior, error-model weights, barriers, TMEM ----
    for (int ii = tid; ii < ni; ii += blockDim.x) {
        const int v = P.internal[ii];
        WsNode e;
        e.slot = P.slot[v];
        e.is_root = v == P.root;
        e.nch = P.cstart[ii + 1] - P.cstart[ii];
        for (int c = 0; c < 2; ++c) {
            e.node[c] = -1;
            e.leaf_col[c] = -1;
            e.cslot[c] = 0;
            if (c < e.nch) {
                const int ch = P.child[P.cstart[ii] + c];
                e.node[c] = ch;
                e.leaf_col[c] = P.leaf_col[ch];
                if (e.leaf_col[c] < 0) e.cslot[c] = P.slot[ch];
            }
        }
        nodes[ii] = e;
    }
    for (int j = tid; j < 256; j += blockDim.x) prior_f[j] = j < a.n_prior ? (float)a.prior[j] : 0.0f;
    if (a.err)
        for (int j = tid; j < 256 * 3; j += blockDim.x) {
            const int n = j / 3, d = j % 3;
            float h = 0.0f, l = 0.0f;
            if (d < a.err_ndev) {
                const double w = a.err[(size_t)(n < a.err_rows ? n : a.err_rows - 1) * a.err_ndev + d];
                if (w > 0) {
                    h = tc::round_tf32((float)w);
                    l = tc::round_tf32((float)w - h);
                }
            }
            errw_hi[j] = h;
            errw_lo[j] = l;
        }
    if (warp == 1) tc::tmem_alloc(&tmem_sh, (uint32_t)a.tmem_cols);
    if (tid == 0) {
        for (int q = 0; q < MAXST; ++q) {
            tc::mbar_init(&bar_full[q], 1);
            tc::mbar_init(&bar_built[q], 1);
            tc::mbar_init(&bar_empty[q], 1);
        }
        for (int x = 0; x < MAXCTX; ++x) {
            tc::mbar_init(&bar_acc[x], 1);
            done_sh[x] = 0;
            ready_sh[x] = 0;
            issued_sh[x] = 0;
            node_g0[x] = node_nc[x] = 0;
        }
        tc::mbar_init(&bar_drain, 1);
        tc::mbar_init_fence();
        abort_sh = 0;
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmem_sh;
    const int G = (int)gridDim.x * NCTX;
    auto tile_of = [&](int x, int r) { return r * G + (int)blockIdx.x * NCTX + x; };
    auto fail = [&](int code) {
        atomicExch(a.status, code);
        atomicExch(&abort_sh, 1);
    };
    const int err_off = a.err ? (a.err_ndev - 1) / 2 : 0;
    const bool timing = a.phase_clocks != nullptr;
    unsigned long long ph[kPhCount];
    for (int q = 0; q < kPhCount; ++q) ph[q] = 0;
    const long long t_kernel = clock64();

    if (warp == 0) {
        // ------------------------------ producer ------------------------------
        // The whole warp walks the schedule (it ORs leaf counts into chunk
        // masks); lane 0 waits on barriers and issues the copies.
        uint32_t g = 0;
        int last_use[MAXST];
        for (int q = 0; q < MAXST; ++q) last_use[q] = -1;
        int r[NCTX], i[NCTX];
        bool act[NCTX];
        for (int x = 0; x < NCTX; ++x) {
            r[x] = 0;
            i[x] = 0;
            act[x] = tile_of(x, 0) < a.n_tiles;
        }
        int last_x = NCTX - 1;
        bool ok = true;
        while (ok) {
            bool any = false;
            for (int x = 0; x < NCTX; ++x) any |= act[x];
            if (!any) break;
            // the next context whose next node may start
            int pick = -1;
            const long long tp0 = timing ? clock64() : 0;
            if (lane == 0) {
                for (int it = 0; pick < 0; ++it) {
                    for (int d = 1; d <= NCTX && pick < 0; ++d) {
                        const int x = (last_x + d) % NCTX;
                        if (act[x] && tc::ld_acquire_shared(&ready_sh[x]) > r[x] &&
                            tc::ld_acquire_shared(&done_sh[x]) >= r[x] * ni + i[x])
                            pick = x;
                    }
                    if (pick >= 0) break;
                    if (*stop) break;
                    if (it > kLimit) {
                        fail(1);
                        break;
                    }
                    if (it > 8) __nanosleep(20);
                }
            }
            pick = __shfl_sync(0xffffffffu, pick, 0);
            if (timing) ph[kPhPick] += clock64() - tp0;
            if (pick < 0) {
                ok = false;
                break;
            }
            last_x = pick;
            const int x = pick;
            const WsNode nd = nodes[i[x]];
            const int* mi = mi_sh + (size_t)x * P.n_nodes;      // the tile's matrix indices
            const int64_t vrow_ctx = a.vrow_base + ((int64_t)blockIdx.x * NCTX + x) * a.n_slots * TM;
            // chunks of every child: all of an internal child's, and a leaf's
            // that hold one of the tile's counts (or its error-model neighbours)
            unsigned mask[2] = {0, 0};
            const unsigned full_mask = (1u << (W / KC)) - 1;
            for (int c = 0; c < nd.nch; ++c) {
                if (nd.leaf_col[c] < 0) {
                    mask[c] = full_mask;
                    continue;
                }
                const uint8_t* cn = cnt8 + ((size_t)x * nl + nd.leaf_col[c]) * TM;
                unsigned bits = 0;
#pragma unroll
                for (int q = 0; q < TM / 32; ++q) {
                    const int n = cn[lane + 32 * q];
                    if (n == kNoCount) continue;
                    for (int d = 0; d < 3; ++d) {
                        const int col = a.err ? n - err_off + d : n;
                        if (col >= 0 && col <= S) bits |= 1u << (col / KC);
                        if (!a.err) break;
                    }
                }
                bits = __reduce_or_sync(0xffffffffu, bits);
                mask[c] = bits ? bits : 1u;   // an all-padding tile still initialises D
            }
            const int last_c = nd.nch - 1;
            // the node's chunk range, for its context's builders
            if (lane == 0) {
                node_g0[x] = (int)g;
                node_nc[x] = __popc(mask[0]) + __popc(mask[1]);
                tc::st_release_shared(&issued_sh[x], r[x] * ni + i[x] + 1);
            }
            for (int c = 0; c < nd.nch && ok; ++c) {
                const bool leaf = nd.leaf_col[c] >= 0;
                const int mrow = (mi[nd.node[c]] & ~kSatBit) * Wm;
                const int vrow = leaf ? 0 : (int)(vrow_ctx + (int64_t)nd.cslot[c] * TM);
                unsigned m = mask[c];
                bool first = true;
                while (m && ok) {
                    const int kc = __ffs(m) - 1;
                    m &= m - 1;
                    const int st = (int)(g % (uint32_t)NS);
                    const uint32_t u = g / (uint32_t)NS;
                    bool okw = true;
                    const long long te0 = timing ? clock64() : 0;
                    if (lane == 0 && g >= (uint32_t)NS) okw = poll_wait(&bar_empty[st], (u - 1) & 1, stop, kLimit);
                    okw = __shfl_sync(0xffffffffu, okw ? 1 : 0, 0) != 0;
                    if (timing) ph[kPhEmpty] += clock64() - te0;
                    if (!okw) {
                        if (lane == 0 && !*stop) fail(1);
                        ok = false;
                        break;
                    }
                    if (lane == 0) {
                        StageDesc dsc;
                        dsc.ctx = x;
                        dsc.acc = c;
                        dsc.kc = kc;
                        dsc.first = first;
                        dsc.last = c == last_c && m == 0;
                        dsc.end = 0;
                        dsc.leaf = leaf ? nd.leaf_col[c] : -1;
                        sdesc[st] = dsc;
                        uint8_t* base = smem + (size_t)st * sbytes;
                        float* Ahi = reinterpret_cast<float*>(base);
                        float* Bhi = Ahi + 2 * TM * KC;
                        float* Blo = Bhi + W * KC;
                        tc::mbar_expect_tx(&bar_full[st], (uint32_t)(((leaf ? 0 : TM) + 2 * W) * KC * sizeof(float)));
                        if (!leaf)
                            for (int q = 0; q < TM / 32; ++q)
                                tc::tma_load_2d(Ahi + q * 32 * KC, &map_vec, kc * KC, vrow + 32 * q, &bar_full[st]);
                        for (int q = 0; q < W / 32; ++q) {
                            tc::tma_load_2d(Bhi + q * 32 * KC, &map_mhi, kc * KC, mrow + 32 * q, &bar_full[st]);
                            tc::tma_load_2d(Blo + q * 32 * KC, &map_mlo, kc * KC, mrow + 32 * q, &bar_full[st]);
                        }
                        last_use[st] = (int)u;
                    }
                    first = false;
                    g++;
                }
            }
            if (!ok) break;
            if (++i[x] == ni) {
                i[x] = 0;
                r[x]++;
                act[x] = tile_of(x, r[x]) < a.n_tiles;
            }
        }
        if (timing) ph[kPhProdAll] += clock64() - t_kernel;
        if (lane == 0) {
            // end marker for the MMA warp
            if (ok) {
                const int st = (int)(g % (uint32_t)NS);
                const uint32_t u = g / (uint32_t)NS;
                if (g >= (uint32_t)NS && !poll_wait(&bar_empty[st], (u - 1) & 1, stop, kLimit)) {
                    if (!*stop) fail(1);
                } else {
                    StageDesc dsc{0, 0, 0, 0, 0, 1, -1};
                    sdesc[st] = dsc;
                    tc::mbar_arrive(&bar_built[st]);
                    g++;
                }
            }
            // no copy of ours may still be landing at teardown
            if (*stop)
                for (int q = 0; q < NS; ++q)
                    if (last_use[q] >= 0) tc::mbar_wait(&bar_full[q], (uint32_t)last_use[q] & 1, kLimit);
        }
    } else if (warp == 1) {
        // ------------------------------ MMA issuer ------------------------------
        if (lane == 0) {
            const uint32_t idesc = tc::idesc_tf32(TM, W);
            for (uint32_t g = 0;; ++g) {
                const int st = (int)(g % (uint32_t)NS);
                const uint32_t u = g / (uint32_t)NS;
                const long long tb0 = timing ? clock64() : 0;
                if (!poll_wait(&bar_built[st], u & 1, stop, kLimit)) {
                    if (!*stop) fail(1);
                    break;
                }
                if (timing) ph[kPhBuilt] += clock64() - tb0;
                const StageDesc d = sdesc[st];
                if (d.end) break;
                const long long ti0 = timing ? clock64() : 0;
                tc::fence_after();
                uint8_t* base = smem + (size_t)st * sbytes;
                const float* Ahi = reinterpret_cast<const float*>(base);
                const float* Alo = Ahi + TM * KC;
                const float* Bhi = Alo + TM * KC;
                const float* Blo = Bhi + W * KC;
                const bool with_lo = d.leaf < 0 || a.err != nullptr;
                const uint32_t dcol = tmem + (uint32_t)(d.ctx * 2 * W + d.acc * W);
#pragma unroll
                for (int ks = 0; ks < KC / 8; ++ks) {
                    const uint64_t ah = tc::desc_sw128(Ahi + ks * 8), al = tc::desc_sw128(Alo + ks * 8);
                    const uint64_t bh = tc::desc_sw128(Bhi + ks * 8), bl = tc::desc_sw128(Blo + ks * 8);
                    tc::mma_tf32(dcol, ah, bh, idesc, (d.first && ks == 0) ? 0u : 1u);
                    tc::mma_tf32(dcol, ah, bl, idesc, 1);
                    if (with_lo) tc::mma_tf32(dcol, al, bh, idesc, 1);
                }
                tc::mma_commit(&bar_empty[st]);
                if (d.last) tc::mma_commit(&bar_acc[d.ctx]);
                if (timing) {
                    ph[kPhIssue] += clock64() - ti0;
                    ph[kPhChunks] += 1;
                }
            }
            // every MMA of ours has completed before TMEM goes away
            tc::mma_commit(&bar_drain);
            tc::mbar_wait(&bar_drain, 0, kLimit);
        }
    } else {
        // -------------------- context: operand builder and epilogue --------------------
        const int x = (warp - 2) >> 2;
        const int quarter = warp & 3;                 // TMEM lane quarter this warp may access
        const int row = quarter * 32 + lane;          // family row of the tile = TMEM lane
        const int bar_id = 1 + x;
        const uint32_t lane_base = (uint32_t)(32 * quarter) << 16;
        int* E_x = Esh + (size_t)x * a.n_slots * TM;
        float* Er_x = Erh + (size_t)x * a.n_slots * TM;
        uint8_t* cn_x = cnt8 + (size_t)x * nl * TM;
        int* mi_x = mi_sh + (size_t)x * P.n_nodes;
        const int64_t vrow_ctx = a.vrow_base + ((int64_t)blockIdx.x * NCTX + x) * a.n_slots * TM;
        const bool lead = row == 0;
        // the lead thread polls; the result reaches the others through the
        // named barrier (an OR of the failures)
        auto ctx_wait = [&](bool got) -> bool { return !tc::named_sync_or(bar_id, 128, !got); };
        uint32_t acc_n = 0;
        int seq = 0;
        bool ok = true;
        for (int rr = 0; ok; ++rr) {
            const int t = tile_of(x, rr);
            if (t >= a.n_tiles) break;
            const long long ts0 = timing ? clock64() : 0;
            const PruneTile tile = a.tiles[t];
            const int k = tile.k;
            const int64_t fam = row < tile.count ? a.perm[tile.first + row] : -1;
            const int Rf = (fam >= 0 && a.fam_R) ? a.fam_R[fam] : tile.R;
            // the tile's counts and matrix indices, staged for the producer and
            // the leaf operands (the previous tile's were all used before its
            // root's GEMMs completed)
            {
                const int32_t* fc = a.counts + (size_t)(fam >= 0 ? fam : 0) * nl;
                for (int l = 0; l < nl; ++l) {
                    const int n = fam >= 0 ? __ldg(fc + l) : -1;
                    cn_x[l * TM + row] = (n >= 0 && n <= S) ? (uint8_t)n : kNoCount;
                }
                const int32_t* mig = a.mat_index + (size_t)k * P.n_nodes;
                for (int v = row; v < P.n_nodes; v += TM) mi_x[v] = __ldg(mig + v);
            }
            tc::named_sync(bar_id, 128);
            if (lead) tc::st_release_shared(&ready_sh[x], rr + 1);
            if (timing) ph[kPhSetup] += clock64() - ts0;
            bool flag = false, dead = false;
            for (int ii = 0; ii < ni && ok; ++ii, ++seq) {
                const WsNode nd = nodes[ii];
                const bool is_root = nd.is_root != 0;

                // ---- build the node's A operands as their chunks land ----
                const long long tb0 = timing ? clock64() : 0;
                {
                    bool got = true;
                    if (lead) got = poll_count(&issued_sh[x], seq + 1, stop, kLimit);
                    if (!ctx_wait(got)) {
                        if (lead && !*stop) fail(2);
                        ok = false;
                        break;
                    }
                }
                const int g0 = node_g0[x], nc = node_nc[x];
                for (int j = 0; j < nc && ok; ++j) {
                    const uint32_t g = (uint32_t)(g0 + j);
                    const int st = (int)(g % (uint32_t)NS);
                    const uint32_t u = g / (uint32_t)NS;
                    bool got = true;
                    if (lead) got = poll_wait(&bar_full[st], u & 1, stop, kLimit);
                    if (!ctx_wait(got)) {
                        if (lead && !*stop) fail(2);
                        ok = false;
                        break;
                    }
                    const StageDesc d = sdesc[st];
                    float* hi = reinterpret_cast<float*>(smem + (size_t)st * sbytes) + (size_t)row * KC;
                    float* lo = hi + TM * KC;
                    float4* h = reinterpret_cast<float4*>(hi);
                    float4* l = reinterpret_cast<float4*>(lo);
                    // this thread's row: 32 FP32, the 16-byte pieces in
                    // 128-byte-swizzled order (piece q at q ^ (row % 8))
                    if (d.leaf < 0) {
#pragma unroll
                        for (int q = 0; q < KC / 4; ++q) {
                            const float4 v = h[q];
                            float4 xh, yl;
                            xh.x = tc::round_tf32_bits(v.x);
                            xh.y = tc::round_tf32_bits(v.y);
                            xh.z = tc::round_tf32_bits(v.z);
                            xh.w = tc::round_tf32_bits(v.w);
                            yl.x = tc::round_tf32_bits(v.x - xh.x);
                            yl.y = tc::round_tf32_bits(v.y - xh.y);
                            yl.z = tc::round_tf32_bits(v.z - xh.z);
                            yl.w = tc::round_tf32_bits(v.w - xh.w);
                            h[q] = xh;
                            l[q] = yl;
                        }
                    } else {
                        const int n = cn_x[d.leaf * TM + row];
                        const int c0 = d.kc * KC;
                        const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
                        for (int q = 0; q < KC / 4; ++q) {
                            h[q] = z;
                            if (a.err) l[q] = z;
                        }
                        if (n != kNoCount) {
                            for (int dd = 0; dd < (a.err ? 3 : 1); ++dd) {
                                const int col = a.err ? n - err_off + dd : n;
                                const int e = col - c0;
                                if (col < 0 || col > S || e < 0 || e >= KC) continue;
                                const int pos = (((e >> 2) ^ (row & 7)) << 2) + (e & 3);
                                hi[pos] = a.err ? errw_hi[n * 3 + dd] : 1.0f;
                                if (a.err) lo[pos] = errw_lo[n * 3 + dd];
                            }
                        }
                    }
                    tc::fence_proxy_async_shared();
                    tc::named_sync(bar_id, 128);
                    if (lead) tc::mbar_arrive(&bar_built[st]);
                }
                if (!ok) break;
                if (timing) ph[kPhBuild] += clock64() - tb0;

                Fac F[2];
                int Eacc = 0;
                bool nflag = false, sat = false;
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    Fac& f = F[c];
                    f.unit = c >= nd.nch;
                    f.leaf = false;
                    f.ue = 0.0f;
                    f.taddr = tmem + lane_base + (uint32_t)(x * 2 * W + c * W);
                    if (f.unit) continue;
                    sat |= (mi_x[nd.node[c]] & kSatBit) != 0;
                    if (nd.leaf_col[c] < 0) {
                        Eacc += E_x[nd.cslot[c] * TM + row];
                        f.ue = Er_x[nd.cslot[c] * TM + row] + (float)(8 * W) * kTiny;
                        continue;
                    }
                    f.leaf = true;
                    f.ue = (a.err ? 8.0f : 2.0f) * kTiny;
                    if (fam >= 0) {
                        // a count none of whose operand columns is inside the bin
                        const int n = cn_x[nd.leaf_col[c] * TM + row];
                        bool any = false;
                        if (n != kNoCount) {
                            if (!a.err) any = true;
                            else
                                for (int dd = 0; dd < 3; ++dd) {
                                    const int col = n - err_off + dd;
                                    any |= col >= 0 && col <= S && errw_hi[n * 3 + dd] > 0.0f;
                                }
                        }
                        if (!any) nflag = true;
                    }
                }
                // the node's GEMMs have landed in TMEM
                const long long ta0 = timing ? clock64() : 0;
                {
                    bool got = true;
                    if (lead)
                        got = poll_wait(&bar_acc[x], acc_n & 1, stop,
                                        a.debug_wait_limit > 0 ? a.debug_wait_limit - 1 : kLimit);
                    acc_n++;
                    if (!ctx_wait(got)) {
                        if (lead && !*stop) fail(2);
                        ok = false;
                        break;
                    }
                    tc::fence_after();
                }
                const long long ta1 = timing ? clock64() : 0;
                if (timing) ph[kPhAcc] += ta1 - ta0;

                // ---- product over the children, rescale ----
                float scl[2] = {1.0f, 1.0f};
                int E = Eacc;
                float maxp, bf, bp, bq, be, fmx[2], fmn[2];
                ws_scan(F, W, is_root, Rf, prior_f, scl, maxp, bf, bp, bq, be, fmx, fmn);
                if (sat && !a.err && !(maxp > 0.0f)) dead = true;
                const bool need = is_root ? !(bf > 0.0f) : !(maxp >= 0x1p-120f);
                if (!is_root && !need && maxp < 0x1p-32f) {
                    const int kk = -bexp(maxp);
                    scl[0] = pow2f(kk);
                    E -= kk;
                }
                if (__any_sync(0xffffffffu, need)) {
                    int maxe = ws_maxexp(F[0], F[1], W, is_root ? 1 : 0, is_root ? Rf + 1 : W);
                    if (need) {
                        if (maxe < -250) {
                            nflag = true;
                            maxe = 0;
                        }
                        const int sh = -maxe, part = sh / 2;
                        scl[0] = pow2f(part + (sh - part * 2));
                        scl[1] = pow2f(part);
                        E = Eacc + maxe;
                    }
                    if (is_root) {
                        float m2, f2, p2, q2, e2, x2[2], n2[2];
                        ws_scan(F, W, true, Rf, prior_f, scl, m2, f2, p2, q2, e2, x2, n2);
                        if (need) {
                            bf = f2;
                            bp = p2;
                            bq = q2;
                            be = e2;
                        }
                    }
                }
                flag |= nflag && !dead;
                const long long ta2 = timing ? clock64() : 0;
                if (timing) ph[kPhScan] += ta2 - ta1;
                if (!is_root) {
                    // ---- the scaled product in FP32, written to the node's slot ----
                    float* vrow = a.vec + (size_t)(vrow_ctx + (int64_t)nd.slot * TM + row) * Wm;
                    for (int col0 = 0; col0 < W; col0 += CW) {
                        uint32_t rg[2][CW];
                        load_facs(F, col0, rg);
                        float p[CW];
#pragma unroll
                        for (int j = 0; j < CW; ++j)
                            p[j] = (__uint_as_float(rg[0][j]) * scl[0]) * (__uint_as_float(rg[1][j]) * scl[1]);
                        float4* dst = reinterpret_cast<float4*>(vrow + col0);
#pragma unroll
                        for (int q = 0; q < CW / 4; ++q) dst[q] = make_float4(p[4 * q], p[4 * q + 1], p[4 * q + 2], p[4 * q + 3]);
                    }
                    // the bound from the factors' maxima: u_A (f_B + u_B) + u_B f_A
                    // over all states, a leaf's u counted only if it fell below
                    // 2^-100 somewhere; plus values flushed on the store
                    float u0 = F[0].ue, u1 = F[1].ue;
                    if (F[0].leaf && !(fmn[0] < 0x1p-100f)) u0 = 0.0f;
                    if (F[1].leaf && !(fmn[1] < 0x1p-100f)) u1 = 0.0f;
                    u0 *= scl[0];
                    u1 *= scl[1];
                    const float ev = u0 * (fmx[1] * scl[1] + u1) + u1 * (fmx[0] * scl[0]);
                    E_x[nd.slot * TM + row] = E;
                    Er_x[nd.slot * TM + row] = fminf(ev + kTiny, 1e30f);
                    // the vector is read next by TMA (the async proxy)
                    tc::fence_proxy_async_global();
                } else if (fam >= 0) {
                    double o = NAN;
                    const double best = (double)bp * (double)bq;
                    if (dead) o = a.model == 0 ? -INFINITY : NAN;
                    else if (best > 0.0 && !flag)
                        o = log(best * a.cat_probs[k]) + (double)E * 0.69314718055994530942;
                    else flag = true;
                    a.out[(size_t)fam * a.K + k] = o;
                    if (a.out_err) a.out_err[(size_t)fam * a.K + k] = (dead || flag || !(bf > 0.0f)) ? 0.0f : be / bf;
                }
                // the node is finished once every TMEM read of the warpgroup
                // and its vector writes are done
                const long long ta3 = timing ? clock64() : 0;
                tc::fence_before();
                tc::named_sync(bar_id, 128);
                if (lead) tc::st_release_shared(&done_sh[x], seq + 1);
                if (timing) {
                    ph[kPhStore] += ta3 - ta2;
                    ph[kPhEnd] += clock64() - ta3;
                    ph[kPhNodes] += 1;
                }
            }
            if (flag && fam >= 0) {
                atomicOr(&a.flags[fam], 1);
                atomicOr(a.status + 3, 1);
            }
        }
    }

    // ---- teardown ----
    if (timing) {
        // one thread per role: producer lane 0, MMA lane 0, row 0 of every context
        const bool rep = (warp == 0 && lane == 0) || (warp == 1 && lane == 0) ||
                         (warp >= 2 && ((warp - 2) & 3) == 0 && lane == 0);
        if (rep) {
            if (warp == 0) ph[kPhKernel] = clock64() - t_kernel;
            for (int q = 0; q < kPhCount; ++q)
                if (ph[q]) atomicAdd(&a.phase_clocks[q], ph[q]);
        }
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (warp == 1) tc::tmem_dealloc(tmem, (uint32_t)a.tmem_cols);
}

}  // namespace

size_t prune_ws_smem_bytes(int W, int n_slots, int stages, int n_internal, int n_leaves, int n_nodes, int nctx,
                           bool err) {
    return (size_t)stages * ws_stage_bytes(W) + (((size_t)nctx * n_leaves * TM + 15) & ~(size_t)15) +
           (((size_t)nctx * n_nodes + 3) & ~(size_t)3) * sizeof(int) +
           (size_t)nctx * n_slots * TM * (sizeof(int) + sizeof(float)) + (size_t)n_internal * sizeof(WsNode) +
           (err ? 2 * 256 * 3 * sizeof(float) : 0) + 1024;
}

// Dynamic shared memory a k_prune_ws CTA may use (the device's opt-in
// limit minus the largest instantiation's static shared memory).
int prune_ws_max_smem() {
    static int cached = -1;
    if (cached < 0) {
        int dev = 0, optin = 0;
        cudaFuncAttributes fa{};
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
            cudaFuncGetAttributes(&fa, (const void*)k_prune_ws<MAXCTX>) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        cached = optin - (int)fa.sharedSizeBytes;
    }
    return cached;
}

cudaError_t prune_ws_init() {
    const int m = prune_ws_max_smem();
    cudaError_t e = cudaFuncSetAttribute(k_prune_ws<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_prune_ws<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_prune_ws<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    return e;
}

cudaError_t launch_prune_ws(const TcMaps& m, const PruneTcArgs& a, int nctx, int n_ctas, size_t smem,
                            cudaStream_t s) {
    if (a.n_tiles <= 0) return cudaSuccess;
    if (smem > (size_t)prune_ws_max_smem()) return cudaErrorInvalidValue;
    if (a.stages < 2 || a.stages > MAXST || a.Ws % KC != 0 || a.Ws > 256 || a.Wm % KC != 0 || a.Ws > a.Wm)
        return cudaErrorInvalidValue;
    if (a.tmem_cols < 2 * nctx * a.Ws || a.tmem_cols > 512) return cudaErrorInvalidValue;
    if (a.err && a.err_ndev > 3) return cudaErrorInvalidValue;
    switch (nctx) {
        case 1: k_prune_ws<1><<<n_ctas, kRoleThreads + 128 * 1, smem, s>>>(m.mat_hi, m.mat_lo, m.vec, a); break;
        case 2: k_prune_ws<2><<<n_ctas, kRoleThreads + 128 * 2, smem, s>>>(m.mat_hi, m.mat_lo, m.vec, a); break;
        case 3: k_prune_ws<3><<<n_ctas, kRoleThreads + 128 * 3, smem, s>>>(m.mat_hi, m.mat_lo, m.vec, a); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace cafe
