// K3/K4 on the tensor cores: split-TF32 (TF32x3) pruning of 128-family tiles
// with FP32 accumulation in TMEM and integer-exponent rescaling.
//
// Same algorithm as k_prune64 (inference_prune, src/core.cpp:134-145 ->
// compute_node_probability, src/probability.cpp:175-234 -> matrix::multiply,
// src/matrix_cache.cpp:32-58; root weighting src/gamma_core.cpp:143-165),
// mapped onto tcgen05:
//
//  * One CTA (4 warps) owns a tile of 128 families of one gamma category and
//    one S-bin of width W and walks the tree in post-order (bins of 384 and
//    512 states, and sparse bins of 128 to 256, share a tile among a
//    cluster of 2 or 4 CTAs, each computing a slice of the output states).
//  * Internal child c: D[f][s] = sum_j L_c[f][j] M_c[s][j] is one
//    M=128 x N=W x K=W GEMM: A = node vectors (128 families x W states,
//    K-major), B = the transition matrix (W x W, K-major: row s, column j).
//    Operands are FP32 pairs hi + lo, each rounded to TF32, and
//    D = A_hi B_hi + A_hi B_lo + A_lo B_hi (the lo*lo term is below the
//    TF32x3 error). K chunks of 32 columns (one 128-byte swizzle row) are
//    staged by TMA in 1 to 4 shared-memory stages, one box per operand: the
//    node vector arrives in FP32 and every thread splits its own row into
//    hi (in place) and lo; the matrix's hi and lo planes arrive in one 3D
//    box. One thread issues TMA and tcgen05.mma; the accumulators of the
//    two children sit side by side in TMEM.
//  * Leaf child: its factor is the matrix column of the observed count (or
//    the error model's weighted sum of three columns): each thread reads its
//    family's column as a row of the transposed FP32 matrix and writes it
//    into the child's TMEM columns (tcgen05.st). Bins up to 64 states read
//    the rows from a W x W block of the transpose that one TMA load puts in
//    shared memory beside the node's first operand chunk; wider bins read
//    them from global memory. A node whose children are both leaves runs no
//    GEMM. Every child's factor then sits in TMEM and the epilogue reads no
//    global memory.
//  * Epilogue (thread f owns family f = TMEM lane f): the product over
//    children is rescaled by the largest per-state sum of the factors'
//    binary exponents, so the product's maximum is ~1 and nothing
//    underflows unless the factors are >2^250 apart; the exponent goes into
//    the family's integer exponent. The node vector is stored in FP32 for
//    the parent's GEMM (bins up to 64 states: one pass over TMEM stages the
//    product and its statistics together). At the root the vector is
//    weighted by the prior in FP64 (root index j = state j + 1) and the
//    category term's natural log is written.
//  * A family whose factors are too far apart, or whose root vector is all
//    zero, is flagged; the host recomputes flagged families in FP64.
//  * FP32 range: a factor value below 2^-126 is flushed (or denormal) where
//    FP64 keeps it, which matters where the children's preferred states are
//    far apart (large counts, short branches). Every node vector carries an
//    absolute error bound E (in its own normalised units): a factor of an
//    internal child is off by at most E_child + 8 W 2^-126 (flushed matrix
//    entries, flushed lo parts and products; rows of M sum to <= 1), a leaf
//    factor by a few 2^-126 where its value is below 2^-100; the product's
//    bound is u_A (f_B + u_B) + u_B f_A per state, scaled like the product.
//    At the root the bound of the best prior-weighted row, relative to it,
//    is written per (family, category); families whose weighted bound
//    exceeds tau |lnL| are recomputed in FP64 (k_range_flags).
//
// Every mbarrier wait is bounded; on time-out the kernel records a status,
// waits (bounded) for its own copies, frees TMEM and returns.
#include "common.cuh"
#include "tc_ptx.cuh"

#include <math.h>

#include <algorithm>
#include <cstring>

namespace cafe {
namespace {

constexpr int TM = 128;   // families per tile = MMA M = TMEM lanes
#ifndef CAFE_TC_KC
#define CAFE_TC_KC 32
#endif
// K per stage: 32 fp32 = one 128-byte swizzle row, or 16 fp32 = one 64-byte
// swizzle row. Shared memory bounds the operand bytes in flight per SM
// either way; 32-column chunks halve the per-chunk issue and barrier costs.
constexpr int KC = CAFE_TC_KC;
static_assert(KC == 32 || KC == 16, "K chunk of 16 or 32 columns");
constexpr int SC = 32;    // columns per staging tile of the epilogue's TMA stores (128-byte swizzle)
constexpr int MAXST = 4;  // pipeline stages at most
constexpr int NTHREADS = 128;
constexpr int kXN = 9;           // values per family in one pair exchange
// root rows the prior table holds: bins up to 256 states in one CTA, up to
// 512 in a pair (the single-CTA kernel keeps the smaller table: four CTAs
// of the 64-state bin fill an SM's shared memory to the last kilobyte)
template <int NSPLIT>
__host__ __device__ constexpr int prior_rows() { return NSPLIT > 1 ? 512 : 256; }

#ifndef CAFE_TC_CW
#define CAFE_TC_CW 16
#endif
#ifndef CAFE_TC_MINB
#define CAFE_TC_MINB 4
#endif
constexpr int CW = CAFE_TC_CW;   // epilogue columns per TMEM load

__host__ __device__ inline size_t stage_bytes(int Ws) { return (size_t)(2 * TM + 2 * Ws) * KC * sizeof(float); }
__device__ __forceinline__ uint64_t desc_k(const void* p) { return KC == 32 ? tc::desc_sw128(p) : tc::desc_sw64(p); }

// Pipeline stages, also home of the epilogue's two 16 KB staging tiles.
__host__ __device__ inline size_t stages_region(int Ws, int stages) {
    const size_t st = (size_t)stages * stage_bytes(Ws), stg = (size_t)2 * TM * SC * sizeof(float);
    return st > stg ? st : stg;
}

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
    int slot;       // scratch slot of an internal child's vector
    int leaf_col;   // >= 0: leaf
    int mat;
    int tcol;       // TMEM column base of the child's factor, in units of W
};

// One internal node of the post-order walk, as the tile's table in shared
// memory holds it (filled once per tile: the matrices depend on the tile's
// category).
struct NodeInfo {
    int slot;
    int nch;
    int is_root;
    int sat;        // a child's matrix is saturated (rows s >= 1 all zero)
    ChildInfo c[2];
};

// Matrix indices carry this bit when the key is saturated (1 - 2a outside
// (0, 1)): such a matrix is delta(s, 0) in row 0 and zero elsewhere.
constexpr int32_t kSatBit = 1 << 30;

// Per-child source of the factor: TMEM columns, or the unit factor of an
// absent second child.
struct Src {
    bool unit;
    uint32_t taddr;
};

template <int NC>
struct NodeSrc {
    Src s[NC];
    int Eacc;     // sum of the internal children's power-of-two exponents
    bool flag;
    float ue[NC]; // absolute error bound of the child's factor (unscaled units): every state of an
                  // internal child; a leaf's only where its value is below 2^-100
    bool leaf[NC];
};

constexpr float kTiny = 0x1p-126f;   // smallest normal FP32 value

// Handshakes among the NSPLIT CTAs of a cluster (NSPLIT > 1).
struct ClusterX {
    uint32_t seq;    // handshakes so far (the same in every thread of every CTA)
    uint32_t rank;   // this CTA's rank in the cluster
    const float* buf;   // the buffer of the last handshake: [NSPLIT - 1][kXN][TM]
};

// One handshake: this thread's N values go to the same family's slot in
// every other CTA's buffer (sender s at position (s - r - 1) mod NSPLIT of
// receiver r), every thread arrives on every other CTA's barrier
// (releasing its stores), then waits (bounded) for the others'
// arrivals. Handshakes alternate between two buffers and two barriers, so
// no CTA can be more than one handshake ahead of what the others have
// read. Returns false in every thread of the CTA when some wait gave up.
template <int NSPLIT, int N>
__device__ __forceinline__ bool cluster_exchange(ClusterX& cx, float* xbuf, uint64_t* bar_x, const float* mine,
                                                 int tid) {
    const uint32_t slot = cx.seq & 1, parity = (cx.seq >> 1) & 1;
    cx.seq++;
    float* buf = xbuf + (size_t)slot * (NSPLIT - 1) * kXN * TM;
#pragma unroll
    for (int d = 1; d < NSPLIT; ++d) {
        const uint32_t r = (cx.rank + d) % NSPLIT;
        const int p = (int)((cx.rank + NSPLIT - r - 1) % NSPLIT);
#pragma unroll
        for (int i = 0; i < N; ++i) tc::st_cluster_f32(tc::mapa(buf + ((size_t)p * kXN + i) * TM + tid, r), mine[i]);
    }
#pragma unroll
    for (int d = 1; d < NSPLIT; ++d) tc::mbar_arrive_remote(tc::mapa(&bar_x[slot], (cx.rank + d) % NSPLIT));
    const bool ok = tc::mbar_wait_cluster(&bar_x[slot], parity);
    cx.buf = buf;
    return __syncthreads_or(!ok) == 0;
}

// Value i of CTA r's last handshake for this thread's family.
template <int NSPLIT>
__device__ __forceinline__ float xval(const ClusterX& cx, uint32_t r, const float* mine, int i, int tid) {
    if (r == cx.rank) return mine[i];
    const int p = (int)((r + NSPLIT - cx.rank - 1) % NSPLIT);
    return cx.buf[((size_t)p * kXN + i) * TM + tid];
}

// Absolute error bound of factor c at a state whose unscaled value is raw.
template <int NC>
__device__ __forceinline__ float fac_err(const NodeSrc<NC>& ns, int c, float raw) {
    return ns.leaf[c] ? (raw < 0x1p-100f ? ns.ue[c] : 0.0f) : ns.ue[c];
}

// Leaf weights of this thread's family as (column, weight) pairs. Only
// col[0] is set now (weight 1): with an error model k_convert_tc has folded
// the model's deviations into that row of the transposed matrix, so the
// multi-column paths below see col[1], col[2] = -1 (kept: removing them
// changes the walk's register allocation, which then spills).
struct LeafW {
    int col[3];
    float w[3];
};

// The leaf weights of a family with count n (a padding row: none). False
// when the count has no column in the bin (the family is recomputed in FP64).
__device__ __forceinline__ bool leaf_weights(const PruneTcArgs& a, int64_t fam, int n, int S, LeafW& L) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        L.col[d] = -1;
        L.w[d] = 0.0f;
    }
    if (fam < 0) return true;
    bool any = false;
    if (a.err) {
        // the transposed matrix's row n holds the error model's weighted sum
        // over columns 0 .. Wm - 1 (k_convert_tc): the same as the bin's own
        // columns 0 .. S when the deviations stay within S (always for
        // per-family bins, whose S is at least the largest count + 20);
        // otherwise, or with no column of positive weight, FP64 recomputes
        const int h = (a.err_ndev - 1) / 2;
        if (n < 0 || n + h > S) return false;
        const double* pr = a.err + (size_t)(n < a.err_rows ? n : a.err_rows - 1) * a.err_ndev;
        for (int d = 0; d < a.err_ndev; ++d) any |= (n - h + d >= 0) && pr[d] > 0;
        if (any) {
            L.col[0] = n;
            L.w[0] = 1.0f;
        }
    } else if (n >= 0 && n <= S) {
        L.col[0] = n;
        L.w[0] = 1.0f;
        any = true;
    }
    return any;
}

template <int NC>
__device__ __forceinline__ void setup_src(const PruneTcArgs& a, const ChildInfo* ch, int nch, const int* Esh,
                                          const float* Erh, uint32_t tmem_lane, int64_t fam, int tid, int S, int W,
                                          int Wt, const int (&count)[NC], NodeSrc<NC>& ns) {
    ns.Eacc = 0;
    ns.flag = false;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        Src& sc = ns.s[c];
        sc.unit = c >= nch;
        sc.taddr = 0;
        ns.ue[c] = 0.0f;
        ns.leaf[c] = false;
        if (sc.unit) continue;
        const ChildInfo ci = ch[c];
        sc.taddr = tmem_lane + (uint32_t)(ci.tcol * Wt);   // Wt TMEM columns per child
        if (ci.leaf_col < 0) {
            ns.Eacc += Esh[ci.slot * TM + tid];
            ns.ue[c] = Erh[ci.slot * TM + tid] + (float)(8 * W) * kTiny;
            continue;
        }
        ns.leaf[c] = true;
        ns.ue[c] = (a.err ? 8.0f : 2.0f) * kTiny;
        LeafW L;
        if (!leaf_weights(a, fam, count[c], S, L)) ns.flag = true;   // a count past the bin: FP64 recomputes
    }
}

// A leaf child's factor into its TMEM columns (warp-collective): column j
// of this thread's row is sum_d w_d M[s_off + j][col_d], read as row col_d
// of the transposed FP32 matrix tr (pitch Wm). A padding row stores zeros.
// A single column (no error model) is loaded 32 states at a time, all
// loads in flight together: one round trip to L2 per 32 states (W is a
// multiple of 32).
__device__ __noinline__ void gather_leaf(const float* __restrict__ tr, int Wm, const LeafW& L, uint32_t taddr, int W,
                                         int s_off) {
    // tcgen05.st is warp-collective: every lane takes the same branch (the
    // weighted one as soon as any lane of the warp has more than one column)
    if (__all_sync(0xffffffffu, L.col[1] < 0 && L.col[2] < 0)) {
        const float w = L.w[0];
        const float4* p = reinterpret_cast<const float4*>(tr + (size_t)(L.col[0] < 0 ? 0 : L.col[0]) * Wm + s_off);
        for (int col0 = 0; col0 < W; col0 += 32) {
            float4 x[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) x[q] = L.col[0] >= 0 ? __ldg(p + col0 / 4 + q) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                float v[16];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    v[4 * q] = w * x[4 * h + q].x;
                    v[4 * q + 1] = w * x[4 * h + q].y;
                    v[4 * q + 2] = w * x[4 * h + q].z;
                    v[4 * q + 3] = w * x[4 * h + q].w;
                }
                tc::tmem_st16(taddr + (uint32_t)(col0 + 16 * h), v);
            }
        }
    } else {
        for (int col0 = 0; col0 < W; col0 += 16) {
            float v[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] = 0.0f;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if (L.col[d] < 0) continue;
                const float4* p = reinterpret_cast<const float4*>(tr + (size_t)L.col[d] * Wm + s_off + col0);
                const float w = L.w[d];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const float4 x = __ldg(p + q);
                    v[4 * q] = fmaf(w, x.x, v[4 * q]);
                    v[4 * q + 1] = fmaf(w, x.y, v[4 * q + 1]);
                    v[4 * q + 2] = fmaf(w, x.z, v[4 * q + 2]);
                    v[4 * q + 3] = fmaf(w, x.w, v[4 * q + 3]);
                }
            }
            tc::tmem_st16(taddr + (uint32_t)col0, v);
        }
    }
    tc::tmem_wait_st();
}

// A leaf child's factor into its TMEM columns (warp-collective), read from
// the W x W block of the transposed FP32 matrix that a TMA load placed in
// shared memory: W / 32 boxes of W rows x 32 columns, 128-byte swizzled
// (box b holds columns 32 b .. 32 b + 31; the 16-byte piece q of row r
// lies at piece q ^ (r & 7)). Column j of this thread's row is
// sum_d w_d tr[col_d][j], summed in the order of the global-memory gather.
__device__ __forceinline__ void gather_leaf_smem(const float* blk, int W, const LeafW& L, uint32_t taddr) {
    for (int col0 = 0; col0 < W; col0 += 16) {
        float v[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = 0.0f;
        const uint8_t* box = reinterpret_cast<const uint8_t*>(blk + (size_t)(col0 / 32) * W * 32);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int r = L.col[d];
            if (r < 0) continue;
            const uint8_t* row = box + (size_t)r * 128;
            const float w = L.w[d];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int piece = ((col0 & 31) >> 2) + q;
                const float4 x = *reinterpret_cast<const float4*>(row + ((piece ^ (r & 7)) << 4));
                v[4 * q] = fmaf(w, x.x, v[4 * q]);
                v[4 * q + 1] = fmaf(w, x.y, v[4 * q + 1]);
                v[4 * q + 2] = fmaf(w, x.z, v[4 * q + 2]);
                v[4 * q + 3] = fmaf(w, x.w, v[4 * q + 3]);
            }
        }
        tc::tmem_st16(taddr + (uint32_t)col0, v);
    }
    tc::tmem_wait_st();
}

// CW values of a child's factor starting at column col0 (issue only for
// TMEM children; the unit factor is filled at once).
__device__ __forceinline__ void load_unit(uint32_t (&out)[CW]) {
#pragma unroll
    for (int j = 0; j < CW; ++j) out[j] = __float_as_uint(1.0f);
}


// Loads CW columns (from col0) of every child's factor.
template <int NC>
__device__ __forceinline__ void load_children(const NodeSrc<NC>& ns, int col0, uint32_t (&r)[NC][CW]) {
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        if (!ns.s[c].unit) tc::tmem_ld_issue(ns.s[c].taddr + (uint32_t)col0, r[c]);
        else load_unit(r[c]);
    }
    tc::tmem_wait();
}

// Pass 1 over the product of the children's factors, each scaled by
// scl[c]: its maximum over the states (inner node), or the largest
// prior-weighted value over root rows 1..Rf (root; index j = state j + 1).
// The W TMEM columns hold states s_off .. s_off + W - 1.
// Warp-collective (TMEM loads).
template <int NC>
__device__ __forceinline__ void epi_scan(const NodeSrc<NC>& ns, int W, int s_off, bool is_root, int Rf,
                                         const float* prior_f,
                                         const float (&scl)[NC], float& maxp, float& best_f, float& best_p,
                                         float& best_q, float& best_err, float (&fmx)[NC], float (&fmn)[NC]) {
    static_assert(NC == 2, "two factors per node");
    maxp = 0.0f;
    best_f = best_p = best_q = best_err = 0.0f;
    fmx[0] = fmx[1] = 0.0f;
    fmn[0] = fmn[1] = 1.0f;
    for (int col0 = 0; col0 < W; col0 += CW) {
        uint32_t r[NC][CW];
        load_children(ns, col0, r);
        float p[CW];
#pragma unroll
        for (int j = 0; j < CW; ++j) p[j] = 1.0f;
#pragma unroll
        for (int c = 0; c < NC; ++c)
#pragma unroll
            for (int j = 0; j < CW; ++j) p[j] *= __uint_as_float(r[c][j]) * scl[c];
        if (!is_root) {
#pragma unroll
            for (int j = 0; j < CW; ++j) {
                maxp = fmaxf(maxp, p[j]);
                const float r0 = __uint_as_float(r[0][j]), r1 = __uint_as_float(r[1][j]);
                fmx[0] = fmaxf(fmx[0], r0);
                fmx[1] = fmaxf(fmx[1], r1);
                fmn[0] = fminf(fmn[0], r0);
                fmn[1] = fminf(fmn[1], r1);
            }
        } else {
#pragma unroll
            for (int j = 0; j < CW; ++j) {
                const int s = s_off + col0 + j;
                if (s >= 1 && s <= Rf) {
                    maxp = fmaxf(maxp, p[j]);
                    const float q = prior_f[s - 1];
                    const float v = p[j] * q;
                    if (v > best_f) {
                        best_f = v;
                        best_p = p[j];
                        best_q = q;
                    }
                    // range-error bound of this row of the root product
                    const float r0 = __uint_as_float(r[0][j]), r1 = __uint_as_float(r[1][j]);
                    const float f0 = r0 * scl[0], f1 = r1 * scl[1];
                    const float u0 = fac_err(ns, 0, r0) * scl[0], u1 = fac_err(ns, 1, r1) * scl[1];
                    best_err = fmaxf(best_err, (u0 * (f1 + u1) + u1 * f0) * q);
                }
            }
        }
    }
}

// Exact path (warp-collective; lanes that do not need it ignore the
// result): the largest per-state sum of the factors' binary exponents over
// states [s_lo, s_hi) (the W TMEM columns hold states s_off ..). Arguments
// travel by value so the caller's copies stay in registers.
template <int NC>
__device__ __noinline__ int epi_maxexp(const NodeSrc<NC> ns, int W, int s_off, int s_lo, int s_hi) {
    int maxe = -100000;
    for (int col0 = 0; col0 < W; col0 += CW) {
        uint32_t r[NC][CW];
        load_children(ns, col0, r);
        int ex[CW];
#pragma unroll
        for (int j = 0; j < CW; ++j) ex[j] = 0;
#pragma unroll
        for (int c = 0; c < NC; ++c)
#pragma unroll
            for (int j = 0; j < CW; ++j) ex[j] += bexp(__uint_as_float(r[c][j]));
#pragma unroll
        for (int j = 0; j < CW; ++j) {
            const int s = s_off + col0 + j;
            if (s >= s_lo && s < s_hi && ex[j] > maxe) maxe = ex[j];
        }
    }
    return maxe;
}

// Columns c32 .. c32 + SC - 1 of this thread's row of the scaled product
// into a staging tile in the 128-byte-swizzled layout (warp-collective:
// TMEM loads; a thread with write = false loads but writes nothing).
template <int NC>
__device__ __forceinline__ void epi_fill_chunk(const NodeSrc<NC>& ns, int c32, const float (&scl)[NC], float* tile,
                                               int tid, bool write = true) {
    uint8_t* row = reinterpret_cast<uint8_t*>(tile) + (size_t)(tid >> 3) * 1024 + (size_t)(tid & 7) * 128;
    for (int col0 = c32; col0 < c32 + SC; col0 += CW) {
        uint32_t r[NC][CW];
        load_children(ns, col0, r);
        float p[CW];
#pragma unroll
        for (int j = 0; j < CW; ++j) p[j] = 1.0f;
#pragma unroll
        for (int c = 0; c < NC; ++c)
#pragma unroll
            for (int j = 0; j < CW; ++j) p[j] *= __uint_as_float(r[c][j]) * scl[c];
        if (!write) continue;
#pragma unroll
        for (int q = 0; q < CW / 4; ++q) {
            const int j = ((col0 - c32) >> 2) + q;          // 16-byte piece of the 128-byte row
            const int off = (j ^ (tid & 7)) << 4;
            *reinterpret_cast<float4*>(row + off) = make_float4(p[4 * q], p[4 * q + 1], p[4 * q + 2], p[4 * q + 3]);
        }
    }
}

// Pass 2 (inner nodes; every thread of the CTA): the scaled product in FP32
// into a staging tile in the 128-byte-swizzled layout, 32 columns at a
// time, written to the node's vector rows by TMA stores (columns x_off ..
// x_off + W - 1). The parent's GEMM splits it into TF32 hi/lo as it loads
// it (split_row_tf32).
template <int NC>
__device__ __forceinline__ void epi_store(const NodeSrc<NC>& ns, int W, const float (&scl)[NC], float* stg, int tid,
                                          const CUtensorMap* map, int vrow, int x_off) {
    static_assert(NC == 2, "two factors per node");
    // two staging tiles of TM x SC floats, used in turn: a chunk waits only
    // for the stores of the chunk two back
    for (int c32 = 0; c32 < W; c32 += SC) {
        const int b = (c32 / SC) & 1;
        float* tile = stg + (size_t)b * TM * SC;
        if (c32 >= 2 * SC) {
            if (tid == 0) tc::bulk_wait_read1();     // the chunk two back has read this tile
            __syncthreads();
        }
        epi_fill_chunk<NC>(ns, c32, scl, tile, tid);
        tc::fence_proxy_async_shared();
        __syncthreads();
        if (tid == 0) {
            tc::tma_store_2d(map, x_off + c32, vrow, tile);     // one TM-row box
            tc::bulk_commit();
        }
    }
}

// One pass for an inner node whose vector fits the two staging tiles
// (W <= 2 SC, one CTA per tile): the statistics of epi_scan and, at the
// same time, the unscaled product into the staging tiles (tile c32 / SC).
// Warp-collective.
template <int NC>
__device__ __forceinline__ void epi_scan_fill(const NodeSrc<NC>& ns, int W, float* stg, int tid, float& maxp,
                                              float (&fmx)[NC], float (&fmn)[NC]) {
    static_assert(NC == 2, "two factors per node");
    maxp = 0.0f;
    fmx[0] = fmx[1] = 0.0f;
    fmn[0] = fmn[1] = 1.0f;
    for (int c32 = 0; c32 < W; c32 += SC) {
        uint8_t* row = reinterpret_cast<uint8_t*>(stg + (size_t)(c32 / SC) * TM * SC) + (size_t)(tid >> 3) * 1024 +
                       (size_t)(tid & 7) * 128;
        for (int col0 = c32; col0 < c32 + SC; col0 += CW) {
            uint32_t r[NC][CW];
            load_children(ns, col0, r);
            float p[CW];
#pragma unroll
            for (int j = 0; j < CW; ++j) {
                const float r0 = __uint_as_float(r[0][j]), r1 = __uint_as_float(r[1][j]);
                p[j] = (1.0f * r0) * r1;      // the same rounding as epi_fill_chunk with unit scales
                maxp = fmaxf(maxp, p[j]);
                fmx[0] = fmaxf(fmx[0], r0);
                fmx[1] = fmaxf(fmx[1], r1);
                fmn[0] = fminf(fmn[0], r0);
                fmn[1] = fminf(fmn[1], r1);
            }
#pragma unroll
            for (int q = 0; q < CW / 4; ++q) {
                const int j = ((col0 - c32) >> 2) + q;
                const int off = (j ^ (tid & 7)) << 4;
                *reinterpret_cast<float4*>(row + off) = make_float4(p[4 * q], p[4 * q + 1], p[4 * q + 2], p[4 * q + 3]);
            }
        }
    }
}

// This thread's staged row times a power of two s (exact unless a value
// was already below the FP32 normal range before the scaling).
__device__ __forceinline__ void rescale_row(float* stg, int tid, int W, float s) {
    for (int c32 = 0; c32 < W; c32 += SC) {
        float4* row = reinterpret_cast<float4*>(reinterpret_cast<uint8_t*>(stg + (size_t)(c32 / SC) * TM * SC) +
                                                (size_t)(tid >> 3) * 1024 + (size_t)(tid & 7) * 128);
#pragma unroll
        for (int q = 0; q < SC / 4; ++q) {
            float4 v = row[q];
            v.x *= s;
            v.y *= s;
            v.z *= s;
            v.w *= s;
            row[q] = v;
        }
    }
}

// Row `row` of an operand chunk holds the FP32 node vector (KC values, the
// 16-byte pieces in swizzled order); write its TF32 hi part in place and the
// lo part at the same position of `lo`: hi = tf32(v), lo = tf32(v - hi).
__device__ __forceinline__ void split_row_tf32(float* hi, float* lo, int row) {
    constexpr int NP = KC / 4;   // 16-byte pieces per row
    float4* h = reinterpret_cast<float4*>(hi + (size_t)row * KC);
    float4* l = reinterpret_cast<float4*>(lo + (size_t)row * KC);
#pragma unroll
    for (int q = 0; q < NP; ++q) {
        const int p = q ^ (row & (NP - 1));   // neighbouring rows start on different banks
        const float4 v = h[p];
        float4 a, b;
        a.x = tc::round_tf32_bits(v.x);
        a.y = tc::round_tf32_bits(v.y);
        a.z = tc::round_tf32_bits(v.z);
        a.w = tc::round_tf32_bits(v.w);
        b.x = tc::round_tf32_bits(v.x - a.x);
        b.y = tc::round_tf32_bits(v.y - a.y);
        b.z = tc::round_tf32_bits(v.z - a.z);
        b.w = tc::round_tf32_bits(v.w - a.w);
        h[p] = a;
        l[p] = b;
    }
}

// NSPLIT = 2 or 4: a cluster of NSPLIT CTAs shares each tile -- bins of
// 384 and 512 states, whose two children's factors would need 2 W > 512
// TMEM columns, and sparse bins of 128 to 256 states, whose few tiles would
// otherwise walk the tree on few SMs. CTA h keeps output states
// [h Wn, h Wn + Wn), Wn = W / NSPLIT, of both children in TMEM (B operand:
// those rows of each matrix; A operand: the child's whole vector). The
// per-family statistics the epilogue's decisions rest on (maxima, minima,
// the best root row, the exponent sums) are exchanged through distributed
// shared memory, so every CTA takes the same decisions and scales its
// states alike; each stores its columns of the node vector, and a
// handshake after the stores' completion lets the parent's GEMM read them
// all. Every handshake wait is bounded.
template <int NSPLIT>
__global__ void __launch_bounds__(NTHREADS, NSPLIT == 1 ? CAFE_TC_MINB : 1)
    k_prune_tc(const __grid_constant__ CUtensorMap map_mat, const __grid_constant__ CUtensorMap map_vec,
               const __grid_constant__ CUtensorMap map_vst, const __grid_constant__ CUtensorMap map_tr,
               const PruneTcArgs a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    __shared__ __align__(8) uint64_t bar_full[MAXST], bar_empty[MAXST], bar_done, bar_drain, bar_leaf;
    __shared__ __align__(8) uint64_t bar_x[2];     // cluster handshakes (NSPLIT > 1), in turn
    // [2][NSPLIT - 1][kXN][TM]: the other CTAs' values, per handshake
    __shared__ float xbuf[NSPLIT > 1 ? 2 * (NSPLIT - 1) * kXN * TM : 1];
    __shared__ uint32_t tmem_sh;
    __shared__ int abort_sh;
    __shared__ float prior_f[prior_rows<NSPLIT>()];

    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t h = NSPLIT > 1 ? tc::cluster_rank() : 0u;   // this CTA's share of the states
    const int cid = (int)blockIdx.x / NSPLIT, n_cl = (int)gridDim.x / NSPLIT;
    const int Wm = a.Wm;
    const int NS = a.stages;
    const TreePlan& P = a.plan;
    const size_t sbytes = stage_bytes(a.Ws);
    int* Esh = reinterpret_cast<int*>(smem + stages_region(a.Ws, NS));   // [n_slots][TM]
    float* Erh = reinterpret_cast<float*>(Esh + (size_t)a.n_slots * TM);   // [n_slots][TM] error bounds
    NodeInfo* nodes = reinterpret_cast<NodeInfo*>(Erh + (size_t)a.n_slots * TM);   // [n_internal]

    for (int j = tid; j < prior_rows<NSPLIT>(); j += NTHREADS) prior_f[j] = j < a.n_prior ? (float)a.prior[j] : 0.0f;
    if (warp == 0) tc::tmem_alloc(&tmem_sh, (uint32_t)a.tmem_cols);
    if (tid == 0) {
        for (int q = 0; q < MAXST; ++q) {
            tc::mbar_init(&bar_full[q], 1);
            tc::mbar_init(&bar_empty[q], 1);
        }
        tc::mbar_init(&bar_done, 1);
        tc::mbar_init(&bar_drain, 1);
        tc::mbar_init(&bar_leaf, 1);
        if (NSPLIT > 1) {
            // one arrival per thread of every other CTA (a count of at least 1)
            tc::mbar_init(&bar_x[0], (NSPLIT > 1 ? NSPLIT - 1 : 1) * NTHREADS);
            tc::mbar_init(&bar_x[1], (NSPLIT > 1 ? NSPLIT - 1 : 1) * NTHREADS);
        }
        tc::mbar_init_fence();
        abort_sh = 0;
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    // every CTA's barriers are initialised before the first remote arrival
    if (NSPLIT > 1) tc::cluster_sync_all();
    ClusterX cx{0u, h, nullptr};
    const uint32_t tmem = tmem_sh;
    const uint32_t lane_base = (uint32_t)(32 * warp) << 16;

    uint32_t g = 0;          // chunks issued so far (same in every thread)
    uint32_t dn = 0;         // completions of bar_done observed (all threads)
    uint32_t ln = 0;         // leaf-block loads issued (all threads)
    int leaf_pending = 0;    // thread 0: a leaf-block load not yet waited for
    int last_full[MAXST] = {0, 0, 0, 0};            // thread 0: stage has a TMA not yet waited for
    uint32_t last_full_parity[MAXST] = {0, 0, 0, 0};
    // node-vector rows of this tile (the CTAs of a cluster share them, each
    // writing its own columns)
    const int64_t vrow_cta = a.vrow_base + (int64_t)cid * a.n_slots * TM;
    // thread 0's clocks (CAFE_TC_PHASES): [0..4] node phases, [5] tile-nodes,
    // [6] waits for a free stage, [7] waits for a chunk's TMA, [8] split and
    // barriers, [9] MMA issue, [10] wait for the node's last MMAs, [11] chunks,
    // [12] wait for the previous node's stores, [13] leaf gathers, [14] the MMA
    // issuer's wait for a chunk, [15] TMA issue, [16] and [17] the barriers
    // after the chunk loop and after the last MMAs
    // (kept in shared memory: only thread 0 touches them, and they cost no registers)
    __shared__ unsigned long long ph[kPhases];
    if (tid == 0)
        for (int q = 0; q < kPhases; ++q) ph[q] = 0;
    const bool timing = a.phase_clocks != nullptr && tid == 0;

    // one CTA per tile: CTAs take tiles from a counter, so a CTA that starts
    // late (its SM was held by another bin's launch) takes fewer; a cluster's
    // CTAs walk their tiles in lockstep and keep the fixed stride
    __shared__ int t_sh;
    auto next_tile = [&](int done) -> int {
        if (NSPLIT > 1 || !a.tile_counter) return done < 0 ? cid : done + n_cl;
        if (tid == 0) t_sh = atomicAdd(a.tile_counter, 1);
        __syncthreads();
        const int t = t_sh;
        __syncthreads();     // (t_sh is rewritten at the next tile)
        return t;
    };
    for (int t = next_tile(-1); t < a.n_tiles; t = next_tile(t)) {
        const PruneTile tile = a.tiles[t];
        const int cnt = tile.count, k = tile.k, S = tile.S, W = tile.S + 1;
        const int Wn = W / NSPLIT;              // output states (TMEM columns) per child in this CTA
        const int s_off = (int)h * Wn;          // this CTA's first output state
        const int64_t fam = tid < cnt ? a.perm[tile.first + tid] : -1;
        const int Rf = (fam >= 0 && a.fam_R) ? a.fam_R[fam] : tile.R;
        const int32_t* mi = a.mat_index + (size_t)k * P.n_nodes;
        const uint32_t idesc = tc::idesc_tf32(TM, Wn);
        bool flag = false;
        bool dead = false;   // an exact zero vector through a saturated branch: the family's term is 0

        // the tile's walk: children, matrices and slots of every internal node
        for (int ii = tid; ii < P.n_internal; ii += NTHREADS) {
            const int v = P.internal[ii];
            NodeInfo e;
            e.slot = P.slot[v];
            e.is_root = v == P.root;
            e.nch = P.cstart[ii + 1] - P.cstart[ii];
            e.sat = 0;
            for (int c = 0; c < 2; ++c) {
                ChildInfo ci{0, -1, 0, c};
                if (c < e.nch) {
                    const int ch = P.child[P.cstart[ii] + c];
                    ci.slot = P.slot[ch];
                    ci.leaf_col = P.leaf_col[ch];
                    ci.mat = mi[ch] & ~kSatBit;
                    e.sat |= (mi[ch] & kSatBit) != 0;
                }
                e.c[c] = ci;
            }
            nodes[ii] = e;
        }
        __syncthreads();
        const int32_t* fam_counts = a.counts + (size_t)(fam >= 0 ? fam : 0) * P.n_leaves;
        int cnt_next[2] = {0, 0};
#pragma unroll
        for (int c = 0; c < 2; ++c)
            if (fam >= 0 && c < nodes[0].nch && nodes[0].c[c].leaf_col >= 0)
                cnt_next[c] = __ldg(fam_counts + nodes[0].c[c].leaf_col);

        for (int ii = 0; ii < P.n_internal; ++ii) {
            const NodeInfo nd = nodes[ii];
            const bool is_root = nd.is_root != 0;
            const int vs = nd.slot;
            const int nch = nd.nch;
            const long long ts = timing ? clock64() : 0;
            // the previous nodes' TMA stores must be complete before this node
            // overwrites their staging tile or reads their rows back (in a
            // cluster: the other CTAs' columns as well)
            if (tid == 0) tc::bulk_wait0();
            if (timing) ph[12] += clock64() - ts;
            if (NSPLIT > 1) {
                if (tid == 0) tc::fence_proxy_async_global();
                __syncthreads();
                if (!cluster_exchange<NSPLIT, 0>(cx, xbuf, bar_x, nullptr, tid)) {
                    if (tid == 0) {
                        atomicExch(a.status, 1);
                        abort_sh = 1;
                    }
                }
                if (tid == 0) tc::fence_proxy_async_global();
            }
            // child sources
            NodeSrc<2> ns2;
            const int cnt_cur[2] = {cnt_next[0], cnt_next[1]};
            setup_src<2>(a, nd.c, nch, Esh, Erh, tmem + lane_base, fam, tid, S, W, Wn, cnt_cur, ns2);
            // counts of the next node's leaves, in flight during this node
            if (ii + 1 < P.n_internal) {
                const NodeInfo& nx = nodes[ii + 1];
#pragma unroll
                for (int c = 0; c < 2; ++c)
                    cnt_next[c] = (fam >= 0 && c < nx.nch && nx.c[c].leaf_col >= 0) ? __ldg(fam_counts + nx.c[c].leaf_col) : 0;
            }
            __syncthreads();

            // ---------------- one GEMM per internal child into TMEM ----------------
            // K chunks of the internal children form one list (CTA-uniform);
            // thread 0 runs the TMA loads up to NS - 1 chunks ahead of the MMAs.
            // Leaf children's factors are gathered into TMEM meanwhile.
            long long t0 = timing ? clock64() : 0;
            {
                const int kpc = W / KC;             // K chunks per child
                int nk[2];
#pragma unroll
                for (int c = 0; c < 2; ++c) nk[c] = (c < nch && nd.c[c].leaf_col < 0) ? kpc : 0;
                const int n0 = nk[0];
                const int n_chunks = n0 + nk[1];
                // leaf factors (CTA-uniform): after the first chunk's loads are
                // issued, or at once when the node runs no GEMM
                // bins of up to 64 states (one CTA per tile): each leaf child's
                // W x W block of the transposed matrix comes by TMA into a free
                // operand area of chunk 0's stage (the lo operand, which chunk
                // 0's split writes only after the gather; a node without GEMMs
                // uses the hi area too), while chunk 0's operands load
                const bool smem_leaf = NSPLIT == 1 && W * W <= TM * KC;
                int n_leaf = 0;
#pragma unroll
                for (int c = 0; c < 2; ++c) n_leaf += (c < nch && nd.c[c].leaf_col >= 0) ? 1 : 0;
                float* leaf_area[2];
                {
                    float* a_hi = reinterpret_cast<float*>(smem + (g % (uint32_t)NS) * sbytes);
                    leaf_area[0] = n_chunks ? a_hi + TM * KC : a_hi;
                    leaf_area[1] = a_hi + TM * KC;
                }
                const bool leaf_tma = smem_leaf && n_leaf > 0;
                if (leaf_tma && tid == 0 && !abort_sh) {
                    tc::fence_proxy_async_shared();     // this CTA's earlier reads of the area come first
                    tc::mbar_expect_tx(&bar_leaf, (uint32_t)(n_leaf * W * W * sizeof(float)));
                    int q = 0;
#pragma unroll
                    for (int c = 0; c < 2; ++c)
                        if (c < nch && nd.c[c].leaf_col >= 0) {
                            for (int b = 0; b < W / 32; ++b)
                                tc::tma_load_2d(leaf_area[q] + (size_t)b * W * 32, &map_tr, 32 * b, nd.c[c].mat * Wm, &bar_leaf);
                            ++q;
                        }
                    leaf_pending = 1;
                }
                auto gather_leaves = [&]() {
                    if (__shfl_sync(0xffffffffu, abort_sh, 0)) return;   // warp-uniform: the stores are collective
                    if (leaf_tma) {
                        const bool ok = tc::mbar_wait(&bar_leaf, ln & 1);
                        if (!__all_sync(0xffffffffu, ok)) {
                            if ((tid & 31) == 0) {
                                atomicExch(a.status, 1);
                                abort_sh = 1;
                            }
                            return;
                        }
                        if (tid == 0) leaf_pending = 0;
                    }
                    int q = 0;
#pragma unroll
                    for (int c = 0; c < 2; ++c)
                        if (c < nch && nd.c[c].leaf_col >= 0) {
                            LeafW L;
                            leaf_weights(a, fam, cnt_cur[c], S, L);
                            if (leaf_tma) gather_leaf_smem(leaf_area[q], W, L, ns2.s[c].taddr);
                            else gather_leaf(a.mat_tr + (size_t)nd.c[c].mat * Wm * Wm, Wm, L, ns2.s[c].taddr, Wn, s_off);
                            ++q;
                        }
                };
                if (n_chunks == 0) {
                    const long long tg = timing ? clock64() : 0;
                    gather_leaves();
                    if (timing) ph[13] += clock64() - tg;
                }
                for (int i = 0; i < n_chunks + NS - 1; ++i) {
                    // ---- produce chunk i ----
                    if (i < n_chunks) {
                        const int c = i < n0 ? 0 : 1;
                        const int kc = c == 0 ? i : i - n0;
                        const ChildInfo chi = nd.c[c];
                        const uint32_t cg = g + (uint32_t)i;
                        const int st = (int)(cg % (uint32_t)NS);
                        const uint32_t u = cg / (uint32_t)NS;
                        uint8_t* base = smem + st * sbytes;
                        float* Ahi = reinterpret_cast<float*>(base);
                        float* Alo = Ahi + TM * KC;
                        float* Bhi = Alo + TM * KC;     // the matrix box lands hi, then lo (Bhi + Ws KC)
                        // the first NS chunks of a node find their stages free: the
                        // previous node's MMAs completed before its epilogue and its
                        // staging-tile stores were waited for at the node start
                        const long long te = timing ? clock64() : 0;
                        if (tid == 0 && !abort_sh && i >= NS && !tc::mbar_wait(&bar_empty[st], (u - 1) & 1)) {
                            atomicExch(a.status, 1);
                            abort_sh = 1;
                        }
                        if (timing) ph[6] += clock64() - te;
                        const long long ti = timing ? clock64() : 0;
                        if (tid == 0 && !abort_sh) {
                            tc::mbar_expect_tx(&bar_full[st], (uint32_t)((TM + 2 * Wn) * KC * sizeof(float)));
                            // the FP32 node vector lands in the hi operand; the
                            // consumer splits it into hi and lo in place
                            // one box each: the vector's TM rows, the matrices' Wn rows
                            // (TMA issue is slow enough per instruction to count)
                            const int vrow = (int)(vrow_cta + (int64_t)chi.slot * TM);
                            tc::tma_load_2d(Ahi, &map_vec, kc * KC, vrow, &bar_full[st]);
                            const int mrow = chi.mat * Wm + s_off;     // this CTA's output states
                            tc::tma_load_3d(Bhi, &map_mat, kc * KC, mrow, 0, &bar_full[st]);   // hi, then lo at Blo
                            last_full[st] = 1;
                            last_full_parity[st] = u & 1;
                        }
                        if (timing) ph[15] += clock64() - ti;
                        if (i == 0) {
                            const long long tg = timing ? clock64() : 0;
                            gather_leaves();
                            // the leaf block lies in chunk 0's lo operand area, which
                            // chunk 0's split overwrites: every thread's reads first
                            if (leaf_tma) __syncthreads();
                            if (timing) ph[13] += clock64() - tg;
                        }
                    }
                    // ---- consume chunk j = i - (NS - 1) ----
                    const int j = i - (NS - 1);
                    // the child's FP32 vector chunk: every thread waits for it
                    // and splits its own row into the TF32 hi/lo operands
                    if (j >= 0) {
                        const uint32_t cg = g + (uint32_t)j;
                        const int st = (int)(cg % (uint32_t)NS);
                        float* Ahi = reinterpret_cast<float*>(smem + st * sbytes);
                        const long long tf = timing ? clock64() : 0;
                        const bool ok = abort_sh || tc::mbar_wait(&bar_full[st], (cg / (uint32_t)NS) & 1);
                        const long long tf1 = timing ? clock64() : 0;
                        // (a thread whose wait gave up stops the CTA: the MMAs are
                        // issued only if no thread did, which the barrier shows)
                        if (!ok) {
                            atomicExch(a.status, 1);
                            abort_sh = 1;
                        } else if (!abort_sh) {
                            split_row_tf32(Ahi, Ahi + TM * KC, tid);
                            tc::fence_proxy_async_shared();
                        }
                        __syncthreads();
                        if (timing) {
                            ph[7] += tf1 - tf;
                            ph[8] += clock64() - tf1;
                            ph[11] += 1;
                        }
                    }
                    if (j >= 0 && tid == 0 && !abort_sh) {
                        const int c = j < n0 ? 0 : 1;
                        const bool first = j == 0 || j == n0;
                        const ChildInfo chi = nd.c[c];
                        const uint32_t cg = g + (uint32_t)j;
                        const int st = (int)(cg % (uint32_t)NS);
                        const uint32_t u = cg / (uint32_t)NS;
                        uint8_t* base = smem + st * sbytes;
                        const float* Ahi = reinterpret_cast<const float*>(base);
                        const float* Alo = Ahi + TM * KC;
                        const float* Bhi = Alo + TM * KC;
                        const float* Blo = Bhi + a.Ws * KC;
                        const long long tm = timing ? clock64() : 0;
                        if (tc::mbar_wait(&bar_full[st], u & 1)) {
                            last_full[st] = 0;
                            tc::fence_after();
                            if (timing) ph[14] += clock64() - tm;
                            const uint32_t d = tmem + (uint32_t)(chi.tcol * Wn);
#pragma unroll
                            for (int ks = 0; ks < KC / 8; ++ks) {
                                const uint64_t ah = desc_k(Ahi + ks * 8), al = desc_k(Alo + ks * 8);
                                const uint64_t bh = desc_k(Bhi + ks * 8), bl = desc_k(Blo + ks * 8);
                                tc::mma_tf32(d, ah, bh, idesc, (first && ks == 0) ? 0u : 1u);
                                tc::mma_tf32(d, ah, bl, idesc, 1);
                                tc::mma_tf32(d, al, bh, idesc, 1);
                            }
                            tc::mma_commit(&bar_empty[st]);
                            if (timing) ph[9] += clock64() - tm;
                        } else {
                            atomicExch(a.status, 1);
                            abort_sh = 1;
                        }
                    }
                }
                if (tid == 0 && !abort_sh) tc::mma_commit(&bar_done);
                g += (uint32_t)n_chunks;        // every thread tracks the stage sequence
                if (leaf_tma) ln++;
                const long long tq = timing ? clock64() : 0;
                __syncthreads();
                const long long td = timing ? clock64() : 0;
                if (timing) ph[16] += td - tq;
                if (!abort_sh) {
                    // (a test hook can make this wait give up after limit - 1 polls)
                    if (!tc::mbar_wait(&bar_done, dn & 1, a.debug_wait_limit > 0 ? a.debug_wait_limit - 1 : (1 << 24))) {
                        atomicExch(a.status, 2);
                        abort_sh = 1;
                    }
                }
                dn++;
                if (timing) ph[10] += clock64() - td;
                tc::fence_after();
            }
            const long long tz = timing ? clock64() : 0;
            __syncthreads();
            if (timing) ph[17] += clock64() - tz;
            if (abort_sh) break;
            long long t1 = timing ? clock64() : 0;

            // ---------------- epilogue: product over children ----------------
            float scl[2] = {1.0f, 1.0f};
            int E = ns2.Eacc;
            bool nflag = ns2.flag;
            float maxp, bf, bp, bq, be, fmx[2], fmn[2];
            // one CTA per tile and a vector that fits the staging tiles: the
            // statistics and the unscaled product in one pass over TMEM
            const bool fused = NSPLIT == 1 && !is_root && Wn <= 2 * SC;
            float* stg = reinterpret_cast<float*>(smem);     // stage 0 holds the two staging tiles
            if (fused) {
                epi_scan_fill<2>(ns2, Wn, stg, tid, maxp, fmx, fmn);
                bf = bp = bq = be = 0.0f;
            } else {
                epi_scan<2>(ns2, Wn, s_off, is_root, Rf, prior_f, scl, maxp, bf, bp, bq, be, fmx, fmn);
            }
            if (NSPLIT > 1) {
                // every CTA's statistics: maxima, minima, the best root row
                // (combined in rank order, so a tie goes to the first in state
                // order, as in one CTA's scan)
                const float mine[kXN] = {maxp, fmx[0], fmx[1], fmn[0], fmn[1], bf, bp, bq, be};
                if (!cluster_exchange<NSPLIT, kXN>(cx, xbuf, bar_x, mine, tid)) {
                    if (tid == 0) {
                        atomicExch(a.status, 1);
                        abort_sh = 1;
                    }
                    cx.buf = nullptr;
                }
                if (cx.buf) {
#pragma unroll
                    for (int r = 0; r < NSPLIT; ++r) {
                        const float f = xval<NSPLIT>(cx, r, mine, 5, tid);
                        maxp = fmaxf(maxp, xval<NSPLIT>(cx, r, mine, 0, tid));
                        fmx[0] = fmaxf(fmx[0], xval<NSPLIT>(cx, r, mine, 1, tid));
                        fmx[1] = fmaxf(fmx[1], xval<NSPLIT>(cx, r, mine, 2, tid));
                        fmn[0] = fminf(fmn[0], xval<NSPLIT>(cx, r, mine, 3, tid));
                        fmn[1] = fminf(fmn[1], xval<NSPLIT>(cx, r, mine, 4, tid));
                        be = fmaxf(be, xval<NSPLIT>(cx, r, mine, 8, tid));
                        if (r == 0 || f > bf) {
                            bf = f;
                            bp = xval<NSPLIT>(cx, r, mine, 6, tid);
                            bq = xval<NSPLIT>(cx, r, mine, 7, tid);
                        }
                    }
                }
            }
            // Without an error model, every state-0 entry is exact: row 0 of
            // every matrix is delta(s, 0), so L[0] is 1 (scaled by a power of
            // two) when all leaves below are 0, else 0, and it is then the
            // vector's largest entry. A saturated child's factor is zero at
            // every state s >= 1, so a product that is zero everywhere here
            // is exactly zero in FP64 as well: the family's term is 0.
            if (nd.sat && !a.err && !(maxp > 0.0f)) dead = true;
            const bool need = is_root ? !(bf > 0.0f) : !(maxp >= 0x1p-120f);
            if (!is_root && !need && maxp < 0x1p-32f) {
                // bring this row's maximum back to [0.5, 1)
                const int kk = -bexp(maxp);
                scl[0] = pow2f(kk);
                E -= kk;
            }
            // (in a pair the decision is the same in both CTAs: it rests on the
            // exchanged statistics of the same families)
            if (NSPLIT > 1 ? __syncthreads_or(need) != 0 : __any_sync(0xffffffffu, need)) {
                // underflow: rescale by the largest per-state exponent sum, so the
                // product's maximum is in [2^-2, 1) unless the factors are more
                // than 2^250 apart (then FP64 recomputes the family)
                int maxe = epi_maxexp<2>(ns2, Wn, s_off, is_root ? 1 : 0, is_root ? Rf + 1 : W);
                if (NSPLIT > 1) {
                    const float mine[1] = {__int_as_float(maxe)};
                    if (cluster_exchange<NSPLIT, 1>(cx, xbuf, bar_x, mine, tid)) {
#pragma unroll
                        for (int r = 0; r < NSPLIT; ++r) maxe = max(maxe, __float_as_int(xval<NSPLIT>(cx, r, mine, 0, tid)));
                    } else if (tid == 0) {
                        atomicExch(a.status, 1);
                        abort_sh = 1;
                    }
                }
                if (need) {
                    if (maxe < -250) {
                        nflag = true;
                        maxe = 0;
                    }
                    const int sh = -maxe, part = sh / 2;
                    scl[0] = pow2f(part + (sh - part * 2));
                    scl[1] = pow2f(part);
                    E = ns2.Eacc + maxe;
                }
                if (is_root) {
                    float m2, f2, p2, q2, e2, x2[2], n2[2];
                    epi_scan<2>(ns2, Wn, s_off, true, Rf, prior_f, scl, m2, f2, p2, q2, e2, x2, n2);
                    if (NSPLIT > 1) {
                        const float mine[4] = {f2, p2, q2, e2};
                        if (cluster_exchange<NSPLIT, 4>(cx, xbuf, bar_x, mine, tid)) {
#pragma unroll
                            for (int r = 0; r < NSPLIT; ++r) {
                                const float f = xval<NSPLIT>(cx, r, mine, 0, tid);
                                e2 = fmaxf(e2, xval<NSPLIT>(cx, r, mine, 3, tid));
                                if (r == 0 || f > f2) {
                                    f2 = f;
                                    p2 = xval<NSPLIT>(cx, r, mine, 1, tid);
                                    q2 = xval<NSPLIT>(cx, r, mine, 2, tid);
                                }
                            }
                        } else if (tid == 0) {
                            atomicExch(a.status, 1);
                            abort_sh = 1;
                        }
                    }
                    if (need) {
                        bf = f2;
                        bp = p2;
                        bq = q2;
                        be = e2;
                    }
                }
            }
            long long t2 = timing ? clock64() : 0;
            flag |= nflag && !dead;
            if (!is_root) {
                float flush = kTiny;   // values flushed on the store, in the stored vector's units
                if (fused) {
                    // a family on the exact path writes its row again with the
                    // factors scaled before the product (the TMEM loads are
                    // warp-collective, the writes its own); a family brought back
                    // to [0.5, 1) is scaled in place, where a value below 2^-126
                    // before the scaling was flushed. Either way a family's row
                    // depends on its own values only.
                    if (__any_sync(0xffffffffu, need)) {
                        for (int c32 = 0; c32 < Wn; c32 += SC)
                            epi_fill_chunk<2>(ns2, c32, scl, stg + (size_t)(c32 / SC) * TM * SC, tid, need);
                    }
                    if (!need && scl[0] != 1.0f) {
                        rescale_row(stg, tid, Wn, scl[0]);
                        flush = kTiny * scl[0];
                    }
                    tc::fence_proxy_async_shared();
                    __syncthreads();
                    if (tid == 0) {
                        const int vrow = (int)(vrow_cta + (int64_t)vs * TM);
                        for (int c32 = 0; c32 < Wn; c32 += SC) tc::tma_store_2d(&map_vst, c32, vrow, stg + (size_t)(c32 / SC) * TM * SC);
                        tc::bulk_commit();
                    }
                } else {
                    epi_store<2>(ns2, Wn, scl, stg, tid, &map_vst, (int)(vrow_cta + (int64_t)vs * TM), s_off);
                }
                Esh[vs * TM + tid] = E;
                // the stored vector's bound, from the factors' maxima: u_A (f_B + u_B)
                // + u_B f_A over all states, with a leaf factor's u counted only
                // if it fell below 2^-100 somewhere; plus values flushed on the store
                float u0 = ns2.ue[0], u1 = ns2.ue[1];
                if (ns2.leaf[0] && !(fmn[0] < 0x1p-100f)) u0 = 0.0f;
                if (ns2.leaf[1] && !(fmn[1] < 0x1p-100f)) u1 = 0.0f;
                u0 *= scl[0];
                u1 *= scl[1];
                const float ev = u0 * (fmx[1] * scl[1] + u1) + u1 * (fmx[0] * scl[0]);
                Erh[vs * TM + tid] = fminf(ev + flush, 1e30f);
            } else if (fam >= 0 && h == 0) {     // (a cluster's first CTA writes the term)
                double o = NAN;
                const double best = (double)bp * (double)bq;
                if (dead) o = a.model == 0 ? -INFINITY : NAN;   // log 0 (base) / a failed family (gamma)
                else if (best > 0.0 && !flag)
                    o = log(best * a.cat_probs[k]) + (double)E * 0.69314718055994530942;
                else flag = true;
                a.out[(size_t)fam * a.K + k] = o;
                if (a.out_err) a.out_err[(size_t)fam * a.K + k] = (dead || flag || !(bf > 0.0f)) ? 0.0f : be / bf;
            }
            long long t3 = timing ? clock64() : 0;
            tc::fence_before();
            __syncthreads();
            tc::fence_after();
            if (timing) {
                const long long t4 = clock64();
                ph[0] += t0 - ts;     // child setup
                ph[1] += t1 - t0;     // GEMMs (issue, TMA and MMA latency)
                ph[2] += t2 - t1;     // epilogue scan (and exact rescale)
                ph[3] += t3 - t2;     // epilogue store (TMA) or root weighting
                ph[4] += t4 - t3;     // end-of-node fence and barrier
                ph[5] += 1;           // tile-nodes
            }
        }
        if (flag && fam >= 0 && h == 0) {
            atomicOr(&a.flags[fam], 1);
            if (a.term_flags) a.term_flags[(size_t)fam * a.K + k] = 1;   // this category term
            atomicOr(a.status + 3, 1);     // "some family is flagged"
        }
        __syncthreads();
        if (abort_sh) break;
    }

    if (timing)
        for (int q = 0; q < kPhases; ++q) atomicAdd(&a.phase_clocks[q], ph[q]);
    // teardown: no copy of ours may still be landing when TMEM goes away
    if (tid == 0) tc::bulk_wait0();
    tc::fence_before();
    __syncthreads();
    // after a time-out the MMAs this thread issued may still be running:
    // they complete before TMEM goes away (a full-length bounded wait)
    if (abort_sh && tid == 0) {
        tc::mma_commit(&bar_drain);
        tc::mbar_wait(&bar_drain, 0, 1 << 24);
    }
    if (abort_sh && tid == 0) {
        for (int q = 0; q < MAXST; ++q)
            if (q < NS && last_full[q]) tc::mbar_wait(&bar_full[q], last_full_parity[q], 1 << 20);
        if (leaf_pending) tc::mbar_wait(&bar_leaf, ln & 1, 1 << 20);
    }
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, (uint32_t)a.tmem_cols);
    // no CTA of a cluster exits while another may still write into its
    // shared memory or arrive on its barriers (every wait before this is
    // bounded)
    if (NSPLIT > 1) tc::cluster_sync_all();
}

// FP64 matrix -> TF32 hi/lo operands (row-major, pitch Wm) and the FP32
// transpose tr[c][s] = M[s][c] (a leaf factor, column c of M, as one row).
// With an error model the transpose's row c is already the leaf factor of
// an observed count c: sum_d w_d(c) M[s][c - h + d] over the model's 2h + 1
// deviations, in deviation order, as FP32 products and sums (the walk then
// reads one row per leaf, whatever the model's width). A block converts a
// band of 32 rows of one matrix, 32 columns (plus h on either side) at a
// time through a shared-memory tile, so the row-major and the transposed
// stores both write whole 128-byte lines. Wm is a multiple of 32.
__global__ void __launch_bounds__(256) k_convert_tc(const ConvertJob* __restrict__ jobs, TcBuffers b) {
    constexpr int TW = 32 + 2 * kMaxErrHalf;
    __shared__ float tile[32][TW + 1];
    __shared__ float wsh[32][2 * kMaxErrHalf + 1];   // the band's rows' deviation weights (0: skipped)
    const int Wm = b.Wm;
    const int bands = Wm / 32;
    const ConvertJob J = jobs[blockIdx.x / bands];
    const int s0 = (int)(blockIdx.x % bands) * 32;
    const size_t base = (size_t)J.mat * Wm * Wm;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int h = b.err ? (b.err_ndev - 1) / 2 : 0;
    // only what the walk reads: hi/lo for internal children's branches, the
    // transpose for leaves' (block-uniform)
    const bool want_hl = (J.what & 1) != 0, want_tr = (J.what & 2) != 0;
    // the deviations' columns either side of a 32-column step (within
    // 0 .. Wm - 1): lane tx < 2h loads column c0 + hoff into tile column hcol
    const bool halo = want_tr && tx < 2 * h;
    const int hoff = tx < h ? tx - h : 32 + (tx - h);
    const int hcol = tx < h ? tx : 32 + tx;
    for (int c0 = 0; c0 < Wm; c0 += 32) {
        // the thread's four rows (ty + 8 i) of this step, and their halo
        // entries, are loaded before any store (the stores might alias the
        // source as far as the compiler knows), so the loads overlap
        const int c = c0 + tx, cc = c0 + hoff;
        float x[4], xh[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) x[i] = (float)J.src[(size_t)(s0 + ty + 8 * i) * J.ld + c];
        if (halo) {
#pragma unroll
            for (int i = 0; i < 4; ++i)
                xh[i] = (cc >= 0 && cc < Wm) ? (float)J.src[(size_t)(s0 + ty + 8 * i) * J.ld + cc] : 0.0f;
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int r = ty + 8 * i, s = s0 + r;
            if (want_hl) {
                const float hi = tc::round_tf32(x[i]);
                b.hi[base + (size_t)s * Wm + c] = hi;
                b.lo[base + (size_t)s * Wm + c] = tc::round_tf32(x[i] - hi);
            }
            if (!want_tr) continue;
            tile[r][h + tx] = x[i];
            if (halo) tile[r][hcol] = xh[i];
        }
        if (!want_tr) continue;
        if (b.err)
            for (int q = threadIdx.x; q < 32 * b.err_ndev; q += blockDim.x) {
                const int r = q / b.err_ndev, d = q % b.err_ndev, c = c0 + r, col = c - h + d;
                const double w = b.err[(size_t)(c < b.err_rows ? c : b.err_rows - 1) * b.err_ndev + d];
                wsh[r][d] = (col >= 0 && col < Wm && w > 0) ? (float)w : 0.0f;
            }
        __syncthreads();
        for (int r = ty; r < 32; r += 8) {
            const int c = c0 + r;      // the count (row of tr); tx: the state s0 + tx
            float v;
            if (!b.err) {
                v = tile[tx][r];
            } else {
                // a skipped deviation has weight 0 here: fmaf(0, x, v) = v
                v = 0.0f;
                for (int d = 0; d < b.err_ndev; ++d) v = fmaf(wsh[r][d], tile[tx][r + d], v);
            }
            b.tr[base + (size_t)c * Wm + s0 + tx] = v;
        }
        __syncthreads();
    }
}

// One block: flagged families of each bin, compacted in permutation order
// (a block-wide prefix sum per 256-family chunk); each bin's range of
// fb_perm goes to fb_bins for k_fallback_tiles.
__global__ void __launch_bounds__(256) k_fallback_plan(FallbackPlanArgs a) {
    __shared__ int scan[256];
    __shared__ int64_t base_sh;
    if (a.any_flag && *a.any_flag == 0) {     // nothing flagged: no work
        if (threadIdx.x == 0) {
            a.out_counts[0] = 0;
            a.out_counts[1] = 0;
        }
        return;
    }
    if (threadIdx.x == 0) base_sh = 0;
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
            a.fb_bins[2 * b] = start;
            a.fb_bins[2 * b + 1] = base_sh - start;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.out_counts[0] = (int32_t)base_sh;
        a.out_counts[1] = 0;      // k_fallback_tiles counts the tiles
    }
}

// A tile for every (32-family chunk of a bin's compacted families, listed
// category) in which some family has that term flagged: one warp per chunk,
// one block per category in turn. Tiles are appended in any order.
__global__ void __launch_bounds__(256) k_fallback_tiles(FallbackPlanArgs a) {
    if (a.any_flag && *a.any_flag == 0) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int q = blockIdx.x; q < a.n_cats; q += gridDim.x) {
        const int k = a.cats[q];
        for (int b = 0; b < a.n_bins; ++b) {
            const int64_t start = a.fb_bins[2 * b], cnt = a.fb_bins[2 * b + 1];
            for (int64_t c0 = (int64_t)warp * 32; c0 < cnt; c0 += 8 * 32) {
                const int64_t i = c0 + lane;
                const bool need = i < cnt && a.term_flags[(size_t)a.fb_perm[start + i] * a.K + k] != 0;
                if (__any_sync(0xffffffffu, need) && lane == 0) {
                    PruneTile t;
                    t.first = (int)(start + c0);
                    t.count = (int)(cnt - c0 < 32 ? cnt - c0 : 32);
                    t.k = k;
                    t.S = a.bin_width[b] - 1;
                    t.R = a.bin_width[b] - 1;
                    t.root_lo = t.pad[0] = t.pad[1] = 0;
                    a.fb_tiles[atomicAdd(&a.out_counts[1], 1)] = t;
                }
            }
        }
    }
}

// One thread per (family, candidate): the category terms' range-error
// bounds weighted by their shares of the family likelihood; a family over
// tau |lnL| is flagged for the FP64 recompute. Terms that are not finite
// (a dead or failed category) carry no weight; a family none of whose
// terms is finite is left to the finish.
__global__ void __launch_bounds__(256) k_range_flags(RangeFlagArgs a) {
    const int n_cand = a.K / a.KC;
    const int64_t n = a.F * n_cand;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t f = i / n_cand;
        const int b = (int)(i % n_cand);
        const double* c = a.cat + (size_t)f * a.K + (size_t)b * a.KC;
        const float* e = a.err + (size_t)f * a.K + (size_t)b * a.KC;
        double m = -INFINITY;
        for (int k = 0; k < a.KC; ++k)
            if (isfinite(c[k])) m = fmax(m, c[k]);
        if (!(m > -INFINITY)) continue;
        double w = 0.0, we = 0.0;
        for (int k = 0; k < a.KC; ++k) {
            if (!isfinite(c[k])) continue;
            const double x = exp(c[k] - m);
            w += x;
            we += x * (double)e[k];
        }
        uint8_t* tf = a.term_flags + (size_t)f * a.K + (size_t)b * a.KC;
        // a term the walk left to the FP64 pass carries no weight here, so the
        // others' shares are unknown: every term of the candidate is recomputed
        bool walk = false;
        for (int k = 0; k < a.KC; ++k) walk |= tf[k] != 0;
        if (walk) {
            for (int k = 0; k < a.KC; ++k) tf[k] = 1;
            continue;      // (the family is flagged already)
        }
        if (!(we != 0.0)) continue;      // no range loss in any term (or a candidate that was not pruned)
        const double lnl = m + log(w);
        const double bound = we / w;
        const double lim = a.tau * fabs(lnl);
        if (!(bound <= lim)) {
            // recompute the terms whose share of the bound is over lim / (2 KC):
            // the others' shares add up to at most lim / 2
            const double each = lim * w / (2.0 * a.KC);
            for (int k = 0; k < a.KC; ++k) {
                const bool fin = isfinite(c[k]);
                const double share = fin ? exp(c[k] - m) * (double)e[k] : 0.0;
                if (!(share <= each) || !(lim > 0.0)) tf[k] = 1;
            }
            atomicOr(&a.flags[f], 2);
            atomicOr(a.any_flag, 1);
        }
    }
}

}  // namespace

cudaError_t launch_range_flags(const RangeFlagArgs& a, cudaStream_t s) {
    const int64_t n = a.F * (a.K / a.KC);
    if (n <= 0) return cudaSuccess;
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, 4096);
    k_range_flags<<<blocks, 256, 0, s>>>(a);
    return cudaGetLastError();
}

// k_prune_tc's dynamic shared-memory limit is raised once, to the most a
// CTA may use, so launches of different widths need no per-launch change.
cudaError_t tc_kernels_init() {
    cudaError_t e = cudaFuncSetAttribute(k_prune_tc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, prune_tc_max_smem(1));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_prune_tc<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, prune_tc_max_smem(2));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_prune_tc<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, prune_tc_max_smem(4));
    return e;
}

cudaError_t launch_fallback_plan(const FallbackPlanArgs& a, cudaStream_t s) {
    k_fallback_plan<<<1, 256, 0, s>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || a.n_cats <= 0) return e;
    k_fallback_tiles<<<a.n_cats < 1024 ? a.n_cats : 1024, 256, 0, s>>>(a);
    return cudaGetLastError();
}

int prune_tc_kchunk() { return KC; }

// Dynamic shared memory one k_prune_tc CTA may use: the device's per-block
// opt-in limit minus the kernel instance's static shared memory (the
// cluster instances hold the handshake buffers).
int prune_tc_max_smem(int nsplit) {
    static int cached[5] = {-1, -1, -1, -1, -1};
    if (nsplit != 1 && nsplit != 2 && nsplit != 4) return 0;
    if (cached[nsplit] < 0) {
        int dev = 0, optin = 0;
        cudaFuncAttributes fa{};
        const void* fn = nsplit == 1 ? (const void*)k_prune_tc<1> : nsplit == 2 ? (const void*)k_prune_tc<2>
                                                                              : (const void*)k_prune_tc<4>;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
            cudaFuncGetAttributes(&fa, fn) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        cached[nsplit] = optin - (int)fa.sharedSizeBytes;
    }
    return cached[nsplit];
}

size_t prune_tc_smem_bytes(int Ws, int n_slots, int stages, int n_internal) {
    return stages_region(Ws, stages) + (size_t)n_slots * TM * (sizeof(int) + sizeof(float)) +
           (size_t)n_internal * sizeof(NodeInfo) + 1024;
}

cudaError_t launch_convert_tc(const ConvertJob* d_jobs, int n_jobs, TcBuffers b, cudaStream_t s) {
    if (n_jobs <= 0) return cudaSuccess;
    if (b.Wm % 32) return cudaErrorInvalidValue;
    k_convert_tc<<<(unsigned)(n_jobs * (b.Wm / 32)), 256, 0, s>>>(d_jobs, b);
    return cudaGetLastError();
}

cudaError_t launch_prune_tc(const TcMaps& m, const PruneTcArgs& a, int n_ctas, size_t smem, cudaStream_t s) {
    if (a.n_tiles <= 0) return cudaSuccess;
    if (smem > (size_t)prune_tc_max_smem(a.nsplit)) return cudaErrorInvalidValue;
    if (a.stages < 1 || a.stages > MAXST) return cudaErrorInvalidValue;
    if (a.nsplit == 1) {
        k_prune_tc<1><<<n_ctas, NTHREADS, smem, s>>>(m.mat, m.vec, m.vst, m.tr, a);
        return cudaGetLastError();
    }
    // a cluster of nsplit CTAs per tile, each with Ws = W / nsplit output
    // states (a multiple of 32: whole 32-row TMA boxes) of both children
    if ((a.nsplit != 2 && a.nsplit != 4) || n_ctas % a.nsplit || a.Ws % 32 || a.Ws > 256 ||
        a.tmem_cols < 2 * a.Ws || a.tmem_cols > 512)
        return cudaErrorInvalidValue;
    cudaLaunchConfig_t cfg;
    std::memset(&cfg, 0, sizeof cfg);
    cfg.gridDim = dim3((unsigned)n_ctas, 1, 1);
    cfg.blockDim = dim3(NTHREADS, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)a.nsplit;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (a.nsplit == 2) return cudaLaunchKernelEx(&cfg, k_prune_tc<2>, m.mat, m.vec, m.vst, m.tr, a);
    return cudaLaunchKernelEx(&cfg, k_prune_tc<4>, m.mat, m.vec, m.vst, m.tr, a);
}

}  // namespace cafe
