// K1: birth-death transition matrices in FP64, one CTA per (lambda, t) key.
//
// Replaces matrix_cache::precalculate_matrices (src/matrix_cache.cpp:113-163)
// over birthdeath_rate_with_log_alpha (src/probability.cpp:104-148), which
// evaluates P(s -> c) = sum_j C(s,j) C(s+c-j-1, s-1) a^(s+c-2j) (1-2a)^j with
// one exp and one pow per term: O(S^3) terms per matrix. On GB300 FP64 is
// the scarcest pipe, so this kernel uses an O(S^2) scheme instead:
//
//  * Row s is the coefficient sequence of G(z)^s, G(z) = (a + b z)/(1 - a z)
//    with a = lt/(1+lt), b = 1 - 2a (the one-lineage law P(1->0) = a,
//    P(1->c) = (1-a)^2 a^(c-1)). From (a + b z)(1 - a z) G_s' = s(1-a)^2 G_s:
//        g_{c+1} = [ ((s-c) b + a^2 (s+c)) g_c + a b (c-1) g_{c-1} ] / (a (c+1))
//    For c < s both coefficients are >= 0, so the forward recurrence only
//    adds non-negative terms and is stable; it starts at g_0 = a^s.
//  * The upper triangle follows from c P(s->c) = s P(c->s) (the two
//    binomial sums differ term by term by the factor s/c): the chain of row
//    s also writes P(c->s) = (c/s) P(s->c) into rows c < s.
//  * Both kinds of store leave each warp as contiguous row segments (the
//    lower triangle through a shared-memory staging tile).
//  * The running value is kept as mantissa * 2^E so rows whose left end
//    underflows FP64 (a^s < 1e-308) still reach their diagonal exactly.
//
// Row 0 is delta(c,0); a key whose 1 - 2a is not in (0, 1) has zero rows
// s >= 1 (the_probability_of_going_from_parent_fam_size_to_c,
// src/probability.cpp:150-167, and the saturation rule of
// matrix_cache.cpp:139-154). Entries are clamped to <= 1 as in
// probability.cpp:147.
#include "common.cuh"

#include <algorithm>

namespace cafe {
namespace {

constexpr double kLn2Hi = 6.93147180369123816490e-01;  // Cody-Waite split of ln 2
constexpr double kLn2Lo = 1.90821492927058770002e-10;

// min(v, 1) for v >= 0 without an FP64 instruction: v >= 1 exactly when
// the high word of its bits is >= that of 1.0.
__device__ __forceinline__ double clamp1(double v) { return __double2hiint(v) >= 0x3ff00000 ? 1.0 : v; }

__device__ __forceinline__ double out_value(double m, int e) { return clamp1(e == 0 ? m : scalbn(m, e)); }

// Per-matrix coefficient tables in shared memory (k = 0..W):
//   p1[c] = (q + alpha) / (c + 1), p2[c] = c (alpha - q) / (c + 1)
//     so that ((s - c) q + alpha (s + c)) / (c + 1) = s p1[c] + p2[c]
//   bb[c] = (1 - 2 alpha) (c - 1) / (c + 1)
struct Coeffs {
    const double* p1;
    const double* p2;
    const double* bb;
};

// One row chain: the coefficients g_c of row s, c = 0..s, as a running
// mantissa m (and the previous one mp) times 2^E; cs = c / s for the
// mirrored entry of row c.
struct RowChain {
    int s, E;
    double m, mp, sd, inv_s, cs;

    __device__ void init(int s_, double la, const double* inv) {
        s = s_;
        const double L0 = (double)s * la;  // log(a^s)
        E = 0;
        if (L0 > -700.0) {
            m = exp(L0);
        } else {
            E = (int)floor(L0 * 1.4426950408889634) + 1;
            m = exp((L0 - (double)E * kLn2Hi) - (double)E * kLn2Lo);
        }
        mp = 0.0;
        sd = (double)s;
        inv_s = inv[s];
        cs = 0.0;
    }
    __device__ __forceinline__ double value() const { return out_value(m, E); }
    // g_c -> g_{c+1}: two FMAs and a product per step
    __device__ __forceinline__ void advance(int c, const Coeffs& k) {
        const double a = fma(sd, k.p1[c], k.p2[c]);
        const double nx = fma(a, m, k.bb[c] * mp);
        mp = m;
        m = nx;
        cs += inv_s;
        if (__double2hiint(m) >= 0x65800000) {   // m >= 2^601
            m *= 0x1p-600;
            mp *= 0x1p-600;
            E += 600;
        }
    }
};

constexpr int kStageCols = 16;   // columns of a warp's staging tile
constexpr int kStagePitch = 33;  // padded row pitch (doubles) of the staging tile

// `parts` CTAs of T threads per matrix, each with an equal share of its row
// pairs (every pair costs about W steps), so a side-512 build spreads over
// the SMs in small CTAs. Thread t of part q owns the row pairs
// p = q T + t + j parts T: the short row 1 + p and the long row W - 1 - p,
// one after the other. Each step c writes two entries of row s's chain:
// the mirror P(c->s) = (c/s) P(s->c) of row c < s, contiguous across the
// warp (neighbouring lanes own neighbouring rows), and P(s->c) itself,
// which is strided across the warp and so goes through a 16-column staging
// tile in shared memory and leaves as contiguous row segments. Row 0 is
// delta(c, 0).
__global__ void __launch_bounds__(128) k_matrix_build(const MatrixJob* __restrict__ jobs, int parts) {
    extern __shared__ double sh[];
    const int part = blockIdx.x % parts;
    const MatrixJob J = jobs[blockIdx.x / parts];
    const int W = J.size;
    double* inv = sh;                  // inv[k] = 1/k, k = 0..W
    double* p1 = sh + (W + 1);         // coefficient tables (Coeffs), k = 0..W
    double* p2 = sh + 2 * (W + 1);
    double* bb = sh + 3 * (W + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* stage = sh + 4 * (W + 1) + (size_t)warp * kStageCols * kStagePitch;
    int* srow = reinterpret_cast<int*>(sh + 4 * (W + 1) + (size_t)(blockDim.x >> 5) * kStageCols * kStagePitch) +
                warp * 32;
    double* M = J.dst;
    const double lt = J.lambda * J.t;
    const double alpha = lt / (1 + lt);
    const double coeff = 1 - 2 * alpha;
    const bool live = (coeff > 0 && coeff != 1);
    const double q = live ? coeff / alpha : 0.0;
    for (int k = threadIdx.x; k <= W; k += blockDim.x) {
        const double ik = 1.0 / (double)(k + 1);
        inv[k] = k ? 1.0 / (double)k : 0.0;
        p1[k] = (q + alpha) * ik;
        p2[k] = (double)k * (alpha - q) * ik;
        bb[k] = coeff * ((double)(k - 1) * ik);
    }
    const Coeffs cf{p1, p2, bb};
    if (part == 0)
        for (int c = threadIdx.x; c < W; c += blockDim.x) M[c] = (c == 0) ? 1.0 : 0.0;
    if (!live) {
        const size_t stride = (size_t)parts * blockDim.x;
        for (size_t i = (size_t)W + (size_t)part * blockDim.x + threadIdx.x; i < (size_t)W * W; i += stride) M[i] = 0.0;
        return;
    }
    __syncthreads();
    const double la = log(alpha);
    const int npairs = W / 2;   // rows 1..W-1 in pairs (the middle row once when W is even)
    for (int p0 = part * blockDim.x + warp * 32; p0 < npairs; p0 += parts * blockDim.x) {
        const int p = p0 + lane;
        for (int set = 0; set < 2; ++set) {
            const int s = set == 0 ? 1 + p : W - 1 - p;
            const bool act = p < npairs && (set == 0 || s != 1 + p);
            srow[lane] = act ? s : 0;
            __syncwarp();
            int maxlen = act ? s : 0;
            for (int o = 16; o > 0; o >>= 1) maxlen = max(maxlen, __shfl_xor_sync(0xffffffffu, maxlen, o));
            RowChain ch;
            if (act) ch.init(s, la, inv);
            for (int c0 = 0; c0 < maxlen; c0 += kStageCols) {
                for (int cc = 0; cc < kStageCols; ++cc) {
                    const int c = c0 + cc;
                    if (act && c < s) {
                        const double v = ch.value();
                        stage[cc * kStagePitch + lane] = v;
                        if (c > 0) M[(size_t)c * W + s] = clamp1(ch.cs * v);
                        ch.advance(c, cf);
                    }
                }
                __syncwarp();
                // the tile's rows, 16 columns each: two rows per warp instruction
                for (int idx = lane; idx < 32 * kStageCols; idx += 32) {
                    const int r = idx / kStageCols, col = idx % kStageCols;
                    const int sr = srow[r];
                    if (c0 + col < sr) M[(size_t)sr * W + c0 + col] = stage[col * kStagePitch + r];
                }
                __syncwarp();
            }
            if (act) M[(size_t)s * W + s] = ch.value();   // the diagonal, g_s
            __syncwarp();
        }
    }
}

}  // namespace

cudaError_t launch_matrix_build(const MatrixJob* d_jobs, int n_jobs, int max_size, cudaStream_t s) {
    if (n_jobs <= 0) return cudaSuccess;
    // one thread per row pair, in whole warps: at most 64 per CTA, and as
    // many CTAs per matrix as its pairs need
    const int pairs = max_size / 2;
    const int threads = std::min(64, std::max(32, (pairs + 31) / 32 * 32));
    const int parts = std::max(1, (pairs + threads - 1) / threads);
    size_t smem = sizeof(double) * (4 * (size_t)(max_size + 1) + (size_t)(threads / 32) * kStageCols * kStagePitch) +
                  sizeof(int) * (size_t)threads;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_matrix_build, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    k_matrix_build<<<n_jobs * parts, threads, smem, s>>>(d_jobs, parts);
    return cudaGetLastError();
}

}  // namespace cafe
