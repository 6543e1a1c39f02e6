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

__device__ __forceinline__ double out_value(double m, int e) {
    double v = (e == 0) ? m : scalbn(m, e);
    return v < 1.0 ? v : 1.0;
}

// Row s of the matrix, columns 0..s, and its mirror: c P(s->c) = s P(c->s)
// gives the upper-triangle entry P(c->s) = (c/s) P(s->c) of row c < s,
// written in the same step. Neighbouring threads own neighbouring rows, so
// the mirror stores of a warp land in one contiguous run of row c.
__device__ void row_chain(double* __restrict__ M, int W, int s, double alpha, double coeff, double q, double la,
                          const double* __restrict__ inv, const double* __restrict__ bq) {
    double L0 = (double)s * la;  // log(a^s)
    int E = 0;
    double m;
    if (L0 > -700.0) {
        m = exp(L0);
    } else {
        E = (int)floor(L0 * 1.4426950408889634) + 1;
        m = exp((L0 - (double)E * kLn2Hi) - (double)E * kLn2Lo);
    }
    double mp = 0.0;
    double sm = (double)s, sp = (double)s;  // s - c, s + c
    const double inv_s = inv[s];
    double* row = M + (size_t)s * W;
    for (int c = 0; c < s; ++c) {
        const double v = out_value(m, E);
        row[c] = v;
        if (c > 0) {
            const double u = (double)c * inv_s * v;
            M[(size_t)c * W + s] = u < 1.0 ? u : 1.0;
        }
        double a = fma(sm, q, alpha * sp) * inv[c + 1];
        double b = coeff * bq[c];
        double nx = fma(a, m, b * mp);
        mp = m;
        m = nx;
        sm -= 1.0;
        sp += 1.0;
        if (m > 0x1p+600) {
            m *= 0x1p-600;
            mp *= 0x1p-600;
            E += 600;
        }
    }
    row[s] = out_value(m, E);
}

// One CTA per matrix; thread p owns rows 1 + p and W - 1 - p (about W
// recurrence steps each). Row 0 and column 0 of rows >= 1 come from the
// chains (P(s -> 0) = a^s); M[0][c] = delta(c, 0).
__global__ void __launch_bounds__(128) k_matrix_build(const MatrixJob* __restrict__ jobs) {
    extern __shared__ double sh[];
    const MatrixJob J = jobs[blockIdx.x];
    const int W = J.size;
    double* inv = sh;          // inv[k] = 1/k, k = 0..W
    double* bq = sh + W + 1;   // bq[c] = (c - 1)/(c + 1), c = 0..W
    for (int k = threadIdx.x; k <= W; k += blockDim.x) {
        inv[k] = k ? 1.0 / (double)k : 0.0;
        bq[k] = (double)(k - 1) / (double)(k + 1);
    }
    double* M = J.dst;
    const double lt = J.lambda * J.t;
    const double alpha = lt / (1 + lt);
    const double coeff = 1 - 2 * alpha;
    const bool live = (coeff > 0 && coeff != 1);
    for (int c = threadIdx.x; c < W; c += blockDim.x) M[c] = (c == 0) ? 1.0 : 0.0;
    if (!live) {
        for (size_t i = (size_t)W + threadIdx.x; i < (size_t)W * W; i += blockDim.x) M[i] = 0.0;
        return;
    }
    __syncthreads();
    const double q = coeff / alpha;
    const double la = log(alpha);
    const int nrows = W - 1;
    for (int p = threadIdx.x; p < (nrows + 1) / 2; p += blockDim.x) {
        const int s1 = 1 + p, s2 = W - 1 - p;
        row_chain(M, W, s1, alpha, coeff, q, la, inv, bq);
        if (s2 != s1) row_chain(M, W, s2, alpha, coeff, q, la, inv, bq);
    }
}

}  // namespace

cudaError_t launch_matrix_build(const MatrixJob* d_jobs, int n_jobs, int max_size, cudaStream_t s) {
    if (n_jobs <= 0) return cudaSuccess;
    size_t smem = sizeof(double) * 2 * (size_t)(max_size + 2);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_matrix_build, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    // one thread per row pair, in whole warps (at most 128)
    const int pairs = max_size / 2;
    const int threads = std::min(128, std::max(32, (pairs + 31) / 32 * 32));
    k_matrix_build<<<n_jobs, threads, smem, s>>>(d_jobs);
    return cudaGetLastError();
}

}  // namespace cafe
