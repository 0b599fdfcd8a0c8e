// prune.cu -- site-pair pruning (HP1) and unpaired column likelihoods on the GPU.
//
// Replaces the kernels of src/cuda/felsenstein.cu used by
// src/FelsensteinCUDA.jl:214-516 (felsensteinleaves16 :117-133,
// felsensteinhelper16 :153-200, sumfinal :428-442, storearr/logsumexparr
// :135-151) with:
//   * build_P16_kernel: P = exp(Qt) per (category, branch) in FP64 from the
//     host eigensystem, stored as FP32 rows (row = parent state);
//   * message rows: what a node passes to its parent is its partial
//     likelihood vector already multiplied by its own branch's matrix,
//     m_v = P_v x_v, so every node update is x_v = m_left * m_right
//     (elementwise) followed by ONE mat-vec, P_v x_v, done once per unique
//     row at v instead of once per parent pair that reads the row (the
//     reference applies both child matrices inside every parent update,
//     felsenstein.cu:170-190); the root needs no mat-vec, only pi . x;
//   * leaf_msg_kernel: the messages of the leaves (P_leaf x indicator rows)
//     per category pass;
//   * prune_msg_kernel: one launch per tree level and category pass; a warp
//     owns 32 unique pairs of one node, gathers the two children's message
//     rows with cp.async (two categories in flight) and does the mat-vec on
//     the tensor cores (3xTF32 mma.sync, operands split into hi/lo in
//     registers).  Rows are rescaled by an exact power of two (exponent kept
//     as an int), which computes the same likelihood as the reference's
//     divide-by-max (felsenstein.cu:193-198);
//   * the root variant folds sumfinal and the category log-sum-exp into the
//     same pass (FP64 log-likelihood reduction);
//   * prune_tc_kernel: the interior update as tcgen05.mma (A in tensor
//     memory, P in shared memory, accumulators in tensor memory), the same
//     bits as prune_msg_kernel; chosen only on request (launch shape 3).
// unpaired_site_kernel + unpaired_mix_kernel restate
// computeunpairedlikelihoodscat (src/FARCE.jl:742-773) in FP64 with the CPU
// rescaling rule.
#include <algorithm>
#include <cmath>

#include "internal.h"

namespace messi {

// P[c][v][a][d] in FP32 (row = parent state), from the FP64 eigensystem:
// P = D^-1/2 U exp(W t) U^T D^1/2.  One CTA per category and run of
// kP16Nodes nodes, a thread per entry: the CTA stages the category's U and
// the ratios sqrt(pi_d) / sqrt(pi_a) once per model group and, per node,
// W[a][k] = U[a][k] exp(w_k t), so an entry is 16 FP64 multiply-adds.  (One
// CTA per node and category staged U for every matrix and divided per entry:
// 26 ms for the 1.28 M matrices of a 256-alignment batch.)
constexpr int kP16Nodes = 32;

__global__ void build_P16_kernel(const double* __restrict__ eig, const double* __restrict__ bl,
                                 const int* __restrict__ nodegrp, int numnodes, int C, float* __restrict__ P)
{
    const int c = blockIdx.x, t = threadIdx.x;
    const int a = t >> 4, d = t & 15;
    const int v0 = blockIdx.y * kP16Nodes, v1 = min(numnodes, v0 + kP16Nodes);
    __shared__ double U[256], W[256], R[256], w[16], ex[16];
    int cur = -1;
    for (int v = v0; v < v1; v++) {
        const int grp = nodegrp ? nodegrp[v] : (v == 0 ? -1 : 0);  // the same in every thread
        const double tl = bl[v];
        __syncthreads();  // the previous node's reads of the staged arrays are done
        if (grp >= 0 && grp != cur) {
            const double* e = eig + ((size_t)grp * C + c) * kEigStride;
            U[t] = e[16 + t];
            R[t] = e[16 + 256 + d] / e[16 + 256 + a];
            if (t < 16) w[t] = e[t];
            cur = grp;
            __syncthreads();
        }
        if (grp >= 0 && t < 16) ex[t] = exp(w[t] * tl);
        __syncthreads();
        if (grp >= 0) W[t] = U[t] * ex[d];  // W[a][k], k = d
        __syncthreads();
        float out;
        if (grp < 0) {
            out = 0.f;  // a root has no branch (gettransitionmatriceslist, src/FARCE.jl:416)
        } else if (tl == 0.0) {
            out = (a == d) ? 1.f : 0.f;
        } else {
            double acc = 0.0;
#pragma unroll
            for (int k = 0; k < 16; k++) acc += W[a * 16 + k] * U[d * 16 + k];
            acc *= R[t];
            out = (acc <= 0.0) ? 0.f : (float)acc;  // absmat clamp (1e-50 rounds to 0 in FP32)
        }
        P[((size_t)c * numnodes + v) * 256 + t] = out;
    }
}

__global__ void build_P4_kernel(const double* __restrict__ eig4, const double* __restrict__ bl,
                                const int* __restrict__ nodegrp, int numnodes, int nsite, double* __restrict__ P4)
{
    const int v = blockIdx.x, s = blockIdx.y, t = threadIdx.x;  // 16 threads
    const int grp = nodegrp ? nodegrp[v] : (v == 0 ? -1 : 0);
    const double* e = eig4 + ((size_t)max(grp, 0) * nsite + s) * kEig4Stride;
    const double tl = bl[v];
    const int a = t >> 2, d = t & 3;
    double out;
    if (grp < 0) {
        out = 0.0;
    } else if (tl == 0.0) {
        out = (a == d) ? 1.0 : 0.0;
    } else {
        double acc = 0.0;
        for (int k = 0; k < 4; k++) acc += e[4 + a * 4 + k] * exp(e[k] * tl) * e[4 + d * 4 + k];
        acc *= e[20 + d] / e[20 + a];
        out = (acc <= 0.0) ? 1e-50 : acc;
    }
    P4[((size_t)s * numnodes + v) * 16 + t] = out;
}

int launch_build_P16(messi_ctx* ctx, const double* d_eig, const double* d_bl, const int* d_nodegrp, int numnodes,
                     int C, float* d_P)
{
    build_P16_kernel<<<dim3(C, (numnodes + kP16Nodes - 1) / kP16Nodes), 256, 0, ctx->stream>>>(d_eig, d_bl, d_nodegrp,
                                                                                              numnodes, C, d_P);
    LAUNCH_CHECK(ctx, "build_P16_kernel");
    return MESSI_OK;
}

int launch_build_P4(messi_ctx* ctx, const double* d_eig4, const double* d_bl, const int* d_nodegrp, int numnodes,
                    int nsite, double* d_P4)
{
    build_P4_kernel<<<dim3(numnodes, nsite), 16, 0, ctx->stream>>>(d_eig4, d_bl, d_nodegrp, numnodes, nsite, d_P4);
    LAUNCH_CHECK(ctx, "build_P4_kernel");
    return MESSI_OK;
}

__device__ __forceinline__ float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

__device__ __forceinline__ double lse_d(double a, double b)
{
    if (b == -INFINITY) return a;
    if (a == -INFINITY) return b;
    return (a < b) ? b + log1p(exp(a - b)) : a + log1p(exp(b - a));
}

// lse_d with the correction log(1 + e^-|a-b|) (in [0, log 2]) formed in FP32
// from the FP64 difference: absolute error ~1e-7 on a sum of log-likelihoods
// of magnitude 10-1000, against an FP64 exp and log1p per call (the band
// preparation of a 256-alignment batch calls it for 9.3e7 cells).
__device__ __forceinline__ double lse_d_fast(double a, double b)
{
    if (b == -INFINITY) return a;
    if (a == -INFINITY) return b;
    const double mx = fmax(a, b);
    return mx + (double)log1pf(expf((float)(fmin(a, b) - mx)));
}

// ---------------------------------------------------------------------------
// Leaf messages: out[cc][r][a] = sum_d P[c0+cc][node(r)][a][d] * rows[r][d]
// (16 threads per row, FP64 accumulation, one FP32 rounding).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) leaf_msg_kernel(const float* __restrict__ rows, const int* __restrict__ rownode,
                                                       long long R, const float* __restrict__ P, int numnodes, int c0,
                                                       int C, float* __restrict__ out)
{
    const long long r = (long long)blockIdx.x * 16 + (threadIdx.x >> 4);
    const int a = threadIdx.x & 15, cc = blockIdx.y;
    if (r >= R) return;
    (void)C;
    const float* p = P + ((size_t)(c0 + cc) * numnodes + __ldg(rownode + r)) * 256 + a * 16;
    const float4* x4 = reinterpret_cast<const float4*>(rows + r * 16);
    float x[16];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const float4 v = __ldg(x4 + q);
        x[4 * q] = v.x;
        x[4 * q + 1] = v.y;
        x[4 * q + 2] = v.z;
        x[4 * q + 3] = v.w;
    }
    // an observed base pair is one nonzero state: its zero terms are skipped
    // (adding +0.0 would leave the sum as it is), the same branch for the 16
    // threads of the row
    double s = 0.0;
#pragma unroll
    for (int d = 0; d < 16; d++)
        if (x[d] != 0.f) s += (double)__ldg(p + d) * (double)x[d];
    out[((size_t)cc * R + r) * 16 + a] = (float)s;
}

int launch_leaf_messages(messi_ctx* ctx, const float* d_rows, const int* d_rownode, int64_t R, const float* d_P,
                         int numnodes, int c0, int nc, int C, float* d_out)
{
    if (R <= 0 || nc <= 0) return MESSI_OK;
    leaf_msg_kernel<<<dim3((unsigned)((R + 15) / 16), nc), 256, 0, ctx->stream>>>(d_rows, d_rownode, R, d_P,
                                                                                  numnodes, c0, C, d_out);
    LAUNCH_CHECK(ctx, "leaf_msg_kernel");
    return MESSI_OK;
}

// ---------------------------------------------------------------------------
// Tensor-core node update (3xTF32 mma.sync).  A warp owns 32 unique pairs of
// one node.  For each category it forms x = m_left * m_right for its pairs
// and, below the root, the product [32 pairs x 16] x [16 x 16]^T with P of
// the node's own branch, as m16n8k8 TF32 MMAs with both operands split
// hi + lo (hi*hi + hi*lo + lo*hi: FP32-level accuracy; all operands are
// non-negative, so there is no cancellation).
// Rounding.  The tensor core rounds each MMA's FP32 result toward zero
// (measured on GB300: 99.9% of outputs equal the truncation of the exact
// sum, mean error -0.44 ulp), so a chain of MMAs loses about half an ulp per
// result, always downwards; over the 62 mat-vecs of a 64-leaf tree that
// shifted every pair log-likelihood by about -1.2e-6.  Each of the two
// k-steps therefore accumulates into its own registers (small cross terms
// first, so their truncation is negligible), the two halves are added in
// FP32 (round to nearest), and half an ulp of the sum is added back, again
// rounded to nearest: a tie, which rounds up or down on the last mantissa
// bit, so the truncation bias of the two halves is returned on average.
// The contraction index d is permuted so that lane (g, t) owns
// d = 4t..4t+3: its A fragment for pair row r is one 16-byte load of each
// child's row, and its B fragment one 16-byte load of P[8nt + g][4t..4t+3].
// Lane (g, t) ends with states {2t, 2t+1, 8+2t, 9+2t} of pairs g, g+8,
// g+16, g+24; lane t keeps the scalar bookkeeping (exponent, mixture) of pair
// g + 8t.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float comp4(const float4& v, int k)
{
    return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// A operand split: hi = x rounded to TF32 (adding half a TF32 ulp to the
// magnitude bits and truncating is round-to-nearest, ties away, the same as
// cvt.rna for the finite values here) and lo = x - hi (exact in FP32), fed
// without conversion: the tensor core reads the top 19 bits of lo, an error
// below 2^-21 |x| of either sign (lo is centred on zero).
__device__ __forceinline__ void split_a(float x, uint32_t& hi, uint32_t& lo)
{
    hi = (__float_as_uint(x) + 0x1000u) & 0xffffe000u;
    lo = __float_as_uint(x - __uint_as_float(hi));
}

// B operand (four entries of P) split the same way, in registers: one FP32
// load per fragment instead of a hi and a lo load.
__device__ __forceinline__ void split_b(const float4& p, float4& hi, float4& lo)
{
    uint32_t h[4], l[4];
    split_a(p.x, h[0], l[0]);
    split_a(p.y, h[1], l[1]);
    split_a(p.z, h[2], l[2]);
    split_a(p.w, h[3], l[3]);
    hi = make_float4(__uint_as_float(h[0]), __uint_as_float(h[1]), __uint_as_float(h[2]), __uint_as_float(h[3]));
    lo = make_float4(__uint_as_float(l[0]), __uint_as_float(l[1]), __uint_as_float(l[2]), __uint_as_float(l[3]));
}

// v + half an ulp of v, rounded to nearest (ties to even): v or v + ulp,
// each for half of the mantissas.  v >= 0.
__device__ __forceinline__ float add_half_ulp(float v)
{
    const int e = (int)(__float_as_uint(v) & 0x7f800000u) - (24 << 23);
    return v + __int_as_float(max(e, 0));
}

// D0[mt][nt] += X x P^T over states k-step 0 (d = 4t, 4t+1), D1 over k-step 1
// (d = 4t+2, 4t+3), each as lo*hi + hi*lo + hi*hi, for rows g + 8k (k = 0..3).
__device__ __forceinline__ void msg_mma(const float4 (&X)[4], const float4 (&Bh)[2], const float4 (&Bl)[2],
                                        float (&D0)[2][2][4], float (&D1)[2][2][4])
{
#pragma unroll
    for (int mt = 0; mt < 2; mt++) {
#pragma unroll
        for (int ks = 0; ks < 2; ks++) {
            const float av[4] = {comp4(X[2 * mt], 2 * ks), comp4(X[2 * mt + 1], 2 * ks), comp4(X[2 * mt], 2 * ks + 1),
                                 comp4(X[2 * mt + 1], 2 * ks + 1)};
            uint32_t ah[4], al[4];
#pragma unroll
            for (int i = 0; i < 4; i++) split_a(av[i], ah[i], al[i]);
#pragma unroll
            for (int nt = 0; nt < 2; nt++) {
                const uint32_t bh0 = __float_as_uint(comp4(Bh[nt], 2 * ks)), bh1 = __float_as_uint(comp4(Bh[nt], 2 * ks + 1));
                const uint32_t bl0 = __float_as_uint(comp4(Bl[nt], 2 * ks)), bl1 = __float_as_uint(comp4(Bl[nt], 2 * ks + 1));
                float (&D)[4] = ks ? D1[mt][nt] : D0[mt][nt];
                mma_tf32(D, al, bh0, bh1);
                mma_tf32(D, ah, bl0, bl1);
                mma_tf32(D, ah, bh0, bh1);
            }
        }
    }
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}

__device__ __forceinline__ void cp_async4(void* smem, const void* gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem));
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }

template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// Exact power-of-two rescale of a row max m > 0: m * 2^-ex in [0.5, 1).
__device__ __forceinline__ void pow2_scale(float m, int& ex, float& sc)
{
    const unsigned bits = __float_as_uint(m);
    const int E = (int)((bits >> 23) & 0xffu);
    if (E >= 1 && E <= 252) {  // normal, and 2^-ex representable
        ex = E - 126;
        sc = __uint_as_float((unsigned)(127 - ex) << 23);
    } else if (m > 0.f) {
        frexpf(m, &ex);
        sc = ldexpf(1.f, -ex);
    } else {
        ex = 0;
        sc = 1.f;
    }
}

// Pipeline shapes: STAGES categories in flight per warp (cp.async), MINB CTAs
// of kTile = 128 threads per SM.  The default, 2 stages x 4 CTAs (16 warps,
// 136 KB of stages per SM), leaves ~90 KB of the SM's L1 to cache the
// gathered child rows, which parent pairs share heavily.

// Per-warp staging of one category: 8 float4 per lane (child rows) + 2 exponents.
struct WarpStage {
    float4 x[8][32];
    int e[2][32];
};

template <bool ROOT, int STAGES, int MINB>
__global__ void __launch_bounds__(kTile, MINB) prune_msg_kernel(
    const NodeDev* __restrict__ nodes, const int2* __restrict__ tiles, const float* __restrict__ P, int numnodes,
    int c0, int nc, int C, const float* __restrict__ pi16, const double* __restrict__ logw,
    const int* __restrict__ lam, int per_lambda)
{
    extern __shared__ float4 smem_raw[];
    const int2 tile = tiles[blockIdx.x];
    const NodeDev& nd = nodes[tile.x];
    const int n = nd.n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int base = tile.y + warp * 32;  // first pair of this warp
    if (base >= n) return;                // whole warp idle (warp-uniform)
    WarpStage* stage = reinterpret_cast<WarpStage*>(smem_raw) + (size_t)warp * STAGES;
    // child rows of pairs g + 8k (clamped to a valid row past the end)
    int li[4], ri[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int u = base + g + 8 * k;
        const int uc = (u < n) ? u : (n - 1);
        li[k] = __ldg(nd.li + uc);
        ri[k] = __ldg(nd.ri + uc);
    }
    const int myu = base + g + 8 * t;  // pair whose scalars this lane keeps
    const bool myvalid = myu < n;
    const int myl = li[0] * (t == 0) + li[1] * (t == 1) + li[2] * (t == 2) + li[3] * (t == 3);
    const int myr = ri[0] * (t == 0) + ri[1] * (t == 1) + ri[2] * (t == 2) + ri[3] * (t == 3);
    const float* lf = nd.lf;
    const float* rf = nd.rf;
    const int* le = nd.le;
    const int* re = nd.re;
    const long long lcs = nd.lcs, rcs = nd.rcs;
    // issue the copies of category cc into its stage (each lane copies what it later reads)
    auto issue = [&](int cc) {
        WarpStage& st = stage[cc % STAGES];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            cp_async16(&st.x[k][lane], lf + ((size_t)cc * lcs + li[k]) * 16 + 4 * t);
            cp_async16(&st.x[4 + k][lane], rf + ((size_t)cc * rcs + ri[k]) * 16 + 4 * t);
        }
        if (le) cp_async4(&st.e[0][lane], le + (size_t)cc * lcs + myl);
        if (re) cp_async4(&st.e[1][lane], re + (size_t)cc * rcs + myr);
    };
#pragma unroll
    for (int s0 = 0; s0 < STAGES - 1; s0++) {
        if (s0 < nc) issue(s0);
        cp_async_commit();
    }
    double mm = -INFINITY;
    float ss = 0.f;
    double lm[kMaxLambda];
    float ls[kMaxLambda];
    if (ROOT) {
#pragma unroll
        for (int q = 0; q < kMaxLambda; q++) { lm[q] = -INFINITY; ls[q] = 0.f; }
    }
    for (int cc = 0; cc < nc; cc++) {
        if (cc + STAGES - 1 < nc) issue(cc + STAGES - 1);
        cp_async_commit();
        cp_async_wait<STAGES - 1>();
        const WarpStage& st = stage[cc % STAGES];
        // x = m_left * m_right: states 4t..4t+3 of pairs g + 8k
        float4 X[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float4 a = st.x[k][lane], b = st.x[4 + k][lane];
            X[k] = make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w);
        }
        const int e = (le ? st.e[0][lane] : 0) + (re ? st.e[1][lane] : 0);
        if (ROOT) {
            const float4 pc = __ldg(reinterpret_cast<const float4*>(pi16 + ((size_t)nd.grp * C + c0 + cc) * 16) + t);
            float dots[4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                float dk = pc.x * X[k].x + pc.y * X[k].y + pc.z * X[k].z + pc.w * X[k].w;
                dk += __shfl_xor_sync(0xffffffffu, dk, 1);
                dk += __shfl_xor_sync(0xffffffffu, dk, 2);
                dots[k] = dk;
            }
            const float dot = dots[0] * (t == 0) + dots[1] * (t == 1) + dots[2] * (t == 2) + dots[3] * (t == 3);
            const double ll = (dot > 0.f) ? (double)logf(dot) + (double)e * 0.69314718055994530942 : -INFINITY;
            if (nd.catll && myvalid) nd.catll[(size_t)(c0 + cc) * n + myu] = ll;
            const double tt = __ldg(logw + (size_t)nd.grp * C + c0 + cc) + ll;
            if (tt > mm) {
                ss = ss * __expf((float)(mm - tt)) + 1.f;
                mm = tt;
            } else if (tt != -INFINITY) {
                ss += __expf((float)(tt - mm));
            }
            if (per_lambda) {
                const int kq = __ldg(lam + c0 + cc);
#pragma unroll
                for (int q = 0; q < kMaxLambda; q++)
                    if (q == kq) {
                        if (tt > lm[q]) {
                            ls[q] = ls[q] * __expf((float)(lm[q] - tt)) + 1.f;
                            lm[q] = tt;
                        } else if (tt != -INFINITY) {
                            ls[q] += __expf((float)(tt - lm[q]));
                        }
                    }
            }
        } else {
            // m_v = P_v x (the node's own branch), then an exact power-of-two rescale
            const float* pv = P + ((size_t)(c0 + cc) * numnodes + nd.self) * 256;
            float4 Bh[2], Bl[2];
#pragma unroll
            for (int nt = 0; nt < 2; nt++) split_b(ldg4(pv + (8 * nt + g) * 16 + 4 * t), Bh[nt], Bl[nt]);
            float D0[2][2][4], D1[2][2][4];
#pragma unroll
            for (int mt = 0; mt < 2; mt++)
#pragma unroll
                for (int nt = 0; nt < 2; nt++)
#pragma unroll
                    for (int i = 0; i < 4; i++) { D0[mt][nt][i] = 0.f; D1[mt][nt][i] = 0.f; }
            msg_mma(X, Bh, Bl, D0, D1);
            // V[k][j]: pair g + 8k, states {2t, 2t+1, 8+2t, 9+2t}; the two
            // k-step halves added, then their truncation returned on average
            float V[4][4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int mt = k >> 1, h = k & 1;
                V[k][0] = add_half_ulp(D0[mt][0][2 * h] + D1[mt][0][2 * h]);
                V[k][1] = add_half_ulp(D0[mt][0][2 * h + 1] + D1[mt][0][2 * h + 1]);
                V[k][2] = add_half_ulp(D0[mt][1][2 * h] + D1[mt][1][2 * h]);
                V[k][3] = add_half_ulp(D0[mt][1][2 * h + 1] + D1[mt][1][2 * h + 1]);
            }
            int exk[4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                float m = fmaxf(fmaxf(V[k][0], V[k][1]), fmaxf(V[k][2], V[k][3]));
                m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 1));
                m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 2));
                int ex;
                float sc;
                pow2_scale(m, ex, sc);
                exk[k] = ex;
                const int u = base + g + 8 * k;
                if (u < n) {
                    float* o = nd.of + ((size_t)cc * nd.ocs + u) * 16;
                    *reinterpret_cast<float2*>(o + 2 * t) = make_float2(V[k][0] * sc, V[k][1] * sc);
                    *reinterpret_cast<float2*>(o + 8 + 2 * t) = make_float2(V[k][2] * sc, V[k][3] * sc);
                }
            }
            if (myvalid) {
                const int ex = exk[0] * (t == 0) + exk[1] * (t == 1) + exk[2] * (t == 2) + exk[3] * (t == 3);
                nd.oe[(size_t)cc * nd.ocs + myu] = e + ex;
            }
        }
    }
    cp_async_wait<0>();
    if (ROOT && myvalid) {
        const double res = (mm == -INFINITY) ? -INFINITY : mm + log((double)ss);
        nd.mix[myu] = (c0 == 0) ? res : lse_d(nd.mix[myu], res);
        if (per_lambda) {
#pragma unroll
            for (int q = 0; q < kMaxLambda; q++) {
                const double rq = (lm[q] == -INFINITY) ? -INFINITY : lm[q] + log((double)ls[q]);
                double* dst = nd.mixlam + (size_t)q * n + myu;
                *dst = (c0 == 0) ? rq : lse_d(*dst, rq);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// tcgen05 form of the interior node update (launch shape 3, chosen only on
// request: MESSI_PRUNE_SHAPE=3).  The CTA's 128 unique pairs of one node are
// the M = 128 rows of one tcgen05.mma (kind::tf32, N = 16 states, K = 8):
//   * the child rows are gathered with cp.async as in prune_msg_kernel, into
//     a stage of whole rows with XOR-ordered quads (Stage), so that both the
//     gathers and thread p's reads of pair p's rows are free of bank
//     conflicts;
//   * thread p forms x = m_left * m_right, splits it into TF32 hi and lo and
//     writes both to its own TMEM lane (tcgen05.st): the A operand comes from
//     tensor memory, not through shared memory;
//   * the node's branch matrix P (B operand, N x K, K-major) is split into hi
//     and lo by the CTA and written to shared memory in the canonical
//     no-swizzle layout: core matrices of 8 rows x 16 bytes, the two 8-row
//     groups of N 128 bytes apart (SBO), the two 4-wide K groups of one MMA
//     256 bytes apart (LBO);
//   * one thread issues, per K half, lo*hi, hi*lo, hi*hi into that half's
//     own accumulator (TMEM columns 32..47 and 48..63), the same split and
//     order as prune_msg_kernel (K half 0 = states {0,1,4,5,8,9,12,13}), and
//     commits them to an mbarrier;
//   * thread p reads its pair's 2 x 16 accumulators back (tcgen05.ld), adds
//     the halves and half an ulp as prune_msg_kernel does, rescales by a power
//     of two and stores the row -- one category late: the MMAs of category c
//     run while the CTA waits for and multiplies the rows of category c + 1,
//     and P is loaded one category ahead.
// TMEM: 64 columns per CTA (A hi 0..15, A lo 16..31, D 32..63); at most 6
// CTAs of this kernel fit on an SM by shared memory (36 KB each), 384 columns.  A wait on
// the mbarrier that gives up (bounded) writes NaN rows, so the likelihood
// that uses them is NaN, and the CTA still frees its TMEM before it returns.
// ---------------------------------------------------------------------------
namespace tc {
constexpr int kStages = 2;
constexpr unsigned kCols = 64;
constexpr unsigned kColAhi = 0, kColAlo = 16, kColD = 32;

// A stage holds each pair's two child rows whole (64 bytes each: the four
// 16-byte copies of one row land side by side, as the gather delivers them),
// with the quads of row p in XOR order q ^ ((p / 2) % 4), so that thread p's
// load of quad q from 32 consecutive rows touches every bank once per
// 128 bytes.
struct Stage {
    float4 x[2][kTile][4];  // [side][pair][quad position]
    int e[2][kTile];
};
__device__ __forceinline__ int qpos(int p, int q) { return q ^ ((p >> 1) & 3); }

struct Smem {
    Stage st[kStages];
    float bhi[256];  // P hi, canonical K-major layout (boff below)
    float blo[256];
    unsigned long long mbar;
    unsigned tmem_base;
    int fail;
};

// Contraction index of column c (0..7) of K half ks: d = 4(c/2) + 2ks + c%2.
__host__ __device__ constexpr int kidx(int ks, int c) { return 4 * (c >> 1) + 2 * ks + (c & 1); }

// Float offset of P[i][d] in the B buffer: K half ks = (d/2)%2 at 128 floats,
// column c = 2(d/4) + d%2 of that half; core matrix (row group i/8, K group
// c/4) at (c/4)*64 + (i/8)*32 floats, row i%8 at 4 floats, element c%4.
__host__ __device__ constexpr int boff(int i, int d)
{
    return ((d >> 1) & 1) * 128 + (((2 * (d >> 2) + (d & 1)) >> 2) * 64) + (i >> 3) * 32 + (i & 7) * 4 +
           ((2 * (d >> 2) + (d & 1)) & 3);
}

// Row and state of P held at float o (even) of the B buffer: the inverse of
// boff, so that a thread storing floats o and o + 1 reads P[row][d..d+1].
__host__ __device__ constexpr int brow(int o) { return (((o & 127) >> 5 & 1) << 3) | (((o & 127) >> 2) & 7); }
__host__ __device__ constexpr int bstate(int o) { return kidx(o >> 7, (((o & 127) >> 6) << 2) | (o & 3)); }

constexpr bool b_layout_ok()
{
    bool seen[256] = {};
    for (int i = 0; i < 16; i++)
        for (int d = 0; d < 16; d++) {
            const int o = boff(i, d);
            if (o < 0 || o >= 256 || seen[o]) return false;
            seen[o] = true;
        }
    for (int o = 0; o < 256; o += 2)
        if ((bstate(o) & 1) || boff(brow(o), bstate(o)) != o || boff(brow(o), bstate(o) + 1) != o + 1) return false;
    return true;
}
static_assert(b_layout_ok(), "B operand layout: boff must be a bijection and brow/bstate its inverse");

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor, no swizzle: start, LBO, SBO in 16-byte
// units; bit 46 = descriptor version 1.
__device__ __forceinline__ unsigned long long bdesc(unsigned addr)
{
    return (unsigned long long)((addr & 0x3FFFFu) >> 4) | ((unsigned long long)(256u >> 4) << 16) |
           ((unsigned long long)(128u >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::tf32: D F32 (bits 4-5 = 1), A and B TF32
// (bits 7-9, 10-12 = 2), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28.
constexpr unsigned kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((16u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void mma_ts(unsigned d, unsigned a, unsigned long long b, unsigned acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(d),
        "r"(a), "l"(b), "r"(kIdesc), "r"(acc));
}

__device__ __forceinline__ void st16(unsigned taddr, const uint32_t (&v)[16])
{
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};\n" ::"r"(
            taddr),
        "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]), "r"(v[9]),
        "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15]));
}

__device__ __forceinline__ void ld32(unsigned taddr, uint32_t (&v)[32])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
        "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
          "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
          "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// Bounded wait for phase `parity` of the mbarrier; false if it gave up.
__device__ __forceinline__ bool mbar_wait(unsigned addr, unsigned parity)
{
    for (int it = 0; it < (1 << 16); it++) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred q;\n\tmbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n\tselp.u32 %0, 1, 0, q;\n\t}\n"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}
}  // namespace tc

__global__ void __launch_bounds__(kTile, 6) prune_tc_kernel(const NodeDev* __restrict__ nodes,
                                                           const int2* __restrict__ tiles,
                                                           const float* __restrict__ P, int numnodes, int c0, int nc)
{
    extern __shared__ float4 smem_raw[];
    tc::Smem& S = *reinterpret_cast<tc::Smem*>(smem_raw);
    const int2 tile = tiles[blockIdx.x];
    const NodeDev& nd = nodes[tile.x];
    const int n = nd.n;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t = lane & 3;
    const unsigned mbar = tc::smem_u32(&S.mbar);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         tc::smem_u32(&S.tmem_base)),
                     "r"(tc::kCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mbar));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        S.fail = 0;
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const unsigned tbase = S.tmem_base;
    const unsigned tlane = tbase + ((unsigned)(32 * warp) << 16);  // this warp's 32 TMEM lanes

    // gathers: lane (g, t) copies state quad t of pairs g + 8k of its warp
    const int wbase = 32 * warp;
    int li[4], ri[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int u = tile.y + wbase + g + 8 * k;
        const int uc = (u < n) ? u : (n - 1);
        li[k] = __ldg(nd.li + uc);
        ri[k] = __ldg(nd.ri + uc);
    }
    const int myl = li[0] * (t == 0) + li[1] * (t == 1) + li[2] * (t == 2) + li[3] * (t == 3);
    const int myr = ri[0] * (t == 0) + ri[1] * (t == 1) + ri[2] * (t == 2) + ri[3] * (t == 3);
    const float* lf = nd.lf;
    const float* rf = nd.rf;
    const int* le = nd.le;
    const int* re = nd.re;
    const long long lcs = nd.lcs, rcs = nd.rcs;
    auto issue = [&](int cc) {
        tc::Stage& st = S.st[cc % tc::kStages];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int pl = wbase + g + 8 * k;
            cp_async16(&st.x[0][pl][tc::qpos(pl, t)], lf + ((size_t)cc * lcs + li[k]) * 16 + 4 * t);
            cp_async16(&st.x[1][pl][tc::qpos(pl, t)], rf + ((size_t)cc * rcs + ri[k]) * 16 + 4 * t);
        }
        if (le) cp_async4(&st.e[0][wbase + g + 8 * t], le + (size_t)cc * lcs + myl);
        if (re) cp_async4(&st.e[1][wbase + g + 8 * t], re + (size_t)cc * rcs + myr);
    };
#pragma unroll
    for (int s0 = 0; s0 < tc::kStages - 1; s0++) {
        if (s0 < nc) issue(s0);
        cp_async_commit();
    }
    const int myu = tile.y + tid;  // the pair this thread finishes
    const bool myvalid = myu < n;
    // this thread's two B entries, in layout order (floats 2 tid and 2 tid + 1
    // of the buffer, the inverse of boff, so the stores are conflict-free): row
    // pi_ of P, states pd and pd + 1
    const int bo = 2 * tid;
    const int pi_ = tc::brow(bo), pd = tc::bstate(bo);
    auto pload = [&](int cc) {
        return __ldg(reinterpret_cast<const float2*>(P + ((size_t)(c0 + cc) * numnodes + nd.self) * 256 + pi_ * 16 +
                                                     pd));
    };
    // category cf's accumulators back from TMEM (its MMAs ran while the next
    // category's rows were read), rescaled and stored with exponent ef
    auto finish = [&](int cf, int ef) {
        const bool ok = __all_sync(0xffffffffu, tc::mbar_wait(mbar, (unsigned)(cf & 1)));
        tc::fence_after();
        float V[16];
        if (ok) {
            uint32_t D[32];
            tc::ld32(tlane + tc::kColD, D);
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            // D[c] / D[16 + c]: K halves 0 and 1 of state c
#pragma unroll
            for (int c = 0; c < 16; c++) V[c] = add_half_ulp(__uint_as_float(D[c]) + __uint_as_float(D[16 + c]));
        } else {
#pragma unroll
            for (int c = 0; c < 16; c++) V[c] = __int_as_float(0x7fc00000);
            if (lane == 0) *(volatile int*)&S.fail = 1;
        }
        tc::fence_before();
        float m = V[0];
#pragma unroll
        for (int c = 1; c < 16; c++) m = fmaxf(m, V[c]);
        int ex;
        float sc;
        pow2_scale(m, ex, sc);
        if (myvalid) {
            // the row as two 32-byte stores: whole sectors
            float* o = nd.of + ((size_t)cf * nd.ocs + myu) * 16;
#pragma unroll
            for (int h = 0; h < 2; h++)
                asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};\n" ::"l"(o + 8 * h),
                             "f"(V[8 * h] * sc), "f"(V[8 * h + 1] * sc), "f"(V[8 * h + 2] * sc),
                             "f"(V[8 * h + 3] * sc), "f"(V[8 * h + 4] * sc), "f"(V[8 * h + 5] * sc),
                             "f"(V[8 * h + 6] * sc), "f"(V[8 * h + 7] * sc)
                             : "memory");
            nd.oe[(size_t)cf * nd.ocs + myu] = ef + ex;
        }
    };
    float2 ppn = (nc > 0) ? pload(0) : make_float2(0.f, 0.f);
    int eprev = 0;
    for (int cc = 0; cc < nc; cc++) {
        if (cc + tc::kStages - 1 < nc) issue(cc + tc::kStages - 1);
        cp_async_commit();
        cp_async_wait<tc::kStages - 1>();
        __syncwarp();
        const float2 pp = ppn;
        if (cc + 1 < nc) ppn = pload(cc + 1);
        const tc::Stage& st = S.st[cc % tc::kStages];
        float x[16];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const float4 a = st.x[0][tid][tc::qpos(tid, q)], b = st.x[1][tid][tc::qpos(tid, q)];
            x[4 * q] = a.x * b.x;
            x[4 * q + 1] = a.y * b.y;
            x[4 * q + 2] = a.z * b.z;
            x[4 * q + 3] = a.w * b.w;
        }
        const int e = (le ? st.e[0][tid] : 0) + (re ? st.e[1][tid] : 0);
        // the previous category's MMAs are done with A, B and D after this
        if (cc > 0) finish(cc - 1, eprev);
        {
            uint32_t hi[16], lo[16];
#pragma unroll
            for (int ks = 0; ks < 2; ks++)
#pragma unroll
                for (int c = 0; c < 8; c++) split_a(x[tc::kidx(ks, c)], hi[8 * ks + c], lo[8 * ks + c]);
            tc::st16(tlane + tc::kColAhi, hi);
            tc::st16(tlane + tc::kColAlo, lo);
        }
        {
            uint32_t h0, l0, h1, l1;
            split_a(pp.x, h0, l0);
            split_a(pp.y, h1, l1);
            *reinterpret_cast<float2*>(S.bhi + bo) = make_float2(__uint_as_float(h0), __uint_as_float(h1));
            *reinterpret_cast<float2*>(S.blo + bo) = make_float2(__uint_as_float(l0), __uint_as_float(l1));
        }
        asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        tc::fence_before();
        __syncthreads();
        if (*(volatile int*)&S.fail) break;  // a wait gave up (uniform: read after the barrier)
        if (tid == 0) {
            tc::fence_after();
            const unsigned bh = tc::smem_u32(S.bhi), bl = tc::smem_u32(S.blo);
#pragma unroll
            for (int ks = 0; ks < 2; ks++) {
                const unsigned d = tbase + tc::kColD + 16 * ks;
                const unsigned long long dh = tc::bdesc(bh + 512 * ks), dl = tc::bdesc(bl + 512 * ks);
                tc::mma_ts(d, tbase + tc::kColAlo + 8 * ks, dh, 0u);
                tc::mma_ts(d, tbase + tc::kColAhi + 8 * ks, dl, 1u);
                tc::mma_ts(d, tbase + tc::kColAhi + 8 * ks, dh, 1u);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
                         : "memory");
        }
        eprev = e;
    }
    // S.fail is uniform here: last written before the final loop barrier
    if (nc > 0 && !*(volatile int*)&S.fail) finish(nc - 1, eprev);
    cp_async_wait<0>();
    tc::fence_before();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tbase), "r"(tc::kCols));
    }
}

static int launch_prune_tc(messi_ctx* ctx, const NodeDev* d_nodes, const int2* d_tiles, int nt, const float* d_P,
                           int numnodes, int c0, int nc)
{
    prune_tc_kernel<<<nt, kTile, sizeof(tc::Smem), ctx->stream>>>(d_nodes, d_tiles, d_P, numnodes, c0, nc);
    LAUNCH_CHECK(ctx, "prune_tc_kernel");
    return MESSI_OK;
}

template <int STAGES, int MINB>
static int launch_prune_shape(messi_ctx* ctx, const NodeDev* d_nodes, const int2* d_tiles, int nt, bool root,
                              const float* d_P, int numnodes, int c0, int nc, int C, const float* d_pi16,
                              const double* d_logw, const int* d_lam, bool per_lambda)
{
    static thread_local int smem_set_device = -1;
    const size_t smem = (size_t)(kTile / 32) * STAGES * sizeof(WarpStage);
    if (smem_set_device != ctx->device) {
        cudaFuncSetAttribute(prune_msg_kernel<false, STAGES, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        cudaFuncSetAttribute(prune_msg_kernel<true, STAGES, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        smem_set_device = ctx->device;
    }
    if (root) {
        prune_msg_kernel<true, STAGES, MINB><<<nt, kTile, smem, ctx->stream>>>(
            d_nodes, d_tiles, d_P, numnodes, c0, nc, C, d_pi16, d_logw, d_lam, per_lambda ? 1 : 0);
        LAUNCH_CHECK(ctx, "prune_msg_kernel<root>");
    } else {
        prune_msg_kernel<false, STAGES, MINB><<<nt, kTile, smem, ctx->stream>>>(
            d_nodes, d_tiles, d_P, numnodes, c0, nc, C, d_pi16, d_logw, d_lam, per_lambda ? 1 : 0);
        LAUNCH_CHECK(ctx, "prune_msg_kernel");
    }
    return MESSI_OK;
}

int launch_prune_tiles(messi_ctx* ctx, const NodeDev* d_nodes, const int2* d_tiles, int nt, bool root,
                       const float* d_P, int numnodes, int c0, int nc, int C, const float* d_pi16,
                       const double* d_logw, const int* d_lam, bool per_lambda)
{
    if (nt <= 0) return MESSI_OK;
    // shapes: 0 = 2 stages x 4 CTAs/SM, 1 = 3 stages x 3 CTAs, 2 = 2 stages x 3 CTAs (the autotuner's
    // candidates); 3 = interior levels in the tcgen05 form, the roots as shape 0 (on request only)
    if (ctx->prune_shape == 3 && !root) return launch_prune_tc(ctx, d_nodes, d_tiles, nt, d_P, numnodes, c0, nc);
    switch (ctx->prune_shape) {
        case 1: return launch_prune_shape<3, 3>(ctx, d_nodes, d_tiles, nt, root, d_P, numnodes, c0, nc, C, d_pi16,
                                                d_logw, d_lam, per_lambda);
        case 2: return launch_prune_shape<2, 3>(ctx, d_nodes, d_tiles, nt, root, d_P, numnodes, c0, nc, C, d_pi16,
                                                d_logw, d_lam, per_lambda);
        default: return launch_prune_shape<2, 4>(ctx, d_nodes, d_tiles, nt, root, d_P, numnodes, c0, nc, C, d_pi16,
                                                 d_logw, d_lam, per_lambda);
    }
}

int run_pairs(messi_ctx* ctx, messi_dataset* ds, const float* d_P, const float* d_pi16, const double* d_logw,
              const int* d_lam, int C, int nlam, bool per_lambda)
{
    (void)nlam;
    const int chunk = ds->chunk;
    for (int c0 = 0; c0 < C; c0 += chunk) {
        const int nc = std::min(chunk, C - c0);
        int rc = launch_leaf_messages(ctx, ds->d_leaf, ds->d_leafnode, ds->leaf_rows, d_P, ds->numnodes, c0, nc, C,
                                      ds->d_leafmsg);
        if (rc) return rc;
        for (int lv = 1; lv <= ds->H; lv++) {
            const int nt = ds->tile_cnt[lv];
            if (nt == 0) continue;
            if (ctx->profiling) {
                double units = 0.0;
                for (int v : ds->level_nodes[lv]) units += (double)ds->nunique[v] * nc;
                prof_begin(ctx, 0, units);
            }
            rc = launch_prune_tiles(ctx, ds->d_nodes, ds->d_tiles + ds->tile_off[lv], nt, lv == ds->H, d_P,
                                    ds->numnodes, c0, nc, C, d_pi16, d_logw, d_lam, per_lambda);
            if (rc) return rc;
            prof_end(ctx);
        }
    }
    return MESSI_OK;
}

// ---------------------------------------------------------------------------
// Unpaired columns: one thread per (column, site-rate category), nodes in
// post-order, partials of every node kept in a [nsite][numnodes][L][4]
// scratch table (FP64; the FP64 pipe is narrow on this part, so the work is
// spread over many small blocks); then the mixture over site rates in the
// reference's order.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(32) unpaired_site_kernel(const uint8_t* __restrict__ masks,
                                                           const int* __restrict__ tree, const int* __restrict__ post,
                                                           int nn, int L, const double* __restrict__ P4, int pstride,
                                                           const double* __restrict__ pi4, double* __restrict__ part,
                                                           double* __restrict__ lmv, double* __restrict__ ll)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int s = blockIdx.y;
    if (x >= L) return;
    const double* Ps = P4 + (size_t)s * pstride * 16;
    double* ps = part + (size_t)s * nn * L * 4;
    double* ls = lmv + (size_t)s * nn * L;
    for (int t = 0; t < nn; t++) {
        const int v = post[t];
        const int c0 = tree[4 * v], c1 = tree[4 * v + 1];
        double* pv = ps + ((size_t)v * L + x) * 4;
        if (c0 < 0) {
            const int m = masks[(size_t)tree[4 * v + 2] * L + x];
#pragma unroll
            for (int a = 0; a < 4; a++) pv[a] = (double)((m >> a) & 1);
            ls[(size_t)v * L + x] = 0.0;
            continue;
        }
        const double* p0 = ps + ((size_t)c0 * L + x) * 4;
        const double* p1 = ps + ((size_t)c1 * L + x) * 4;
        const double* P0 = Ps + (size_t)c0 * 16;
        const double* P1 = Ps + (size_t)c1 * 16;
        double l[4], r[4], o[4], m = -INFINITY;
#pragma unroll
        for (int a = 0; a < 4; a++) { l[a] = p0[a]; r[a] = p1[a]; }
#pragma unroll
        for (int a = 0; a < 4; a++) {
            double sl = 0.0, sr = 0.0;
#pragma unroll
            for (int d = 0; d < 4; d++) {
                sl += __ldg(P0 + a * 4 + d) * l[d];
                sr += __ldg(P1 + a * 4 + d) * r[d];
            }
            o[a] = sl * sr;
            m = fmax(m, o[a]);
        }
        double lm = ls[(size_t)c0 * L + x] + ls[(size_t)c1 * L + x];
        if (m < 1e-20) {  // src/FARCE.jl:2226-2238
#pragma unroll
            for (int a = 0; a < 4; a++) o[a] /= m;
            lm += log(m);
        }
#pragma unroll
        for (int a = 0; a < 4; a++) pv[a] = o[a];
        ls[(size_t)v * L + x] = lm;
    }
    const double* pr = ps + (size_t)x * 4;  // root = node 0
    double tot = 0.0;
#pragma unroll
    for (int a = 0; a < 4; a++) tot += pi4[a] * pr[a];
    ll[(size_t)s * L + x] = log(tot) + ls[x];
}

__global__ void unpaired_mix_kernel(const double* __restrict__ ll, const double* __restrict__ logw_site, int nsite,
                                    int L, double* __restrict__ u)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= L) return;
    double acc = -INFINITY;
    for (int s = 0; s < nsite; s++) {
        const double v = ll[(size_t)s * L + x] + logw_site[s];
        acc = (s == 0) ? v : lse_d(acc, v);
    }
    u[x] = acc;
}

int launch_unpaired(messi_ctx* ctx, messi_dataset* ds, const double* d_P4, int pstride, const double* d_pi4,
                    const double* d_logw_site, int nsite, double* d_u, double* d_scratch)
{
    // d_scratch: nsite * (numnodes * L * 5 + L) doubles, or nullptr for the context's buffer
    const size_t n = (size_t)ds->numnodes * ds->L;
    if (!d_scratch) {
        void* scratch;
        int rc = ensure(ctx, 20, ((size_t)nsite * (n * 5 + ds->L)) * sizeof(double), &scratch);
        if (rc) return rc;
        d_scratch = (double*)scratch;
    }
    double* part = d_scratch;
    double* lmv = part + (size_t)nsite * n * 4;
    double* ll = lmv + (size_t)nsite * n;
    const int bs = 32;
    unpaired_site_kernel<<<dim3((ds->L + bs - 1) / bs, nsite), bs, 0, ctx->stream>>>(
        ds->d_masks, ds->d_tree, ds->d_post, ds->numnodes, ds->L, d_P4, pstride, d_pi4, part, lmv, ll);
    LAUNCH_CHECK(ctx, "unpaired_site_kernel");
    unpaired_mix_kernel<<<(ds->L + 127) / 128, 128, 0, ctx->stream>>>(ll, d_logw_site, nsite, ds->L, d_u);
    LAUNCH_CHECK(ctx, "unpaired_mix_kernel");
    return MESSI_OK;
}

// ---------------------------------------------------------------------------
// Output layouts
// ---------------------------------------------------------------------------
__global__ void scatter_dense_kernel(const int* __restrict__ bandidx, const double* __restrict__ vals,
                                     const double* __restrict__ u, double addw, int L, int W,
                                     double* __restrict__ out)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)L * L) return;
    const int x = (int)(idx % L), y = (int)(idx / L);
    const int k = (x > y) ? x - y : y - x;
    const int i = (x < y) ? x : y;
    double val = -INFINITY;
    if (k >= 1 && k <= W) {
        const int b = bandidx[(size_t)i * (W + 1) + k];
        if (b >= 0) {
            if (vals) val = vals[b];
            if (addw != -INFINITY) val = lse_d(val, addw + u[i] + u[i + k]);
        }
    }
    out[idx] = val;
}

int launch_scatter_dense(messi_ctx* ctx, messi_dataset* ds, const double* d_vals, const double* d_u, double addw,
                         double* d_out)
{
    const long long n = (long long)ds->L * ds->L;
    const int bs = 256;
    if (addw != -INFINITY && !d_u) return fail(ctx, MESSI_EINVAL, "scatter: factorised term without unpaired values");
    scatter_dense_kernel<<<(unsigned)((n + bs - 1) / bs), bs, 0, ctx->stream>>>(ds->d_bandidx, d_vals, d_u, addw,
                                                                                ds->L, ds->W, d_out);
    LAUNCH_CHECK(ctx, "scatter_dense_kernel");
    return MESSI_OK;
}

// Banded log-odds pair scores from the root mixtures (device-resident path),
// with maskgapped! (src/RNATools.jl:441-451) folded in.
// The factorised lambda categories add logwF + u[i] + u[j] to the mixture
// (logwF read from d_logwF when given: a replayed graph then sees each call's
// value).
__global__ void bandprep_from_mix_kernel(const int* __restrict__ bandidx, const double* __restrict__ mix, int L, int W,
                                         int Wb, int RS, const uint8_t* __restrict__ gapmask,
                                         const double* __restrict__ u, double logwF_value,
                                         const double* __restrict__ d_logwF, const double* __restrict__ b, double B,
                                         float* __restrict__ pb)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)L * RS) return;
    const double logwF = d_logwF ? *d_logwF : logwF_value;
    const int i = (int)(idx / RS), k = (int)(idx % RS);
    float out = -INFINITY;
    if (k >= 1 && k <= Wb && i + k < L && k <= W) {
        const int bi = bandidx[(size_t)i * (W + 1) + k];
        if (bi >= 0 && !(gapmask && (gapmask[i] || gapmask[i + k]))) {
            double p = mix[bi];
            if (logwF != -INFINITY) p = lse_d_fast(p, logwF + u[i] + u[i + k]);
            if (p != -INFINITY) out = (float)(B * p - b[i] - b[i + k]);
        }
    }
    pb[idx] = out;
}

int launch_bandprep_from_mix(messi_ctx* ctx, messi_dataset* ds, const Band& t, const uint8_t* d_gapmask, double B,
                             double logwF, const double* d_logwF)
{
    const long long n = (long long)t.L * t.RS;
    const int bs = 256;
    bandprep_from_mix_kernel<<<(unsigned)((n + bs - 1) / bs), bs, 0, ctx->stream>>>(
        ds->d_bandidx, ds->d_mix, ds->L, ds->W, t.Wb, t.RS, d_gapmask, t.u, logwF, d_logwF, t.b, B, t.pb);
    LAUNCH_CHECK(ctx, "bandprep_from_mix_kernel");
    return MESSI_OK;
}

// ---------------------------------------------------------------------------
// Fixed-structure likelihood: sum of the unpaired columns and of the pairs
// (one block, FP64, fixed reduction order).  On return u holds the unpaired
// log-likelihood of unpaired columns and 0 on paired ones (the reference's
// computeunpairedlikelihoods(..., paired), src/FARCE.jl:1222-1250), pairll
// the pair log-likelihood at the first column of each pair and 0 elsewhere.
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// Site-rate conditionals (felsensteinposteriorsiterateconditionalscuda,
// src/FelsensteinCUDA.jl:518-717): for column x and site-rate category s,
//   LSE( log w_s + log single[x] + u_s[x],
//        over band partners y > x, categories with s1 = s:
//            log pair[x,y] + log w_c + ll_c(x, y),
//        over band partners y < x, categories with s2 = s:
//            log pair[y,x] + log w_c + ll_c(y, x) )
// One thread per (column, category); categories in the order s1, s2, lambda.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double lse_acc(double a, double b)
{
    if (b == -INFINITY) return a;
    if (a == -INFINITY) return b;
    return (a < b) ? b + log1p(exp(a - b)) : a + log1p(exp(b - a));
}

__global__ void siterate_cond_kernel(const int* __restrict__ bandidx, int L, int W, const double* __restrict__ catll,
                                     int nroot, const double* __restrict__ logw, int ns, int nl,
                                     const double* __restrict__ single, const double* __restrict__ pair,
                                     const double* __restrict__ ull, const double* __restrict__ logw_site,
                                     double* __restrict__ out)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int s = blockIdx.y;
    if (x >= L) return;
    double acc = -INFINITY;
    const double us = ull[(size_t)s * L + x];
    if (us != -INFINITY) acc = lse_acc(acc, logw_site[s] + log(single[x]) + us);
    for (int k = 1; k <= W && x + k < L; k++) {
        const int b = bandidx[(size_t)x * (W + 1) + k];
        if (b < 0) continue;
        const double pp = pair[(size_t)x + (size_t)(x + k) * L];
        if (!(pp > 0.0)) continue;
        const double lp = log(pp);
        for (int s2 = 0; s2 < ns; s2++)
            for (int l = 0; l < nl; l++) {
                const int c = (s * ns + s2) * nl + l;
                acc = lse_acc(acc, lp + logw[c] + catll[(size_t)c * nroot + b]);
            }
    }
    for (int k = 1; k <= W && k <= x; k++) {
        const int y = x - k;
        const int b = bandidx[(size_t)y * (W + 1) + k];
        if (b < 0) continue;
        const double pp = pair[(size_t)y + (size_t)x * L];
        if (!(pp > 0.0)) continue;
        const double lp = log(pp);
        for (int s1 = 0; s1 < ns; s1++)
            for (int l = 0; l < nl; l++) {
                const int c = (s1 * ns + s) * nl + l;
                acc = lse_acc(acc, lp + logw[c] + catll[(size_t)c * nroot + b]);
            }
    }
    out[(size_t)s + (size_t)x * ns] = acc;
}

int launch_siterate_conditionals(messi_ctx* ctx, messi_dataset* ds, const double* d_catll, const double* d_logw,
                                 int nsite, int nlam, const double* d_single, const double* d_pair,
                                 const double* d_ull, const double* d_logw_site, double* d_out)
{
    const int bs = 64;
    siterate_cond_kernel<<<dim3((ds->L + bs - 1) / bs, nsite), bs, 0, ctx->stream>>>(
        ds->d_bandidx, ds->L, ds->W, d_catll, (int)ds->nroot, d_logw, nsite, nlam, d_single, d_pair, d_ull,
        d_logw_site, d_out);
    LAUNCH_CHECK(ctx, "siterate_cond_kernel");
    return MESSI_OK;
}

// colu[c]: unique root pair of the pair opened at column c (>= 0), -2 on the
// closing column of a pair, -1 on an unpaired column; partner[c] the other
// column of the pair opened at c.  The factorised lambda categories add
// logwF + u[c] + u[partner] to each pair, so the unpaired values of paired
// columns are read before they are cleared.
__global__ void __launch_bounds__(1024) structure_sum_kernel(double* __restrict__ u, const int* __restrict__ colu,
                                                             const int* __restrict__ partner, int L,
                                                             const double* __restrict__ mix, double logwF,
                                                             double* __restrict__ total, double* __restrict__ pairll)
{
    __shared__ double part[1024];
    double acc = 0.0;
    for (int c = threadIdx.x; c < L; c += blockDim.x) {
        const int k = colu[c];
        double pv = 0.0;
        if (k >= 0) {
            pv = mix[k];
            if (logwF != -INFINITY) pv = lse_d(pv, logwF + u[c] + u[partner[c]]);
        }
        if (k == -1) acc += u[c];
        pairll[c] = pv;
        acc += pv;
    }
    __syncthreads();
    for (int c = threadIdx.x; c < L; c += blockDim.x)
        if (colu[c] != -1) u[c] = 0.0;
    part[threadIdx.x] = acc;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) part[threadIdx.x] += part[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) total[0] = part[0];
}

int launch_structure_sum(messi_ctx* ctx, int L, double* d_u, const int* d_colu, const int* d_partner,
                         const double* d_mix, double logwF, double* d_total, double* d_pairll)
{
    structure_sum_kernel<<<1, 1024, 0, ctx->stream>>>(d_u, d_colu, d_partner, L, d_mix, logwF, d_total, d_pairll);
    LAUNCH_CHECK(ctx, "structure_sum_kernel");
    return MESSI_OK;
}

}  // namespace messi
