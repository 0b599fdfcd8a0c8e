// mlp.cu -- the learned MCMC proposal network (HP3): a BF16 MLP with a
// Gaussian-mixture head, trained and evaluated on the GPU.
//
// The reference's MCMC moves (src/MCMC.jl:1307-1674) have no learned part;
// this network is the proposal described for the learned chain: input = the
// current model parameters (transformed) + alignment summary statistics,
// output = a K-component diagonal Gaussian mixture over the free parameters.
//
// Layout: three linear layers in -> H -> H -> out with SiLU after the first
// two.  Weights are kept in FP32 (Adam master copy) and BF16 (the copy the
// forward/backward kernels read); activations are BF16, and so are the
// gradient operands of the backward GEMMs (rounded while a tile is staged);
// every product is accumulated in FP32.  Every GEMM runs on the tensor cores
// (gemm_bf16_kernel: 32 x 32 CTA tiles, four warps of 16 x 16, BF16
// mma.sync m16n8k16 with FP32 accumulators) with its epilogue fused: bias,
// bias + SiLU (writing the FP32 pre-activation and the BF16 activation), or
// the SiLU derivative of the backward pass.  The network is small (batch a
// few hundred, width 256), so a GEMM is latency bound: small tiles for more
// CTAs, a 256-wide K chunk staged per barrier, and the fused epilogues
// remove the elementwise launches between the GEMMs.
//
// Head per sample: [K logits | K*D means | K*D log-sd]; the loss is the
// negative log-likelihood of a target vector under the mixture.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"

struct messi_mlp {
    int in = 0, H = 0, out = 0, K = 0, D = 0;
    int cap = 0;                       // batch capacity of the activation buffers
    // parameters: W1[H][in] b1[H] W2[H][H] b2[H] W3[out][H] b3[out]
    int nparam = 0;
    float* p32 = nullptr;              // FP32 master
    __nv_bfloat16* p16 = nullptr;      // BF16 copy
    float* grad = nullptr;
    float* m1 = nullptr;               // Adam moments
    float* m2 = nullptr;
    int64_t steps = 0;
    // activations
    __nv_bfloat16 *x = nullptr, *a1 = nullptr, *a2 = nullptr;   // inputs / post-SiLU (BF16)
    float *z1 = nullptr, *z2 = nullptr, *y = nullptr;           // pre-activations, head (FP32)
    float *dy = nullptr, *d2 = nullptr, *d1 = nullptr;          // gradients w.r.t. y, a2/z2, a1/z1
    float* target = nullptr;
    float* loss = nullptr;             // [cap]
    float* stage = nullptr;            // host-pinned staging
};

namespace messi {

namespace {

__device__ __forceinline__ float silu(float z);
__device__ __forceinline__ float dsilu(float z);

__device__ __forceinline__ __nv_bfloat16 to_bf(float v) { return __float2bfloat16(v); }
__device__ __forceinline__ __nv_bfloat16 to_bf(__nv_bfloat16 v) { return v; }


// CTA tile 32 x 32 (four warps of 16 x 16), the K extent staged in chunks of
// kBK: the GEMMs of this network are a few hundred rows, so the CTA count,
// not the per-CTA rate, bounds them; a whole chunk's loads are issued before
// the one CTA barrier, so a chunk costs one memory round trip.
constexpr int kBM = 32, kBN = 32, kBK = 256, kPad = 8;

// Four consecutive elements (16 B of FP32 or 8 B of BF16), rounded to BF16.
__device__ __forceinline__ void load4_bf(const float* p, __nv_bfloat16 (&o)[4])
{
    const float4 v = __ldg(reinterpret_cast<const float4*>(p));
    o[0] = __float2bfloat16(v.x);
    o[1] = __float2bfloat16(v.y);
    o[2] = __float2bfloat16(v.z);
    o[3] = __float2bfloat16(v.w);
}
__device__ __forceinline__ void load4_bf(const __nv_bfloat16* p, __nv_bfloat16 (&o)[4])
{
    const uint2 v = __ldg(reinterpret_cast<const uint2*>(p));
    const __nv_bfloat16* b = reinterpret_cast<const __nv_bfloat16*>(&v);
    o[0] = b[0];
    o[1] = b[1];
    o[2] = b[2];
    o[3] = b[3];
}

// Stage rows r0.. of one operand tile, [rows][k] in shared memory (rows of
// kBK + kPad): X(r, k) = X[r*srow + k*sk].  With vec (unit stride along the
// fast index, the other stride a multiple of 4, the base aligned), four
// consecutive elements of the fast index come in one load.
template <int ROWS, typename T>
__device__ __forceinline__ void stage_tile(__nv_bfloat16 (*dst)[kBK + 8], const T* __restrict__ X, long long srow,
                                           long long sk, int r0, int nrows, int k0, int kc, int kc16, bool vec)
{
    const bool k_fast = (sk == 1);
    if (vec) {
        for (int e = threadIdx.x; e < ROWS * kBK / 4; e += blockDim.x) {
            // groups of four along the fast index
            const int r = k_fast ? e / (kBK / 4) : 4 * (e % (ROWS / 4));
            const int c = k_fast ? 4 * (e % (kBK / 4)) : e / (ROWS / 4);
            if (c >= kc16) continue;
            __nv_bfloat16 v[4];
            const int rr = r0 + r, kk = k0 + c;
            if (k_fast) {
                if (rr < nrows && c + 3 < kc) load4_bf(X + rr * srow + kk, v);
                else
                    for (int q = 0; q < 4; q++)
                        v[q] = (rr < nrows && c + q < kc) ? to_bf(X[rr * srow + kk + q]) : __float2bfloat16(0.f);
                for (int q = 0; q < 4; q++) dst[r][c + q] = v[q];
            } else {
                if (rr + 3 < nrows && c < kc) load4_bf(X + rr + kk * sk, v);
                else
                    for (int q = 0; q < 4; q++)
                        v[q] = (rr + q < nrows && c < kc) ? to_bf(X[(rr + q) + kk * sk]) : __float2bfloat16(0.f);
                for (int q = 0; q < 4; q++) dst[r + q][c] = v[q];
            }
        }
    } else {
        for (int e = threadIdx.x; e < ROWS * kBK; e += blockDim.x) {
            const int r = k_fast ? e / kBK : e % ROWS, c = k_fast ? e % kBK : e / ROWS;
            if (c >= kc16) continue;
            const int rr = r0 + r, kk = k0 + c;
            dst[r][c] = (rr < nrows && c < kc) ? to_bf(X[rr * srow + kk * sk]) : __float2bfloat16(0.f);
        }
    }
}

template <typename T>
__host__ __device__ inline bool vec_ok(const T* p, long long srow, long long sk)
{
    const size_t align = sizeof(T) * 4;
    const bool unit = (srow == 1) != (sk == 1) && (srow == 1 || sk == 1);
    const long long other = (sk == 1) ? srow : sk;
    return unit && other % 4 == 0 && (reinterpret_cast<size_t>(p) % align) == 0;
}

// GEMM epilogues
enum GemmMode {
    kStoreBias = 0,  // C = acc + bias[n]
    kAccumulate = 1, // C += acc
    kBiasSilu = 2,   // z = acc + bias[n]; C = z (FP32); act = bf16(silu(z))
    kDsilu = 3       // C = acc * dsilu(z[m][n])
};

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// C[m][n] (row stride scm) = epilogue(sum_k A(m, k) * B(k, n)) with
// A(m,k) = A[m*sam + k*sak], B(k,n) = B[k*sbk + n*sbn]; operands are rounded
// to BF16 as they are staged in shared memory ([row][k], k contiguous, rows
// padded by 8 so the fragment loads hit 32 distinct banks).
template <typename TA, typename TB>
__global__ void __launch_bounds__(128) gemm_bf16_kernel(int M, int N, int K, const TA* __restrict__ A, long long sam,
                                                        long long sak, const TB* __restrict__ B, long long sbk,
                                                        long long sbn, const float* __restrict__ bias,
                                                        float* __restrict__ C, long long scm, int mode,
                                                        const float* __restrict__ z, __nv_bfloat16* __restrict__ act)
{
    __shared__ __align__(16) __nv_bfloat16 As[kBM][kBK + kPad];
    __shared__ __align__(16) __nv_bfloat16 Bs[kBN][kBK + kPad];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int wm = (warp >> 1) * 16, wn = (warp & 1) * 16;
    const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
    float acc[2][4];
#pragma unroll
    for (int j = 0; j < 2; j++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[j][q] = 0.f;
    // consecutive threads walk the operand's unit-stride index (coalesced)
    const bool va = vec_ok(A, sam, sak), vb = vec_ok(B, sbn, sbk);
    for (int k0 = 0; k0 < K; k0 += kBK) {
        const int kc = min(kBK, K - k0);
        const int kc16 = (kc + 15) & ~15;  // chunk rounded up to whole k16 steps (zero padded)
        if (k0 > 0) __syncthreads();
        stage_tile<kBM>(As, A, sam, sak, m0, M, k0, kc, kc16, va);
        stage_tile<kBN>(Bs, B, sbn, sbk, n0, N, k0, kc, kc16, vb);
        __syncthreads();
        for (int ks = 0; ks < kc16; ks += 16) {
            uint32_t af[4], bf[2][2];
            const int r = wm + g;
            af[0] = *reinterpret_cast<const uint32_t*>(&As[r][ks + 2 * t]);
            af[1] = *reinterpret_cast<const uint32_t*>(&As[r + 8][ks + 2 * t]);
            af[2] = *reinterpret_cast<const uint32_t*>(&As[r][ks + 2 * t + 8]);
            af[3] = *reinterpret_cast<const uint32_t*>(&As[r + 8][ks + 2 * t + 8]);
#pragma unroll
            for (int nt = 0; nt < 2; nt++) {
                const int c = wn + nt * 8 + g;
                bf[nt][0] = *reinterpret_cast<const uint32_t*>(&Bs[c][ks + 2 * t]);
                bf[nt][1] = *reinterpret_cast<const uint32_t*>(&Bs[c][ks + 2 * t + 8]);
            }
#pragma unroll
            for (int nt = 0; nt < 2; nt++) mma_bf16(acc[nt], af, bf[nt][0], bf[nt][1]);
        }
    }
#pragma unroll
    for (int nt = 0; nt < 2; nt++)
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int m = m0 + wm + g + 8 * (q >> 1);
            const int n = n0 + wn + nt * 8 + 2 * t + (q & 1);
            if (m >= M || n >= N) continue;
            const long long o = m * scm + n;
            const float v = acc[nt][q];
            if (mode == kStoreBias) {
                C[o] = v + (bias ? bias[n] : 0.f);
            } else if (mode == kAccumulate) {
                C[o] += v;
            } else if (mode == kBiasSilu) {
                const float zz = v + (bias ? bias[n] : 0.f);
                C[o] = zz;
                act[o] = __float2bfloat16(silu(zz));
            } else {
                C[o] = v * dsilu(z[o]);
            }
        }
}

template <typename TA, typename TB>
int gemm(messi_ctx* ctx, int M, int N, int K, const TA* A, long long sam, long long sak, const TB* B, long long sbk,
         long long sbn, const float* bias, float* C, long long scm, int mode, const float* z = nullptr,
         __nv_bfloat16* act = nullptr)
{
    dim3 grid((N + kBN - 1) / kBN, (M + kBM - 1) / kBM);
    gemm_bf16_kernel<TA, TB><<<grid, 128, 0, ctx->stream>>>(M, N, K, A, sam, sak, B, sbk, sbn, bias, C, scm, mode, z,
                                                            act);
    LAUNCH_CHECK(ctx, "gemm_bf16_kernel");
    return MESSI_OK;
}

__device__ __forceinline__ float silu(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z)
{
    const float s = 1.f / (1.f + __expf(-z));
    return s * (1.f + z * (1.f - s));
}

__global__ void to_bf16_kernel(const float* __restrict__ s, __nv_bfloat16* __restrict__ d, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = __float2bfloat16(s[i]);
}

__global__ void colsum_kernel(const float* __restrict__ dY, int M, int N, float* __restrict__ db)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.f;
    for (int m = 0; m < M; m++) s += dY[(long long)m * N + n];
    db[n] += s;
}

// Mixture negative log-likelihood per sample and its gradient w.r.t. the head.
// y: [K logits | K*D means | K*D log-sd], log-sd clamped to [-7, 5].
__global__ void mixture_nll_kernel(const float* __restrict__ y, const float* __restrict__ tgt, int M, int K, int D,
                                   float* __restrict__ loss, float* __restrict__ dy, float inv_batch)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    const int O = K + 2 * K * D;
    const float* ym = y + (long long)m * O;
    const float* x = tgt + (long long)m * D;
    float* g = dy + (long long)m * O;
    float lw[8], lp[8];
    float mx = -INFINITY;
    for (int k = 0; k < K; k++) mx = fmaxf(mx, ym[k]);
    float se = 0.f;
    for (int k = 0; k < K; k++) se += __expf(ym[k] - mx);
    const float lse_w = mx + __logf(se);
    const float c = -0.91893853320467274f * D;  // -D/2 log(2 pi)
    float best = -INFINITY;
    for (int k = 0; k < K; k++) {
        lw[k] = ym[k] - lse_w;
        float s = c;
        for (int d = 0; d < D; d++) {
            const float ls = fminf(fmaxf(ym[K + K * D + k * D + d], -7.f), 5.f);
            const float r = (x[d] - ym[K + k * D + d]) * __expf(-ls);
            s += -0.5f * r * r - ls;
        }
        lp[k] = lw[k] + s;
        best = fmaxf(best, lp[k]);
    }
    float tot = 0.f;
    for (int k = 0; k < K; k++) tot += __expf(lp[k] - best);
    const float ll = best + __logf(tot);
    loss[m] = -ll;
    for (int k = 0; k < K; k++) {
        const float r_k = __expf(lp[k] - ll);        // responsibility
        const float w_k = __expf(lw[k]);
        g[k] = (w_k - r_k) * inv_batch;              // d(-ll)/d logit
        for (int d = 0; d < D; d++) {
            const float raw = ym[K + K * D + k * D + d];
            const float ls = fminf(fmaxf(raw, -7.f), 5.f);
            const float iv = __expf(-2.f * ls);
            const float diff = x[d] - ym[K + k * D + d];
            g[K + k * D + d] = -r_k * diff * iv * inv_batch;
            const float gls = -r_k * (diff * diff * iv - 1.f);
            g[K + K * D + k * D + d] = (raw > -7.f && raw < 5.f) ? gls * inv_batch : 0.f;
        }
    }
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ gr, float* __restrict__ m1,
                            float* __restrict__ m2, __nv_bfloat16* __restrict__ p16, int n, float lr, float b1,
                            float b2, float c1, float c2, float eps, float clip_scale)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = gr[i] * clip_scale;
    const float a = b1 * m1[i] + (1.f - b1) * g;
    const float b = b2 * m2[i] + (1.f - b2) * g * g;
    m1[i] = a;
    m2[i] = b;
    const float v = p[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
    p[i] = v;
    p16[i] = __float2bfloat16(v);
}

__global__ void sumsq_kernel(const float* __restrict__ g, int n, float* __restrict__ out)
{
    __shared__ float red[256];
    float s = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) s += g[i] * g[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(out, red[0]);
}

}  // namespace

static int mlp_offsets(const messi_mlp* m, size_t off[6])
{
    off[0] = 0;                                    // W1
    off[1] = off[0] + (size_t)m->H * m->in;        // b1
    off[2] = off[1] + m->H;                        // W2
    off[3] = off[2] + (size_t)m->H * m->H;         // b2
    off[4] = off[3] + m->H;                        // W3
    off[5] = off[4] + (size_t)m->out * m->H;       // b3
    return (int)(off[5] + m->out);
}

static int mlp_reserve(messi_ctx* ctx, messi_mlp* m, int batch)
{
    if (batch <= m->cap) return MESSI_OK;
    cudaFree(m->x);
    cudaFree(m->a1);
    cudaFree(m->a2);
    cudaFree(m->z1);
    cudaFree(m->z2);
    cudaFree(m->y);
    cudaFree(m->dy);
    cudaFree(m->d2);
    cudaFree(m->d1);
    cudaFree(m->target);
    cudaFree(m->loss);
    cudaFreeHost(m->stage);
    const size_t B = (size_t)batch;
    cudaError_t e = cudaSuccess;
    auto al = [&](void** p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
    };
    al((void**)&m->x, B * m->in * 2);
    al((void**)&m->a1, B * m->H * 2);
    al((void**)&m->a2, B * m->H * 2);
    al((void**)&m->z1, B * m->H * 4);
    al((void**)&m->z2, B * m->H * 4);
    al((void**)&m->y, B * m->out * 4);
    al((void**)&m->dy, B * m->out * 4);
    al((void**)&m->d2, B * m->H * 4);
    al((void**)&m->d1, B * m->H * 4);
    al((void**)&m->target, B * m->D * 4);
    al((void**)&m->loss, B * 4 + 64);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&m->stage, B * (m->in + m->out + m->D + 2) * 4 + 64);
    if (e != cudaSuccess) {
        m->cap = 0;
        return cuda_fail(ctx, e, "mlp activations");
    }
    m->cap = batch;
    return MESSI_OK;
}

static inline unsigned blocks(long long n) { return (unsigned)((n + 255) / 256); }

// forward pass on the batch already in m->x (BF16)
static int mlp_forward_dev(messi_ctx* ctx, messi_mlp* m, int Bn)
{
    size_t off[6];
    mlp_offsets(m, off);
    const __nv_bfloat16* W1 = m->p16 + off[0];
    const __nv_bfloat16* W2 = m->p16 + off[2];
    const __nv_bfloat16* W3 = m->p16 + off[4];
    int rc;
    // z1 = x W1^T + b1 : A = x [B x in], B(k, n) = W1[n][k]
    // (z1, a1) = (x W1^T + b1, silu); the same for layer 2; y = a2 W3^T + b3
    if ((rc = gemm(ctx, Bn, m->H, m->in, m->x, m->in, 1, W1, 1, m->in, m->p32 + off[1], m->z1, m->H, kBiasSilu,
                   nullptr, m->a1)))
        return rc;
    if ((rc = gemm(ctx, Bn, m->H, m->H, m->a1, m->H, 1, W2, 1, m->H, m->p32 + off[3], m->z2, m->H, kBiasSilu,
                   nullptr, m->a2)))
        return rc;
    return gemm(ctx, Bn, m->out, m->H, m->a2, m->H, 1, W3, 1, m->H, m->p32 + off[5], m->y, m->out, kStoreBias);
}

// loss + gradients into m->grad (zeroed first); returns via m->loss
static int mlp_backward_dev(messi_ctx* ctx, messi_mlp* m, int Bn)
{
    size_t off[6];
    mlp_offsets(m, off);
    const __nv_bfloat16* W2 = m->p16 + off[2];
    const __nv_bfloat16* W3 = m->p16 + off[4];
    cudaError_t e = cudaMemsetAsync(m->grad, 0, sizeof(float) * m->nparam, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "grad reset");
    mixture_nll_kernel<<<blocks(Bn), 256, 0, ctx->stream>>>(m->y, m->target, Bn, m->K, m->D, m->loss, m->dy,
                                                            1.f / (float)Bn);
    LAUNCH_CHECK(ctx, "mixture_nll_kernel");
    int rc;
    // layer 3: dW3[o][h] = sum_b dy[b][o] a2[b][h]; db3 = colsum dy; d2 = dy W3
    if ((rc = gemm(ctx, m->out, m->H, Bn, m->dy, 1, m->out, m->a2, m->H, 1, nullptr, m->grad + off[4], m->H,
                   kAccumulate)))
        return rc;
    colsum_kernel<<<blocks(m->out), 256, 0, ctx->stream>>>(m->dy, Bn, m->out, m->grad + off[5]);
    LAUNCH_CHECK(ctx, "colsum_kernel");
    // d2 = (dy W3) * silu'(z2)
    if ((rc = gemm(ctx, Bn, m->H, m->out, m->dy, m->out, 1, W3, m->H, 1, nullptr, m->d2, m->H, kDsilu, m->z2)))
        return rc;
    // layer 2
    if ((rc = gemm(ctx, m->H, m->H, Bn, m->d2, 1, m->H, m->a1, m->H, 1, nullptr, m->grad + off[2], m->H,
                   kAccumulate)))
        return rc;
    colsum_kernel<<<blocks(m->H), 256, 0, ctx->stream>>>(m->d2, Bn, m->H, m->grad + off[3]);
    LAUNCH_CHECK(ctx, "colsum_kernel");
    if ((rc = gemm(ctx, Bn, m->H, m->H, m->d2, m->H, 1, W2, m->H, 1, nullptr, m->d1, m->H, kDsilu, m->z1)))
        return rc;
    // layer 1
    if ((rc = gemm(ctx, m->H, m->in, Bn, m->d1, 1, m->H, m->x, m->in, 1, nullptr, m->grad + off[0], m->in,
                   kAccumulate)))
        return rc;
    colsum_kernel<<<blocks(m->H), 256, 0, ctx->stream>>>(m->d1, Bn, m->H, m->grad + off[1]);
    LAUNCH_CHECK(ctx, "colsum_kernel");
    return MESSI_OK;
}

static int upload_batch(messi_ctx* ctx, messi_mlp* m, int Bn, const float* x, const float* target)
{
    int rc;
    if ((rc = mlp_reserve(ctx, m, Bn))) return rc;
    float* st = m->stage;
    std::memcpy(st, x, sizeof(float) * Bn * m->in);
    cudaError_t e = cudaMemcpyAsync(m->z1, st, sizeof(float) * Bn * m->in, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "mlp input upload");
    // inputs to BF16 (z1 is free at this point and large enough: H >= in)
    to_bf16_kernel<<<blocks((long long)Bn * m->in), 256, 0, ctx->stream>>>(m->z1, m->x, (long long)Bn * m->in);
    LAUNCH_CHECK(ctx, "to_bf16_kernel");
    if (target) {
        float* sp = st + (size_t)Bn * m->in;
        std::memcpy(sp, target, sizeof(float) * Bn * m->D);
        e = cudaMemcpyAsync(m->target, sp, sizeof(float) * Bn * m->D, cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "mlp target upload");
    }
    return MESSI_OK;
}

}  // namespace messi

using namespace messi;

extern "C" {

int messi_mlp_create(messi_ctx* ctx, int32_t in_dim, int32_t width, int32_t ncomp, int32_t dim, uint64_t seed,
                     messi_mlp** out)
{
    if (!ctx || !out || in_dim < 1 || width < 1 || ncomp < 1 || ncomp > 8 || dim < 1) return MESSI_EINVAL;
    if (width < in_dim) return fail(ctx, MESSI_EINVAL, "mlp: width must be >= input size");
    cudaSetDevice(ctx->device);
    messi_mlp* m = new messi_mlp();
    m->in = in_dim;
    m->H = width;
    m->K = ncomp;
    m->D = dim;
    m->out = ncomp + 2 * ncomp * dim;
    size_t off[6];
    m->nparam = mlp_offsets(m, off);
    // He-style initialisation from a splitmix64 stream (deterministic in seed)
    std::vector<float> p(m->nparam, 0.f);
    uint64_t st = seed ? seed : 0x9E3779B97F4A7C15ull;
    auto next = [&]() {
        st += 0x9E3779B97F4A7C15ull;
        uint64_t z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    auto fill = [&](size_t o, size_t n, double scale) {
        for (size_t i = 0; i < n; i++) p[o + i] = (float)((2.0 * next() - 1.0) * scale);
    };
    fill(off[0], (size_t)m->H * m->in, std::sqrt(3.0 / m->in));
    fill(off[2], (size_t)m->H * m->H, std::sqrt(3.0 / m->H));
    fill(off[4], (size_t)m->out * m->H, 0.1 * std::sqrt(3.0 / m->H));
    cudaError_t e = cudaMalloc((void**)&m->p32, sizeof(float) * m->nparam);
    if (e == cudaSuccess) e = cudaMalloc((void**)&m->p16, sizeof(__nv_bfloat16) * m->nparam);
    if (e == cudaSuccess) e = cudaMalloc((void**)&m->grad, sizeof(float) * (m->nparam + 16));
    if (e == cudaSuccess) e = cudaMalloc((void**)&m->m1, sizeof(float) * m->nparam);
    if (e == cudaSuccess) e = cudaMalloc((void**)&m->m2, sizeof(float) * m->nparam);
    if (e == cudaSuccess) e = cudaMemcpy(m->p32, p.data(), sizeof(float) * m->nparam, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(m->m1, 0, sizeof(float) * m->nparam);
    if (e == cudaSuccess) e = cudaMemset(m->m2, 0, sizeof(float) * m->nparam);
    if (e != cudaSuccess) {
        messi_mlp_destroy(m);
        return cuda_fail(ctx, e, "mlp parameters");
    }
    to_bf16_kernel<<<blocks(m->nparam), 256, 0, ctx->stream>>>(m->p32, m->p16, m->nparam);
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        messi_mlp_destroy(m);
        return cuda_fail(ctx, e, "mlp init");
    }
    *out = m;
    return MESSI_OK;
}

int messi_mlp_destroy(messi_mlp* m)
{
    if (!m) return MESSI_EINVAL;
    void* ptrs[] = {m->p32, m->p16, m->grad, m->m1, m->m2, m->x, m->a1, m->a2, m->z1,
                    m->z2,  m->y,   m->dy,   m->d2, m->d1, m->target, m->loss};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (m->stage) cudaFreeHost(m->stage);
    delete m;
    return MESSI_OK;
}

int messi_mlp_nparams(messi_mlp* m, int32_t* n)
{
    if (!m || !n) return MESSI_EINVAL;
    *n = m->nparam;
    return MESSI_OK;
}

int messi_mlp_get_params(messi_ctx* ctx, messi_mlp* m, float* host)
{
    if (!ctx || !m || !host) return MESSI_EINVAL;
    cudaSetDevice(ctx->device);
    cudaError_t e = cudaMemcpy(host, m->p32, sizeof(float) * m->nparam, cudaMemcpyDeviceToHost);
    return (e == cudaSuccess) ? MESSI_OK : cuda_fail(ctx, e, "mlp get params");
}

int messi_mlp_set_params(messi_ctx* ctx, messi_mlp* m, const float* host)
{
    if (!ctx || !m || !host) return MESSI_EINVAL;
    cudaSetDevice(ctx->device);
    cudaError_t e = cudaMemcpy(m->p32, host, sizeof(float) * m->nparam, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "mlp set params");
    to_bf16_kernel<<<blocks(m->nparam), 256, 0, ctx->stream>>>(m->p32, m->p16, m->nparam);
    e = cudaStreamSynchronize(ctx->stream);
    return (e == cudaSuccess) ? MESSI_OK : cuda_fail(ctx, e, "mlp set params");
}

int messi_mlp_forward(messi_ctx* ctx, messi_mlp* m, int32_t batch, const float* x, float* y)
{
    if (!ctx || !m || batch < 1 || !x || !y) return MESSI_EINVAL;
    ctx->launches = 0;
    cudaSetDevice(ctx->device);
    int rc;
    if ((rc = upload_batch(ctx, m, batch, x, nullptr))) return rc;
    if ((rc = mlp_forward_dev(ctx, m, batch))) return rc;
    cudaError_t e = cudaMemcpyAsync(y, m->y, sizeof(float) * batch * m->out, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return (e == cudaSuccess) ? MESSI_OK : cuda_fail(ctx, e, "mlp forward");
}

int messi_mlp_gradients(messi_ctx* ctx, messi_mlp* m, int32_t batch, const float* x, const float* target,
                        float* loss, float* grads)
{
    if (!ctx || !m || batch < 1 || !x || !target) return MESSI_EINVAL;
    ctx->launches = 0;
    cudaSetDevice(ctx->device);
    int rc;
    if ((rc = upload_batch(ctx, m, batch, x, target))) return rc;
    if ((rc = mlp_forward_dev(ctx, m, batch))) return rc;
    if ((rc = mlp_backward_dev(ctx, m, batch))) return rc;
    std::vector<float> l(batch);
    cudaError_t e = cudaMemcpyAsync(l.data(), m->loss, sizeof(float) * batch, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess && grads)
        e = cudaMemcpyAsync(grads, m->grad, sizeof(float) * m->nparam, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "mlp gradients");
    if (loss) {
        double s = 0.0;
        for (float v : l) s += v;
        *loss = (float)(s / batch);
    }
    return MESSI_OK;
}

int messi_mlp_train_step(messi_ctx* ctx, messi_mlp* m, int32_t batch, const float* x, const float* target, float lr,
                         float max_grad_norm, float* loss)
{
    int rc = messi_mlp_gradients(ctx, m, batch, x, target, loss, nullptr);
    if (rc) return rc;
    float* d_norm = m->grad + m->nparam;  // spare slot
    cudaMemsetAsync(d_norm, 0, sizeof(float), ctx->stream);
    sumsq_kernel<<<64, 256, 0, ctx->stream>>>(m->grad, m->nparam, d_norm);
    LAUNCH_CHECK(ctx, "sumsq_kernel");
    float h = 0.f;
    cudaError_t e = cudaMemcpyAsync(&h, d_norm, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "grad norm");
    const float gn = std::sqrt(h);
    const float clip = (max_grad_norm > 0.f && gn > max_grad_norm) ? max_grad_norm / gn : 1.f;
    m->steps++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)m->steps), c2 = 1.f - std::pow(b2, (float)m->steps);
    adam_kernel<<<blocks(m->nparam), 256, 0, ctx->stream>>>(m->p32, m->grad, m->m1, m->m2, m->p16, m->nparam, lr, b1,
                                                            b2, c1, c2, 1e-8f, clip);
    LAUNCH_CHECK(ctx, "adam_kernel");
    e = cudaStreamSynchronize(ctx->stream);
    return (e == cudaSuccess) ? MESSI_OK : cuda_fail(ctx, e, "adam");
}

}  // extern "C"
