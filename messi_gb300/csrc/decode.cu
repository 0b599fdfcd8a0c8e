// decode.cu -- structures from the SCFG tables: maximum-expected-accuracy
// posterior decoding and stochastic sampling of structures.
//
// Posterior decoding replaces computeposteriordecodingcuda
// (src/InsideCUDA.jl:183-215, kernel posteriordecoding of
// src/cuda/inside.cu:286-321, one launch per span) and the CPU traceback
// posteriordecodingtraceback (src/RNATools.jl:43-72).  The recursion, in FP32
// as the reference's GPU path computes it:
//     e(i,i) = 0
//     e(i,j) = max( single[i] + e(i+1,j),                                  s = -1
//                   alpha*pair(i,j) + e(i+1,j-1),                          s = -2
//                   max_k alpha*pair(i,k) + e(i+1,k-1) + e(k+1,j) )        s = k+1
// with ties to the first alternative and the smallest k.  One persistent
// cooperative launch walks the spans (grid barrier between spans); a cell's
// split maximum is reduced by a group of lanes with a (value, k) arg-max.  e
// is kept twice (row-major and column-major) so both operand streams of the
// split are unit-stride; s is written column-major, the layout the Julia
// caller reads.  The traceback runs on the device in one thread.
//
// Structure sampling replaces samplestructure / samplestructurehelper
// (src/InsideOutsideAlgorithm.jl:570-635): a stochastic traceback through the
// banded inside tables of scfg.cu.  One warp draws one structure: for a span
// (x, y) with parent nonterminal P it weighs every bifurcation x..h | h+1..y
// (P = S, F) and the pair (x, y) (P = S, F, L) by rule x inside x inside,
// samples one by inverse CDF and pushes the sub-spans on a per-warp stack.
// The log-odds baseline of the banded tables is the same for every option
// of a span, so the weights are the reference's up to a common factor.
// Random numbers: SplitMix64 (Steele, Lea and Flood, OOPSLA 2014) over
// (seed, structure, draw).
#include <climits>
#include <cmath>

#include "internal.h"
#include "wave.cuh"

namespace messi {

namespace {

__device__ __forceinline__ void amax_merge(float& v, int& k, float v2, int k2)
{
    if (v2 > v || (v2 == v && k2 < k)) {
        v = v2;
        k = k2;
    }
}

}  // namespace

__global__ void to_float_kernel(const double* __restrict__ in, float* __restrict__ out, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (float)in[i];
}

__global__ void to_double_kernel(const float* __restrict__ in, double* __restrict__ out, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (double)in[i];
}

// pair: L x L as uploaded from the Julia matrix (column-major); it is read as
// pair[i*L + k], the reference kernel's indexing (the matrix is symmetric).
//
// Cell (i, j = i+d): the best split over k = i+1 .. j-1 of
// alpha*pair(i,k) + e(i+1,k-1) + e(k+1,j), e2 = alpha*pair(i,j) + e(i+1,j-1)
// and e1 = single(i) + e(i+1,j).  Split point k reads spans k-i-2 and j-k-1.
// Diagonals go two per grid barrier, (dA, dB) = (2p-1, 2p): decode_split_t
// takes the split points k = i+KLO .. j-KHI, whose spans are <= 2p-4 and so
// complete before the wait on the barrier that completes 2p-2 (dA: KLO = 2,
// KHI = 1; dB: KLO = 3, KHI = 2), as a lane-group (value, k) arg-max;
// decode_finish_t adds the outer split points in ascending k, e2 and e1 and
// writes the cell.  The maximum is exact and ties go to the smallest k (the
// reference's loop order) however the points are split, so the bits are the
// reference kernel's.
struct DecodePart {
    float bv;
    int bk;
};

template <int KLO, int KHI>
__device__ __forceinline__ DecodePart decode_split_t(const float* __restrict__ pair, const float* erow,
                                                     const float* ecol, int L, float alpha, int i, int d,
                                                     bool valid, int lane, int G)
{
    DecodePart p{-1e10f, 0};  // the reference's initial maximum and index
    const int j = i + d;
    if (valid) {
        const float* prow = pair + (size_t)i * L;
        const float* er = erow + (size_t)(i + 1) * L;  // e(i+1, k-1)
        const float* ec = ecol + (size_t)j * L;        // e(k+1, j)
        const int kend = j - KHI;
        int k = i + KLO + lane;
        // four splits per step, loads issued together, compared in ascending k
        for (; k + 3 * G <= kend; k += 4 * G) {
            float v[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int kq = k + q * G;
                v[q] = __fmaf_rn(alpha, __ldg(prow + kq), __ldcg(er + kq - 1)) + __ldcg(ec + kq + 1);
            }
#pragma unroll
            for (int q = 0; q < 4; q++)
                if (v[q] > p.bv) {
                    p.bv = v[q];
                    p.bk = k + q * G;
                }
        }
        for (; k <= kend; k += G) {
            const float v = __fmaf_rn(alpha, __ldg(prow + k), __ldcg(er + k - 1)) + __ldcg(ec + k + 1);
            if (v > p.bv) {
                p.bv = v;
                p.bk = k;
            }
        }
    }
    if (__any_sync(0xffffffffu, valid))
        for (int off = G >> 1; off > 0; off >>= 1) {
            const float v2 = __shfl_xor_sync(0xffffffffu, p.bv, off);
            const int k2 = __shfl_xor_sync(0xffffffffu, p.bk, off);
            amax_merge(p.bv, p.bk, v2, k2);
        }
    return p;
}

template <int KLO, int KHI>
__device__ __forceinline__ void decode_finish_t(const float* __restrict__ single, const float* __restrict__ pair,
                                                float* erow, float* ecol, int* scol, int L, float alpha, int i,
                                                int d, bool valid, DecodePart p)
{
    if (!valid) return;
    const int j = i + d;
    const float* prow = pair + (size_t)i * L;
    const float* er = erow + (size_t)(i + 1) * L;
    const float* ec = ecol + (size_t)j * L;
    // the outer split points, ascending k (ties to the smaller k)
    for (int k = i + 1; k <= min(i + KLO - 1, j - 1); k++)
        amax_merge(p.bv, p.bk, __fmaf_rn(alpha, __ldg(prow + k), __ldcg(er + k - 1)) + __ldcg(ec + k + 1), k);
    for (int k = max(i + KLO, j - KHI + 1); k <= j - 1; k++)
        amax_merge(p.bv, p.bk, __fmaf_rn(alpha, __ldg(prow + k), __ldcg(er + k - 1)) + __ldcg(ec + k + 1), k);
    const float e2 = __fmaf_rn(alpha, __ldg(prow + j), __ldcg(er + j - 1));
    const float e1 = __ldg(single + i) + __ldcg(er + j);
    float mv = e1;
    int sv = -1;
    if (e2 > mv) {
        mv = e2;
        sv = -2;
    }
    if (p.bv > mv) {
        mv = p.bv;
        sv = p.bk + 1;
    }
    erow[(size_t)i * L + j] = mv;
    ecol[(size_t)j * L + i] = mv;
    scol[(size_t)j * L + i] = sv;
}

// The cells of one diagonal with rows [r0, end), by all warps of the CTA:
// split parts of the first two rows of every lane group before the wait,
// their finishing parts (lanes 0 and 1 of a group side by side) and any
// further rows whole after it.
struct DecodeRows {
    DecodePart c[2];
};

template <int KLO, int KHI>
__device__ __forceinline__ DecodeRows decode_rows_split(const float* __restrict__ pair, const float* erow,
                                                        const float* ecol, int L, float alpha, int d, int r0,
                                                        int end)
{
    DecodeRows p;
    const int G = group_width(d - 1), gpb = blockDim.x / G;
    const int lane = threadIdx.x & (G - 1), g = threadIdx.x / G;
#pragma unroll
    for (int it = 0; it < 2; it++) {
        const int i = r0 + g + it * gpb;
        p.c[it] = decode_split_t<KLO, KHI>(pair, erow, ecol, L, alpha, i, d, i < end, lane, G);
    }
    return p;
}

template <int KLO, int KHI>
__device__ __forceinline__ void decode_rows_finish(const float* __restrict__ single, const float* __restrict__ pair,
                                                   float* erow, float* ecol, int* scol, int L, float alpha, int d,
                                                   int r0, int end, const DecodeRows& p)
{
    const int G = group_width(d - 1), gpb = blockDim.x / G;
    const int lane = threadIdx.x & (G - 1), g = threadIdx.x / G;
    if (G >= 2) {
        const int it = lane & 1;
        const int i = r0 + g + it * gpb;
        decode_finish_t<KLO, KHI>(single, pair, erow, ecol, scol, L, alpha, i, d, lane < 2 && i < end,
                                  it ? p.c[1] : p.c[0]);
    } else {
#pragma unroll
        for (int it = 0; it < 2; it++) {
            const int i = r0 + g + it * gpb;
            decode_finish_t<KLO, KHI>(single, pair, erow, ecol, scol, L, alpha, i, d, i < end, p.c[it]);
        }
    }
    for (int base = r0 + 2 * gpb; base < end; base += gpb) {
        const int i = base + g;
        const DecodePart c = decode_split_t<KLO, KHI>(pair, erow, ecol, L, alpha, i, d, i < end, lane, G);
        decode_finish_t<KLO, KHI>(single, pair, erow, ecol, scol, L, alpha, i, d, i < end && lane == 0, c);
    }
}

// All diagonals, two per grid barrier.  CTA b owns rows [b*R, (b+1)*R) of
// every diagonal (R = ceil(L / CTAs)); for the pair (dA, dB) it computes dA
// for its rows plus row (b+1)*R (which the next CTA also computes, to the
// same bits) and then, after a CTA barrier, dB, whose e1 reads dA at row
// i+1, its own.
__global__ void __launch_bounds__(kWaveMaxThreads) decode_wave_kernel(const float* __restrict__ single,
                                                          const float* __restrict__ pair, int L, float alpha,
                                                          float* __restrict__ erow, float* __restrict__ ecol,
                                                          int* __restrict__ scol, unsigned int* sync)
{
    unsigned int gen = 0;
    grid_arrive(sync);  // spans 0 and -1 are the zero-filled tables
    const int rows = (L + gridDim.x - 1) / gridDim.x;
    const int r0 = blockIdx.x * rows;
    for (int dA = 1; dA < L; dA += 2) {
        const int dB = dA + 1;
        const int endA = min(r0 + rows + 1, L - dA);
        const int endB = (dB < L) ? min(r0 + rows, L - dB) : r0;
        const DecodeRows pa = decode_rows_split<2, 1>(pair, erow, ecol, L, alpha, dA, r0, endA);
        const DecodeRows pb = decode_rows_split<3, 2>(pair, erow, ecol, L, alpha, dB, r0, endB);
        if (!grid_wait(sync, gen)) return;
        decode_rows_finish<2, 1>(single, pair, erow, ecol, scol, L, alpha, dA, r0, endA, pa);
        __syncthreads();  // diagonal dA of this CTA's rows before dB reads it
        decode_rows_finish<3, 2>(single, pair, erow, ecol, scol, L, alpha, dB, r0, endB, pb);
        grid_arrive(sync);
    }
}

// posteriordecodingtraceback (src/RNATools.jl:43-72) on the column-major s:
// paired[c] = 1-based partner of column c, 0 when unpaired.  One thread;
// stack: 2 * (L + 1) ints of scratch.
__global__ void decode_traceback_kernel(const int* __restrict__ scol, int L, int* __restrict__ paired,
                                        int* __restrict__ stack)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int c = 0; c < L; c++) paired[c] = 0;
    int top = 0;
    stack[top++] = 1;
    stack[top++] = L;
    while (top > 0 && top + 2 <= 2 * (L + 1)) {
        const int j = stack[--top];
        const int i = stack[--top];
        const int k = scol[(size_t)(j - 1) * L + (i - 1)];
        if (k == -1) {
            stack[top++] = i + 1;
            stack[top++] = j;
        } else if (k == -2) {
            paired[i - 1] = j;
            paired[j - 1] = i;
            if (i + 1 < j - 1) {
                stack[top++] = i + 1;
                stack[top++] = j - 1;
            }
        } else if (k > 0 && k <= L) {
            if (i < k) {
                paired[i - 1] = k;
                paired[k - 1] = i;
            }
            if (i + 1 <= k - 1) {
                stack[top++] = i + 1;
                stack[top++] = k - 1;
            }
            if (k + 1 <= j) {
                stack[top++] = k + 1;
                stack[top++] = j;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// structure sampling
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__device__ __forceinline__ double uniform01(unsigned long long seed, unsigned long long stream, unsigned long long n)
{
    const unsigned long long h = splitmix64(splitmix64(seed ^ (stream * 0xD1B54A32D192ED03ull)) + n);
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

// Weight of option o of span (x, y) under parent P (0 = S, 1 = F, 2 = L):
// o < nsplit: bifurcation at h = x + o; o == nsplit: the pair (x, y).
__device__ __forceinline__ float option_weight(const Band& t, const Rules& R, int P, int x, int y, int o, int nsplit)
{
    if (o < nsplit) {
        const int h = x + o;
        const float lv = __ldg(t.Lrow + (size_t)x * t.RS + (h - x));
        const int span = y - h - 1;
        float sv;
        // column layout: consecutive h of a warp read consecutive addresses
        if (span <= t.Wb) sv = __ldg(t.Scol + (size_t)y * t.RS + span);
        else if (y == t.L - 1) sv = __ldg(t.Ssuf + h + 1);
        else sv = -INFINITY;
        return ((P == 0) ? R.r[0] : R.r[4]) + lv + sv;
    }
    const int span = y - x;
    if (span < 2 || span > t.Wb) return -INFINITY;
    const float pv = __ldg(t.pb + (size_t)x * t.RS + span);
    const float fv = __ldg(t.Frow + (size_t)(x + 1) * t.RS + (span - 2));
    return ((P == 0) ? R.r[2] : (P == 1 ? R.r[3] : R.r[6])) + pv + fv;
}

constexpr int kCachedRounds = 32;  // options of a span kept in registers: 32 per lane

// One warp per structure.  stack: [nstruct][3 * (L + 1)] ints;
// paired: [nstruct][L] (1-based partners, 0 = unpaired).
// KH99 log rule probabilities in FP64 (the prior of a sampled structure is
// the sum over its derivation: src/InsideOutsideAlgorithm.jl:86-144 parses
// the same rules, unfolded).
struct PriorRules {
    double r[7];
};

__global__ void __launch_bounds__(128) sample_structures_kernel(Band t, Rules R, PriorRules PR, int nstruct,
                                                                unsigned long long seed, int* __restrict__ paired,
                                                                int* __restrict__ stack, double* __restrict__ prior,
                                                                unsigned int* __restrict__ status)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nstruct) return;
    const int L = t.L;
    int* out = paired + (size_t)warp * L;
    int* stk = stack + (size_t)warp * 3 * (L + 1);
    for (int c = lane; c < L; c += 32) out[c] = 0;
    __syncwarp();
    int top = 0;  // entries of 3 ints: parent, x, y (kept in lane 0's view; every lane follows)
    if (lane == 0) {
        stk[0] = 0;
        stk[1] = 0;
        stk[2] = L - 1;
    }
    top = 1;
    unsigned long long draw = 0;
    double lp = 0.0;  // log prior of the derivation (lane 0's copy is the result)
    while (top > 0) {
        __syncwarp();
        top--;
        const int P = stk[3 * top], x = stk[3 * top + 1], y = stk[3 * top + 2];
        __syncwarp();
        if (x == y) lp += (P == 0) ? PR.r[1] : (P == 2 ? PR.r[5] : -INFINITY);  // S -> s, L -> s
        if (x >= y) continue;
        // bifurcations x..h | h+1..y with L(x, h) in the band; then the pair.
        // Up to kCached options per span keep their weights in registers (one
        // pass of loads); longer option lists are re-read per pass.
        const int nsplit = (P == 2) ? 0 : min(y - x, t.Wb + 1);
        const int nopt = nsplit + 1;
        const bool cached = nopt <= 32 * kCachedRounds;
        float wv[kCachedRounds];
        float m = -INFINITY;
        if (cached) {
#pragma unroll
            for (int q = 0; q < kCachedRounds; q++) {
                const int o = lane + 32 * q;
                wv[q] = (o < nopt) ? option_weight(t, R, P, x, y, o, nsplit) : -INFINITY;
                m = fmaxf(m, wv[q]);
            }
        } else {
            for (int o = lane; o < nopt; o += 32) m = fmaxf(m, option_weight(t, R, P, x, y, o, nsplit));
        }
        for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
        if (m == -INFINITY) {
            if (lane == 0) atomicOr(status, 2u);  // a span with no derivation: the tables are inconsistent
            break;
        }
        double tot = 0.0;
        if (cached) {
#pragma unroll
            for (int q = 0; q < kCachedRounds; q++) tot += (double)__expf(wv[q] - m);
        } else {
            for (int o = lane; o < nopt; o += 32) tot += (double)__expf(option_weight(t, R, P, x, y, o, nsplit) - m);
        }
        for (int off = 16; off > 0; off >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, off);
        const double target = uniform01(seed, (unsigned long long)warp, draw++) * tot;
        // inverse CDF in rounds of 32 options; if rounding leaves the target
        // past the last cumulative sum, the last option of non-zero weight
        int pick = -1, last = -1;
        double run = 0.0;
        // one round of 32 options: returns true once the pick is found
        auto round = [&](int r0, float wo) {
            const int o = r0 + lane;
            const double w = (o < nopt) ? (double)__expf(wo - m) : 0.0;
            double inc = w;
            for (int off = 1; off < 32; off <<= 1) {
                const double n = __shfl_up_sync(0xffffffffu, inc, off);
                if (lane >= off) inc += n;
            }
            const unsigned int pos = __ballot_sync(0xffffffffu, w > 0.0);
            if (pos) last = r0 + 31 - __clz((int)pos);
            const unsigned int ball = __ballot_sync(0xffffffffu, (w > 0.0) && (run + inc > target));
            if (ball) {
                pick = r0 + __ffs(ball) - 1;
                return true;
            }
            run += __shfl_sync(0xffffffffu, inc, 31);
            return false;
        };
        if (cached) {
            bool found = false;
#pragma unroll
            for (int q = 0; q < kCachedRounds; q++)
                if (!found && 32 * q < nopt) found = round(32 * q, wv[q]);
        } else {
            for (int r0 = 0; r0 < nopt; r0 += 32)
                if (round(r0, (r0 + lane < nopt) ? option_weight(t, R, P, x, y, r0 + lane, nsplit) : -INFINITY)) break;
        }
        if (pick < 0) pick = last;
        const int npush = (pick < nsplit) ? 2 : 1;
        if (pick < 0 || top + npush > L) {
            if (lane == 0) atomicOr(status, 4u);
            break;
        }
        if (pick < nsplit) lp += (P == 0) ? PR.r[0] : PR.r[4];                   // S -> LS, F -> LS
        else lp += (P == 0) ? PR.r[2] : (P == 1 ? PR.r[3] : PR.r[6]);            // pair rules
        if (lane == 0) {
            if (pick < nsplit) {
                const int h = x + pick;
                // the reference pushes the left part, then the right part
                stk[3 * top] = 2;  // L(x, h)
                stk[3 * top + 1] = x;
                stk[3 * top + 2] = h;
                stk[3 * top + 3] = 0;  // S(h+1, y)
                stk[3 * top + 4] = h + 1;
                stk[3 * top + 5] = y;
            } else {
                out[x] = y + 1;
                out[y] = x + 1;
                stk[3 * top] = 1;  // F(x+1, y-1)
                stk[3 * top + 1] = x + 1;
                stk[3 * top + 2] = y - 1;
            }
        }
        top += npush;
    }
    if (lane == 0 && prior) prior[warp] = lp;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int run_posterior_decoding(messi_ctx* ctx, int L, const double* d_single, const double* d_pair, double alpha,
                           float* d_work, int* d_scol, unsigned int* d_sync, int* d_paired, int* d_stack,
                           double* d_eout)
{
    // d_work: single (L) | pair (L*L) | erow (L*L) | ecol (L*L) floats
    const long long LL = (long long)L * L;
    float* f_single = d_work;
    float* f_pair = d_work + L;
    float* erow = f_pair + LL;
    float* ecol = erow + LL;
    const int bs = 256;
    to_float_kernel<<<(unsigned)((L + bs - 1) / bs), bs, 0, ctx->stream>>>(d_single, f_single, L);
    LAUNCH_CHECK(ctx, "to_float_kernel");
    to_float_kernel<<<(unsigned)((LL + bs - 1) / bs), bs, 0, ctx->stream>>>(d_pair, f_pair, LL);
    LAUNCH_CHECK(ctx, "to_float_kernel");
    cudaError_t e = cudaMemsetAsync(erow, 0, sizeof(float) * 2 * LL, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_scol, 0, sizeof(int) * LL, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_sync, 0, kSyncWords * sizeof(unsigned int), ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "decoding tables reset");
    if (L > 1) {
        const float a = (float)alpha;
        int Lv = L;
        void* args[] = {(void*)&f_single, (void*)&f_pair, &Lv, (void*)&a, &erow, &ecol, &d_scol, &d_sync};
        // paired shape: a CTA's two diagonals of a pair (2 x rows + 1 cells)
        // in one pass of its warps where the CTA can grow to hold them
        const int rc = launch_wave(ctx, (const void*)decode_wave_kernel, args, d_sync, L, 0.5 * (double)L * L,
                                   "decode_wave_kernel", 2);
        if (rc) return rc;
    }
    if (d_paired) {
        decode_traceback_kernel<<<1, 32, 0, ctx->stream>>>(d_scol, L, d_paired, d_stack);
        LAUNCH_CHECK(ctx, "decode_traceback_kernel");
    }
    if (d_eout) {
        // the column-major copy is the Julia matrix e[i, j] (zeros below the diagonal)
        to_double_kernel<<<(unsigned)((LL + bs - 1) / bs), bs, 0, ctx->stream>>>(ecol, d_eout, LL);
        LAUNCH_CHECK(ctx, "to_double_kernel");
    }
    if (ctx->status_host) {
        e = cudaMemcpyAsync(ctx->status_host, d_sync + 2, sizeof(unsigned int), cudaMemcpyDeviceToHost, ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "status readback");
    }
    return MESSI_OK;
}

int run_sample_structures(messi_ctx* ctx, const Band& t, double B, int nstruct, unsigned long long seed,
                          int* d_paired, int* d_stack, double* d_prior, unsigned int* d_status)
{
    Rules R = make_rules(B);
    PriorRules PR;
    for (int k = 0; k < 7; k++) PR.r[k] = std::log(kKH99Prob[k]);
    cudaError_t e = cudaMemsetAsync(d_status, 0, sizeof(unsigned int), ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "sampler status reset");
    const int warps_per_block = 4;
    const int blocks = (nstruct + warps_per_block - 1) / warps_per_block;
    sample_structures_kernel<<<blocks, 32 * warps_per_block, 0, ctx->stream>>>(t, R, PR, nstruct, seed, d_paired,
                                                                                d_stack, d_prior, d_status);
    LAUNCH_CHECK(ctx, "sample_structures_kernel");
    return MESSI_OK;
}

}  // namespace messi
