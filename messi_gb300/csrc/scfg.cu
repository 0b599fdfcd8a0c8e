// scfg.cu -- KH99 SCFG inside/outside passes and base-pairing posteriors (HP2).
//
// Replaces initialiseinside / insidealgorithm / insidez / outsidealgorithm of
// src/cuda/inside.cu (driven by src/InsideCUDA.jl:87-181, 301-389) and the
// CPU computebasepairprobs (src/InsideOutsideAlgorithm.jl:486-533).
//
// Representation.  Cells are stored as FP32 log-odds against a per-column
// baseline b_k = B*(u_k + log r1 + log r6) (u_k: unpaired log-likelihood):
//     Xbar(i,j) = X(i,j) - sum_{k=i..j} b_k.
// The baseline is additive over the split point, so the recurrences keep
// their form with pair scores pbar_ij = B*p_ij - b_i - b_j; an all-unpaired
// span keeps Sbar constant, which keeps FP32 magnitudes small.  The prefix
// sums of b and Z = Sbar(0, L-1) + sum_k b_k are FP64.
//
// Banding.  With every pair of span > Wb forbidden, only cells of span <= Wb
// and the S cells of the last column (the "suffix") reach Z
// (S->LS chains end at j = L-1; F and L need an enclosing or own pair), so
// the pass keeps a band of Wb+1 diagonals plus one suffix column.
//
// Layouts (row stride RS floats, RS >= Wb+1, multiple of 32):
//   Lrow[i][k] = Lbar(i, i+k)     Lcol[j][k] = Lbar(j-k, j)
//   Srow[i][k] = Sbar(i, i+k)     Scol[j][k] = Sbar(j-k, j)
//   Frow[i][k] = Fbar(i, i+k)     pb[i][k]   = pbar(i, i+k)
//   Ssuf[i]    = Sbar(i, L-1)
// so the split sum of cell (i, j) reads row i of L and column j of S with
// unit stride.  Outside tables mirror them (OSrow/OScol/OFrow/OFcol/OLrow/Osuf).
//
// Schedule.  One persistent cooperative launch walks the band diagonals (a
// wavefront): all cells of a span are independent, so each diagonal is spread
// over the whole grid and grid barriers separate diagonals (the inside pass
// takes two diagonals per barrier: a CTA owns a block of rows and the second
// diagonal of a pair reads the first only at the CTA's own rows).  The
// barrier spins with a bounded iteration count; on timeout it raises an
// error flag, every CTA leaves, Z becomes NaN and the host returns
// MESSI_ETIMEOUT.  A cell's split sum is reduced by a group of G lanes (G
// grows with the number of split points) with shuffle log-sum-exp; its
// middle split points, which do not read the diagonals just finished, are
// summed while a barrier is in progress.  The suffix recurrences run in one
// CTA in blocks of 32 cells: the terms that reach outside the block are
// summed by 32 warps in parallel, the in-block triangle by one warp.
#include <algorithm>
#include <cmath>

#include "internal.h"
#include "wave.cuh"

namespace messi {

namespace {

__device__ __forceinline__ void lse_add(float& m, float& s, float x)
{
    if (x > m) {
        s = s * __expf(m - x) + 1.f;
        m = x;
    } else if (x != -INFINITY) {
        s += __expf(x - m);
    }
}

// Four terms at once: the loads feeding them are independent, so a lane keeps
// four L2 requests in flight instead of one.
__device__ __forceinline__ void lse_add4(float& m, float& s, float x0, float x1, float x2, float x3)
{
    const float mx = fmaxf(fmaxf(x0, x1), fmaxf(x2, x3));
    if (mx == -INFINITY) return;
    if (mx > m) {
        s *= __expf(m - mx);
        m = mx;
    }
    s += (__expf(x0 - m) + __expf(x1 - m)) + (__expf(x2 - m) + __expf(x3 - m));
}

// Eight terms at once (sixteen independent loads in flight per lane).
// Without branches: the rescale of (m, s) always runs (exp(0) = 1 leaves s
// exactly as it is when the block brings no larger term, and a block of
// -inf terms adds exact zeros), so lanes of a warp never diverge here.
__device__ __forceinline__ void lse_add8(float& m, float& s, const float (&x)[8])
{
    // the maximum as a tree (three dependent steps instead of seven; exact)
    const float mx = fmaxf(fmaxf(fmaxf(x[0], x[1]), fmaxf(x[2], x[3])), fmaxf(fmaxf(x[4], x[5]), fmaxf(x[6], x[7])));
    const float nm = fmaxf(m, mx);
    const float base = (nm == -INFINITY) ? 0.f : nm;
    s *= __expf(m - base);
    m = nm;
    float a = 0.f, b = 0.f;
#pragma unroll
    for (int q = 0; q < 8; q += 2) {
        a += __expf(x[q] - base);
        b += __expf(x[q + 1] - base);
    }
    s += a + b;
}

__device__ __forceinline__ void lse_merge(float& m, float& s, float m2, float s2)
{
    if (m2 > m) {
        s = s * __expf(m - m2) + s2;
        m = m2;
    } else if (m2 != -INFINITY) {
        s += s2 * __expf(m2 - m);
    }
}

__device__ __forceinline__ float lse_val(float m, float s) { return (m == -INFINITY) ? -INFINITY : m + __logf(s); }

__device__ __forceinline__ float lse2f(float a, float b)
{
    const float m = fmaxf(a, b);
    if (m == -INFINITY) return -INFINITY;
    return m + __logf(__expf(a - m) + __expf(b - m));
}

// Adds sl * exp(x0) to the log-sum-exp (m, s) without branches (x0, m may
// be -inf): the serial triangle of the suffix recurrences, where a branch
// would split the warp on every step.
__device__ __forceinline__ void lse_add_scaled(float& m, float& s, float x0, float sl)
{
    const float mx = fmaxf(m, x0);
    const float base = (mx == -INFINITY) ? 0.f : mx;
    s = s * __expf(m - base) + sl * __expf(x0 - base);
    m = mx;
}

template <int G>
__device__ __forceinline__ void group_reduce(float& m, float& s)
{
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) {
        const float m2 = __shfl_xor_sync(0xffffffffu, m, off);
        const float s2 = __shfl_xor_sync(0xffffffffu, s, off);
        lse_merge(m, s, m2, s2);
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// workspace
// ---------------------------------------------------------------------------
int band_alloc(messi_ctx* ctx, int L, int Wb, bool outside, Band* t)
{
    t->L = L;
    t->Wb = Wb;
    t->RS = ((Wb + 1 + 31) / 32) * 32;
    const size_t tab = (size_t)L * t->RS * sizeof(float);
    void* p;
    int rc;
    float** in_tabs[6] = {&t->Lrow, &t->Lcol, &t->Srow, &t->Scol, &t->Frow, &t->pb};
    for (int k = 0; k < 6; k++) {
        if ((rc = ensure(ctx, k, tab, &p))) return rc;
        *in_tabs[k] = (float*)p;
    }
    if ((rc = ensure(ctx, 6, (size_t)(L + 1) * sizeof(float) * 2, &p))) return rc;
    t->Ssuf = (float*)p;
    t->Osuf = t->Ssuf + (L + 1);
    if ((rc = ensure(ctx, 7, (size_t)(3 * L + 8 + kSyncWords / 2) * sizeof(double), &p))) return rc;
    t->b = (double*)p;
    t->cb = t->b + L;
    t->u = t->cb + (L + 1);
    t->Zd = t->u + L;
    t->maxspan = (int*)(t->Zd + 2);
    t->sync = (unsigned int*)(t->Zd + 4);
    if (outside) {
        float** out_tabs[6] = {&t->OSrow, &t->OScol, &t->OFrow, &t->OFcol, &t->OLrow, &t->PP};
        for (int k = 0; k < 6; k++) {
            if ((rc = ensure(ctx, 8 + k, tab, &p))) return rc;
            *out_tabs[k] = (float*)p;
        }
        if ((rc = ensure(ctx, 14, (size_t)3 * L * sizeof(float), &p))) return rc;
        t->SL = (float*)p;
        t->nrm = t->SL + L;
        t->OSlast = t->nrm + L;
    } else {
        t->OSrow = t->OScol = t->OFrow = t->OFcol = t->OLrow = t->PP = t->SL = t->nrm = t->OSlast = nullptr;
    }
    return MESSI_OK;
}

Rules make_rules(double B)
{
    Rules r;
    for (int k = 0; k < 7; k++) r.r[k] = (float)(B * std::log(kKH99Prob[k]));
    return r;
}

static double baseline_c() { return std::log(0.868534) + std::log(0.894603); }

// ---------------------------------------------------------------------------
// baseline b_k and prefix sums cb (one block, deterministic FP64 scan)
// ---------------------------------------------------------------------------
__device__ void baseline_body(const double* __restrict__ u, int L, double B, double c, double* __restrict__ b,
                              double* __restrict__ cb)
{
    __shared__ double part[1024];
    const int t = threadIdx.x, nt = blockDim.x;
    const int per = (L + nt - 1) / nt;
    const int lo = min(L, t * per), hi = min(L, lo + per);
    double s = 0.0;
    for (int k = lo; k < hi; k++) {
        const double uk = u[k];
        const double bk = B * ((isfinite(uk) ? uk : 0.0) + c);
        b[k] = bk;
        s += bk;
    }
    part[t] = s;
    __syncthreads();
    for (int off = 1; off < nt; off <<= 1) {
        const double v = (t >= off) ? part[t - off] : 0.0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    double run = (t == 0) ? 0.0 : part[t - 1];
    for (int k = lo; k < hi; k++) {
        cb[k] = run;
        run += b[k];
    }
    if (t == nt - 1) cb[L] = part[nt - 1];
}

__global__ void baseline_kernel(const double* __restrict__ u, int L, double B, double c, double* __restrict__ b,
                                double* __restrict__ cb)
{
    baseline_body(u, L, B, c, b, cb);
}

// one block per alignment of a batch
__global__ void baseline_batch_kernel(const Band* __restrict__ bands, double B, double c)
{
    const Band t = bands[blockIdx.x];
    baseline_body(t.u, t.L, B, c, t.b, t.cb);
}

int launch_baseline(messi_ctx* ctx, const Band& t, double B)
{
    baseline_kernel<<<1, 1024, 0, ctx->stream>>>(t.u, t.L, B, baseline_c(), t.b, t.cb);
    LAUNCH_CHECK(ctx, "baseline_kernel");
    return MESSI_OK;
}

// ---------------------------------------------------------------------------
// pair-score preparation from a dense host matrix
// ---------------------------------------------------------------------------
__global__ void maxspan_kernel(const double* __restrict__ p, int L, int* __restrict__ out)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int best = 0;
    if (idx < (long long)L * L) {
        const int i = (int)(idx % L), j = (int)(idx / L);
        if (i < j && isfinite(p[idx])) best = j - i;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, off));
    if ((threadIdx.x & 31) == 0 && best > 0) atomicMax(out, best);
}

int launch_maxspan(messi_ctx* ctx, int L, const double* d_dense, int* d_out)
{
    cudaError_t e = cudaMemsetAsync(d_out, 0, sizeof(int), ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "memset maxspan");
    const long long n = (long long)L * L;
    maxspan_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(d_dense, L, d_out);
    LAUNCH_CHECK(ctx, "maxspan_kernel");
    return MESSI_OK;
}

// pb[i][k] from the upper triangle p(i, i+k) of a dense column-major matrix.
// Threads walk i fastest for a fixed column j so the dense reads coalesce.
__global__ void bandprep_from_dense_kernel(const double* __restrict__ p, int L, int Wb, int RS,
                                           const double* __restrict__ b, double B, float* __restrict__ pb)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)L * RS) return;
    const int j = (int)(idx / RS), r = (int)(idx % RS);
    // r enumerates rows i = j - RS + 1 + r .. j; k = j - i
    const int k = RS - 1 - r;
    const int i = j - k;
    if (i < 0) return;
    float out = -INFINITY;
    if (k >= 1 && k <= Wb) {
        const double v = p[(size_t)i + (size_t)j * L];
        if (v != -INFINITY && !isnan(v)) out = (float)(B * v - b[i] - b[j]);
    }
    pb[(size_t)i * RS + k] = out;
}

__global__ void fill_kernel(float* __restrict__ a, long long n, float v)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < n) a[idx] = v;
}

static int fill(messi_ctx* ctx, float* a, long long n, float v)
{
    fill_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(a, n, v);
    LAUNCH_CHECK(ctx, "fill_kernel");
    return MESSI_OK;
}

int launch_bandprep_from_dense(messi_ctx* ctx, const Band& t, const double* d_dense, double B)
{
    int rc = fill(ctx, t.pb, (long long)t.L * t.RS, -INFINITY);
    if (rc) return rc;
    const long long n = (long long)t.L * t.RS;
    bandprep_from_dense_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(d_dense, t.L, t.Wb, t.RS, t.b,
                                                                                      B, t.pb);
    LAUNCH_CHECK(ctx, "bandprep_from_dense_kernel");
    return MESSI_OK;
}

// ---------------------------------------------------------------------------
// inside
// ---------------------------------------------------------------------------
// Ssuf[i] for spans beyond the band (i < T = L-1-Wb), descending i:
// Ssuf[i] = r1 + LSE_{k=0..Wb} (Lrow[i][k] + Ssuf[i+k+1]), a recurrence
// whose every cell waits for the Wb+1 cells after it.  One CTA, blocks of 32
// cells from the top.  Every cell keeps a running log-sum-exp (m, s) of the
// terms whose S cell is already final, in shared memory over a window of
// cells (slot c % win): first the terms into the band's last column (j >= T),
// then, each time a block is final, its 32 values are pushed into the cells
// that reference them.  A push of S cell j into cell c adds L(c, j-1) +
// Ssuf[j]; for fixed j, L(c, j-1) = Lcol[j-1][j-1-c] is contiguous in c, so
// threads that own consecutive cells load consecutive words.  Warp 0 pushes
// into the next block's cells and solves that block's in-block triangle by
// column-oriented substitution; meanwhile the other warps push into the
// farther cells; one CTA barrier per block.  (The former form pulled each
// block's Wb+1 terms per cell from global memory after the block above was
// final: 2.7 ms for the 8,199 suffix cells of a 9,000-column alignment with
// span 800.)
constexpr int kSuffixMaxWindow = 24576;  // cells of the shared-memory window (192 KB)
// threads of a suffix CTA (16 warps: 128 registers each, so warp 0 keeps its
// 32 prefetched terms in registers across the triangle)
constexpr int kSuffixThreads = 512;

__host__ __device__ inline int suffix_window(int Wb) { return Wb + 64; }

// Asks L2 to fetch rows [r0, r1] of a band table (RS floats per row) from
// DRAM, `nlines` 128-byte lines from the start of each row, by threads tid
// of nthr; rows outside [0, L) are skipped.  The suffix recurrences walk the
// band tables one 32-row block at a time, and when the inside wavefront's
// tables exceed L2 each block's rows would otherwise arrive at DRAM latency
// on the single CTA's critical path.
__device__ __forceinline__ void prefetch_rows_l2(const float* tab, int RS, int L, int r0, int r1, int nlines, int tid,
                                                 int nthr)
{
    r0 = max(r0, 0);
    r1 = min(r1, L - 1);
    if (r1 < r0) return;
    const int n = (r1 - r0 + 1) * nlines;
    for (int x = tid; x < n; x += nthr) {
        const float* p = tab + (size_t)(r0 + x / nlines) * RS + (size_t)(x % nlines) * 32;
        asm volatile("prefetch.global.L2 [%0];" ::"l"(__cvta_generic_to_global(p)));
    }
}

// A read-only global load under a predicate (`dflt` where it is false),
// written as one predicated instruction so that a run of them stays a run of
// independent loads in flight (a conditional expression may become a branch
// around each load, and the loads one after another).  `p` is never read
// when `pred` is false.
__device__ __forceinline__ float ldg_if(const float* p, bool pred, float dflt)
{
    float v;
    asm("{\n\t.reg .pred q;\n\t"
        "setp.ne.b32 q, %2, 0;\n\t"
        "mov.f32 %0, %3;\n\t"
        "@q ld.global.nc.f32 %0, [%1];\n\t}"
        : "=f"(v)
        : "l"(__cvta_generic_to_global(p)), "r"((int)pred), "f"(dflt));
    return v;
}

// ldg_if through L2 only (ld.global.cg): for the wavefronts' tables, which
// other CTAs write during the launch.
__device__ __forceinline__ float ldcg_if(const float* p, bool pred, float dflt)
{
    float v;
    asm("{\n\t.reg .pred q;\n\t"
        "setp.ne.b32 q, %2, 0;\n\t"
        "mov.f32 %0, %3;\n\t"
        "@q ld.global.cg.f32 %0, [%1];\n\t}"
        : "=f"(v)
        : "l"(__cvta_generic_to_global(p)), "r"((int)pred), "f"(dflt));
    return v;
}

// Adds to (m, s) the terms col[u] + vals[u] for the block's values u < nb,
// where col[u] = tab[(jbase + dj*u) * RS + kbase - u] (the L cell that joins
// this thread's cell to value u; skipped when its band offset kbase - u is
// outside 0..Wb): the valid u are one range, computed once, and the
// addresses one base plus u times a stride, so a load costs two compares and
// an address step; the 32 loads are issued together, then summed in blocks
// of eight.
__device__ __forceinline__ void suffix_push_terms(float& m, float& s, const float* __restrict__ tab, int RS,
                                                  int jbase, int dj, int kbase, const float* vals, int nb, int Wb)
{
    const int ulo = max(0, kbase - Wb), uhi = min(nb - 1, kbase);
    const long long step = (long long)dj * RS - 1;
    const float* base = tab + ((ulo <= uhi) ? (long long)jbase * RS + kbase : 0);
    float x[32];
#pragma unroll
    for (int u = 0; u < 32; u++) {
        const bool on = u >= ulo && u <= uhi;
        x[u] = ldg_if(base + (on ? u * step : 0), on, -INFINITY);
    }
#pragma unroll
    for (int u = 0; u < 32; u++) x[u] += vals[u];
#pragma unroll
    for (int u = 0; u < 32; u += 8) {
        const float y[8] = {x[u], x[u + 1], x[u + 2], x[u + 3], x[u + 4], x[u + 5], x[u + 6], x[u + 7]};
        lse_add8(m, s, y);
    }
}

// In-block triangle of a suffix recurrence, by one warp: lane q owns cell q
// of the block (nb cells) and enters with the log-sum-exp (m, s) of its
// terms from outside the block; once cell l is final it adds
// tri[q][q-l-1] + r1 + value_l to every later lane q (recv: the lane takes
// in-block terms).  Returns every lane's final (m, s).
// Linear form first: values relative to the block's largest accumulator in
// FP32, the factors E = exp(tri + r1) staged beside tri by the staging warp,
// so a step of the serial chain is one broadcast and one multiply-add (the
// log form's step, two exponentials and their max, took ~290 cycles).  Where
// a value leaves [1e-30, 1e30] of the reference (FP32 would lose digits or
// overflow) the block is redone in the log-sum-exp form.
__device__ __forceinline__ void suffix_triangle(float& m, float& s, const float (&tri)[32][33],
                                                const float (&etri)[32][33], int nb, bool recv, int Wb, float r1,
                                                int lane)
{
    float mx = m;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    const float ref = (mx == -INFINITY) ? 0.f : mx;
    float A = (m == -INFINITY) ? 0.f : s * __expf(m - ref);
    // the factors exp(tri + r1), staged with tri (unconditional shared
    // loads at a clamped index, then the selects)
    float E[32];
#pragma unroll
    for (int l = 0; l < 32; l++) E[l] = etri[lane][max(lane - l - 1, 0)];
#pragma unroll
    for (int l = 0; l < 32; l++) {
        const int k = lane - l - 1;
        E[l] = (recv && l < lane && k <= Wb) ? E[l] : 0.f;
    }
    // the serial chain: lane l's A is final at step l (full blocks without
    // the per-step bound check)
    if (nb == 32) {
#pragma unroll
        for (int l = 0; l < 32; l++) A = fmaf(E[l], __shfl_sync(0xffffffffu, A, l), A);
    } else {
#pragma unroll
        for (int l = 0; l < 32; l++)
            if (l < nb) A = fmaf(E[l], __shfl_sync(0xffffffffu, A, l), A);
    }
    // whether the lane has any term (a zero A is then an underflow), off the chain
    bool any = (m != -INFINITY);
#pragma unroll
    for (int l = 0; l < 32; l++) {
        const float V = __shfl_sync(0xffffffffu, A, l);
        any = any || (l < nb && E[l] > 0.f && V > 0.f);
    }
    const bool bad = (lane < nb) && (!(A <= 1e30f) || (any && A < 1e-30f));
    if (!__any_sync(0xffffffffu, bad)) {
        if (A > 0.f) {
            m = ref;
            s = A;
        } else {
            m = -INFINITY;
            s = 0.f;
        }
        return;
    }
#pragma unroll
    for (int l = 0; l < 32; l++) {
        if (l < nb) {
            const float ml = __shfl_sync(0xffffffffu, m, l), sl = __shfl_sync(0xffffffffu, s, l);
            const int k = lane - l - 1;
            if (recv && lane > l && k <= Wb) lse_add_scaled(m, s, tri[lane][k] + r1 + ml, sl);
        }
    }
}

__device__ void inside_suffix_body(const Band& t, const Rules& R, float* am, float* as, int win)
{
    const int L = t.L, Wb = t.Wb, RS = t.RS;
    const int T = L - 1 - Wb;
    if (T <= 0) return;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    // tri[q][k] = Lrow[i0 - q][k]: the in-block terms of the block's cells,
    // double-buffered (warp 1 stages the next block's while warp 0 solves)
    __shared__ float tri2[2][32][33];
    __shared__ float etri2[2][32][33];  // exp(tri + r1), staged with tri
    // finished block values, double-buffered: the far pushes of one block may
    // still read them while warp 0 solves the next block
    __shared__ float vals2[2][32];
    // xs[u][q]: the L value joining next-block cell lo-1-q to this block's
    // cell i0-u (warp 0's push after the triangle), staged a block ahead by
    // warp 1 and read into registers at the top of the block
    __shared__ float xs2[2][32][33];
    int parity = 0, tb = 0;
    for (int c = threadIdx.x; c < win; c += blockDim.x) {
        am[c] = -INFINITY;
        as[c] = 0.f;
    }
    __syncthreads();
    // terms into the band's last column: cells T-1 down to T-1-Wb, a warp per cell
    const int c_first = max(0, T - 1 - Wb);
    for (int c = T - 1 - w; c >= c_first; c -= nw) {
        float m = -INFINITY, s = 0.f;
        const float* lrow = t.Lrow + (size_t)c * RS;
        const int k1 = min(L - 1, c + Wb + 1) - c - 1;
        for (int k = (T - c - 1) + lane; k <= k1; k += 512) {
            float x[16];
#pragma unroll
            for (int q = 0; q < 16; q++) {
                const int kq = k + 32 * q;
                x[q] = (kq <= k1) ? __ldg(lrow + kq) + t.Ssuf[c + kq + 1] : -INFINITY;
            }
            const float y0[8] = {x[0], x[1], x[2], x[3], x[4], x[5], x[6], x[7]};
            const float y1[8] = {x[8], x[9], x[10], x[11], x[12], x[13], x[14], x[15]};
            lse_add8(m, s, y0);
            lse_add8(m, s, y1);
        }
        group_reduce<32>(m, s);
        if (lane == 0) {
            am[c % win] = m;
            as[c % win] = s;
        }
    }
    int i0 = T - 1, lo = max(0, i0 - 31);
    // the first two blocks' pushes (Lcol rows lo-33 .. i0-1) and the second
    // block's in-block terms (first line of Lrow rows lo-32 .. lo-1)
    prefetch_rows_l2(t.Lcol, RS, L, lo - 33, i0 - 1, RS / 32, threadIdx.x, blockDim.x);
    prefetch_rows_l2(t.Lrow, RS, L, lo - 32, lo - 1, 1, threadIdx.x, blockDim.x);
    if (w == 1) {
        for (int q = 0; q < 32; q++) {
            const float v = (i0 - q >= lo && lane <= Wb) ? __ldg(t.Lrow + (size_t)(i0 - q) * RS + lane) : -INFINITY;
            tri2[0][q][lane] = v;
            etri2[0][q][lane] = __expf(v + R.r[0]);
        }
        const int nb0 = i0 - lo + 1, nlo0 = max(0, lo - 32), c = lo - 1 - lane;
        for (int u = 0; u < 32; u++) {
            const int k = i0 - 1 - c - u;
            xs2[0][u][lane] = (lo > 0 && c >= nlo0 && u < nb0 && k <= Wb) ? __ldg(t.Lcol + (size_t)(i0 - 1 - u) * RS + k)
                                                                          : -INFINITY;
        }
    }
    __syncthreads();
    float cm = -INFINITY, cs = 0.f;  // warp 0: accumulator of cell i0 - lane
    if (w == 0 && i0 - lane >= lo) {
        cm = am[(i0 - lane) % win];
        cs = as[(i0 - lane) % win];
    }
    for (;;) {
        const int nb = i0 - lo + 1;
        const int nlo = max(0, lo - 32);
        float* vals = vals2[parity];
        parity ^= 1;
        float x[32];  // warp 0: L values joining its next-block cell to this block's cells
        if (w == 0) {
            // column-oriented substitution: lane q owns cell i0 - q
            float m = (lane < nb) ? cm : -INFINITY, s = (lane < nb) ? cs : 0.f;
            suffix_triangle(m, s, tri2[tb], etri2[tb], nb, lane < nb, Wb, R.r[0], lane);
            // the block's values, formed and stored by all lanes at once
            if (lane < nb) {
                const float sv = R.r[0] + lse_val(m, s);
                t.Ssuf[i0 - lane] = sv;
                vals[lane] = sv;
            }
            // the push operands, before the barrier: warp 1 refills this
            // buffer in the next block
#pragma unroll
            for (int u = 0; u < 32; u++) x[u] = xs2[tb][u][lane];
        } else if (w == 1 && lo > 0) {
            // the next block's in-block terms and push operands: all 64 loads
            // first, then the stores (one memory round trip)
            const int i0n = lo - 1, nbn = lo - nlo, nlon = max(0, nlo - 32), c = nlo - 1 - lane;
            float v[32], y[32];
#pragma unroll
            for (int q = 0; q < 32; q++) {
                const bool onv = lo - 1 - q >= nlo && lane <= Wb;
                v[q] = ldg_if(t.Lrow + (onv ? (size_t)(lo - 1 - q) * RS + lane : 0), onv, -INFINITY);
                const int k = i0n - 1 - c - q;
                const bool ony = nlo > 0 && c >= nlon && q < nbn && k <= Wb;
                y[q] = ldg_if(t.Lcol + (ony ? (size_t)(i0n - 1 - q) * RS + k : 0), ony, -INFINITY);
            }
#pragma unroll
            for (int q = 0; q < 32; q++) {
                tri2[tb ^ 1][q][lane] = v[q];
                etri2[tb ^ 1][q][lane] = __expf(v[q] + R.r[0]);
                xs2[tb ^ 1][q][lane] = y[q];
            }
        } else if (w >= 2) {
            // the block after the next one: its pushes read Lcol rows
            // lo-65 .. lo-34, its in-block terms Lrow rows lo-64 .. lo-33
            prefetch_rows_l2(t.Lcol, RS, L, lo - 65, lo - 34, RS / 32, threadIdx.x - 64, blockDim.x - 64);
            prefetch_rows_l2(t.Lrow, RS, L, lo - 64, lo - 33, 1, threadIdx.x - 64, blockDim.x - 64);
        }
        __syncthreads();
        if (lo == 0) break;
        // push the block [lo, i0] (value u = S cell i0 - u) into the cells
        // lo-1 .. lo-1-Wb; a cell's first push starts it afresh unless the
        // band already gave it terms
        if (w == 0) {
            const int c = lo - 1 - lane;
            cm = -INFINITY;
            cs = 0.f;
            if (c >= nlo) {
                const bool fresh = (c < c_first) && (c + Wb + 1 <= i0);
                if (!fresh) {
                    cm = am[c % win];
                    cs = as[c % win];
                }
#pragma unroll
                for (int u = 0; u < 32; u += 8) {
                    const float y[8] = {x[u] + vals[u], x[u + 1] + vals[u + 1], x[u + 2] + vals[u + 2],
                                        x[u + 3] + vals[u + 3], x[u + 4] + vals[u + 4], x[u + 5] + vals[u + 5],
                                        x[u + 6] + vals[u + 6], x[u + 7] + vals[u + 7]};
                    lse_add8(cm, cs, y);
                }
            }
        } else if (w >= 2) {
            for (int c = nlo - 1 - (threadIdx.x - 64); c >= max(0, lo - 1 - Wb); c -= (int)blockDim.x - 64) {
                const bool fresh = (c < c_first) && (c + Wb + 1 <= i0);
                float m = fresh ? -INFINITY : am[c % win], s = fresh ? 0.f : as[c % win];
                suffix_push_terms(m, s, t.Lcol, RS, i0 - 1, -1, i0 - 1 - c, vals, nb, Wb);
                am[c % win] = m;
                as[c % win] = s;
            }
        }
        tb ^= 1;
        i0 = lo - 1;
        lo = nlo;
    }
}

// Blocks of 32 cells pulled from global memory (bands wider than the
// shared-memory window of the pushing form).
__device__ void inside_suffix_body_pull(const Band& t, const Rules& R)
{
    const int T = t.L - 1 - t.Wb;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __shared__ float known[32];
    __shared__ float tri[32][33];  // Lrow[i0 - l][k], k < 32: the in-block terms, read by the serial warp
    for (int i0 = T - 1; i0 >= 0; i0 -= 32) {
        const int lo = max(0, i0 - 31);
        const int i = i0 - w;
        tri[w][lane] = (i >= lo && lane <= t.Wb) ? t.Lrow[(size_t)i * t.RS + lane] : -INFINITY;
        if (i >= lo) {
            float m = -INFINITY, s = 0.f;
            const float* lrow = t.Lrow + (size_t)i * t.RS;
            int k = (i0 - i) + lane;
            for (; k + 96 <= t.Wb; k += 128)
                lse_add4(m, s, lrow[k] + t.Ssuf[i + k + 1], lrow[k + 32] + t.Ssuf[i + k + 33],
                         lrow[k + 64] + t.Ssuf[i + k + 65], lrow[k + 96] + t.Ssuf[i + k + 97]);
            for (; k <= t.Wb; k += 32) lse_add(m, s, lrow[k] + t.Ssuf[i + k + 1]);
            group_reduce<32>(m, s);
            if (lane == 0) known[w] = lse_val(m, s);
        }
        __syncthreads();
        if (w == 0) {
            // column-oriented substitution: lane q owns cell i0 - q; once cell l
            // is final it is broadcast and every later cell adds its term
            const int nb = i0 - lo + 1;
            float am = (lane < nb) ? known[lane] : -INFINITY, as = (am == -INFINITY) ? 0.f : 1.f;
            for (int l = 0; l < nb; l++) {
                const float sv = __shfl_sync(0xffffffffu, R.r[0] + lse_val(am, as), l);
                if (lane == 0) t.Ssuf[i0 - l] = sv;
                const int k = lane - l - 1;
                if (lane > l && lane < nb && k <= t.Wb) lse_add(am, as, tri[lane][k] + sv);
            }
        }
        __syncthreads();
    }
}

__device__ void inside_suffix_any(const Band& t, const Rules& R, float* smem, int win)
{
    if (suffix_window(t.Wb) <= win) inside_suffix_body(t, R, smem, smem + win, win);
    else inside_suffix_body_pull(t, R);
}

// win: cells of the dynamic shared-memory window (2 * win floats)
__global__ void __launch_bounds__(kSuffixThreads) inside_suffix_kernel(Band t, Rules R, int win)
{
    extern __shared__ float suffix_smem[];
    inside_suffix_any(t, R, suffix_smem, win);
}

// one block per alignment of a batch (alignments whose band reaches the last column skip)
__global__ void __launch_bounds__(kSuffixThreads) inside_suffix_batch_kernel(const Band* __restrict__ bands, Rules R,
                                                                           int win)
{
    extern __shared__ float suffix_smem[];
    const Band t = bands[blockIdx.x];
    if (t.L - 1 > t.Wb) inside_suffix_any(t, R, suffix_smem, win);
}

// Window for the largest band that needs a suffix (0: none fits, the pull form runs).
static int suffix_launch_window(int maxWb)
{
    const int win = suffix_window(maxWb);
    return (win <= kSuffixMaxWindow) ? win : 0;
}

// The window for a batch: the widest band among those that take the pushing
// form (a band too wide for any window takes the pull form in a single call
// too, so both paths give the same bits).
static int suffix_batch_window(const BandBatch& bb)
{
    int win = 0;
    for (const Band& t : bb.host)
        if (t.L - 1 > t.Wb && suffix_window(t.Wb) <= kSuffixMaxWindow) win = std::max(win, suffix_window(t.Wb));
    return win;
}

static cudaError_t suffix_smem_attr(int win)
{
    const int bytes = 2 * win * (int)sizeof(float);
    cudaError_t e = cudaFuncSetAttribute(inside_suffix_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         std::max(bytes, 0));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(inside_suffix_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 std::max(bytes, 0));
    return e;
}

__global__ void finish_Z_kernel(Band t)
{
    if (threadIdx.x == 0 && blockIdx.x == 0)
        t.Zd[0] = (t.sync[2] != 0u) ? (double)NAN : (double)t.Ssuf[0] + t.cb[t.L];
}

__global__ void finish_Z_batch_kernel(const Band* __restrict__ bands, int n, const unsigned int* __restrict__ sync,
                                      double* __restrict__ Z)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    const Band& t = bands[b];
    Z[b] = (sync[2] != 0u) ? (double)NAN : (double)t.Ssuf[0] + t.cb[t.L];
}

int launch_finish_Z(messi_ctx* ctx, const Band& t)
{
    finish_Z_kernel<<<1, 32, 0, ctx->stream>>>(t);
    LAUNCH_CHECK(ctx, "finish_Z_kernel");
    return queue_status_readback(ctx, t);
}


// Log-sum-exp over a group of G lanes: the group's maximum by a butterfly,
// one rescale per lane, then a butterfly sum (max and sum are commutative,
// so every lane of the group ends with the same bits) -- about a third of the
// instructions of a pairwise merge per round.
__device__ __forceinline__ void group_reduce_rt(float& m, float& s, int G)
{
    float mx = m;
    for (int off = G >> 1; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    const float base = (mx == -INFINITY) ? 0.f : mx;
    float v = s * __expf(m - base);
    for (int off = G >> 1; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    m = mx;
    s = v;
}

// Span-0 cells of row i.
__device__ __forceinline__ void inside_init_cell(const Band& t, int i, const Rules& R, double B)
{
    const double ui = t.u[i];
    const float S = (ui == -INFINITY) ? -INFINITY : (float)(B * ui + (double)R.r[1] - t.b[i]);
    const float Lv = (ui == -INFINITY) ? -INFINITY : (float)(B * ui + (double)R.r[5] - t.b[i]);
    const size_t o = (size_t)i * t.RS;
    t.Srow[o] = S;
    t.Scol[o] = S;
    t.Lrow[o] = Lv;
    t.Lcol[o] = Lv;
    t.Frow[o] = -INFINITY;
    if (i == t.L - 1) t.Ssuf[i] = S;
}

// Cell (i, i+d) in two parts, by a group of G lanes (every lane of the warp
// calls both, `valid` false for padding groups: the shuffles need the whole
// warp).  The split sum runs over k = 0 .. d-1 of L(i, i+k) + S(i+k+1, j),
// spans k and d-1-k.  The partial part sums the middle split points k =
// NLO .. d-NHI-1 (both spans <= d-1-min(NLO, NHI)), reduces them over the
// group and loads the pair score; the finishing part (lane 0) adds the
// outer split points k < NLO and k >= d-NHI in ascending order, the enclosed
// F (span d-2) and writes the cell.  Odd spans use NLO = NHI = 2, even spans
// 3: the partial sums of a diagonal pair (2p-1, 2p) then read spans <= 2p-4
// only, which the paired wavefront has before its wait, and every kernel
// splits a cell the same way, so all of them give the same bits.
struct CellPartial {
    float m, s, pbv;
};

// Sixteen split points of a lane that are all in range (two blocks of eight,
// summed in order): no predicates, and with the group width a constant the
// 32 loads take immediate offsets from two base addresses.  Long spans spend
// most of their points here; the integer pipe (addresses, range checks,
// selects) was the busiest one in the predicated form.
template <int GS>
__device__ __forceinline__ void split_full16(float& m, float& s, const float* lrow, const float* scol, int k)
{
    const float* pa = lrow + k;
    const float* pb = scol - k;
    float a[16], b[16];
#pragma unroll
    for (int q = 0; q < 16; q++) {
        a[q] = __ldcg(pa + q * GS);
        b[q] = __ldcg(pb - q * GS);
    }
    float x0[8], x1[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
        x0[q] = a[q] + b[q];
        x1[q] = a[8 + q] + b[8 + q];
    }
    lse_add8(m, s, x0);
    lse_add8(m, s, x1);
}

// The last rem points (1..16) of a lane at G = 32, in one or two blocks of
// eight (TWO), summed in order: predicated loads at constant offsets from two
// base addresses, the absent points -inf.  Most of a lane's points on bands
// up to 800 wide fall here (at most 25 per lane).
template <bool TWO>
__device__ __forceinline__ void split_tail32(float& m, float& s, const float* lrow, const float* scol, int k,
                                             int rem)
{
    constexpr int NQ = TWO ? 16 : 8;
    const float* pa = lrow + k;
    const float* pb = scol - k;
    float a[NQ], b[NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) {
        const bool on = q < rem;
        a[q] = ldcg_if(pa + q * 32, on, -INFINITY);
        b[q] = ldcg_if(pb - q * 32, on, -INFINITY);
    }
    float x0[8];
#pragma unroll
    for (int q = 0; q < 8; q++) x0[q] = a[q] + b[q];
    lse_add8(m, s, x0);
    if (TWO) {
        float x1[8];
#pragma unroll
        for (int q = 0; q < 8; q++) x1[q] = a[(8 + q) % NQ] + b[(8 + q) % NQ];
        lse_add8(m, s, x1);
    }
}

template <int NLO, int NHI, bool WIDE>
__device__ __forceinline__ CellPartial cell_partial_t(const Band& t, int i, int d, bool valid, int lane, int G)
{
    const int RS = t.RS;
    CellPartial c{-INFINITY, 0.f, -INFINITY};
    // lanes 0 and 1: either may finish the cell (rows_finish)
    if (valid && lane < 2 && d >= 2) c.pbv = t.pb[(size_t)i * RS + d];
    const int kend = d - NHI;
    if (valid && kend > NLO) {
        const float* lrow = t.Lrow + (size_t)i * RS;
        const float* scol = t.Scol + (size_t)(i + d) * RS + (d - 1);
        // blocks of eight split points per lane, summed in order.  WIDE: while
        // a lane has more than eight points left, two blocks' 32 loads are
        // issued together (one L2 round trip for sixteen points: long spans
        // have up to 47 points per lane); the narrow form keeps 16 loads in
        // flight for kernels without the registers.  Points past the end are
        // -inf, which lse_add8 skips exactly, so both forms give the same bits.
        int k = NLO + lane;
        if (G == 32) {  // warp-uniform: one cell per warp, constant strides
            int rem;
            if (WIDE) {
                for (; k + 15 * 32 < kend; k += 16 * 32) split_full16<32>(c.m, c.s, lrow, scol, k);
                rem = (kend - k + 31) / 32;  // points left (<= 0: none)
                if (rem > 8) {
                    split_tail32<true>(c.m, c.s, lrow, scol, k, rem);
                    rem = 0;
                }
            } else {
                rem = (kend - k + 31) / 32;
            }
            for (; rem > 0; rem -= 8, k += 8 * 32) split_tail32<false>(c.m, c.s, lrow, scol, k, rem);
        } else {
            if (WIDE) {
                for (; k + 8 * G < kend; k += 16 * G) {
                    float a[16], b[16];
#pragma unroll
                    for (int q = 0; q < 16; q++) {
                        const int kq = k + q * G;
                        const bool on = kq < kend;
                        a[q] = ldcg_if(lrow + kq, on, -INFINITY);
                        b[q] = ldcg_if(scol - kq, on, -INFINITY);
                    }
                    float x0[8], x1[8];
#pragma unroll
                    for (int q = 0; q < 8; q++) {
                        x0[q] = a[q] + b[q];
                        x1[q] = a[8 + q] + b[8 + q];
                    }
                    lse_add8(c.m, c.s, x0);
                    lse_add8(c.m, c.s, x1);
                }
            }
            for (; k < kend; k += 8 * G) {
                float x[8];
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    const int kq = k + q * G;
                    const bool on = kq < kend;
                    x[q] = ldcg_if(lrow + kq, on, -INFINITY) + ldcg_if(scol - kq, on, -INFINITY);
                }
                lse_add8(c.m, c.s, x);
            }
        }
    }
    // the shuffles only where some lane group of the warp has a cell (the
    // callers pass every lane of the warp; an empty slot's result is unused)
    if (__any_sync(0xffffffffu, valid)) group_reduce_rt(c.m, c.s, G);
    return c;
}

// cell_partial_t in two steps, for a wavefront that issues a cell's loads
// one phase before it needs them: partial_issue loads the pair score and the
// operands of the first two blocks (sixteen split points per lane) without
// using them, so that the loads stay in flight; partial_complete adds them
// and any further blocks in the same order and reduces over the group, so the
// result has the bits of cell_partial_t.
struct PartialPre {
    float a[16], b[16];
    float pbv;
};

template <int NLO, int NHI>
__device__ __forceinline__ void partial_issue(const Band& t, int i, int d, bool valid, int lane, int G,
                                              PartialPre& pp)
{
    const int RS = t.RS;
    pp.pbv = (valid && lane == 0 && d >= 2) ? t.pb[(size_t)i * RS + d] : -INFINITY;
    const int kend = d - NHI;
    const float* lrow = t.Lrow + (size_t)i * RS;
    const float* scol = t.Scol + (size_t)(i + d) * RS + (d - 1);
    if (G == 32) {  // constant strides from two base addresses
        const float* pa = lrow + NLO + lane;
        const float* pb = scol - NLO - lane;
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const bool on = valid && NLO + lane + q * 32 < kend;
            pp.a[q] = ldcg_if(pa + q * 32, on, -INFINITY);
            pp.b[q] = ldcg_if(pb - q * 32, on, -INFINITY);
        }
    } else {
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const int kq = NLO + lane + q * G;
            const bool on = valid && kq < kend;
            pp.a[q] = ldcg_if(lrow + kq, on, -INFINITY);
            pp.b[q] = ldcg_if(scol - kq, on, -INFINITY);
        }
    }
}

template <int NLO, int NHI>
__device__ __forceinline__ CellPartial partial_complete(const Band& t, int i, int d, bool valid, int lane, int G,
                                                        const PartialPre& pp)
{
    CellPartial c{-INFINITY, 0.f, pp.pbv};
    const int kend = d - NHI;
    if (valid && kend > NLO) {
        // a block that cell_partial_t would not reach is all -inf: lse_add8 leaves (m, s) as they are
        float x0[8], x1[8];
#pragma unroll
        for (int q = 0; q < 8; q++) {
            x0[q] = pp.a[q] + pp.b[q];
            x1[q] = pp.a[8 + q] + pp.b[8 + q];
        }
        lse_add8(c.m, c.s, x0);
        lse_add8(c.m, c.s, x1);
        const float* lrow = t.Lrow + (size_t)i * t.RS;
        const float* scol = t.Scol + (size_t)(i + d) * t.RS + (d - 1);
        for (int k = NLO + lane + 16 * G; k < kend; k += 8 * G) {
            float x[8];
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const int kq = k + q * G;
                x[q] = (kq < kend) ? __ldcg(lrow + kq) + __ldcg(scol - kq) : -INFINITY;
            }
            lse_add8(c.m, c.s, x);
        }
    }
    // the shuffles only where some lane group of the warp has a cell (the
    // callers pass every lane of the warp; an empty slot's result is unused)
    if (__any_sync(0xffffffffu, valid)) group_reduce_rt(c.m, c.s, G);
    return c;
}

// Operands of a cell's outer split points, k < NLO and k >= hb = max(NLO,
// d-NHI) in ascending k: L(i, i+k) and S(i+k+1, j), both -inf where the
// split point is absent (an absent term is then -inf, which lse_add skips
// exactly), and the enclosed F(i+1, j-1).
template <int NLO, int NHI>
struct Outer {
    float l[NLO + NHI], s[NLO + NHI], fin;
};

// defer: leave L(i, i+d-1) and S(i+1, j), the two operands on diagonal d-1,
// to outer_patch.
template <int NLO, int NHI>
__device__ __forceinline__ Outer<NLO, NHI> outer_load(const Band& t, int i, int d, bool defer)
{
    Outer<NLO, NHI> o;
    const int RS = t.RS;
    const float* lrow = t.Lrow + (size_t)i * RS;
    const float* scol = t.Scol + (size_t)(i + d) * RS + (d - 1);
    const int hb = max(NLO, d - NHI);
#pragma unroll
    for (int q = 0; q < NLO + NHI; q++) {
        const int k = (q < NLO) ? q : hb + (q - NLO);
        const bool present = k < d;
        o.l[q] = !present ? -INFINITY : ((defer && k == d - 1) ? 0.f : __ldcg(lrow + k));
        o.s[q] = !present ? -INFINITY : ((defer && k == 0) ? 0.f : __ldcg(scol - k));
    }
    o.fin = (d >= 2) ? __ldcg(t.Frow + (size_t)(i + 1) * RS + (d - 2)) : -INFINITY;
    return o;
}

template <int NLO, int NHI>
__device__ __forceinline__ void outer_patch(Outer<NLO, NHI>& o, int d, float l_last, float s_first)
{
    const int hb = max(NLO, d - NHI);
#pragma unroll
    for (int q = 0; q < NLO + NHI; q++) {
        const int k = (q < NLO) ? q : hb + (q - NLO);
        if (k < d && k == d - 1) o.l[q] = l_last;
        if (k < d && k == 0) o.s[q] = s_first;
    }
}

// Adds the outer split points to the partial sum and writes cell (i, i+d);
// lv/sv, when given, also receive its L and S.
template <int NLO, int NHI>
__device__ __forceinline__ void cell_write_t(const Band& t, int i, int d, CellPartial c, const Outer<NLO, NHI>& o,
                                             const Rules& R, float* lv = nullptr, float* sv = nullptr)
{
    const int RS = t.RS;
    const int j = i + d;
    // the outer split points as one block (one max, independent exponentials:
    // this is the serial part of a cell after the barrier)
    float x[8];
#pragma unroll
    for (int q = 0; q < 8; q++) x[q] = (q < NLO + NHI) ? o.l[q % (NLO + NHI)] + o.s[q % (NLO + NHI)] : -INFINITY;
    lse_add8(c.m, c.s, x);
    const float tmp = lse_val(c.m, c.s);
    const float v = c.pbv + o.fin;
    const float S = lse2f(R.r[0] + tmp, R.r[2] + v);
    const float F = lse2f(R.r[4] + tmp, R.r[3] + v);
    const float Lv = R.r[6] + v;
    t.Lrow[(size_t)i * RS + d] = Lv;
    t.Lcol[(size_t)j * RS + d] = Lv;
    t.Srow[(size_t)i * RS + d] = S;
    t.Scol[(size_t)j * RS + d] = S;
    t.Frow[(size_t)i * RS + d] = F;
    if (j == t.L - 1) t.Ssuf[i] = S;
    if (lv) {
        *lv = Lv;
        *sv = S;
    }
}

template <int NLO, int NHI>
__device__ __forceinline__ void cell_finish_t(const Band& t, int i, int d, bool valid, int lane, CellPartial c,
                                              const Rules& R)
{
    if (!(valid && lane == 0)) return;
    cell_write_t<NLO, NHI>(t, i, d, c, outer_load<NLO, NHI>(t, i, d, false), R);
}

template <bool WIDE>
__device__ __forceinline__ CellPartial inside_cell_partial(const Band& t, int i, int d, bool valid, int lane, int G)
{
    return (d & 1) ? cell_partial_t<2, 2, WIDE>(t, i, d, valid, lane, G) : cell_partial_t<3, 3, WIDE>(t, i, d, valid, lane, G);
}

__device__ __forceinline__ void inside_cell_finish(const Band& t, int i, int d, bool valid, int lane, CellPartial c,
                                                   const Rules& R)
{
    if (d & 1) cell_finish_t<2, 2>(t, i, d, valid, lane, c, R);
    else cell_finish_t<3, 3>(t, i, d, valid, lane, c, R);
}

template <bool WIDE>
__device__ __forceinline__ void inside_cell(const Band& t, int i, int d, bool valid, int lane, int G, const Rules& R)
{
    inside_cell_finish(t, i, d, valid, lane, inside_cell_partial<WIDE>(t, i, d, valid, lane, G), R);
}

// The cells of one diagonal that a CTA owns (rows [r0, end)), computed by the
// CTA's warps [w0, w0 + nw) in two phases: partial sums of the first two rows
// of every group, then (after the caller's wait) their finishing parts and any
// further rows whole.  Which warp computes a cell does not change its bits.
struct RowsPart {
    CellPartial c[2];
};

struct WarpSet {
    int w0, nw;
    __device__ __forceinline__ bool mine() const
    {
        const int w = threadIdx.x >> 5;
        return w >= w0 && w < w0 + nw;
    }
};

template <bool WIDE>
__device__ __forceinline__ RowsPart rows_partial(const Band& t, int d, int r0, int end, WarpSet ws)
{
    RowsPart p;
    p.c[0] = p.c[1] = CellPartial{-INFINITY, 0.f, -INFINITY};
    if (!ws.mine()) return p;  // warp-uniform: the group shuffles stay within the warp
    const int G = group_width(d), gpb = ws.nw * (32 / G);
    const int lane = threadIdx.x & (G - 1), g = (threadIdx.x - 32 * ws.w0) / G;
#pragma unroll
    for (int it = 0; it < 2; it++) {
        const int i = r0 + g + it * gpb;
        p.c[it] = inside_cell_partial<WIDE>(t, i, d, i < end, lane, G);
    }
    return p;
}

template <bool WIDE>
__device__ __forceinline__ void rows_finish(const Band& t, int d, int r0, int end, const RowsPart& p, const Rules& R,
                                            WarpSet ws)
{
    if (!ws.mine()) return;
    const int G = group_width(d), gpb = ws.nw * (32 / G);
    const int lane = threadIdx.x & (G - 1), g = (threadIdx.x - 32 * ws.w0) / G;
    if (G >= 2) {
        // every lane of a group holds both reduced partial sums: lanes 0 and 1
        // finish the group's two cells side by side
        const int it = lane & 1;
        const int i = r0 + g + it * gpb;
        inside_cell_finish(t, i, d, lane < 2 && i < end, 0, it ? p.c[1] : p.c[0], R);
    } else {
#pragma unroll
        for (int it = 0; it < 2; it++) {
            const int i = r0 + g + it * gpb;
            inside_cell_finish(t, i, d, i < end, lane, p.c[it], R);
        }
    }
    for (int base = r0 + 2 * gpb; base < end; base += gpb) {
        const int i = base + g;
        inside_cell<WIDE>(t, i, d, i < end, lane, G, R);
    }
}

// All band diagonals of the inside pass, two per grid barrier.  CTA b owns
// rows [b*R, (b+1)*R) of every diagonal (R = ceil(L / CTAs)).  For the pair
// (2p-1, 2p) it computes diagonal 2p-1 for its rows plus row (b+1)*R (which
// the next CTA also computes, to the same bits) and then, after a CTA
// barrier, diagonal 2p, whose cells read diagonal 2p-1 only at rows i and
// i+1, its own.  The partial sums of both diagonals read spans <= 2p-4 and
// are computed between the CTA's arrival at the barrier that completes
// diagonal 2p-2 and its wait there; every warp computes both diagonals'
// cells, one after the other.
__global__ void __launch_bounds__(kWaveMaxThreads) inside_wave_kernel(Band t, Rules R, double B)
{
    unsigned int gen = 0;
    const int L = t.L;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L; i += gridDim.x * blockDim.x) inside_init_cell(t, i, R, B);
    grid_arrive(t.sync);
    const int rows = (L + gridDim.x - 1) / gridDim.x;
    const int r0 = blockIdx.x * rows;
    const WarpSet all{0, (int)(blockDim.x >> 5)};
    for (int eA = 1; eA <= t.Wb; eA += 2) {
        const int eB = eA + 1;
        const int endA = min(r0 + rows + 1, L - eA);
        const int endB = (eB <= t.Wb) ? min(r0 + rows, L - eB) : r0;
        const RowsPart pa = rows_partial<true>(t, eA, r0, endA, all);
        const RowsPart pb = rows_partial<true>(t, eB, r0, endB, all);
        if (!grid_wait(t.sync, gen)) return;
        // further rows (short spans only) in the narrow form: the wide one
        // would spill beside the partial sums held across the wait
        rows_finish<false>(t, eA, r0, endA, pa, R, all);
        __syncthreads();  // diagonal 2p-1 of this CTA's rows before diagonal 2p reads it
        rows_finish<false>(t, eB, r0, endB, pb, R, all);
        grid_arrive(t.sync);
    }
}

// inside_wave_kernel when the CTA's rows fit one per warp in each half of
// the CTA (the host launches it only then): the odd diagonals' cells go to
// the first half, the even ones' to the second, one cell per lane group.
// The wait that completes diagonal 2p-2 also completes every span that the
// next pair's partial sums read (<= 2p-2), so a warp issues the loads of its
// next cell's partial sum as soon as its current cell is finished, before
// the arrival, and adds them after it.
__global__ void __launch_bounds__(kWaveMaxThreads) inside_wave_pipe_kernel(Band t, Rules R, double B)
{
    __shared__ float s_lv[kWaveMaxThreads / 64], s_sv[kWaveMaxThreads / 64];
    unsigned int gen = 0;
    const int L = t.L, Wb = t.Wb;
    const int rows = (L + gridDim.x - 1) / gridDim.x;
    const int r0 = blockIdx.x * rows;
    const int half = (int)(blockDim.x >> 6);
    if (half < rows + 1) {  // not launched so; leave with the launch marked failed
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicExch(&t.sync[2], 1u);
        return;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L; i += gridDim.x * blockDim.x) inside_init_cell(t, i, R, B);
    grid_arrive(t.sync);
    const bool odd = (int)(threadIdx.x >> 5) < half;
    const int tid = (int)threadIdx.x - (odd ? 0 : 32 * half);
    // this warp's diagonal of pair p is 2p-1 (odd) or 2p; its cell's row r0 + g
    auto row_end = [&](int d) {
        return (d > Wb) ? r0 : (odd ? min(r0 + rows + 1, L - d) : min(r0 + rows, L - d));
    };
    int d = odd ? 1 : 2;
    int G = group_width(d), lane = tid & (G - 1), i = r0 + tid / G;
    bool valid = i < row_end(d);
    CellPartial c;
    {
        PartialPre pp;
        if (odd) {
            partial_issue<2, 2>(t, i, d, valid, lane, G, pp);
            c = partial_complete<2, 2>(t, i, d, valid, lane, G, pp);
        } else {
            partial_issue<3, 3>(t, i, d, valid, lane, G, pp);
            c = partial_complete<3, 3>(t, i, d, valid, lane, G, pp);
        }
    }
    for (int eA = 1; eA <= Wb; eA += 2) {
        if (!grid_wait(t.sync, gen)) return;
        const int dn = d + 2;
        const int Gn = group_width(dn), lanen = tid & (Gn - 1), in = r0 + tid / Gn;
        const bool validn = in < row_end(dn);
        PartialPre pn;
        int ib = -1;
        Outer<3, 3> ob;
        if (odd) {
            if (valid && lane == 0)
                cell_write_t<2, 2>(t, i, d, c, outer_load<2, 2>(t, i, d, false), R, s_lv + (i - r0), s_sv + (i - r0));
        } else if (valid && lane == 0) {
            ob = outer_load<3, 3>(t, i, d, true);
            ib = i;
        }
        __syncthreads();  // diagonal 2p-1 of this CTA's rows in s_lv / s_sv
        if (ib >= 0) {
            outer_patch<3, 3>(ob, d, s_lv[ib - r0], s_sv[ib + 1 - r0]);
            cell_write_t<3, 3>(t, ib, d, c, ob, R);
        }
        // the next cell's loads go out after the current cells' (issued
        // earlier they queue ahead of the finishing loads, which are on the
        // critical path) and stay in flight across the arrival
        if (odd) partial_issue<2, 2>(t, in, dn, validn, lanen, Gn, pn);
        else partial_issue<3, 3>(t, in, dn, validn, lanen, Gn, pn);
        // the last warp never has a cell (its group index is >= rows), so no
        // loads in flight for the fence to wait for; the CTA barrier also
        // orders these reads before the next pair's writes
        grid_arrive(t.sync, blockDim.x - 1);
        c = odd ? partial_complete<2, 2>(t, in, dn, validn, lanen, Gn, pn)
                : partial_complete<3, 3>(t, in, dn, validn, lanen, Gn, pn);
        d = dn;
        G = Gn;
        lane = lanen;
        i = in;
        valid = validn;
    }
}

// Batched inside over n alignments in one persistent launch: diagonal d of
// every alignment whose band reaches it is one step of the wavefront.  Bands
// are sorted by band width, descending, so the alignments active at span d
// are a prefix [0, nact) and the cells of diagonal d, flattened in band order,
// start at cumL[b] - d*b for band b (cumL: exclusive prefix of the lengths).
__device__ __forceinline__ int batch_active(const int* __restrict__ wbs, int n, int d)
{
    int lo = 0, hi = n;  // first band with Wb < d
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (wbs[mid] >= d) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ int batch_band(const long long* __restrict__ cumL, int nact, int d, long long item)
{
    int lo = 0, hi = nact - 1;  // last band b with cumL[b] - d*b <= item
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (cumL[mid] - (long long)d * mid <= item) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(kWaveMaxThreads) inside_wave_batch_kernel(const Band* __restrict__ bands,
                                                                const long long* __restrict__ cumL,
                                                                const int* __restrict__ wbs, int n, Rules R,
                                                                double B, unsigned int* sync)
{
    unsigned int gen = 0;
    {
        const long long total = cumL[n];
        for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < total;
             it += (long long)gridDim.x * blockDim.x) {
            const int b = batch_band(cumL, n, 0, it);
            inside_init_cell(bands[b], (int)(it - cumL[b]), R, B);
        }
    }
    grid_arrive(sync);
    const int maxW = n > 0 ? wbs[0] : 0;
    for (int d = 1; d <= maxW; d++) {
        const int nact = batch_active(wbs, n, d);
        const long long ncell = cumL[nact] - (long long)d * nact;
        const int G = group_width(d);
        const int gpb = blockDim.x / G;
        const long long total = (long long)gridDim.x * gpb;
        const int lane = threadIdx.x & (G - 1);
        const long long gid0 = (long long)blockIdx.x * gpb + threadIdx.x / G;
        // first cells: partial sums before the wait (as in inside_wave_kernel)
        const bool v0 = gid0 < ncell;
        const int b0 = v0 ? batch_band(cumL, nact, d, gid0) : 0;
        const int i0 = v0 ? (int)(gid0 - (cumL[b0] - (long long)d * b0)) : 0;
        const CellPartial c = inside_cell_partial<true>(bands[b0], i0, d, v0, lane, G);
        if (!grid_wait(sync, gen)) return;
        inside_cell_finish(bands[b0], i0, d, v0, lane, c, R);
        for (long long base = total; base < ncell; base += total) {
            const long long it = base + gid0;
            const bool valid = it < ncell;
            const int b = valid ? batch_band(cumL, nact, d, it) : 0;
            inside_cell<true>(bands[b], valid ? (int)(it - (cumL[b] - (long long)d * b)) : 0, d, valid, lane, G, R);
        }
        grid_arrive(sync);
    }
}

// Outside cell (i, j = i+d): the parent sums run over q of OS/OF(i, j+1+q) *
// S(j+1, j+1+q) (side 0, "L") and of OS/OF(i-1-q, j) * L(i-1-q, i-1) (side
// 1, "S"), spans d+1+q.  Each sum is computed apart, by its own lane group
// (outside_sum_t: q >= Q and the suffix-column terms, reduced over the
// group); the finishing part (outside_finish_t, one thread) adds q = 0 ..
// Q-1 of both sums in ascending order, forms the F value from the enclosing
// pair (i-1, j+1) (span d+2) and writes the cell.  Diagonals go two per
// barrier, (e, e-1), with Q = 2 for e and Q = 3 for e-1: the sums then read
// spans >= e+3 only, which are complete before the wait that completes e+2
// and e+1.  A cell's bits depend only on its span (the group width), not on
// which CTA, warp or thread computes it.
struct SumPartial {
    float m, s;
};

// Eight points of one sum that are all in range (two blocks of four points,
// eight terms each, summed in order): no range checks, and with the group
// width a constant the 24 loads take immediate offsets.
template <int GS>
__device__ __forceinline__ void outside_full8(float& m, float& s, const float* o1, const float* o2, const float* in,
                                              int q, const Rules& R)
{
    const float* p1 = o1 + q;
    const float* p2 = o2 + q;
    const float* p3 = in + q;
    float a[8], b[8], v[8];
#pragma unroll
    for (int u = 0; u < 8; u++) {
        a[u] = __ldcg(p1 + u * GS);
        b[u] = __ldcg(p2 + u * GS);
        v[u] = p3[u * GS];
    }
    float x0[8], x1[8];
#pragma unroll
    for (int u = 0; u < 4; u++) {
        x0[2 * u] = R.r[0] + a[u] + v[u];
        x0[2 * u + 1] = R.r[4] + b[u] + v[u];
        x1[2 * u] = R.r[0] + a[4 + u] + v[4 + u];
        x1[2 * u + 1] = R.r[4] + b[4 + u] + v[4 + u];
    }
    lse_add8(m, s, x0);
    lse_add8(m, s, x1);
}

template <int Q>
__device__ __forceinline__ SumPartial outside_sum_t(const Band& t, int i, int d, int side, bool valid, int lane,
                                                    int G, const Rules& R)
{
    const int L = t.L, Wb = t.Wb, RS = t.RS;
    const int j = i + d;
    SumPartial c{-INFINITY, 0.f};
    if (valid) {
        int n;
        const float *o1, *o2, *in;
        float extra = -INFINITY;
        if (side == 0) {
            const bool has = j + 1 <= L - 1;
            n = has ? min(i + Wb, L - 1) - j : 0;
            o1 = t.OSrow + (size_t)i * RS + d + 1;
            o2 = t.OFrow + (size_t)i * RS + d + 1;
            in = t.Srow + (size_t)min(j + 1, L - 1) * RS;
            if (lane == 0 && has && L - 1 > i + Wb) extra = R.r[0] + __ldcg(t.Osuf + i) + t.Ssuf[j + 1];
        } else {
            const bool has = i >= 1;
            n = has ? i - max(0, j - Wb) : 0;
            o1 = t.OScol + (size_t)j * RS + d + 1;
            o2 = t.OFcol + (size_t)j * RS + d + 1;
            in = t.Lcol + (size_t)max(i - 1, 0) * RS;
            // the last column's parents beyond the band, summed before the launch
            if (lane == 0 && has && j == L - 1) extra = t.OSlast[i];
        }
        int q = Q + lane;
        if (G == 32) {  // warp-uniform: one sum per warp, constant strides
            for (; q + 7 * 32 < n; q += 8 * 32) outside_full8<32>(c.m, c.s, o1, o2, in, q, R);
            const int rem = (n - q + 31) / 32;  // points left (0..7)
            if (rem > 0) {
                const float* p1 = o1 + q;
                const float* p2 = o2 + q;
                const float* p3 = in + q;
                float x0[8], x1[8];
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const bool on = u < rem;
                    const float v = ldg_if(p3 + u * 32, on, 0.f);
                    const float a = ldcg_if(p1 + u * 32, on, -INFINITY);
                    const float b = ldcg_if(p2 + u * 32, on, -INFINITY);
                    float* x = (u < 4) ? x0 : x1;
                    x[2 * (u & 3)] = R.r[0] + a + v;
                    x[2 * (u & 3) + 1] = R.r[4] + b + v;
                }
                lse_add8(c.m, c.s, x0);
                lse_add8(c.m, c.s, x1);
            }
            q = n;
        }
        for (; q < n; q += 8 * G) {
            float x0[8], x1[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int qq = q + u * G;
                const bool on = qq < n;
                const float v = on ? in[qq] : 0.f;
                const float a = on ? __ldcg(o1 + qq) : -INFINITY;
                const float b = on ? __ldcg(o2 + qq) : -INFINITY;
                float* x = (u < 4) ? x0 : x1;
                x[2 * (u & 3)] = R.r[0] + a + v;
                x[2 * (u & 3) + 1] = R.r[4] + b + v;
            }
            lse_add8(c.m, c.s, x0);
            lse_add8(c.m, c.s, x1);
        }
        lse_add(c.m, c.s, extra);
    }
    // the shuffles only where some lane group of the warp has a cell (the
    // callers pass every lane of the warp; an empty slot's result is unused)
    if (__any_sync(0xffffffffu, valid)) group_reduce_rt(c.m, c.s, G);
    return c;
}

template <int Q>
__device__ __forceinline__ void outside_finish_t(const Band& t, int i, int d, SumPartial cl, SumPartial cs,
                                                 const Rules& R)
{
    const int L = t.L, Wb = t.Wb, RS = t.RS;
    const int j = i + d;
    const bool hasL = j + 1 <= L - 1, hasS = i >= 1;
    const int nL = hasL ? min(i + Wb, L - 1) - j : 0;
    const int nS = hasS ? i - max(0, j - Wb) : 0;
    // every operand first (one round trip), then the sums in ascending q
    float sib[Q], osl[Q], ofl[Q], lft[Q], oss[Q], ofs[Q];
    const size_t orow = (size_t)i * RS + d + 1, ocol = (size_t)j * RS + d + 1;
    const size_t srow = (size_t)min(j + 1, L - 1) * RS, lc = (size_t)max(i - 1, 0) * RS;
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const bool onL = q < nL, onS = q < nS;
        sib[q] = onL ? t.Srow[srow + q] : 0.f;
        osl[q] = onL ? __ldcg(t.OSrow + orow + q) : -INFINITY;
        ofl[q] = onL ? __ldcg(t.OFrow + orow + q) : -INFINITY;
        lft[q] = onS ? t.Lcol[lc + q] : 0.f;
        oss[q] = onS ? __ldcg(t.OScol + ocol + q) : -INFINITY;
        ofs[q] = onS ? __ldcg(t.OFcol + ocol + q) : -INFINITY;
    }
    const bool enc = hasS && j <= L - 2 && d + 2 <= Wb;
    const size_t pr = (size_t)max(i - 1, 0) * RS + d + 2;
    const float pp = enc ? t.pb[pr] : -INFINITY;
    const float fa = enc ? __ldcg(t.OSrow + pr) : -INFINITY;
    const float fb = enc ? __ldcg(t.OFrow + pr) : -INFINITY;
    const float fc = enc ? __ldcg(t.OLrow + pr) : -INFINITY;
    float oF = -INFINITY;
    if (pp != -INFINITY) {
        float m = -INFINITY, s = 0.f;
        lse_add4(m, s, R.r[2] + pp + fa, R.r[3] + pp + fb, R.r[6] + pp + fc, -INFINITY);
        oF = lse_val(m, s);
    }
    // the near parents of each sum as one block (one max, independent exponentials)
    float xl[8], xs[8];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const bool on = q < Q;
        const int qq = on ? q : 0;
        xl[2 * q] = on ? R.r[0] + osl[qq] + sib[qq] : -INFINITY;
        xl[2 * q + 1] = on ? R.r[4] + ofl[qq] + sib[qq] : -INFINITY;
        xs[2 * q] = on ? R.r[0] + oss[qq] + lft[qq] : -INFINITY;
        xs[2 * q + 1] = on ? R.r[4] + ofs[qq] + lft[qq] : -INFINITY;
    }
    lse_add8(cl.m, cl.s, xl);
    lse_add8(cs.m, cs.s, xs);
    const float oL = lse_val(cl.m, cl.s);
    float oS = lse_val(cs.m, cs.s);
    if (i == 0 && j == L - 1) oS = 0.f;
    t.OSrow[(size_t)i * RS + d] = oS;
    t.OScol[(size_t)j * RS + d] = oS;
    t.OFrow[(size_t)i * RS + d] = oF;
    t.OFcol[(size_t)j * RS + d] = oF;
    t.OLrow[(size_t)i * RS + d] = oL;
    if (j == L - 1) t.Osuf[i] = oS;
}

// The sums of one diagonal's rows [start, start + nrows) before the wait:
// task tau = 2r + side (row r, one of its two sums) goes to lane group
// (first + tau) mod (groups per CTA), two tasks per group, each group's
// result to slot[tau].  The second diagonal of a pair starts on the groups
// the first one leaves idle.
template <int Q>
__device__ __forceinline__ void out_sums_partial(const Band& t, int d, int start, int nrows, int first,
                                                 float2* slot, const Rules& R)
{
    const int G = group_width(2 * (t.Wb - d) + 2), gpb = blockDim.x / G;
    const int lane = threadIdx.x & (G - 1), g = (threadIdx.x / G + gpb - first % gpb) % gpb;
    const int ntask = 2 * min(nrows, gpb);
#pragma unroll
    for (int it = 0; it < 2; it++) {
        const int tau = g + it * gpb;
        const bool valid = tau < ntask;
        const SumPartial c = outside_sum_t<Q>(t, start + (tau >> 1), d, tau & 1, valid, lane, G, R);
        if (valid && lane == 0) slot[tau] = make_float2(c.m, c.s);
    }
}

// After the wait: one thread per row finishes the rows whose sums are in the
// slots; rows beyond the groups of the CTA are computed whole, both sums by
// one group and the cell finished by its lane 0.
template <int Q>
__device__ __forceinline__ void out_sums_finish(const Band& t, int d, int start, int nrows, const float2* slot,
                                                const Rules& R)
{
    const int G = group_width(2 * (t.Wb - d) + 2), gpb = blockDim.x / G;
    const int np = min(nrows, gpb);
    for (int r = threadIdx.x; r < np; r += blockDim.x) {
        const float2 a = slot[2 * r], b = slot[2 * r + 1];
        outside_finish_t<Q>(t, start + r, d, SumPartial{a.x, a.y}, SumPartial{b.x, b.y}, R);
    }
    const int lane = threadIdx.x & (G - 1), g = threadIdx.x / G;
    for (int base = np; base < nrows; base += gpb) {
        const int r = base + g;
        const bool valid = r < nrows;
        const SumPartial cl = outside_sum_t<Q>(t, start + r, d, 0, valid, lane, G, R);
        const SumPartial cs = outside_sum_t<Q>(t, start + r, d, 1, valid, lane, G, R);
        if (valid && lane == 0) outside_finish_t<Q>(t, start + r, d, cl, cs, R);
    }
}

// Suffix-column terms of the outside S sums of the last column's band cells:
// cell (i, L-1) has the parents (ip, L-1) beyond the band, ip = max(0, i-1-Wb)
// .. L-2-Wb, each adding r1 + OS(ip, L-1) + L(ip, i-1).  They read only the
// suffix column and the inside tables, so one launch before the wavefront
// sums them for every row, a warp per row: inside the wavefront the cell of
// diagonal d has d+1 of them, summed by the single lane group of a long
// diagonal while every other CTA waited at the next barrier.
__global__ void outside_lastcol_kernel(Band t, Rules R)
{
    const int L = t.L, Wb = t.Wb, RS = t.RS;
    const int lane = threadIdx.x & 31;
    const int i = max(1, L - 1 - Wb) + (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (i > L - 1) return;  // warp-uniform
    const int a = max(0, i - 1 - Wb), bnd = min(i - 1, L - 2 - Wb);
    const float* lcol = t.Lcol + (size_t)(i - 1) * RS;
    float m = -INFINITY, s = 0.f;
    for (int ip = a + lane; ip <= bnd; ip += 256) {
        float x[8];
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int iq = ip + 32 * q;
            x[q] = (iq <= bnd) ? R.r[0] + t.Osuf[iq] + lcol[i - 1 - iq] : -INFINITY;
        }
        lse_add8(m, s, x);
    }
    group_reduce<32>(m, s);
    if (lane == 0) t.OSlast[i] = lse_val(m, s);
}

// All band diagonals of the outside pass, descending spans, two per grid
// barrier.  CTA b owns rows [b*R, (b+1)*R) of every diagonal (R = ceil(L /
// CTAs)).  For the pair (e, e-1) it computes diagonal e for its rows plus row
// b*R - 1 (which the previous CTA also computes, to the same bits) and then,
// after a CTA barrier, diagonal e-1, whose cells read diagonal e only at rows
// i and i-1.  The sums of both diagonals read spans >= e+3 and are computed
// between the CTA's arrival at the barrier that completes e+1 and its wait
// there; the finishing parts follow the wait.
__global__ void __launch_bounds__(kWaveMaxThreads) outside_wave_kernel(Band t, Rules R)
{
    __shared__ float2 slotA[2 * kWaveMaxThreads], slotB[2 * kWaveMaxThreads];
    unsigned int gen = 0;
    const int L = t.L, Wb = t.Wb;
    const int rows = (L + gridDim.x - 1) / gridDim.x;
    const int r0 = blockIdx.x * rows;
    grid_arrive(t.sync);  // the suffix column was written by the previous launch
    for (int eA = Wb; eA >= 0; eA -= 2) {
        const int eB = eA - 1;
        const int sA = max(r0 - 1, 0), nA = min(r0 + rows, L - eA) - sA;
        const int nB = (eB >= 0) ? min(r0 + rows, L - eB) - r0 : 0;
        out_sums_partial<2>(t, eA, sA, nA, 0, slotA, R);
        if (eB >= 0) out_sums_partial<3>(t, eB, r0, nB, 2 * max(nA, 0), slotB, R);
        if (!grid_wait(t.sync, gen)) return;
        out_sums_finish<2>(t, eA, sA, nA, slotA, R);
        if (eB >= 0) {
            __syncthreads();  // diagonal e of rows r0-1 .. before diagonal e-1 reads it
            out_sums_finish<3>(t, eB, r0, nB, slotB, R);
        }
        grid_arrive(t.sync);  // begins with a CTA barrier: the slots are free again
    }
}

// CTA size of a persistent wavefront launch.  The split sums are bound by
// the latency of their L2 loads: long bands need many warps per SM to keep
// enough loads in flight, short ones pay more for the larger CTA barrier
// than they gain (GB300: 256 threads best at L x W = 0.5e6, 1024 at 7e6).
int wave_threads(const messi_ctx* ctx, double cells)
{
    const int t = ctx->wave_threads;
    if (t == 256 || t == 512 || t == 1024) return t;
    return cells < 1.5e6 ? 256 : (cells < 4e6 ? 512 : kWaveMaxThreads);
}

int wave_grid(messi_ctx* ctx, const void* kernel, int L, int threads)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    int sms = ctx->num_sms;
    if (sms <= 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        ctx->num_sms = sms;
    }
    // one CTA per SM at most keeps the barrier cheap; a context may cap it lower
    const int useful = (int)std::min<long long>((long long)L * 32 / threads + 1, (long long)per_sm * sms);
    int grid = std::max(1, std::min(useful, sms));
    if (ctx->wave_ctas > 0) grid = std::min(grid, ctx->wave_ctas);
    return grid;
}

// CTAs for which a CTA's ceil(L / CTAs) rows plus one fit one per warp in
// `warps` warps.
static int ctas_for_rows(int L, int warps) { return (warps > 1) ? (L + warps - 2) / (warps - 1) : L; }

// Launch a persistent wavefront kernel (cooperative: every CTA resident).
// share > 0 (paired kernels): the CTA owns ceil(L / grid) rows of every
// diagonal plus one, and a row wants `share` warps per diagonal pair (the
// inside pass: one per diagonal, 2; the outside pass: one per parent sum of
// each diagonal, 4).  The CTA grows (up to 1,024 threads, unless its size is
// set) to the smallest size at which warps / share of its warps hold those
// rows one per warp with at most one CTA per SM (inside: the pipelined halves
// kernel then runs; GB300, band of 500: 23-29% faster for 1,200-2,000
// columns than 256- or 512-thread CTAs of the plain kernel); the grid then
// grows (up to one CTA per SM) until the rows fit, or else fit one per warp
// of the whole CTA.
int launch_wave(messi_ctx* ctx, const void* kernel, void** args, unsigned int* sync, int L, double band_cells,
                const char* what, int share, const void* halves_kernel)
{
    int threads = wave_threads(ctx, band_cells);
    cudaError_t e = cudaMemsetAsync(sync, 0, kSyncWords * sizeof(unsigned int), ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "barrier reset");
    int grid = wave_grid(ctx, kernel, L, threads);  // also sets ctx->num_sms
    if (share > 0 && ctx->wave_ctas <= 0) {
        for (int t2 = threads; t2 <= (ctx->wave_threads ? threads : kWaveMaxThreads); t2 *= 2)
            if (ctas_for_rows(L, t2 / 32 / share) <= ctx->num_sms) {
                if (t2 != threads) {
                    threads = t2;
                    grid = wave_grid(ctx, kernel, L, threads);
                }
                break;
            }
        const int warps = threads / 32;
        const int half = ctas_for_rows(L, warps / share);
        const int want = (half <= ctx->num_sms) ? half : ctas_for_rows(L, warps);
        grid = std::max(grid, std::min(want, ctx->num_sms));
        // the halves shape (rows + 1 <= warps / 2 for ceil(L / grid) rows)
        const int rows = (L + grid - 1) / grid;
        if (halves_kernel && rows + 1 <= warps / 2) kernel = halves_kernel;
    }
    e = cudaLaunchCooperativeKernel(kernel, dim3(grid), dim3(threads), args, 0, ctx->stream);
    ctx->launches++;
    if (e != cudaSuccess) return cuda_fail(ctx, e, what);
    return MESSI_OK;
}

// Self-test of the bounded grid barrier: CTA 1 never arrives, so CTA 0's wait
// gives up after `limit` polls, raises the error flag (sync[2]) and returns.
// Nothing faults and nothing waits unboundedly; the context stays usable.
__global__ void barrier_selftest_kernel(unsigned int* sync, unsigned int limit)
{
    if (blockIdx.x != 0) return;
    unsigned int gen = 0;
    grid_sync(sync, gen, limit);
}

int launch_barrier_selftest(messi_ctx* ctx, unsigned int* d_sync)
{
    cudaError_t e = cudaMemsetAsync(d_sync, 0, kSyncWords * sizeof(unsigned int), ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "barrier self-test reset");
    barrier_selftest_kernel<<<2, 32, 0, ctx->stream>>>(d_sync, 1u << 12);
    LAUNCH_CHECK(ctx, "barrier_selftest_kernel");
    return MESSI_OK;
}

int queue_status_readback(messi_ctx* ctx, const Band& t)
{
    if (!ctx->status_host) return MESSI_OK;
    cudaError_t e = cudaMemcpyAsync(ctx->status_host, t.sync + 2, sizeof(unsigned int), cudaMemcpyDeviceToHost,
                                    ctx->stream);
    return (e == cudaSuccess) ? MESSI_OK : cuda_fail(ctx, e, "status readback");
}

int run_inside(messi_ctx* ctx, const Band& t, double B)
{
    Rules R = make_rules(B);
    Band tt = t;
    double Bv = B;
    void* args[] = {&tt, &R, &Bv};
    prof_begin(ctx, 1, (double)t.L * (t.Wb + 1) - 0.5 * t.Wb * (t.Wb + 1.0));
    int rc = launch_wave(ctx, (const void*)inside_wave_kernel, args, t.sync, t.L, (double)t.L * (t.Wb + 1),
                         "inside_wave_kernel", 2, (const void*)inside_wave_pipe_kernel);
    if (rc) return rc;
    prof_end(ctx);
    if (t.L - 1 > t.Wb) {
        prof_begin(ctx, 2, (double)(t.L - 1 - t.Wb));
        const int win = suffix_launch_window(t.Wb);
        cudaError_t e = suffix_smem_attr(win);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "inside_suffix_kernel attributes");
        inside_suffix_kernel<<<1, kSuffixThreads, (size_t)2 * win * sizeof(float), ctx->stream>>>(t, R, win);
        LAUNCH_CHECK(ctx, "inside_suffix_kernel");
        prof_end(ctx);
    }
    return launch_finish_Z(ctx, t);
}

// ---------------------------------------------------------------------------
// batched inside
// ---------------------------------------------------------------------------
int bandbatch_alloc(const std::vector<int>& L, const std::vector<int>& Wb, BandBatch* bb, std::string* err)
{
    const int n = (int)L.size();
    bb->n = n;
    bb->order.resize(n);
    for (int a = 0; a < n; a++) bb->order[a] = a;
    std::stable_sort(bb->order.begin(), bb->order.end(), [&](int x, int y) { return Wb[x] > Wb[y]; });
    bb->slot.assign(n, 0);
    for (int k = 0; k < n; k++) bb->slot[bb->order[k]] = k;
    // one allocation: per band 6 tables, Ssuf/Osuf, b/cb/u/Zd; then the batch arrays
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    std::vector<size_t> off_tab(n), off_suf(n), off_dbl(n);
    size_t bytes = 0;
    for (int k = 0; k < n; k++) {
        const int a = bb->order[k];
        const size_t RS = ((size_t)Wb[a] + 1 + 31) / 32 * 32;
        off_tab[k] = bytes;
        bytes = al(bytes + 6 * (size_t)L[a] * RS * sizeof(float));
        off_suf[k] = bytes;
        bytes = al(bytes + (size_t)(L[a] + 1) * 2 * sizeof(float));
        off_dbl[k] = bytes;
        bytes = al(bytes + (size_t)(3 * L[a] + 8) * sizeof(double));
    }
    const size_t off_bands = bytes;
    bytes = al(bytes + (size_t)n * sizeof(Band));
    const size_t off_cum = bytes;
    bytes = al(bytes + (size_t)(n + 1) * sizeof(long long));
    const size_t off_wbs = bytes;
    bytes = al(bytes + (size_t)n * sizeof(int));
    const size_t off_sync = bytes;
    bytes = al(bytes + kSyncWords * sizeof(unsigned int));
    const size_t off_Z = bytes;
    bytes = al(bytes + (size_t)n * sizeof(double));
    cudaError_t e = cudaMalloc(&bb->mem, bytes);
    if (e != cudaSuccess) {
        bb->mem = nullptr;
        *err = std::string("batch band tables: ") + cudaGetErrorString(e);
        return MESSI_ENOMEM;
    }
    bb->bytes = bytes;
    char* base = (char*)bb->mem;
    bb->host.assign(n, Band{});
    std::vector<long long> cum(n + 1, 0);
    std::vector<int> wbs(n);
    bb->d_sync = (unsigned int*)(base + off_sync);
    for (int k = 0; k < n; k++) {
        const int a = bb->order[k];
        Band& t = bb->host[k];
        t.L = L[a];
        t.Wb = Wb[a];
        t.RS = ((Wb[a] + 1 + 31) / 32) * 32;
        const size_t tab = (size_t)t.L * t.RS;
        float* f = (float*)(base + off_tab[k]);
        t.Lrow = f;
        t.Lcol = f + tab;
        t.Srow = f + 2 * tab;
        t.Scol = f + 3 * tab;
        t.Frow = f + 4 * tab;
        t.pb = f + 5 * tab;
        t.Ssuf = (float*)(base + off_suf[k]);
        t.Osuf = t.Ssuf + (t.L + 1);
        t.b = (double*)(base + off_dbl[k]);
        t.cb = t.b + t.L;
        t.u = t.cb + (t.L + 1);
        t.Zd = t.u + t.L;
        t.maxspan = nullptr;
        t.sync = bb->d_sync;
        t.OSrow = t.OScol = t.OFrow = t.OFcol = t.OLrow = t.PP = t.SL = t.nrm = t.OSlast = nullptr;
        cum[k + 1] = cum[k] + t.L;
        wbs[k] = t.Wb;
    }
    bb->total_cols = cum[n];
    bb->d_bands = (Band*)(base + off_bands);
    bb->d_cumL = (long long*)(base + off_cum);
    bb->d_wbs = (int*)(base + off_wbs);
    bb->d_Z = (double*)(base + off_Z);
    e = cudaMemcpy(bb->d_bands, bb->host.data(), (size_t)n * sizeof(Band), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(bb->d_cumL, cum.data(), (size_t)(n + 1) * sizeof(long long), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(bb->d_wbs, wbs.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        *err = std::string("batch band descriptors: ") + cudaGetErrorString(e);
        return MESSI_ECUDA;
    }
    return MESSI_OK;
}

void bandbatch_free(BandBatch* bb)
{
    if (bb->mem) cudaFree(bb->mem);
    bb->mem = nullptr;
    bb->host.clear();
}

int launch_baseline_batch(messi_ctx* ctx, const BandBatch& bb, double B)
{
    if (bb.n == 0) return MESSI_OK;
    baseline_batch_kernel<<<bb.n, 1024, 0, ctx->stream>>>(bb.d_bands, B, baseline_c());
    LAUNCH_CHECK(ctx, "baseline_batch_kernel");
    return MESSI_OK;
}

int run_inside_batch(messi_ctx* ctx, const BandBatch& bb, double B)
{
    if (bb.n == 0) return MESSI_OK;
    Rules R = make_rules(B);
    const Band* bands = bb.d_bands;
    const long long* cum = bb.d_cumL;
    const int* wbs = bb.d_wbs;
    int n = bb.n;
    double Bv = B;
    unsigned int* sync = bb.d_sync;
    void* args[] = {&bands, &cum, &wbs, &n, &R, &Bv, &sync};
    double cells = 0.0, band = 0.0;
    for (const Band& t : bb.host) {
        cells += (double)t.L * (t.Wb + 1) - 0.5 * t.Wb * (t.Wb + 1.0);
        band += (double)t.L * (t.Wb + 1);
    }
    const int threads = wave_threads(ctx, band);
    const int grid = wave_grid(ctx, (const void*)inside_wave_batch_kernel,
                               (int)std::min<long long>(bb.total_cols, 1 << 30), threads);
    prof_begin(ctx, 1, cells);
    cudaError_t e = cudaMemsetAsync(sync, 0, kSyncWords * sizeof(unsigned int), ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "barrier reset");
    e = cudaLaunchCooperativeKernel((const void*)inside_wave_batch_kernel, dim3(grid), dim3(threads), args, 0,
                                    ctx->stream);
    ctx->launches++;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "inside_wave_batch_kernel");
    prof_end(ctx);
    prof_begin(ctx, 2, 0.0);
    const int win = suffix_batch_window(bb);
    e = suffix_smem_attr(win);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "inside_suffix_batch_kernel attributes");
    inside_suffix_batch_kernel<<<n, kSuffixThreads, (size_t)2 * win * sizeof(float), ctx->stream>>>(bands, R, win);
    LAUNCH_CHECK(ctx, "inside_suffix_batch_kernel");
    prof_end(ctx);
    finish_Z_batch_kernel<<<(n + 127) / 128, 128, 0, ctx->stream>>>(bands, n, sync, bb.d_Z);
    LAUNCH_CHECK(ctx, "finish_Z_batch_kernel");
    if (!ctx->status_host) return MESSI_OK;
    e = cudaMemcpyAsync(ctx->status_host, sync + 2, sizeof(unsigned int), cudaMemcpyDeviceToHost, ctx->stream);
    return (e == cudaSuccess) ? MESSI_OK : cuda_fail(ctx, e, "status readback");
}

// ---------------------------------------------------------------------------
// outside
// ---------------------------------------------------------------------------
// Osuf[i] for spans beyond the band on the last column, ascending i:
// Osuf[0] = 0;  Osuf[i] = r1 + LSE_{k=0..Wb, i-k-1>=0} (Osuf[i-k-1] + Lcol[i-1][k]).
// Osuf[i] (outside of S(i, L-1) beyond the band, i < T = L-1-Wb), ascending
// i: Osuf[0] = 0, Osuf[i] = r1 + LSE_{k=0..min(Wb, i-1)} (Osuf[i-k-1] +
// Lcol[i-1][k]).  The mirror of the inside suffix: blocks of 32 cells from
// the bottom, every finished block pushed into the next Wb+1 cells'
// shared-memory accumulators (warp 0 into the next block and its triangle,
// the other warps into the farther cells, one barrier per block).
__device__ void outside_suffix_body(const Band& t, const Rules& R, float* am, float* as, int win)
{
    const int Wb = t.Wb, RS = t.RS;
    const int T = t.L - 1 - Wb;
    if (T <= 0) return;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // tri[q][k] = Lcol[i0 + q - 1][k] for the block's cells i0 + q, double-buffered
    __shared__ float tri2[2][32][33];
    __shared__ float etri2[2][32][33];  // exp(tri + r1), staged with tri
    __shared__ float vals2[2][32];
    // xs[u][q]: the L value joining next-block cell hi+1+q to this block's
    // cell i0+u (warp 0's push after the triangle), staged a block ahead by warp 1
    __shared__ float xs2[2][32][33];
    int parity = 0, tb = 0;
    for (int c = threadIdx.x; c < win; c += blockDim.x) {
        am[c] = -INFINITY;
        as[c] = 0.f;
    }
    int i0 = 0, hi = min(T - 1, 31);
    // the first two blocks' pushes (Lrow rows i0 .. hi+32) and the second
    // block's in-block terms (first line of Lcol rows hi .. hi+31)
    prefetch_rows_l2(t.Lrow, RS, t.L, i0, hi + 32, RS / 32, threadIdx.x, blockDim.x);
    prefetch_rows_l2(t.Lcol, RS, t.L, hi, hi + 31, 1, threadIdx.x, blockDim.x);
    if (w == 1) {
        for (int q = 0; q < 32; q++) {
            const int c = i0 + q;
            const float v = (c <= hi && c >= 1 && lane <= Wb) ? __ldg(t.Lcol + (size_t)(c - 1) * RS + lane) : -INFINITY;
            tri2[0][q][lane] = v;
            etri2[0][q][lane] = __expf(v + R.r[0]);
        }
        const int nb0 = hi - i0 + 1, nhi0 = min(T - 1, hi + 32), c = hi + 1 + lane;
        for (int u = 0; u < 32; u++) {
            const int k = c - 1 - i0 - u;
            xs2[0][u][lane] = (hi < T - 1 && c <= nhi0 && u < nb0 && k >= 0 && k <= Wb)
                                  ? __ldg(t.Lrow + (size_t)(i0 + u) * RS + k)
                                  : -INFINITY;
        }
    }
    __syncthreads();
    float cm = -INFINITY, cs = 0.f;
    for (;;) {
        const int nb = hi - i0 + 1;
        const int nhi = min(T - 1, hi + 32);
        float* vals = vals2[parity];
        parity ^= 1;
        float x[32];  // warp 0: L values joining its next-block cell to this block's cells
        if (w == 0) {
            // column-oriented substitution (lane q owns cell i0 + q); Osuf[0]
            // = 0 is (m, s) = (-r1, 1), so every value is r1 + m + log s
            float m = (lane < nb) ? cm : -INFINITY, s = (lane < nb) ? cs : 0.f;
            if (i0 + lane == 0) {
                m = -R.r[0];
                s = 1.f;
            }
            suffix_triangle(m, s, tri2[tb], etri2[tb], nb, lane < nb && i0 + lane >= 1, Wb, R.r[0], lane);
            // the block's values, stored by all lanes at once
            if (lane < nb) {
                const float sv = (i0 + lane == 0) ? 0.f : R.r[0] + lse_val(m, s);
                t.Osuf[i0 + lane] = sv;
                vals[lane] = sv;
            }
            // the push operands, before the barrier: warp 1 refills this
            // buffer in the next block
#pragma unroll
            for (int u = 0; u < 32; u++) x[u] = xs2[tb][u][lane];
        } else if (w == 1 && hi < T - 1) {
            // the next block's in-block terms and push operands: all 64 loads
            // first, then the stores (one memory round trip)
            const int i0n = hi + 1, nbn = nhi - hi, nhin = min(T - 1, nhi + 32), c = nhi + 1 + lane;
            float v[32], y[32];
#pragma unroll
            for (int q = 0; q < 32; q++) {
                const int cq = hi + 1 + q;
                const bool onv = cq <= nhi && lane <= Wb;
                v[q] = ldg_if(t.Lcol + (onv ? (size_t)(cq - 1) * RS + lane : 0), onv, -INFINITY);
                const int k = c - 1 - i0n - q;
                const bool ony = nhi < T - 1 && c <= nhin && q < nbn && k >= 0 && k <= Wb;
                y[q] = ldg_if(t.Lrow + (ony ? (size_t)(i0n + q) * RS + k : 0), ony, -INFINITY);
            }
#pragma unroll
            for (int q = 0; q < 32; q++) {
                tri2[tb ^ 1][q][lane] = v[q];
                etri2[tb ^ 1][q][lane] = __expf(v[q] + R.r[0]);
                xs2[tb ^ 1][q][lane] = y[q];
            }
        } else if (w >= 2) {
            // the block after the next one: its pushes read Lrow rows
            // hi+33 .. hi+64, its in-block terms Lcol rows hi+32 .. hi+63
            prefetch_rows_l2(t.Lrow, RS, t.L, hi + 33, hi + 64, RS / 32, threadIdx.x - 64, blockDim.x - 64);
            prefetch_rows_l2(t.Lcol, RS, t.L, hi + 32, hi + 63, 1, threadIdx.x - 64, blockDim.x - 64);
        }
        __syncthreads();
        if (hi == T - 1) break;
        // push the block [i0, hi] (value u = cell i0 + u) into the cells
        // hi+1 .. hi+1+Wb: L(i0 + u, c - 1) = Lrow[i0 + u][c - 1 - i0 - u],
        // contiguous in c; a cell's first push (from the block holding its
        // smallest referenced cell) starts it afresh
        if (w == 0) {
            const int c = hi + 1 + lane;
            cm = -INFINITY;
            cs = 0.f;
            if (c <= nhi) {
                const bool fresh = i0 <= max(0, c - 1 - Wb);
                if (!fresh) {
                    cm = am[c % win];
                    cs = as[c % win];
                }
#pragma unroll
                for (int u = 0; u < 32; u += 8) {
                    const float y[8] = {x[u] + vals[u], x[u + 1] + vals[u + 1], x[u + 2] + vals[u + 2],
                                        x[u + 3] + vals[u + 3], x[u + 4] + vals[u + 4], x[u + 5] + vals[u + 5],
                                        x[u + 6] + vals[u + 6], x[u + 7] + vals[u + 7]};
                    lse_add8(cm, cs, y);
                }
            }
        } else if (w >= 2) {
            for (int c = nhi + 1 + (threadIdx.x - 64); c <= min(T - 1, hi + 1 + Wb); c += (int)blockDim.x - 64) {
                const bool fresh = i0 <= max(0, c - 1 - Wb);
                float m = fresh ? -INFINITY : am[c % win], s = fresh ? 0.f : as[c % win];
                suffix_push_terms(m, s, t.Lrow, RS, i0, 1, c - 1 - i0, vals, nb, Wb);
                am[c % win] = m;
                as[c % win] = s;
            }
        }
        tb ^= 1;
        i0 = hi + 1;
        hi = nhi;
    }
}

// Blocks of 32 cells pulled from global memory (bands wider than the window).
__device__ void outside_suffix_body_pull(const Band& t, const Rules& R)
{
    const int T = t.L - 1 - t.Wb;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __shared__ float known[32];
    __shared__ float tri[32][33];  // Lcol[i0 + l - 1][k], k < 32: the in-block terms
    for (int i0 = 0; i0 < T; i0 += 32) {
        const int hi = min(T - 1, i0 + 31);
        const int i = i0 + w;
        tri[w][lane] = (i <= hi && i >= 1 && lane <= t.Wb) ? t.Lcol[(size_t)(i - 1) * t.RS + lane] : -INFINITY;
        if (i <= hi) {
            float m = -INFINITY, s = 0.f;
            if (i >= 1) {
                const float* lcol = t.Lcol + (size_t)(i - 1) * t.RS;
                const int kmax = min(t.Wb, i - 1);
                int k = (i - i0) + lane;
                for (; k + 96 <= kmax; k += 128)
                    lse_add4(m, s, t.Osuf[i - k - 1] + lcol[k], t.Osuf[i - k - 33] + lcol[k + 32],
                             t.Osuf[i - k - 65] + lcol[k + 64], t.Osuf[i - k - 97] + lcol[k + 96]);
                for (; k <= kmax; k += 32) lse_add(m, s, t.Osuf[i - k - 1] + lcol[k]);
            }
            group_reduce<32>(m, s);
            if (lane == 0) known[w] = lse_val(m, s);
        }
        __syncthreads();
        if (w == 0) {
            // column-oriented substitution (lane q owns cell i0 + q); Osuf[0] = 0
            const int nb = hi - i0 + 1;
            float am = (lane < nb) ? known[lane] : -INFINITY, as = (am == -INFINITY) ? 0.f : 1.f;
            for (int l = 0; l < nb; l++) {
                const int ic = i0 + l;
                const float fin = (ic == 0) ? 0.f : R.r[0] + lse_val(am, as);
                const float sv = __shfl_sync(0xffffffffu, fin, l);
                if (lane == 0) t.Osuf[ic] = sv;
                const int k = lane - l - 1;
                if (lane > l && lane < nb && k <= t.Wb && i0 + lane >= 1) lse_add(am, as, tri[lane][k] + sv);
            }
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kSuffixThreads) outside_suffix_kernel(Band t, Rules R, int win)
{
    extern __shared__ float suffix_smem[];
    if (suffix_window(t.Wb) <= win) outside_suffix_body(t, R, suffix_smem, suffix_smem + win, win);
    else outside_suffix_body_pull(t, R);
}

int run_outside(messi_ctx* ctx, const Band& t, double B)
{
    Rules R = make_rules(B);
    if (t.L - 1 > t.Wb) {
        const int win = suffix_launch_window(t.Wb);
        cudaError_t e = cudaFuncSetAttribute(outside_suffix_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             2 * win * (int)sizeof(float));
        if (e != cudaSuccess) return cuda_fail(ctx, e, "outside_suffix_kernel attributes");
        outside_suffix_kernel<<<1, kSuffixThreads, (size_t)2 * win * sizeof(float), ctx->stream>>>(t, R, win);
        LAUNCH_CHECK(ctx, "outside_suffix_kernel");
    }
    {
        const int rows = t.L - std::max(1, t.L - 1 - t.Wb);  // last-column band cells with i >= 1
        if (rows > 0) {
            outside_lastcol_kernel<<<(rows + 7) / 8, 256, 0, ctx->stream>>>(t, R);
            LAUNCH_CHECK(ctx, "outside_lastcol_kernel");
        }
    }
    Band tt = t;
    void* args[] = {&tt, &R};
    prof_begin(ctx, 3, (double)t.L * (t.Wb + 1) - 0.5 * t.Wb * (t.Wb + 1.0));
    // paired: the two sums of each cell of a CTA's diagonal pair (2 x (2 x
    // rows + 1) sums) in one pass of its warps where the CTA can grow to hold them
    int rc = launch_wave(ctx, (const void*)outside_wave_kernel, args, t.sync, t.L, (double)t.L * (t.Wb + 1),
                         "outside_wave_kernel", 4);
    if (rc) return rc;
    prof_end(ctx);
    return queue_status_readback(ctx, t);
}

// ---------------------------------------------------------------------------
// posteriors (computebasepairprobs, row-normalised)
// ---------------------------------------------------------------------------
__global__ void post_cells_kernel(Band t, Rules R, double B)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)t.L * t.RS) return;
    const int j = (int)(idx / t.RS), d = (int)(idx % t.RS);
    const float Zbar = t.Ssuf[0];
    if (d == 0) {
        float m = -INFINITY, s = 0.f;
        lse_add(m, s, t.OSrow[(size_t)j * t.RS] + R.r[1]);
        lse_add(m, s, t.OLrow[(size_t)j * t.RS] + R.r[5]);
        const double uj = t.u[j];
        t.SL[j] = (uj == -INFINITY) ? -INFINITY : (float)((double)lse_val(m, s) + B * uj - t.b[j]) - Zbar;
        t.PP[idx] = -INFINITY;
        return;
    }
    float out = -INFINITY;
    if (d <= t.Wb && j + d < t.L) {
        const float pp = t.pb[idx];
        const float fin = (d >= 2) ? t.Frow[(size_t)(j + 1) * t.RS + (d - 2)] : -INFINITY;
        if (pp != -INFINITY && fin != -INFINITY) {
            float m = -INFINITY, s = 0.f;
            lse_add(m, s, t.OSrow[idx] + R.r[2]);
            lse_add(m, s, t.OFrow[idx] + R.r[3]);
            lse_add(m, s, t.OLrow[idx] + R.r[6]);
            out = lse_val(m, s) + fin + pp - Zbar;
        }
    }
    t.PP[idx] = out;
}

// one warp per row x: log normaliser over the unpaired term and every partner
__global__ void post_norm_kernel(Band t)
{
    const int x = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (x >= t.L) return;
    float m = -INFINITY, s = 0.f;
    if (lane == 0) lse_add(m, s, t.SL[x]);
    for (int d = 1 + lane; d <= t.Wb; d += 32) {
        if (x + d < t.L) lse_add(m, s, t.PP[(size_t)x * t.RS + d]);
        if (x - d >= 0) lse_add(m, s, t.PP[(size_t)(x - d) * t.RS + d]);
    }
    group_reduce<32>(m, s);
    if (lane == 0) t.nrm[x] = lse_val(m, s);
}

__global__ void post_dense_kernel(Band t, double* __restrict__ single, double* __restrict__ pair)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int L = t.L;
    if (idx >= (long long)L * L) return;
    const int x = (int)(idx % L), y = (int)(idx / L);
    const int k = (x > y) ? x - y : y - x;
    double v = 0.0;
    if (k >= 1 && k <= t.Wb) {
        const int i = (x < y) ? x : y;
        const float pp = t.PP[(size_t)i * t.RS + k];
        if (pp != -INFINITY) v = exp((double)pp - (double)t.nrm[x]);
    }
    pair[idx] = v;
    if (y == 0) single[x] = exp((double)t.SL[x] - (double)t.nrm[x]);
}

int run_posteriors(messi_ctx* ctx, const Band& t, double B, double* d_single, double* d_pair)
{
    const Rules R = make_rules(B);
    const long long n = (long long)t.L * t.RS;
    post_cells_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(t, R, B);
    LAUNCH_CHECK(ctx, "post_cells_kernel");
    post_norm_kernel<<<(unsigned)(((long long)t.L * 32 + 255) / 256), 256, 0, ctx->stream>>>(t);
    LAUNCH_CHECK(ctx, "post_norm_kernel");
    const long long nn = (long long)t.L * t.L;
    post_dense_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, ctx->stream>>>(t, d_single, d_pair);
    LAUNCH_CHECK(ctx, "post_dense_kernel");
    return MESSI_OK;
}

// ---------------------------------------------------------------------------
// dense (Julia-layout) tables <-> band tables
// ---------------------------------------------------------------------------
__global__ void dense_inside_kernel(Band t, double* __restrict__ out)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int L = t.L;
    if (idx >= (long long)L * L) return;
    const int i = (int)(idx % L), j = (int)(idx / L);
    double S = -INFINITY, F = -INFINITY, Lv = -INFINITY;
    if (j >= i) {
        const int d = j - i;
        const double base = t.cb[j + 1] - t.cb[i];
        if (d <= t.Wb) {
            const size_t o = (size_t)i * t.RS + d;
            S = (double)t.Srow[o] + base;
            F = (double)t.Frow[o] + base;
            Lv = (double)t.Lrow[o] + base;
        } else if (j == L - 1) {
            S = (double)t.Ssuf[i] + base;
        }
    }
    out[3 * idx] = S;
    out[3 * idx + 1] = F;
    out[3 * idx + 2] = Lv;
}

__global__ void dense_outside_kernel(Band t, double* __restrict__ out)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int L = t.L;
    if (idx >= (long long)L * L) return;
    const int i = (int)(idx % L), j = (int)(idx / L);
    double S = -INFINITY, F = -INFINITY, Lv = -INFINITY;
    if (j >= i) {
        const int d = j - i;
        const double base = t.cb[L] - (t.cb[j + 1] - t.cb[i]);
        if (d <= t.Wb) {
            const size_t o = (size_t)i * t.RS + d;
            S = (double)t.OSrow[o] + base;
            F = (double)t.OFrow[o] + base;
            Lv = (double)t.OLrow[o] + base;
        } else if (j == L - 1) {
            S = (double)t.Osuf[i] + base;
        }
    }
    out[3 * idx] = S;
    out[3 * idx + 1] = F;
    out[3 * idx + 2] = Lv;
}

int launch_dense_inside(messi_ctx* ctx, const Band& t, double* d_out)
{
    const long long n = (long long)t.L * t.L;
    dense_inside_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(t, d_out);
    LAUNCH_CHECK(ctx, "dense_inside_kernel");
    return MESSI_OK;
}

int launch_dense_outside(messi_ctx* ctx, const Band& t, double* d_out)
{
    const long long n = (long long)t.L * t.L;
    dense_outside_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(t, d_out);
    LAUNCH_CHECK(ctx, "dense_outside_kernel");
    return MESSI_OK;
}

__global__ void band_from_dense_inside_kernel(Band t, const double* __restrict__ in)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int L = t.L;
    if (idx >= (long long)L * L) return;
    const int i = (int)(idx % L), j = (int)(idx / L);
    if (j < i) return;
    const int d = j - i;
    const double base = t.cb[j + 1] - t.cb[i];
    const double S = in[3 * idx], F = in[3 * idx + 1], Lv = in[3 * idx + 2];
    if (d <= t.Wb) {
        const float s = (float)(S - base), f = (float)(F - base), l = (float)(Lv - base);
        t.Srow[(size_t)i * t.RS + d] = s;
        t.Scol[(size_t)j * t.RS + d] = s;
        t.Frow[(size_t)i * t.RS + d] = f;
        t.Lrow[(size_t)i * t.RS + d] = l;
        t.Lcol[(size_t)j * t.RS + d] = l;
    }
    if (j == L - 1) t.Ssuf[i] = (float)(S - base);
}

__global__ void band_from_dense_outside_kernel(Band t, const double* __restrict__ in)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int L = t.L;
    if (idx >= (long long)L * L) return;
    const int i = (int)(idx % L), j = (int)(idx / L);
    if (j < i) return;
    const int d = j - i;
    if (d > t.Wb) return;
    const double base = t.cb[L] - (t.cb[j + 1] - t.cb[i]);
    const size_t o = (size_t)i * t.RS + d;
    t.OSrow[o] = (float)(in[3 * idx] - base);
    t.OFrow[o] = (float)(in[3 * idx + 1] - base);
    t.OLrow[o] = (float)(in[3 * idx + 2] - base);
}

int launch_band_from_dense_inside(messi_ctx* ctx, const Band& t, const double* d_in)
{
    const long long n = (long long)t.L * t.L;
    band_from_dense_inside_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(t, d_in);
    LAUNCH_CHECK(ctx, "band_from_dense_inside_kernel");
    return MESSI_OK;
}

int launch_band_from_dense_outside(messi_ctx* ctx, const Band& t, const double* d_out)
{
    const long long n = (long long)t.L * t.L;
    band_from_dense_outside_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(t, d_out);
    LAUNCH_CHECK(ctx, "band_from_dense_outside_kernel");
    return MESSI_OK;
}

}  // namespace messi
