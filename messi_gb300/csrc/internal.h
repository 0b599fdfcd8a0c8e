// internal.h -- shared declarations of the messi_gb300 library (not part of the ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/messi_gb300.h"

namespace messi {

constexpr int kTile = 256;          // unique pairs per CTA in the pruning kernels
constexpr int kMaxLambda = 8;       // per-lambda conditionals kept in registers
constexpr int kMaxStack = 512;      // tree height limit of the unpaired kernel
constexpr int kEigStride = 16 + 256 + 16;  // eigenvalues, U (row-major), sqrt(pi)
constexpr int kEig4Stride = 4 + 16 + 4;

// Grow-only device buffer.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

// Per-internal-node descriptor of one pruning step (device resident).
struct NodeDev {
    const int* li;     // [n] row of the left child for each unique pair
    const int* ri;     // [n]
    const float* lf;   // left child rows (16 floats each)
    const int* le;     // left child exponents (nullptr for leaves: exponent 0)
    long long lcs;     // left child category stride in rows (0 for leaves)
    const float* rf;
    const int* re;
    long long rcs;
    float* of;         // output rows (unused at the root)
    int* oe;
    long long ocs;
    int n;             // unique pairs at this node
    int left;          // child node ids (index of their transition matrices)
    int right;
    int pad;
};

// Discretised model categories built on the host for one call.
struct Categories {
    int C = 0, nsite = 0, nlam = 0;
    std::vector<double> eig;      // [C][kEigStride]
    std::vector<float> pi16;      // [C][16]
    std::vector<double> logw;     // [C]
    std::vector<int> lam;         // [C] lambda category of each category
    std::vector<double> eig4;     // [nsite][kEig4Stride]
    std::vector<double> logw_site;  // [nsite]
    double pi4[4];
};

// Banded SCFG workspace (device pointers into context scratch).
struct Band {
    int L = 0, Wb = 0, RS = 0;    // length, band width, row stride (floats)
    float *Lrow, *Lcol, *Srow, *Scol, *Frow, *pb, *Ssuf;
    float *OSrow, *OScol, *OFrow, *OFcol, *OLrow, *Osuf;
    float *PP, *SL, *nrm;
    double *b, *cb, *u, *Zd;
    int* maxspan;
    unsigned int* sync;  // grid barrier of the wavefront kernels: count, generation, error flag, spare
};

// Rule log-probabilities times B (index 0..6 = r1..r7).
struct Rules {
    float r[7];
};

}  // namespace messi

namespace messi {
struct ProfRec {
    int kernel;
    cudaEvent_t a, b;
    double units;
};
constexpr int kProfKernels = 4;
}  // namespace messi

struct messi_ctx {
    int device = 0;
    // pair node-update kernel: 0 = tensor cores (3xTF32 mma.sync), 1 = FP32 FMA
    int prune_kernel = 0;
    // per-kernel event timing (messi_ctx_profile)
    bool profiling = false;
    std::vector<messi::ProfRec> prof_pending;
    std::vector<cudaEvent_t> prof_pool;
    double prof_ms[messi::kProfKernels] = {0, 0, 0, 0};
    int64_t prof_count[messi::kProfKernels] = {0, 0, 0, 0};
    double prof_units[messi::kProfKernels] = {0, 0, 0, 0};
    cudaStream_t stream = nullptr;
    int64_t launches = 0;
    std::string last_error;
    int num_sms = 0;
    // scratch buffers (grow-only)
    messi::DevBuf scratch[24];
    void* pinned = nullptr;
    size_t pinned_bytes = 0;
    unsigned int* status_host = nullptr;  // pinned word: wavefront barrier status of the last call
};

struct messi_dataset {
    messi_ctx* ctx = nullptr;
    int N = 0, L = 0, numnodes = 0, W = 0;
    std::vector<int> children, seqindex, parent, level, postorder;
    std::vector<uint8_t> masks;
    int H = 0;                         // number of levels (root level)
    int64_t band_pairs = 0, nroot = 0, executed = 0, naive = 0, arena_rows = 0;
    std::vector<int64_t> nunique;      // per node
    std::vector<int64_t> row_off;      // arena row offset per internal non-root node
    std::vector<std::vector<int>> level_nodes;  // internal nodes per level (index = level)
    std::vector<int> tile_off, tile_cnt;        // per level: offset/count into d_tiles
    int chunk = 0;                     // categories per pass (0 = arena not allocated yet)
    int arena_C = 0;                   // category count the arena was laid out for
    // device
    int* d_bandidx = nullptr;          // [L][W+1]
    int* d_lr = nullptr;               // concatenated li/ri arrays
    float* d_leaf = nullptr;           // concatenated leaf tables
    messi::NodeDev* d_nodes = nullptr; // [numnodes]
    int2* d_tiles = nullptr;
    uint8_t* d_masks = nullptr;        // [N][L]
    int* d_tree = nullptr;             // [numnodes][4]: child0, child1, seqindex, pad
    int* d_post = nullptr;             // [numnodes] post-order
    float* d_arena_f = nullptr;
    int* d_arena_e = nullptr;
    double* d_mix = nullptr;           // [nroot]
    double* d_mixlam = nullptr;        // [kMaxLambda][nroot]
    std::vector<messi::NodeDev> nodes_host;
    std::vector<int64_t> lr_off;       // per internal node offset into d_lr (li at off, ri at off+n)
    std::vector<int64_t> leaf_off;     // per leaf offset (rows) into d_leaf
};

namespace messi {

#define LAUNCH_CHECK(ctx, what)                                   \
    do {                                                          \
        (ctx)->launches++;                                        \
        cudaError_t e_ = cudaGetLastError();                      \
        if (e_ != cudaSuccess) return cuda_fail((ctx), e_, what); \
    } while (0)

// ---- error helpers (api.cu) ----
int fail(messi_ctx* ctx, int code, const std::string& msg);
int cuda_fail(messi_ctx* ctx, cudaError_t e, const char* what);
int ensure(messi_ctx* ctx, int slot, size_t bytes, void** p);
int ensure_pinned(messi_ctx* ctx, size_t bytes, void** p);
// Event pair around one launch of a timed kernel family (no-op unless profiling).
int prof_begin(messi_ctx* ctx, int kernel, double units);
void prof_end(messi_ctx* ctx);

// ---- host model (host_model.cpp) ----
int build_categories(const messi_model* m, int numnodes, Categories* out, std::string* err);
void host_gtr(const double* q, const double* piv, double* Q);
void host_musefreqs(const double* pi4, double lGC, double lAT, double lGT, double* out16);
void host_muse(double lGC, double lAT, double lGT, const double* q, const double* pi4, double sr1, double sr2,
               double* Q);
int host_reversible_eig(int n, const double* Q, const double* pi, double* w, double* U);

// ---- plan (plan.cpp) ----
int build_plan(messi_dataset* ds, const messi_alignment* aln, int W, const uint8_t* pairmask, std::string* err);
int allocate_arena(messi_dataset* ds, int C, std::string* err);

// ---- pruning kernels (prune.cu) ----
int launch_build_P16(messi_ctx* ctx, const double* d_eig, const double* d_bl, int numnodes, int C, float* d_P);
int launch_build_P4(messi_ctx* ctx, const double* d_eig4, const double* d_bl, int numnodes, int nsite,
                    double* d_P4);
int run_pairs(messi_ctx* ctx, messi_dataset* ds, const float* d_P, const float* d_pi16, const double* d_logw,
              const int* d_lam, int C, int nlam, bool per_lambda);
int launch_unpaired(messi_ctx* ctx, messi_dataset* ds, const double* d_P4, const double* d_pi4,
                    const double* d_logw_site, int nsite, double* d_u);
int launch_scatter_dense(messi_ctx* ctx, messi_dataset* ds, const double* d_vals, double* d_out);
int launch_bandprep_from_mix(messi_ctx* ctx, messi_dataset* ds, const Band& t, const uint8_t* d_gapmask,
                             double B);

// ---- SCFG kernels (scfg.cu) ----
int band_alloc(messi_ctx* ctx, int L, int Wb, bool outside, Band* t);
int launch_baseline(messi_ctx* ctx, const Band& t, double B);
int launch_bandprep_from_dense(messi_ctx* ctx, const Band& t, const double* d_dense, double B);
int launch_maxspan(messi_ctx* ctx, int L, const double* d_dense, int* d_out);
int run_inside(messi_ctx* ctx, const Band& t, double B);
int run_outside(messi_ctx* ctx, const Band& t, double B);
int run_posteriors(messi_ctx* ctx, const Band& t, double B, double* d_single, double* d_pair);
int launch_dense_inside(messi_ctx* ctx, const Band& t, double* d_out);
int launch_dense_outside(messi_ctx* ctx, const Band& t, double* d_out);
int launch_band_from_dense_inside(messi_ctx* ctx, const Band& t, const double* d_in);
int launch_band_from_dense_outside(messi_ctx* ctx, const Band& t, const double* d_out);
int launch_finish_Z(messi_ctx* ctx, const Band& t);
// Queue a copy of the wavefront barrier status into ctx->status_host.
int queue_status_readback(messi_ctx* ctx, const Band& t);

}  // namespace messi
