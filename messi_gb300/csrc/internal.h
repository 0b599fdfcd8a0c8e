// internal.h -- shared declarations of the messi_gb300 library (not part of the ABI).
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/messi_gb300.h"

namespace messi {

constexpr int kTile = 128;          // unique pairs per CTA in the pruning kernels
// Grid-barrier words of the wavefront kernels: [0] = arrivals, [2] =
// host-visible error flag (wave.cuh).
constexpr int kSyncWords = 4;
constexpr int kMaxLambda = 8;       // per-lambda conditionals kept in registers
constexpr int kMaxStack = 512;      // tree height limit of the unpaired kernel
constexpr int kEigStride = 16 + 256 + 16;  // eigenvalues, U (row-major), sqrt(pi)
constexpr int kEig4Stride = 4 + 16 + 4;

// Grow-only device buffer.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

// Host staging of several arrays for one host-to-device copy (16-byte aligned).
struct Staged {
    size_t off = 0;
    std::vector<char> host;
    template <typename T>
    size_t add(const T* src, size_t n)
    {
        off = (off + 15) & ~size_t(15);
        size_t at = off;
        host.resize(off + n * sizeof(T));
        if (n) std::memcpy(host.data() + at, src, n * sizeof(T));
        off += n * sizeof(T);
        return at;
    }
};

// Per-internal-node descriptor of one pruning step (device resident).  Rows
// are messages: the row a node sends to its parent is its partial likelihood
// vector multiplied by its own branch's transition matrix, so a node update
// is the elementwise product of its two children's messages followed by one
// mat-vec (none at the root).
struct NodeDev {
    const int* li;     // [n] row of the left child for each unique pair
    const int* ri;     // [n]
    const float* lf;   // left child message rows (16 floats each)
    const int* le;     // left child exponents (nullptr for leaves: exponent 0)
    long long lcs;     // left child category stride in rows
    const float* rf;
    const int* re;
    long long rcs;
    float* of;         // output message rows (unused at the root)
    int* oe;
    long long ocs;
    double* mix;       // root only: [n] category mixture per unique root pair
    double* mixlam;    // root only: [kMaxLambda][n] per-lambda mixtures (nullable)
    double* catll;     // root only: [C][n] per-category log-likelihoods (nullable)
    int n;             // unique pairs at this node
    int self;          // this node's id (index of its branch's transition matrices)
    int grp;           // model group (index of the category tables pi16/logw)
    int pad;
};

// Discretised model categories built on the host for one call.
struct Categories {
    int C = 0, nsite = 0, nlam = 0;  // C = categories pruned with 16 states
    std::vector<double> eig;      // [C][kEigStride]
    std::vector<float> pi16;      // [C][16]
    std::vector<double> logw;     // [C]
    std::vector<int> lam;         // [C] lambda category of each category
    // Lambda categories with lambda_GC = lambda_AT = lambda_GT = 1 left out of
    // the 16-state pruning when factorising: their pair likelihood is the
    // product of the two unpaired columns, so over the site rates they add
    // log(sum of their weights) + u[x] + u[y] to the mixture.
    uint32_t lamF = 0;             // bit l: lambda category l is factorised
    double logwF = -INFINITY;      // log of the summed weights of those categories
    std::vector<double> logw_lam;  // [nlam] log lambda weight
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
    float* OSlast;  // suffix-column terms of the outside S sums of the last column's band cells
    double *b, *cb, *u, *Zd;
    int* maxspan;
    unsigned int* sync;  // kSyncWords grid-barrier words of the wavefront kernels
};

// Band tables of a batch of alignments for the batched inside pass.  Bands
// are kept sorted by band width, descending (band k holds alignment order[k]).
struct BandBatch {
    int n = 0;
    long long total_cols = 0;
    std::vector<Band> host;
    std::vector<int> order, slot;  // slot[alignment] = band index
    Band* d_bands = nullptr;
    long long* d_cumL = nullptr;   // [n+1] exclusive prefix of the lengths
    int* d_wbs = nullptr;          // [n] band widths
    unsigned int* d_sync = nullptr;
    double* d_Z = nullptr;         // [n] in band order
    void* mem = nullptr;           // one device allocation holding all of the above
    size_t bytes = 0;
};

// KH99 rule probabilities (src/InsideOutsideAlgorithm.jl:40-53):
// S->LS, S->s, S->dFd, F->dFd, F->LS, L->s, L->dFd.
constexpr double kKH99Prob[7] = {0.868534, 0.117609877998, 0.013856122002, 0.787640, 0.21236, 0.894603, 0.105397};

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

namespace messi {
// What a captured likelihood launch sequence depends on besides the staged
// model bytes: the dataset, the category layout, the gap mask's presence and
// every device pointer (through the context's allocation epoch).
struct LikelihoodKey {
    const void* ds = nullptr;
    int C = -1, nsite = -1, nlam = -1, Wb = -1;
    uint32_t lamF = 0;
    bool gapmask = false;
    size_t staged = 0;
    uint64_t epoch = 0, arena_gen = 0;
    // launch shapes the captured sequence was recorded with
    int wave_ctas = -1, wave_threads = -1, prune_shape = -1;
    bool operator==(const LikelihoodKey& o) const
    {
        return ds == o.ds && C == o.C && nsite == o.nsite && nlam == o.nlam && Wb == o.Wb && lamF == o.lamF &&
               gapmask == o.gapmask && staged == o.staged && epoch == o.epoch && arena_gen == o.arena_gen &&
               wave_ctas == o.wave_ctas && wave_threads == o.wave_threads && prune_shape == o.prune_shape;
    }
};
// Launch-shape autotuning of one workload (a dataset or a batch at a
// category count): the first kTuneCalls evaluations run with candidate shapes
// (pruning pipeline shape k % 3, wavefront CTA size k % 4) and time the
// pruning and the inside pass with CUDA events; then the fastest of each is
// kept (the default unless another is at least 2% faster).  Results do not
// depend on the shapes.
constexpr int kTuneCalls = 4;
constexpr int kPruneShapes = 3;
constexpr int kWaveCands = 4;
constexpr int kWaveThreadCands[kWaveCands] = {0, 256, 512, 1024};  // 0: chosen by band size
struct TuneSlot {
    int k = 0;                       // evaluations timed so far
    bool done = false;
    double prune_ms[kPruneShapes] = {INFINITY, INFINITY, INFINITY};
    double wave_ms[kWaveCands] = {INFINITY, INFINITY, INFINITY, INFINITY};
    int prune_shape = 0, wave_threads = 0;  // chosen
};
struct LikelihoodGraph {
    cudaGraphExec_t exec = nullptr;
    LikelihoodKey key;      // of exec
    LikelihoodKey seen;     // of the last eager call (capture on the second identical call)
    int64_t launches = 0;   // kernel launches in exec
};
}  // namespace messi

struct messi_ctx {
    int device = 0;
    // CTAs of the persistent wavefront kernels (0 = one per SM, fewer for short
    // sequences) and their size (256, 512 or 1024 threads; 0 = by band size)
    int wave_ctas = 0;
    int wave_threads = 0;
    // pair node-update pipeline (128-pair tiles): 0 = 2 stages x 4 CTAs/SM,
    // 1 = 3 stages x 3 CTAs/SM, 2 = 2 stages x 3 CTAs/SM
    int prune_shape = 0;
    // per-kernel event timing (messi_ctx_profile)
    bool profiling = false;
    std::vector<messi::ProfRec> prof_pending;
    std::vector<cudaEvent_t> prof_pool;
    double prof_ms[messi::kProfKernels] = {0, 0, 0, 0};
    int64_t prof_count[messi::kProfKernels] = {0, 0, 0, 0};
    double prof_units[messi::kProfKernels] = {0, 0, 0, 0};
    cudaStream_t stream = nullptr;
    // second stream for work independent of the pair pruning (unpaired
    // columns, baselines), forked from and joined back to `stream` by events
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    int64_t launches = 0;
    std::string last_error;
    int num_sms = 0;
    // scratch buffers (grow-only)
    messi::DevBuf scratch[32];
    void* pinned = nullptr;
    size_t pinned_bytes = 0;
    unsigned int* status_host = nullptr;  // pinned word: wavefront barrier status of the last call
    // device buffers are reallocated only when they grow; every reallocation
    // bumps the epoch, so a captured launch sequence knows its pointers are stale
    uint64_t alloc_epoch = 0;
    // CUDA graph of messi_likelihood's device work (MESSI_GRAPHS=0 disables)
    bool graphs = true;
    messi::LikelihoodGraph lgraph;
    int64_t graph_replays = 0;
    // launch-shape autotuning (MESSI_AUTOTUNE=0 turns it off; an explicit
    // MESSI_PRUNE_SHAPE or MESSI_WAVE_THREADS fixes that knob)
    bool autotune = true, fixed_prune = false, fixed_wave = false;
    std::map<std::pair<const void*, int>, messi::TuneSlot> tune;
    cudaEvent_t tev[4] = {nullptr, nullptr, nullptr, nullptr};
    bool tune_timing = false;        // record tev[] around the pruning and the inside pass of this call
    int tune_saved[2] = {0, 0};      // context shapes restored after a tuned call
    int last_prune_shape = 0, last_wave_threads = 0;
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
    uint64_t arena_gen = 0;            // bumped whenever the arena and node descriptors are rewritten
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
    int64_t leaf_rows = 0;             // rows of d_leaf (unique pairs summed over the leaves)
    std::vector<float> leaf_host;      // [leaf_rows][16] host copy of d_leaf
    std::vector<int> leafnode_host;    // [leaf_rows] leaf node of each row
    int* d_leafnode = nullptr;         // device copy of leafnode_host
    float* d_leafmsg = nullptr;        // [chunk][leaf_rows][16] leaf messages of the current pass
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
// Start of every entry point (device, counters) and its end (stream sync, status checks).
int begin(messi_ctx* ctx);
int finish(messi_ctx* ctx);
int h2d(messi_ctx* ctx, void* dst, const void* src, size_t bytes);
int d2h(messi_ctx* ctx, void* dst, const void* src, size_t bytes);
// Event pair around one launch of a timed kernel family (no-op unless profiling).
int prof_begin(messi_ctx* ctx, int kernel, double units);
void prof_end(messi_ctx* ctx);

// ---- host model (host_model.cpp) ----
// pairs = false skips the 16-state eigensystems (unpaired-only calls);
// threads = false keeps the eigensystems on the calling thread (callers that
// build many models in parallel themselves).
int build_categories(const messi_model* m, int numnodes, Categories* out, std::string* err, bool pairs = true,
                     bool factorise = false, bool threads = true);
void host_gtr(const double* q, const double* piv, double* Q);
void host_musefreqs(const double* pi4, double lGC, double lAT, double lGT, double* out16);
void host_muse(double lGC, double lAT, double lGT, const double* q, const double* pi4, double sr1, double sr2,
               double* Q);
int host_reversible_eig(int n, const double* Q, const double* pi, double* w, double* U);

// ---- plan (plan.cpp) ----
// Plan of the band pairs (y - x <= W, pairmask non-zero), or with `pairs`
// of exactly those pairs (pair_unique[p] = unique root pair of pairs[p]; no
// band index map).
int build_plan(messi_dataset* ds, const messi_alignment* aln, int W, const uint8_t* pairmask, std::string* err,
               const std::vector<int2>* pairs = nullptr, std::vector<int32_t>* pair_unique = nullptr);
int allocate_arena(messi_dataset* ds, int C, std::string* err);

// Node descriptors of one dataset whose message rows live at `arena_f/e` +
// row_base rows, category stride `cstride` rows, and whose leaf messages live
// at `leafmsg` + leaf_base rows, category stride `leaf_cstride` rows;
// transition matrices of local node v are those of node node_base + v; model
// group `grp`.
void fill_node_descriptors(const messi_dataset* ds, float* arena_f, int* arena_e, int64_t row_base, int64_t cstride,
                           float* leafmsg, int64_t leaf_base, int64_t leaf_cstride, int node_base, int grp,
                           NodeDev* out);

// ---- pruning kernels (prune.cu) ----
// nodegrp: [numnodes] model group of each node, -1 for a root (nullptr: one
// tree, root = node 0, group 0).  Category tables are [group][C][...].
// d_P: FP32 matrices [C][numnodes][256] (the pruning kernel splits them into
// TF32 hi/lo parts in registers).
int launch_build_P16(messi_ctx* ctx, const double* d_eig, const double* d_bl, const int* d_nodegrp, int numnodes,
                     int C, float* d_P);
int launch_build_P4(messi_ctx* ctx, const double* d_eig4, const double* d_bl, const int* d_nodegrp, int numnodes,
                    int nsite, double* d_P4);
// Leaf messages of categories c0 .. c0+nc-1: out[cc][r] = P[c0+cc][rownode[r]]
// x rows[r] for the R leaf rows (FP64 accumulation, stored FP32); d_P holds
// C categories.
int launch_leaf_messages(messi_ctx* ctx, const float* d_rows, const int* d_rownode, int64_t R, const float* d_P,
                         int numnodes, int c0, int nc, int C, float* d_out);
// The tensor-core node update over `nt` tiles of one level (root tiles when root).
int launch_prune_tiles(messi_ctx* ctx, const NodeDev* d_nodes, const int2* d_tiles, int nt, bool root,
                       const float* d_P, int numnodes, int c0, int nc, int C, const float* d_pi16,
                       const double* d_logw, const int* d_lam, bool per_lambda);
int run_pairs(messi_ctx* ctx, messi_dataset* ds, const float* d_P, const float* d_pi16, const double* d_logw,
              const int* d_lam, int C, int nlam, bool per_lambda);
// Unpaired column likelihoods of one tree whose transition matrices start at
// d_P4 with node stride `pstride` (nodes of all site categories: [s][pstride][16]).
// d_scratch: nsite * (numnodes * L * 5 + L) doubles, or nullptr for the
// context's buffer (reused in stream order).
int launch_unpaired(messi_ctx* ctx, messi_dataset* ds, const double* d_P4, int pstride, const double* d_pi4,
                    const double* d_logw_site, int nsite, double* d_u, double* d_scratch);
// Site-rate conditionals (prune.cu): catll [C][nroot] per-category root
// log-likelihoods, ull [nsite][L] per-site unpaired log-likelihoods, single
// [L] and pair [L x L] (column-major) posteriors; out [nsite x L] column-major.
int launch_siterate_conditionals(messi_ctx* ctx, messi_dataset* ds, const double* d_catll, const double* d_logw,
                                 int nsite, int nlam, const double* d_single, const double* d_pair,
                                 const double* d_ull, const double* d_logw_site, double* d_out);
// Fixed-structure sums (prune.cu, structure_sum_kernel); d_partner[c] is the
// 0-based partner of column c (or -1), logwF the factorised lambda weight.
int launch_structure_sum(messi_ctx* ctx, int L, double* d_u, const int* d_colu, const int* d_partner,
                         const double* d_mix, double logwF, double* d_total, double* d_pairll);
// Work on the context's side stream (api.cu): fork_side makes the side
// stream wait for everything queued on the main stream so far; while a
// SideLaunches is alive the launch helpers (which use ctx->stream) queue on
// the side stream; join_side makes the main stream wait for the side
// stream's work.
int fork_side(messi_ctx* ctx);
int join_side(messi_ctx* ctx);
struct SideLaunches {
    messi_ctx* ctx;
    cudaStream_t main;
    explicit SideLaunches(messi_ctx* c) : ctx(c), main(c->stream) { ctx->stream = ctx->side; }
    ~SideLaunches() { ctx->stream = main; }
};

// Bounded-wait self-test (scfg.cu): a two-CTA grid barrier that one CTA never
// reaches; d_sync[2] becomes 1 when the other CTA's wait gives up.
int launch_barrier_selftest(messi_ctx* ctx, unsigned int* d_sync);
// Dense L x L pair matrix: vals (nullable) of the unique root pairs, mixed with
// addw + u[x] + u[y] when addw is finite (the factorised lambda categories).
int launch_scatter_dense(messi_ctx* ctx, messi_dataset* ds, const double* d_vals, const double* d_u, double addw,
                         double* d_out);
// Banded pair scores from the root mixtures of ds, with the factorised term
// logwF + u[i] + u[j] (u = t.u) when logwF is finite; d_logwF (nullable)
// holds logwF on the device instead.
int launch_bandprep_from_mix(messi_ctx* ctx, messi_dataset* ds, const Band& t, const uint8_t* d_gapmask,
                             double B, double logwF, const double* d_logwF = nullptr);

// ---- column patterns on the device (ingest.cu) ----
// d_refs: [numnodes][L] first-column pattern ids; d_out_julia (nullable):
// [numnodes x L] column-major, 1-based (the reference's subcolumnrefs).
int run_subcolumnrefs(messi_ctx* ctx, messi_dataset* ds, int* d_refs, int* d_out_julia, void* d_work,
                      size_t work_bytes);
size_t subcolumnrefs_work_bytes(const messi_dataset* ds);

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
// KH99 rule log-probabilities times B.
Rules make_rules(double B);
// Posterior decoding (decode.cu).  d_work: (L + 3 L^2) floats; d_scol: L^2
// ints (the column-major s output); d_sync: 4 uints; d_paired (nullable):
// [L]; d_stack: 2 (L + 1) ints; d_eout (nullable): L^2 doubles.
int run_posterior_decoding(messi_ctx* ctx, int L, const double* d_single, const double* d_pair, double alpha,
                           float* d_work, int* d_scol, unsigned int* d_sync, int* d_paired, int* d_stack,
                           double* d_eout);
// Structure sampling through the inside band tables of t (computed with B).
// d_paired: [nstruct][L]; d_stack: [nstruct][3 (L + 1)] ints; d_prior
// (nullable): [nstruct] log KH99 prior of each structure; d_status: 1 uint.
int run_sample_structures(messi_ctx* ctx, const Band& t, double B, int nstruct, unsigned long long seed,
                          int* d_paired, int* d_stack, double* d_prior, unsigned int* d_status);
// Grid and CTA size of a persistent wavefront kernel (cooperative launch).
int wave_threads(const messi_ctx* ctx, double band_cells);
int wave_grid(messi_ctx* ctx, const void* kernel, int L, int threads);
int bandbatch_alloc(const std::vector<int>& L, const std::vector<int>& Wb, BandBatch* bb, std::string* err);
void bandbatch_free(BandBatch* bb);
int launch_baseline_batch(messi_ctx* ctx, const BandBatch& bb, double B);
int run_inside_batch(messi_ctx* ctx, const BandBatch& bb, double B);
// Autotuning around one evaluation of `key` with C categories (api.cu):
// tune_begin sets the context's launch shapes for this call (a candidate, or
// the chosen ones) and arms the timing events; tune_mark(i) records event i
// (0/1 around the pruning, 2/3 around the inside pass) when armed;
// tune_end reads the events after the call's stream synchronise.
void tune_begin(messi_ctx* ctx, const void* key, int C);
void tune_mark(messi_ctx* ctx, int i);
void tune_end(messi_ctx* ctx, const void* key, int C);
void tune_forget(messi_ctx* ctx, const void* key);
// Queue a copy of the wavefront barrier status into ctx->status_host.
int queue_status_readback(messi_ctx* ctx, const Band& t);
// Cooperative launch of a persistent wavefront kernel (scfg.cu): resets the
// barrier words, picks the CTA size and grid; share > 0 for kernels that own
// rows of diagonal pairs (warps per row and pair).
int launch_wave(messi_ctx* ctx, const void* kernel, void** args, unsigned int* sync, int L, double band_cells,
                const char* what, int share = 0, const void* halves_kernel = nullptr);

}  // namespace messi
