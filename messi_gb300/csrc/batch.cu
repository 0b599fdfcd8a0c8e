// batch.cu -- many alignments in one evaluation.
//
// The reference evaluates one alignment per call (src/FelsensteinCUDA.jl:214,
// src/InsideCUDA.jl:23, driven from src/FARCE.jl:2322-2345).  A batch keeps
// the per-alignment pair plans of plan.cpp and runs them together:
//   * pruning: the alignments form groups (contiguous in batch order) whose
//     message arena holds every category at once; within a group the tree
//     levels of all alignments are merged, so level l of every tree in the
//     group is one launch (plus one for the roots that sit at level l), and
//     the groups reuse one arena one after another.  (One arena for the whole
//     batch would have to run the categories in several passes, each
//     re-reading the gather indices and refilling the copy pipeline: 17%
//     slower per node update on 256 alignments of up to 1,500 columns);
//   * transition matrices of every node of every tree come from one launch,
//     with one eigensystem set per distinct model (models that differ only
//     in their branch lengths share it);
//   * the inside passes of all alignments run in one persistent wavefront
//     (inside_wave_batch_kernel): diagonal d of every alignment whose band
//     reaches it is one step, so the number of grid barriers is the largest
//     band width in the batch instead of the sum over alignments;
//   * the device work of a step is captured as a CUDA graph on the second
//     call with the same layout and replayed from then on (per-call values
//     travel in the staged model bytes).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <thread>

#include "internal.h"

using namespace messi;

struct messi_batch {
    messi_ctx* ctx = nullptr;
    int n = 0;
    std::vector<messi_dataset*> ds;
    std::vector<int> node_base;
    std::vector<int64_t> col_base;
    int total_nodes = 0;
    int64_t total_cols = 0;
    int H = 0;
    // groups of alignments [a0, a1) pruned together; per group and level the
    // non-root and root tile ranges in d_tiles
    struct Group {
        int a0 = 0, a1 = 0, H = 0;
        int64_t rows = 0, leaf0 = 0, leaf_rows = 0;
        std::vector<int> tile_off, tile_cnt, rtile_off, rtile_cnt;
    };
    std::vector<Group> groups;
    int64_t max_group_rows = 0, max_group_leaf_rows = 0;
    int2* d_tiles = nullptr;
    NodeDev* d_nodes = nullptr;
    std::vector<NodeDev> nodes_host;
    std::vector<int> desc_grp;  // model group the descriptors were written for
    float* d_arena_f = nullptr;
    int* d_arena_e = nullptr;
    std::vector<int64_t> row_base;
    int64_t total_rows = 0;
    // leaf rows of every alignment, concatenated, with their global node ids,
    // and the leaf messages of the current category pass
    std::vector<int64_t> leaf_base;
    int64_t total_leaf_rows = 0;
    float* d_leafrows = nullptr;
    int* d_leafnode = nullptr;
    float* d_leafmsg = nullptr;
    int chunk = 0, arena_C = 0;
    BandBatch bands;
    DevBuf stage, P16, P4;
    int64_t executed = 0, naive = 0, band_pairs = 0, nroot = 0;
    // bumped whenever a device buffer the step uses is reallocated or the
    // node descriptors are rewritten (a captured graph holds their pointers)
    uint64_t gen = 0;
    // captured step: launch shapes and layout it was recorded with
    struct Key {
        int C = -1, G = -1, nsite = -1;
        uint32_t lamF = 0;
        bool gap = false;
        size_t staged = 0;
        uint64_t epoch = 0, gen = 0;
        int prune_shape = -1, wave_threads = -1, wave_ctas = -1;
        bool operator==(const Key& o) const
        {
            return C == o.C && G == o.G && nsite == o.nsite && lamF == o.lamF && gap == o.gap && staged == o.staged &&
                   epoch == o.epoch && gen == o.gen && prune_shape == o.prune_shape &&
                   wave_threads == o.wave_threads && wave_ctas == o.wave_ctas;
        }
    };
    cudaGraphExec_t graph = nullptr;
    Key graph_key, seen_key;
    int64_t graph_launches = 0;
};

namespace {

int grow(DevBuf& b, size_t bytes, void** p)
{
    if (b.bytes < bytes) {
        if (b.p) cudaFree(b.p);
        b.p = nullptr;
        b.bytes = 0;
        if (cudaMalloc(&b.p, bytes) != cudaSuccess) return MESSI_ENOMEM;
        b.bytes = bytes;
    }
    *p = b.p;
    return MESSI_OK;
}

bool same_arrays(const double* a, const double* b, int n)
{
    return std::memcmp(a, b, sizeof(double) * (size_t)n) == 0;
}

// Models that differ only in their branch lengths share categories.
bool same_parameters(const messi_model& a, const messi_model& b)
{
    return same_arrays(a.freqs, b.freqs, 4) && same_arrays(a.q, b.q, 6) && a.nsite == b.nsite &&
           a.nlambda == b.nlambda && same_arrays(a.siteRates, b.siteRates, a.nsite) &&
           same_arrays(a.siteWeights, b.siteWeights, a.nsite) && same_arrays(a.lambdaGC, b.lambdaGC, a.nlambda) &&
           same_arrays(a.lambdaAT, b.lambdaAT, a.nlambda) && same_arrays(a.lambdaGT, b.lambdaGT, a.nlambda) &&
           same_arrays(a.lambdaWeights, b.lambdaWeights, a.nlambda);
}

void destroy_batch(messi_batch* b)
{
    if (!b) return;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (messi_dataset* d : b->ds)
        if (d) messi_dataset_destroy(d);
    void* bufs[] = {b->d_tiles, b->d_nodes, b->d_arena_f, b->d_arena_e, b->stage.p, b->P16.p, b->P4.p,
                    b->d_leafrows, b->d_leafnode, b->d_leafmsg};
    for (void* p : bufs)
        if (p) cudaFree(p);
    bandbatch_free(&b->bands);
    delete b;
}

// Message arena for C categories, sized for the largest group (as many
// categories per pass as fit; every category at once unless one group alone
// is larger than the memory budget).
int prepare_batch_arena(messi_ctx* ctx, messi_batch* b, int C)
{
    if (b->chunk != 0 && b->arena_C == C) return MESSI_OK;
    if (b->d_arena_f) cudaFree(b->d_arena_f);
    if (b->d_arena_e) cudaFree(b->d_arena_e);
    if (b->d_leafmsg) cudaFree(b->d_leafmsg);
    b->d_arena_f = nullptr;
    b->d_arena_e = nullptr;
    b->d_leafmsg = nullptr;
    b->chunk = 0;
    b->gen++;
    size_t freeb = 0, totalb = 0;
    cudaMemGetInfo(&freeb, &totalb);
    const size_t row_bytes = 16 * sizeof(float) + sizeof(int);
    const int64_t rows = std::max<int64_t>(b->max_group_rows, 1);
    const int64_t leaf_rows = std::max<int64_t>(b->max_group_leaf_rows, 1);
    int chunk = C;
    while (chunk > 1 && (size_t)chunk * (rows + leaf_rows) * row_bytes > freeb / 2) chunk = (chunk + 1) / 2;
    cudaError_t e = cudaMalloc((void**)&b->d_arena_f, (size_t)chunk * rows * 16 * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_arena_e, (size_t)chunk * rows * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_leafmsg, (size_t)chunk * leaf_rows * 16 * sizeof(float));
    if (e != cudaSuccess) return cuda_fail(ctx, e, "batch message arena");
    b->chunk = chunk;
    b->arena_C = C;
    b->desc_grp.clear();  // descriptors point into the old arena
    return MESSI_OK;
}

int write_descriptors(messi_ctx* ctx, messi_batch* b, const std::vector<int>& grp)
{
    if (b->desc_grp == grp) return MESSI_OK;
    b->nodes_host.assign(b->total_nodes, NodeDev{});
    const int64_t cs = std::max<int64_t>(b->max_group_rows, 1);
    for (const messi_batch::Group& gr : b->groups)
        for (int a = gr.a0; a < gr.a1; a++)
            fill_node_descriptors(b->ds[a], b->d_arena_f, b->d_arena_e, b->row_base[a], cs, b->d_leafmsg,
                                  b->leaf_base[a] - gr.leaf0, std::max<int64_t>(gr.leaf_rows, 1), b->node_base[a],
                                  grp[a], b->nodes_host.data() + b->node_base[a]);
    b->gen++;
    cudaError_t e = cudaMemcpyAsync(b->d_nodes, b->nodes_host.data(), sizeof(NodeDev) * b->total_nodes,
                                    cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "batch node descriptors");
    // the host copy must outlive the asynchronous copy: keep it until the next call
    b->desc_grp = grp;
    return MESSI_OK;
}

// Device pointers and per-call values of one batch step (host staging done).
struct BatchStep {
    void* stage_dev = nullptr;
    const void* stage_host = nullptr;
    size_t stage_bytes = 0;
    const double *eig = nullptr, *eig4 = nullptr, *logw = nullptr, *pi4 = nullptr, *lws = nullptr, *bl = nullptr;
    const double* logwF = nullptr;  // [model group] factorised lambda weight, on the device
    const float* pi16 = nullptr;
    const int *lam = nullptr, *grp = nullptr;
    const uint8_t* gap = nullptr;
    float* P = nullptr;
    double* P4 = nullptr;
    double* unpaired_scratch = nullptr;
    int C = 0, nsite = 0;
    const std::vector<int>* grp_of = nullptr;
    const std::vector<Categories>* cats = nullptr;
};

// Every device step of a batch evaluation: model upload, transition matrices,
// unpaired columns and baselines on the side stream, pruning group by group,
// banded scores, the batched inside pass.
int enqueue_batch(messi_ctx* ctx, messi_batch* b, const BatchStep& s)
{
    int rc;
    const int n = b->n, C = s.C, nsite = s.nsite;
    if ((rc = h2d(ctx, s.stage_dev, s.stage_host, s.stage_bytes))) return rc;
    if ((rc = launch_build_P16(ctx, s.eig, s.bl, s.grp, b->total_nodes, C, s.P))) return rc;
    if ((rc = launch_build_P4(ctx, s.eig4, s.bl, s.grp, b->total_nodes, nsite, s.P4))) return rc;
    if ((rc = fork_side(ctx))) return rc;
    {
        SideLaunches side(ctx);
        for (int a = 0; a < n; a++) {
            const Band& t = b->bands.host[b->bands.slot[a]];
            const int g = (*s.grp_of)[a];
            if ((rc = launch_unpaired(ctx, b->ds[a], s.P4 + (size_t)b->node_base[a] * 16, b->total_nodes,
                                      s.pi4 + 4 * g, s.lws + (size_t)nsite * g, nsite, t.u, s.unpaired_scratch)))
                return rc;
        }
        if ((rc = launch_baseline_batch(ctx, b->bands, 1.0))) return rc;
    }
    tune_mark(ctx, 0);
    for (const messi_batch::Group& gr : b->groups) {
        for (int c0 = 0; c0 < C; c0 += b->chunk) {
            const int nc = std::min(b->chunk, C - c0);
            if ((rc = launch_leaf_messages(ctx, b->d_leafrows + (size_t)gr.leaf0 * 16, b->d_leafnode + gr.leaf0,
                                           gr.leaf_rows, s.P, b->total_nodes, c0, nc, C, b->d_leafmsg)))
                return rc;
            for (int lv = 1; lv <= gr.H; lv++) {
                for (int root = 0; root < 2; root++) {
                    const int nt = root ? gr.rtile_cnt[lv] : gr.tile_cnt[lv];
                    if (nt == 0) continue;
                    const int2* tl = b->d_tiles + (root ? gr.rtile_off[lv] : gr.tile_off[lv]);
                    if (ctx->profiling) {
                        double units = 0.0;
                        for (int a = gr.a0; a < gr.a1; a++) {
                            const messi_dataset* d = b->ds[a];
                            if (lv > d->H || (root != 0) != (lv == d->H)) continue;
                            for (int v : d->level_nodes[lv]) units += (double)d->nunique[v] * nc;
                        }
                        prof_begin(ctx, 0, units);
                    }
                    if ((rc = launch_prune_tiles(ctx, b->d_nodes, tl, nt, root != 0, s.P, b->total_nodes, c0, nc, C,
                                                 s.pi16, s.logw, s.lam, false)))
                        return rc;
                    prof_end(ctx);
                }
            }
        }
    }
    tune_mark(ctx, 1);
    if ((rc = join_side(ctx))) return rc;
    for (int a = 0; a < n; a++) {
        const Band& t = b->bands.host[b->bands.slot[a]];
        const int g = (*s.grp_of)[a];
        if ((rc = launch_bandprep_from_mix(ctx, b->ds[a], t, s.gap ? s.gap + b->col_base[a] : nullptr, 1.0,
                                           (*s.cats)[g].logwF, s.logwF + g)))
            return rc;
    }
    tune_mark(ctx, 2);
    if ((rc = run_inside_batch(ctx, b->bands, 1.0))) return rc;
    tune_mark(ctx, 3);
    return MESSI_OK;
}

// Capture enqueue_batch into b->graph; on any capture error graphs are
// switched off for the context and the caller runs the steps eagerly.
bool capture_batch(messi_ctx* ctx, messi_batch* b, const BatchStep& s, const messi_batch::Key& key)
{
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    const int64_t l0 = ctx->launches;
    bool ok = false;
    if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        const int rc = enqueue_batch(ctx, b, s);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
        cudaGraphExec_t ex = nullptr;
        if (rc == MESSI_OK && e == cudaSuccess && g && cudaGraphInstantiate(&ex, g, 0) == cudaSuccess) {
            b->graph = ex;
            b->graph_key = key;
            b->graph_launches = ctx->launches - l0;
            ok = true;
        }
        if (g) cudaGraphDestroy(g);
    }
    if (!ok) {
        cudaGetLastError();
        ctx->graphs = false;
        ctx->last_error.clear();
    }
    ctx->launches = l0;
    return ok;
}

}  // namespace

extern "C" {

int messi_batch_create(messi_ctx* ctx, int32_t n, const messi_alignment* alns, const int32_t* maxbasepairdistance,
                       messi_batch** out)
{
    int rc = begin(ctx);
    if (rc) return rc;
    if (n < 1 || !alns || !out) return fail(ctx, MESSI_EINVAL, "batch: need n >= 1 alignments and an output");
    *out = nullptr;
    messi_batch* b = new (std::nothrow) messi_batch();
    if (!b) return fail(ctx, MESSI_ENOMEM, "batch: host allocation");
    b->ctx = ctx;
    b->n = n;
    b->ds.assign(n, nullptr);
    // per-alignment plans, built on host threads
    std::vector<int> rcs(n, MESSI_OK);
    std::vector<std::string> errs(n);
    const int nthreads = (int)std::max(1u, std::min<unsigned>((unsigned)n, std::thread::hardware_concurrency()));
    auto work = [&](int tid) {
        cudaSetDevice(ctx->device);
        for (int a = tid; a < n; a += nthreads) {
            messi_dataset* d = new (std::nothrow) messi_dataset();
            if (!d) { rcs[a] = MESSI_ENOMEM; errs[a] = "batch: host allocation"; continue; }
            d->ctx = ctx;
            b->ds[a] = d;
            const int W = maxbasepairdistance ? maxbasepairdistance[a] : alns[a].numcols - 1;
            rcs[a] = build_plan(d, &alns[a], W, nullptr, &errs[a]);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nthreads; t++) pool.emplace_back(work, t);
    work(0);
    for (auto& th : pool) th.join();
    for (int a = 0; a < n; a++)
        if (rcs[a] != MESSI_OK) {
            std::string msg = "batch alignment " + std::to_string(a) + ": " + errs[a];
            destroy_batch(b);
            return fail(ctx, rcs[a], msg);
        }
    // merged levels
    b->node_base.resize(n);
    b->col_base.resize(n);
    b->row_base.resize(n);
    b->leaf_base.resize(n);
    for (int a = 0; a < n; a++) {
        const messi_dataset* d = b->ds[a];
        b->leaf_base[a] = b->total_leaf_rows;
        b->total_leaf_rows += d->leaf_rows;
        b->node_base[a] = b->total_nodes;
        b->total_nodes += d->numnodes;
        b->col_base[a] = b->total_cols;
        b->total_cols += d->L;
        b->row_base[a] = b->total_rows;
        b->total_rows += d->arena_rows;
        b->H = std::max(b->H, d->H);
        b->executed += d->executed;
        b->naive += d->naive;
        b->band_pairs += d->band_pairs;
        b->nroot += d->nroot;
    }
    // groups: contiguous runs of alignments whose messages for every
    // category fit in half of the free memory (45 categories: 3 site rates
    // squared times 5 lambda categories, the most a default model prunes)
    {
        size_t freeb = 0, totalb = 0;
        cudaMemGetInfo(&freeb, &totalb);
        const size_t row_bytes = 16 * sizeof(float) + sizeof(int);
        const int64_t budget_rows = (int64_t)(freeb / 2 / (45 * row_bytes));
        int a = 0;
        while (a < n) {
            messi_batch::Group gr;
            gr.a0 = a;
            gr.leaf0 = b->leaf_base[a];
            int64_t rows = 0, lrows = 0;
            while (a < n) {
                const int64_t r = b->ds[a]->arena_rows, l = b->ds[a]->leaf_rows;
                if (a > gr.a0 && rows + r + lrows + l > budget_rows) break;
                b->row_base[a] = rows;  // group-local
                rows += r;
                lrows += l;
                gr.H = std::max(gr.H, b->ds[a]->H);
                a++;
            }
            gr.a1 = a;
            gr.rows = rows;
            gr.leaf_rows = lrows;
            b->max_group_rows = std::max(b->max_group_rows, rows);
            b->max_group_leaf_rows = std::max(b->max_group_leaf_rows, lrows);
            b->groups.push_back(std::move(gr));
        }
    }
    std::vector<int2> tiles;
    for (messi_batch::Group& gr : b->groups) {
        gr.tile_off.assign(gr.H + 1, 0);
        gr.tile_cnt.assign(gr.H + 1, 0);
        gr.rtile_off.assign(gr.H + 1, 0);
        gr.rtile_cnt.assign(gr.H + 1, 0);
        for (int lv = 1; lv <= gr.H; lv++) {
            gr.tile_off[lv] = (int)tiles.size();
            for (int a = gr.a0; a < gr.a1; a++) {
                const messi_dataset* d = b->ds[a];
                if (lv >= d->H) continue;
                for (int v : d->level_nodes[lv])
                    for (int64_t s = 0; s < d->nunique[v]; s += kTile)
                        tiles.push_back(make_int2(b->node_base[a] + v, (int)s));
            }
            gr.tile_cnt[lv] = (int)tiles.size() - gr.tile_off[lv];
            gr.rtile_off[lv] = (int)tiles.size();
            for (int a = gr.a0; a < gr.a1; a++) {
                const messi_dataset* d = b->ds[a];
                if (lv != d->H) continue;
                for (int64_t s = 0; s < d->nunique[0]; s += kTile) tiles.push_back(make_int2(b->node_base[a], (int)s));
            }
            gr.rtile_cnt[lv] = (int)tiles.size() - gr.rtile_off[lv];
        }
    }
    if (tiles.empty()) tiles.push_back(make_int2(0, 0));
    cudaError_t e = cudaMalloc((void**)&b->d_tiles, tiles.size() * sizeof(int2));
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_tiles, tiles.data(), tiles.size() * sizeof(int2), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_nodes, sizeof(NodeDev) * std::max(1, b->total_nodes));
    {
        // leaf rows of all alignments and their global node ids
        const size_t R = (size_t)std::max<int64_t>(b->total_leaf_rows, 1);
        std::vector<float> rows(R * 16, 0.f);
        std::vector<int> rownode(R, 0);
        for (int a = 0; a < n; a++) {
            const messi_dataset* d = b->ds[a];
            std::copy(d->leaf_host.begin(), d->leaf_host.begin() + (size_t)d->leaf_rows * 16,
                      rows.begin() + (size_t)b->leaf_base[a] * 16);
            for (int64_t r = 0; r < d->leaf_rows; r++) rownode[b->leaf_base[a] + r] = b->node_base[a] + d->leafnode_host[r];
        }
        if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_leafrows, R * 16 * sizeof(float));
        if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_leafnode, R * sizeof(int));
        if (e == cudaSuccess) e = cudaMemcpy(b->d_leafrows, rows.data(), R * 16 * sizeof(float), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(b->d_leafnode, rownode.data(), R * sizeof(int), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        destroy_batch(b);
        return cuda_fail(ctx, e, "batch upload");
    }
    std::vector<int> Ls(n), Wbs(n);
    for (int a = 0; a < n; a++) {
        Ls[a] = b->ds[a]->L;
        Wbs[a] = std::max(0, std::min(b->ds[a]->W, b->ds[a]->L - 1));
    }
    std::string err;
    if ((rc = bandbatch_alloc(Ls, Wbs, &b->bands, &err))) {
        destroy_batch(b);
        return fail(ctx, rc, err);
    }
    *out = b;
    return MESSI_OK;
}

int messi_batch_destroy(messi_batch* b)
{
    if (!b) return MESSI_EINVAL;
    if (b->ctx) {
        cudaSetDevice(b->ctx->device);
        cudaStreamSynchronize(b->ctx->stream);
        tune_forget(b->ctx, b);
    }
    destroy_batch(b);
    return MESSI_OK;
}

int messi_batch_stats(messi_batch* b, int64_t* out, int32_t nout)
{
    if (!b || !out || nout < 0) return MESSI_EINVAL;
    const int64_t v[8] = {b->band_pairs, b->nroot, b->executed, b->naive, b->H, b->total_rows, b->chunk,
                          b->total_nodes};
    for (int k = 0; k < nout && k < 8; k++) out[k] = v[k];
    return MESSI_OK;
}

int messi_batch_likelihood(messi_ctx* ctx, messi_batch* b, const messi_model* models, const double* gapfrequency,
                           double gapcutoff, double* Z)
{
    int rc = begin(ctx);
    if (rc) return rc;
    if (!b || !models || !Z) return fail(ctx, MESSI_EINVAL, "batch likelihood: null argument");
    if (b->ctx != ctx) return fail(ctx, MESSI_ESTATE, "batch likelihood: batch belongs to another context");
    const int n = b->n;
    // model groups
    std::vector<int> grp(n), reps;
    for (int a = 0; a < n; a++) {
        int g = -1;
        for (int k = 0; k < (int)reps.size() && g < 0; k++)
            if (same_parameters(models[a], models[reps[k]])) g = k;
        if (g < 0) {
            g = (int)reps.size();
            reps.push_back(a);
        }
        grp[a] = g;
    }
    const int G = (int)reps.size();
    std::vector<Categories> cats(G);
    // lambda = 1 categories are factorised when every model group leaves out
    // the same ones (the merged launches share one category list); the
    // models' eigensystems are built on the host threads, one model per
    // thread (256 models of 36 categories are 9,216 16-state eigensystems)
    std::vector<int> rcs(G);
    std::vector<std::string> errs(G);
    for (int pass = 0; pass < 2; pass++) {
        const bool factorise = (pass == 0);
#pragma omp parallel for schedule(dynamic, 1) if (G >= 4)
        for (int g = 0; g < G; g++) {
            const int a = reps[g];
            rcs[g] = build_categories(&models[a], b->ds[a]->numnodes, &cats[g], &errs[g], true, factorise, G < 4);
        }
        bool same = true;
        for (int g = 0; g < G; g++) {
            if (rcs[g]) return fail(ctx, rcs[g], errs[g]);
            same = same && cats[g].lamF == cats[0].lamF;
        }
        if (same) break;
    }
    for (int g = 0; g < G; g++)
        if (cats[g].C != cats[0].C || cats[g].nsite != cats[0].nsite)
            return fail(ctx, MESSI_EINVAL, "batch likelihood: models must have the same category counts");
    for (int a = 0; a < n; a++)
        for (int v = 0; v < b->ds[a]->numnodes; v++)
            if (!models[a].branchlengths || !(models[a].branchlengths[v] >= 0.0) ||
                !std::isfinite(models[a].branchlengths[v]))
                return fail(ctx, MESSI_EINVAL, "batch likelihood: branch lengths must be finite and non-negative");
    const int C = cats[0].C, nsite = cats[0].nsite;
    // staged upload: eigensystems, category tables, branch lengths, node groups, gap masks
    std::vector<double> eig, eig4, logw, pi4, lws, bl(b->total_nodes), logwF(G);
    std::vector<float> pi16;
    std::vector<int> nodegrp(b->total_nodes);
    for (int g = 0; g < G; g++) {
        logwF[g] = cats[g].logwF;
        eig.insert(eig.end(), cats[g].eig.begin(), cats[g].eig.end());
        eig4.insert(eig4.end(), cats[g].eig4.begin(), cats[g].eig4.end());
        pi16.insert(pi16.end(), cats[g].pi16.begin(), cats[g].pi16.end());
        logw.insert(logw.end(), cats[g].logw.begin(), cats[g].logw.end());
        pi4.insert(pi4.end(), cats[g].pi4, cats[g].pi4 + 4);
        lws.insert(lws.end(), cats[g].logw_site.begin(), cats[g].logw_site.end());
    }
    for (int a = 0; a < n; a++)
        for (int v = 0; v < b->ds[a]->numnodes; v++) {
            bl[b->node_base[a] + v] = models[a].branchlengths[v];
            nodegrp[b->node_base[a] + v] = (v == 0) ? -1 : grp[a];
        }
    std::vector<uint8_t> gm;
    if (gapfrequency) {
        gm.resize(b->total_cols);
        for (int64_t k = 0; k < b->total_cols; k++) gm[k] = (gapfrequency[k] >= gapcutoff) ? 1 : 0;
    }
    Staged st;
    const size_t o_eig = st.add(eig.data(), eig.size());
    const size_t o_eig4 = st.add(eig4.data(), eig4.size());
    const size_t o_pi16 = st.add(pi16.data(), pi16.size());
    const size_t o_logw = st.add(logw.data(), logw.size());
    const size_t o_lam = st.add(cats[0].lam.data(), cats[0].lam.size());
    const size_t o_pi4 = st.add(pi4.data(), pi4.size());
    const size_t o_lws = st.add(lws.data(), lws.size());
    const size_t o_bl = st.add(bl.data(), bl.size());
    const size_t o_lwF = st.add(logwF.data(), logwF.size());
    const size_t o_grp = st.add(nodegrp.data(), nodegrp.size());
    const size_t o_gap = gapfrequency ? st.add(gm.data(), gm.size()) : 0;
    // ---- host staging and every allocation first
    void *pin, *dev, *pt, *p4, *ps;
    if ((rc = ensure_pinned(ctx, st.host.size(), &pin))) return rc;
    const void* old_stage = b->stage.p;
    const void* old_P = b->P16.p;
    const void* old_P4 = b->P4.p;
    if (grow(b->stage, st.host.size(), &dev)) return fail(ctx, MESSI_ENOMEM, "batch model staging");
    if (grow(b->P16, (size_t)C * b->total_nodes * 256 * sizeof(float), &pt))
        return fail(ctx, MESSI_ENOMEM, "batch transition matrices");
    if (grow(b->P4, (size_t)nsite * b->total_nodes * 16 * sizeof(double), &p4))
        return fail(ctx, MESSI_ENOMEM, "batch unpaired transition matrices");
    if (b->stage.p != old_stage || b->P16.p != old_P || b->P4.p != old_P4) b->gen++;
    {
        // unpaired scratch: one buffer sized for the largest alignment, reused in stream order
        size_t scratch = 0;
        for (int a = 0; a < n; a++)
            scratch = std::max(scratch, (size_t)nsite * ((size_t)b->ds[a]->numnodes * b->ds[a]->L * 5 + b->ds[a]->L));
        if ((rc = ensure(ctx, 20, scratch * sizeof(double), &ps))) return rc;
    }
    if ((rc = prepare_batch_arena(ctx, b, C))) return rc;
    if ((rc = write_descriptors(ctx, b, grp))) return rc;
    std::memcpy(pin, st.host.data(), st.host.size());
    char* base = (char*)dev;
    BatchStep step;
    step.stage_dev = dev;
    step.stage_host = pin;
    step.stage_bytes = st.host.size();
    step.eig = (const double*)(base + o_eig);
    step.eig4 = (const double*)(base + o_eig4);
    step.pi16 = (const float*)(base + o_pi16);
    step.logw = (const double*)(base + o_logw);
    step.lam = (const int*)(base + o_lam);
    step.pi4 = (const double*)(base + o_pi4);
    step.lws = (const double*)(base + o_lws);
    step.bl = (const double*)(base + o_bl);
    step.logwF = (const double*)(base + o_lwF);
    step.grp = (const int*)(base + o_grp);
    step.gap = gapfrequency ? (const uint8_t*)(base + o_gap) : nullptr;
    step.P = (float*)pt;
    step.P4 = (double*)p4;
    step.unpaired_scratch = (double*)ps;
    step.C = C;
    step.nsite = nsite;
    step.grp_of = &grp;
    step.cats = &cats;
    // ---- device work: replay a captured graph when the layout is unchanged
    tune_begin(ctx, b, C);
    messi_batch::Key key;
    key.C = C;
    key.G = G;
    key.nsite = nsite;
    key.lamF = cats[0].lamF;
    key.gap = gapfrequency != nullptr;
    key.staged = st.host.size();
    key.epoch = ctx->alloc_epoch;
    key.gen = b->gen;
    key.prune_shape = ctx->prune_shape;
    key.wave_threads = ctx->wave_threads;
    key.wave_ctas = ctx->wave_ctas;
    const bool graphs = ctx->graphs && !ctx->profiling && !ctx->tune_timing;
    bool replay = graphs && b->graph && b->graph_key == key;
    if (!replay && graphs && b->seen_key == key) replay = capture_batch(ctx, b, step, key);
    if (replay) {
        cudaError_t e = cudaGraphLaunch(b->graph, ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "batch graph launch");
        ctx->launches += b->graph_launches;
        ctx->graph_replays++;
    } else {
        if ((rc = enqueue_batch(ctx, b, step))) return rc;
        b->seen_key = key;
    }
    std::vector<double> zb(n);
    if ((rc = d2h(ctx, zb.data(), b->bands.d_Z, sizeof(double) * n))) return rc;
    rc = finish(ctx);
    tune_end(ctx, b, C);
    if (rc) return rc;
    for (int a = 0; a < n; a++) Z[a] = zb[b->bands.slot[a]];
    return MESSI_OK;
}

}  // extern "C"
