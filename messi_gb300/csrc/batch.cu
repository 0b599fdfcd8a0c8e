// batch.cu -- many alignments in one evaluation.
//
// The reference evaluates one alignment per call (src/FelsensteinCUDA.jl:214,
// src/InsideCUDA.jl:23, driven from src/FARCE.jl:2322-2345).  A batch keeps
// the per-alignment pair plans of plan.cpp and runs them together:
//   * pruning: the tree levels of all alignments are merged, so level l of
//     every tree is one launch (plus one for the roots that sit at level l);
//     all partial rows share one arena with a common category stride;
//   * transition matrices of every node of every tree come from one launch,
//     with one eigensystem set per distinct model (models that differ only
//     in their branch lengths share it);
//   * the inside passes of all alignments run in one persistent wavefront
//     (inside_wave_batch_kernel): diagonal d of every alignment whose band
//     reaches it is one step, so the number of grid barriers is the largest
//     band width in the batch instead of the sum over alignments.
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
    std::vector<int> tile_off, tile_cnt, rtile_off, rtile_cnt;  // per level: non-root and root tiles
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
    for (messi_dataset* d : b->ds)
        if (d) messi_dataset_destroy(d);
    void* bufs[] = {b->d_tiles, b->d_nodes, b->d_arena_f, b->d_arena_e, b->stage.p, b->P16.p, b->P4.p,
                    b->d_leafrows, b->d_leafnode, b->d_leafmsg};
    for (void* p : bufs)
        if (p) cudaFree(p);
    bandbatch_free(&b->bands);
    delete b;
}

// Partial-row arena of the whole batch for C categories (as many per pass as fit).
int prepare_batch_arena(messi_ctx* ctx, messi_batch* b, int C)
{
    if (b->chunk != 0 && b->arena_C == C) return MESSI_OK;
    size_t freeb = 0, totalb = 0;
    cudaMemGetInfo(&freeb, &totalb);
    const size_t row_bytes = 16 * sizeof(float) + sizeof(int);
    const int64_t leaf_rows = std::max<int64_t>(b->total_leaf_rows, 1);
    int chunk = C;
    while (chunk > 1 && (size_t)chunk * (b->total_rows + leaf_rows) * row_bytes > freeb / 2) chunk = (chunk + 1) / 2;
    if (b->d_arena_f) cudaFree(b->d_arena_f);
    if (b->d_arena_e) cudaFree(b->d_arena_e);
    if (b->d_leafmsg) cudaFree(b->d_leafmsg);
    b->d_arena_f = nullptr;
    b->d_arena_e = nullptr;
    b->d_leafmsg = nullptr;
    b->chunk = 0;
    cudaError_t e = cudaMalloc((void**)&b->d_arena_f, (size_t)chunk * b->total_rows * 16 * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_arena_e, (size_t)chunk * b->total_rows * sizeof(int));
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
    for (int a = 0; a < b->n; a++)
        fill_node_descriptors(b->ds[a], b->d_arena_f, b->d_arena_e, b->row_base[a], b->total_rows, b->d_leafmsg,
                              b->leaf_base[a], std::max<int64_t>(b->total_leaf_rows, 1), b->node_base[a], grp[a],
                              b->nodes_host.data() + b->node_base[a]);
    cudaError_t e = cudaMemcpyAsync(b->d_nodes, b->nodes_host.data(), sizeof(NodeDev) * b->total_nodes,
                                    cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "batch node descriptors");
    // the host copy must outlive the asynchronous copy: keep it until the next call
    b->desc_grp = grp;
    return MESSI_OK;
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
    std::vector<int2> tiles;
    b->tile_off.assign(b->H + 1, 0);
    b->tile_cnt.assign(b->H + 1, 0);
    b->rtile_off.assign(b->H + 1, 0);
    b->rtile_cnt.assign(b->H + 1, 0);
    for (int lv = 1; lv <= b->H; lv++) {
        b->tile_off[lv] = (int)tiles.size();
        for (int a = 0; a < n; a++) {
            const messi_dataset* d = b->ds[a];
            if (lv >= d->H) continue;
            for (int v : d->level_nodes[lv])
                for (int64_t s = 0; s < d->nunique[v]; s += kTile) tiles.push_back(make_int2(b->node_base[a] + v, (int)s));
        }
        b->tile_cnt[lv] = (int)tiles.size() - b->tile_off[lv];
        b->rtile_off[lv] = (int)tiles.size();
        for (int a = 0; a < n; a++) {
            const messi_dataset* d = b->ds[a];
            if (lv != d->H) continue;
            for (int64_t s = 0; s < d->nunique[0]; s += kTile) tiles.push_back(make_int2(b->node_base[a], (int)s));
        }
        b->rtile_cnt[lv] = (int)tiles.size() - b->rtile_off[lv];
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
    std::string err;
    // lambda = 1 categories are factorised when every model group leaves out
    // the same ones (the merged launches share one category list)
    for (int pass = 0; pass < 2; pass++) {
        const bool factorise = (pass == 0);
        bool same = true;
        for (int g = 0; g < G; g++) {
            const int a = reps[g];
            if ((rc = build_categories(&models[a], b->ds[a]->numnodes, &cats[g], &err, true, factorise)))
                return fail(ctx, rc, err);
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
    std::vector<double> eig, eig4, logw, pi4, lws, bl(b->total_nodes);
    std::vector<float> pi16;
    std::vector<int> nodegrp(b->total_nodes);
    for (int g = 0; g < G; g++) {
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
    const size_t o_grp = st.add(nodegrp.data(), nodegrp.size());
    const size_t o_gap = gapfrequency ? st.add(gm.data(), gm.size()) : 0;
    void *pin, *dev;
    if ((rc = ensure_pinned(ctx, st.host.size(), &pin))) return rc;
    if (grow(b->stage, st.host.size(), &dev)) return fail(ctx, MESSI_ENOMEM, "batch model staging");
    std::memcpy(pin, st.host.data(), st.host.size());
    if ((rc = h2d(ctx, dev, pin, st.host.size()))) return rc;
    char* base = (char*)dev;
    const float* d_pi16 = (const float*)(base + o_pi16);
    const double* d_logw = (const double*)(base + o_logw);
    const int* d_lam = (const int*)(base + o_lam);
    const double* d_pi4 = (const double*)(base + o_pi4);
    const double* d_lws = (const double*)(base + o_lws);
    const double* d_bl = (const double*)(base + o_bl);
    const int* d_grp = (const int*)(base + o_grp);
    const uint8_t* d_gap = gapfrequency ? (const uint8_t*)(base + o_gap) : nullptr;
    void *pt, *p4;
    if (grow(b->P16, (size_t)3 * C * b->total_nodes * 256 * sizeof(float), &pt))
        return fail(ctx, MESSI_ENOMEM, "batch transition matrices");
    if (grow(b->P4, (size_t)nsite * b->total_nodes * 16 * sizeof(double), &p4))
        return fail(ctx, MESSI_ENOMEM, "batch unpaired transition matrices");
    const float* d_P = (const float*)pt;
    if ((rc = launch_build_P16(ctx, (const double*)(base + o_eig), d_bl, d_grp, b->total_nodes, C, (float*)pt)))
        return rc;
    if ((rc = launch_build_P4(ctx, (const double*)(base + o_eig4), d_bl, d_grp, b->total_nodes, nsite,
                              (double*)p4)))
        return rc;
    if ((rc = prepare_batch_arena(ctx, b, C))) return rc;
    if ((rc = write_descriptors(ctx, b, grp))) return rc;
    // unpaired columns (one scratch buffer, sized for the largest alignment
    // and reused in stream order) and baselines do not need the pairs: they
    // run on the side stream under the pruning
    {
        size_t scratch = 0;
        for (int a = 0; a < n; a++)
            scratch = std::max(scratch, (size_t)nsite * ((size_t)b->ds[a]->numnodes * b->ds[a]->L * 5 + b->ds[a]->L));
        void* ps;
        if ((rc = ensure(ctx, 20, scratch * sizeof(double), &ps))) return rc;
        if ((rc = fork_side(ctx))) return rc;
        SideLaunches side(ctx);
        for (int a = 0; a < n; a++) {
            const Band& t = b->bands.host[b->bands.slot[a]];
            if ((rc = launch_unpaired(ctx, b->ds[a], (const double*)p4 + (size_t)b->node_base[a] * 16,
                                      b->total_nodes, d_pi4 + 4 * grp[a], d_lws + (size_t)nsite * grp[a], nsite,
                                      t.u, (double*)ps)))
                return rc;
        }
        if ((rc = launch_baseline_batch(ctx, b->bands, 1.0))) return rc;
    }
    // pair pruning over the merged levels
    for (int c0 = 0; c0 < C; c0 += b->chunk) {
        const int nc = std::min(b->chunk, C - c0);
        if ((rc = launch_leaf_messages(ctx, b->d_leafrows, b->d_leafnode, b->total_leaf_rows, d_P, b->total_nodes, c0,
                                       nc, C, b->d_leafmsg)))
            return rc;
        for (int lv = 1; lv <= b->H; lv++) {
            for (int root = 0; root < 2; root++) {
                const int nt = root ? b->rtile_cnt[lv] : b->tile_cnt[lv];
                if (nt == 0) continue;
                const int2* tl = b->d_tiles + (root ? b->rtile_off[lv] : b->tile_off[lv]);
                if (ctx->profiling) {
                    double units = 0.0;
                    for (int a = 0; a < n; a++) {
                        const messi_dataset* d = b->ds[a];
                        if (lv > d->H || (root != 0) != (lv == d->H)) continue;
                        for (int v : d->level_nodes[lv]) units += (double)d->nunique[v] * nc;
                    }
                    prof_begin(ctx, 0, units);
                }
                if ((rc = launch_prune_tiles(ctx, b->d_nodes, tl, nt, root != 0, d_P, b->total_nodes, c0, nc, C,
                                             d_pi16, d_logw, d_lam, false)))
                    return rc;
                prof_end(ctx);
            }
        }
    }
    // banded pair scores, batched inside
    if ((rc = join_side(ctx))) return rc;
    for (int a = 0; a < n; a++) {
        const Band& t = b->bands.host[b->bands.slot[a]];
        if ((rc = launch_bandprep_from_mix(ctx, b->ds[a], t, d_gap ? d_gap + b->col_base[a] : nullptr, 1.0,
                                           cats[grp[a]].logwF)))
            return rc;
    }
    if ((rc = run_inside_batch(ctx, b->bands, 1.0))) return rc;
    std::vector<double> zb(n);
    if ((rc = d2h(ctx, zb.data(), b->bands.d_Z, sizeof(double) * n))) return rc;
    if ((rc = finish(ctx))) return rc;
    for (int a = 0; a < n; a++) Z[a] = zb[b->bands.slot[a]];
    return MESSI_OK;
}

}  // extern "C"
