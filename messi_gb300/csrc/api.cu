// api.cu -- C ABI entry points (include/messi_gb300.h): contexts, dataset
// handles and the orchestration of each call on the context's stream.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstddef>
#include <cstring>
#include <new>

#include "internal.h"

namespace messi {

int fail(messi_ctx* ctx, int code, const std::string& msg)
{
    if (ctx) ctx->last_error = msg;
    return code;
}

int cuda_fail(messi_ctx* ctx, cudaError_t e, const char* what)
{
    return fail(ctx, (e == cudaErrorMemoryAllocation) ? MESSI_ENOMEM : MESSI_ECUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

int ensure(messi_ctx* ctx, int slot, size_t bytes, void** p)
{
    DevBuf& b = ctx->scratch[slot];
    if (bytes == 0) bytes = 16;
    if (b.bytes < bytes) {
        ctx->alloc_epoch++;
        if (b.p) cudaFree(b.p);
        b.p = nullptr;
        b.bytes = 0;
        cudaError_t e = cudaMalloc(&b.p, bytes);
        if (e != cudaSuccess) {
            b.p = nullptr;
            return cuda_fail(ctx, e, "scratch allocation");
        }
        b.bytes = bytes;
    }
    *p = b.p;
    return MESSI_OK;
}

int ensure_pinned(messi_ctx* ctx, size_t bytes, void** p)
{
    if (ctx->pinned_bytes < bytes) {
        ctx->alloc_epoch++;
        if (ctx->pinned) cudaFreeHost(ctx->pinned);
        ctx->pinned = nullptr;
        ctx->pinned_bytes = 0;
        cudaError_t e = cudaMallocHost(&ctx->pinned, bytes);
        if (e != cudaSuccess) {
            ctx->pinned = nullptr;
            return cuda_fail(ctx, e, "pinned staging allocation");
        }
        ctx->pinned_bytes = bytes;
    }
    *p = ctx->pinned;
    return MESSI_OK;
}

static cudaEvent_t prof_event(messi_ctx* ctx)
{
    if (!ctx->prof_pool.empty()) {
        cudaEvent_t e = ctx->prof_pool.back();
        ctx->prof_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

int prof_begin(messi_ctx* ctx, int kernel, double units)
{
    if (!ctx->profiling) return -1;
    ProfRec r{kernel, prof_event(ctx), prof_event(ctx), units};
    cudaEventRecord(r.a, ctx->stream);
    ctx->prof_pending.push_back(r);
    return (int)ctx->prof_pending.size() - 1;
}

void prof_end(messi_ctx* ctx)
{
    if (!ctx->profiling || ctx->prof_pending.empty()) return;
    cudaEventRecord(ctx->prof_pending.back().b, ctx->stream);
}

static void prof_collect(messi_ctx* ctx)
{
    for (ProfRec& r : ctx->prof_pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess && r.kernel >= 0 && r.kernel < kProfKernels) {
            ctx->prof_ms[r.kernel] += ms;
            ctx->prof_count[r.kernel] += 1;
            ctx->prof_units[r.kernel] += r.units;
        }
        ctx->prof_pool.push_back(r.a);
        ctx->prof_pool.push_back(r.b);
    }
    ctx->prof_pending.clear();
}

namespace {

// Scratch slots (grow-only, per context).  0..14 belong to the band tables.
enum Slot {
    kSlotStage = 15, kSlotP16 = 16, kSlotDense = 17, kSlotVec = 18, kSlotTable = 19, kSlotP4 = 21,
    kSlotDecodeF = 22, kSlotDecodeI = 23, kSlotCatLL = 24, kSlotCond = 25
};

struct ModelDev {
    Categories cat;
    float* P16 = nullptr;
    double* P4 = nullptr;
    float* pi16 = nullptr;
    double* logw = nullptr;
    int* lam = nullptr;
    double* pi4 = nullptr;
    double* logw_site = nullptr;
    uint8_t* gapmask = nullptr;
    double* logwF = nullptr;  // device copy of cat.logwF
    // staged copy (pinned -> device) and the transition-matrix builds, queued
    // by enqueue_model (separately, so that a captured graph can replay them)
    void* stage_host = nullptr;
    void* stage_dev = nullptr;
    size_t stage_bytes = 0;
    const double *eig = nullptr, *eig4 = nullptr, *bl = nullptr;
    bool pairs = false, unpaired = false;
};

// Queues the staged model's copy to the device and the transition-matrix
// builds on ctx->stream.
int enqueue_model(messi_ctx* ctx, messi_dataset* ds, ModelDev* md)
{
    int rc;
    cudaError_t e = cudaMemcpyAsync(md->stage_dev, md->stage_host, md->stage_bytes, cudaMemcpyHostToDevice,
                                    ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "model upload");
    if (md->pairs && (rc = launch_build_P16(ctx, md->eig, md->bl, nullptr, ds->numnodes, md->cat.C, md->P16)))
        return rc;
    if (md->unpaired && (rc = launch_build_P4(ctx, md->eig4, md->bl, nullptr, ds->numnodes, md->cat.nsite, md->P4)))
        return rc;
    return MESSI_OK;
}

// Builds categories on the host, stages them in pinned memory and (with
// enqueue) queues their upload and the transition-matrix builds.
// factorise: leave the lambda = 1 categories out of the 16-state pruning (the
// caller then adds md->cat.logwF + u[x] + u[y] to every pair mixture).
int upload_model(messi_ctx* ctx, messi_dataset* ds, const messi_model* m, bool pairs, bool unpaired,
                 const uint8_t* gapmask, ModelDev* md, bool factorise = false, bool enqueue = true)
{
    std::string err;
    int rc = build_categories(m, ds->numnodes, &md->cat, &err, pairs, factorise && pairs && unpaired);
    if (rc) return fail(ctx, rc, err);
    Categories& c = md->cat;
    Staged st;
    size_t o_eig = st.add(c.eig.data(), c.eig.size());
    size_t o_bl = st.add(m->branchlengths, (size_t)ds->numnodes);
    size_t o_pi16 = st.add(c.pi16.data(), c.pi16.size());
    size_t o_logw = st.add(c.logw.data(), c.logw.size());
    size_t o_lam = st.add(c.lam.data(), c.lam.size());
    size_t o_eig4 = st.add(c.eig4.data(), c.eig4.size());
    size_t o_pi4 = st.add(c.pi4, 4);
    size_t o_lws = st.add(c.logw_site.data(), c.logw_site.size());
    size_t o_lwF = st.add(&c.logwF, 1);
    size_t o_gap = gapmask ? st.add(gapmask, (size_t)ds->L) : 0;
    void *pin, *dev;
    if ((rc = ensure_pinned(ctx, st.host.size(), &pin))) return rc;
    if ((rc = ensure(ctx, kSlotStage, st.host.size(), &dev))) return rc;
    std::memcpy(pin, st.host.data(), st.host.size());
    md->stage_host = pin;
    md->stage_dev = dev;
    md->stage_bytes = st.host.size();
    md->pairs = pairs;
    md->unpaired = unpaired;
    char* base = (char*)dev;
    md->logwF = (double*)(base + o_lwF);
    md->pi16 = (float*)(base + o_pi16);
    md->logw = (double*)(base + o_logw);
    md->lam = (int*)(base + o_lam);
    md->pi4 = (double*)(base + o_pi4);
    md->logw_site = (double*)(base + o_lws);
    md->gapmask = gapmask ? (uint8_t*)(base + o_gap) : nullptr;
    md->bl = (const double*)(base + o_bl);
    md->eig = (const double*)(base + o_eig);
    md->eig4 = (const double*)(base + o_eig4);
    if (pairs) {
        void* p;
        if ((rc = ensure(ctx, kSlotP16, (size_t)c.C * ds->numnodes * 256 * sizeof(float), &p))) return rc;
        md->P16 = (float*)p;
    }
    if (unpaired) {
        void* p;
        if ((rc = ensure(ctx, kSlotP4, (size_t)c.nsite * ds->numnodes * 16 * sizeof(double), &p))) return rc;
        md->P4 = (double*)p;
    }
    return enqueue ? enqueue_model(ctx, ds, md) : MESSI_OK;
}

int prepare_arena(messi_ctx* ctx, messi_dataset* ds, int C)
{
    std::string err;
    if (ds->chunk == 0 || ds->arena_C != C) {
        int rc = allocate_arena(ds, C, &err);
        if (rc) return fail(ctx, rc, err);
        ds->arena_C = C;
    }
    return MESSI_OK;
}

}  // namespace

int finish(messi_ctx* ctx)
{
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "stream synchronize");
    if (!ctx->prof_pending.empty()) prof_collect(ctx);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(ctx, e, "kernel execution");
    if (ctx->status_host && *ctx->status_host != 0u)
        return fail(ctx, MESSI_ETIMEOUT, "wavefront grid barrier gave up waiting (bounded spin)");
    return MESSI_OK;
}

void tune_begin(messi_ctx* ctx, const void* key, int C)
{
    ctx->tune_timing = false;
    ctx->tune_saved[0] = ctx->prune_shape;
    ctx->tune_saved[1] = ctx->wave_threads;
    if (!ctx->autotune || (ctx->fixed_prune && ctx->fixed_wave) || ctx->profiling) return;
    TuneSlot& s = ctx->tune[std::make_pair(key, C)];
    if (s.done) {
        if (!ctx->fixed_prune) ctx->prune_shape = s.prune_shape;
        if (!ctx->fixed_wave) ctx->wave_threads = s.wave_threads;
    } else {
        if (!ctx->fixed_prune) ctx->prune_shape = s.k % kPruneShapes;
        if (!ctx->fixed_wave) ctx->wave_threads = kWaveThreadCands[s.k % kWaveCands];
        for (int i = 0; i < 4; i++)
            if (!ctx->tev[i]) cudaEventCreate(&ctx->tev[i]);
        ctx->tune_timing = true;
    }
}

void tune_mark(messi_ctx* ctx, int i)
{
    if (ctx->tune_timing) cudaEventRecord(ctx->tev[i], ctx->stream);
}

void tune_end(messi_ctx* ctx, const void* key, int C)
{
    // the shapes of this workload apply to this call only
    ctx->last_prune_shape = ctx->prune_shape;
    ctx->last_wave_threads = ctx->wave_threads;
    ctx->prune_shape = ctx->tune_saved[0];
    ctx->wave_threads = ctx->tune_saved[1];
    if (!ctx->tune_timing) return;
    ctx->tune_timing = false;
    TuneSlot& s = ctx->tune[std::make_pair(key, C)];
    float p = 0.f, w = 0.f;
    if (cudaEventElapsedTime(&p, ctx->tev[0], ctx->tev[1]) != cudaSuccess ||
        cudaEventElapsedTime(&w, ctx->tev[2], ctx->tev[3]) != cudaSuccess) {
        cudaGetLastError();
        s.done = true;  // timing unavailable: keep the defaults
        return;
    }
    s.prune_ms[s.k % kPruneShapes] = std::min(s.prune_ms[s.k % kPruneShapes], (double)p);
    s.wave_ms[s.k % kWaveCands] = std::min(s.wave_ms[s.k % kWaveCands], (double)w);
    if (++s.k < kTuneCalls) return;
    s.done = true;
    int bp = 0, bw = 0;
    for (int i = 1; i < kPruneShapes; i++)
        if (s.prune_ms[i] < s.prune_ms[bp]) bp = i;
    for (int i = 1; i < kWaveCands; i++)
        if (s.wave_ms[i] < s.wave_ms[bw]) bw = i;
    s.prune_shape = (s.prune_ms[bp] < 0.98 * s.prune_ms[0]) ? bp : 0;
    s.wave_threads = (s.wave_ms[bw] < 0.98 * s.wave_ms[0]) ? kWaveThreadCands[bw] : 0;
}

void tune_forget(messi_ctx* ctx, const void* key)
{
    for (auto it = ctx->tune.begin(); it != ctx->tune.end();)
        it = (it->first.first == key) ? ctx->tune.erase(it) : std::next(it);
}

int begin(messi_ctx* ctx)
{
    if (!ctx) return MESSI_EINVAL;
    ctx->launches = 0;
    ctx->last_error.clear();
    if (ctx->status_host) *ctx->status_host = 0u;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
    return MESSI_OK;
}

int h2d(messi_ctx* ctx, void* dst, const void* src, size_t bytes)
{
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
    return (e == cudaSuccess) ? MESSI_OK : cuda_fail(ctx, e, "host to device copy");
}

int d2h(messi_ctx* ctx, void* dst, const void* src, size_t bytes)
{
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    return (e == cudaSuccess) ? MESSI_OK : cuda_fail(ctx, e, "device to host copy");
}

int fork_side(messi_ctx* ctx)
{
    cudaError_t e = cudaEventRecord(ctx->fork_ev, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->side, ctx->fork_ev, 0);
    return (e == cudaSuccess) ? MESSI_OK : cuda_fail(ctx, e, "side stream fork");
}

int join_side(messi_ctx* ctx)
{
    cudaError_t e = cudaEventRecord(ctx->join_ev, ctx->side);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->stream, ctx->join_ev, 0);
    return (e == cudaSuccess) ? MESSI_OK : cuda_fail(ctx, e, "side stream join");
}

// Every device step of one likelihood evaluation after the host staging:
// model upload and transition matrices, unpaired columns and baselines on the
// side stream, pair pruning, banded pair scores, inside pass.
int enqueue_likelihood(messi_ctx* ctx, messi_dataset* ds, ModelDev& md, const Band& t)
{
    int rc;
    if ((rc = enqueue_model(ctx, ds, &md))) return rc;
    // the unpaired columns and the baselines do not need the pairs: they run
    // on the side stream under the pruning
    if ((rc = fork_side(ctx))) return rc;
    {
        SideLaunches side(ctx);
        if ((rc = launch_unpaired(ctx, ds, md.P4, ds->numnodes, md.pi4, md.logw_site, md.cat.nsite, t.u, nullptr)))
            return rc;
        if ((rc = launch_baseline(ctx, t, 1.0))) return rc;
    }
    tune_mark(ctx, 0);
    if ((rc = run_pairs(ctx, ds, md.P16, md.pi16, md.logw, md.lam, md.cat.C, md.cat.nlam, false))) return rc;
    tune_mark(ctx, 1);
    if ((rc = join_side(ctx))) return rc;
    if ((rc = launch_bandprep_from_mix(ctx, ds, t, md.gapmask, 1.0, md.cat.logwF, md.logwF))) return rc;
    tune_mark(ctx, 2);
    if ((rc = run_inside(ctx, t, 1.0))) return rc;
    tune_mark(ctx, 3);
    return MESSI_OK;
}

// Capture enqueue_likelihood into ctx->lgraph (key: what its pointers and
// launch shapes depend on).  On any capture error graphs are switched off for
// the context and the caller runs the steps eagerly.
bool capture_likelihood(messi_ctx* ctx, messi_dataset* ds, ModelDev& md, const Band& t, const LikelihoodKey& key)
{
    if (ctx->lgraph.exec) {
        cudaGraphExecDestroy(ctx->lgraph.exec);
        ctx->lgraph.exec = nullptr;
    }
    const int64_t l0 = ctx->launches;
    bool ok = false;
    if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        const int rc = enqueue_likelihood(ctx, ds, md, t);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
        cudaGraphExec_t ex = nullptr;
        if (rc == MESSI_OK && e == cudaSuccess && g && cudaGraphInstantiate(&ex, g, 0) == cudaSuccess) {
            ctx->lgraph.exec = ex;
            ctx->lgraph.key = key;
            ctx->lgraph.launches = ctx->launches - l0;
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

// Upload a dense L x L pair matrix, pick the band width, prepare the band.
int dense_pairs_to_band(messi_ctx* ctx, int L, const double* unpaired, const double* paired, int maxspan,
                        double B, bool outside, Band* t)
{
    int rc;
    void* p;
    if ((rc = ensure(ctx, kSlotDense, (size_t)L * L * sizeof(double), &p))) return rc;
    double* d_dense = (double*)p;
    if ((rc = h2d(ctx, d_dense, paired, (size_t)L * L * sizeof(double)))) return rc;
    int Wb = maxspan;
    if (maxspan < 0) {
        void* q;
        if ((rc = ensure(ctx, kSlotVec, 64, &q))) return rc;
        if ((rc = launch_maxspan(ctx, L, d_dense, (int*)q))) return rc;
        int host = 0;
        if ((rc = d2h(ctx, &host, q, sizeof(int)))) return rc;
        if ((rc = finish(ctx))) return rc;
        Wb = host;
    }
    Wb = std::max(0, std::min(Wb, L - 1));
    if ((rc = band_alloc(ctx, L, Wb, outside, t))) return rc;
    if ((rc = h2d(ctx, t->u, unpaired, (size_t)L * sizeof(double)))) return rc;
    if ((rc = launch_baseline(ctx, *t, B))) return rc;
    return launch_bandprep_from_dense(ctx, *t, d_dense, B);
}

}  // namespace messi

using namespace messi;

extern "C" {

const char* messi_strerror(int status)
{
    switch (status) {
        case MESSI_OK: return "ok";
        case MESSI_EINVAL: return "invalid argument";
        case MESSI_ENOMEM: return "out of memory";
        case MESSI_ECUDA: return "CUDA error";
        case MESSI_ETIMEOUT: return "bounded device wait timed out";
        case MESSI_ESTATE: return "object used in the wrong state";
        case MESSI_ETOOBIG: return "problem exceeds the fixed scratch size of this entry point";
        default: return "unknown status";
    }
}

int messi_version(void) { return 100; }

int messi_ctx_create(int device, messi_ctx** out)
{
    if (!out) return MESSI_EINVAL;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return MESSI_ECUDA;
    if (device < 0 || device >= n) return MESSI_EINVAL;
    messi_ctx* ctx = new (std::nothrow) messi_ctx();
    if (!ctx) return MESSI_ENOMEM;
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) !=
                                                    cudaSuccess) {
        delete ctx;
        return MESSI_ECUDA;
    }
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->join_ev, cudaEventDisableTiming) != cudaSuccess) {
        if (ctx->fork_ev) cudaEventDestroy(ctx->fork_ev);
        if (ctx->side) cudaStreamDestroy(ctx->side);
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return MESSI_ECUDA;
    }
    if (cudaMallocHost((void**)&ctx->status_host, 64) != cudaSuccess) {
        cudaEventDestroy(ctx->fork_ev);
        cudaEventDestroy(ctx->join_ev);
        cudaStreamDestroy(ctx->side);
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return MESSI_ENOMEM;
    }
    *ctx->status_host = 0u;
    {
        const char* w = std::getenv("MESSI_WAVE_CTAS");
        if (w) ctx->wave_ctas = std::max(0, std::atoi(w));
        const char* wt = std::getenv("MESSI_WAVE_THREADS");
        if (wt) {
            ctx->wave_threads = std::atoi(wt);
            ctx->fixed_wave = true;
        }
        const char* gr = std::getenv("MESSI_GRAPHS");
        if (gr && std::atoi(gr) == 0) ctx->graphs = false;
        const char* ps = std::getenv("MESSI_PRUNE_SHAPE");
        if (ps) {
            const int v = std::atoi(ps);
            ctx->prune_shape = (v >= 0 && v <= 3) ? v : 0;
            ctx->fixed_prune = true;
        }
        const char* at = std::getenv("MESSI_AUTOTUNE");
        if (at && std::atoi(at) == 0) ctx->autotune = false;
    }
    *out = ctx;
    return MESSI_OK;
}

int messi_ctx_profile(messi_ctx* ctx, int enable)
{
    if (!ctx) return MESSI_EINVAL;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    prof_collect(ctx);
    ctx->profiling = enable != 0;
    for (int k = 0; k < kProfKernels; k++) {
        ctx->prof_ms[k] = 0.0;
        ctx->prof_count[k] = 0;
        ctx->prof_units[k] = 0.0;
    }
    return MESSI_OK;
}

int messi_ctx_profile_read(messi_ctx* ctx, int kernel, double* total_ms, int64_t* launches, double* units)
{
    if (!ctx || kernel < 0 || kernel >= kProfKernels) return MESSI_EINVAL;
    if (total_ms) *total_ms = ctx->prof_ms[kernel];
    if (launches) *launches = ctx->prof_count[kernel];
    if (units) *units = ctx->prof_units[kernel];
    return MESSI_OK;
}

int messi_ctx_destroy(messi_ctx* ctx)
{
    if (!ctx) return MESSI_EINVAL;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    prof_collect(ctx);
    for (cudaEvent_t e : ctx->prof_pool) cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->tev)
        if (e) cudaEventDestroy(e);
    for (auto& b : ctx->scratch)
        if (b.p) cudaFree(b.p);
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    if (ctx->status_host) cudaFreeHost(ctx->status_host);
    if (ctx->lgraph.exec) cudaGraphExecDestroy(ctx->lgraph.exec);
    cudaStreamSynchronize(ctx->side);
    cudaEventDestroy(ctx->fork_ev);
    cudaEventDestroy(ctx->join_ev);
    cudaStreamDestroy(ctx->side);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return MESSI_OK;
}

int messi_ctx_stream(messi_ctx* ctx, void** stream)
{
    if (!ctx || !stream) return MESSI_EINVAL;
    *stream = (void*)ctx->stream;
    return MESSI_OK;
}

int messi_ctx_graph_replays(messi_ctx* ctx, int64_t* replays)
{
    if (!ctx || !replays) return MESSI_EINVAL;
    *replays = ctx->graph_replays;
    return MESSI_OK;
}

int messi_selftest_bounded_wait(messi_ctx* ctx, int32_t* status)
{
    int rc = begin(ctx);
    if (rc) return rc;
    if (!status) return fail(ctx, MESSI_EINVAL, "bounded-wait self-test: null argument");
    void* p;
    if ((rc = ensure(ctx, kSlotVec, kSyncWords * sizeof(unsigned int), &p))) return rc;
    unsigned int flag = 0;
    if ((rc = launch_barrier_selftest(ctx, (unsigned int*)p))) return rc;
    if ((rc = d2h(ctx, &flag, (unsigned int*)p + 2, sizeof(unsigned int)))) return rc;
    if ((rc = finish(ctx))) return rc;
    *status = flag ? MESSI_ETIMEOUT : MESSI_OK;
    return MESSI_OK;
}

int messi_host_reversible_eig(int32_t n, const double* Q, const double* pi, double* w, double* U)
{
    if (n < 1 || n > 16 || !Q || !pi || !w || !U) return MESSI_EINVAL;
    return host_reversible_eig(n, Q, pi, w, U);
}

int messi_ctx_launch_shapes(messi_ctx* ctx, int32_t* prune_shape, int32_t* wave_threads, int32_t* tuned)
{
    if (!ctx) return MESSI_EINVAL;
    if (prune_shape) *prune_shape = ctx->last_prune_shape;
    if (wave_threads) *wave_threads = ctx->last_wave_threads;
    if (tuned) {
        int n = 0;
        for (const auto& kv : ctx->tune) n += kv.second.done ? 1 : 0;
        *tuned = n;
    }
    return MESSI_OK;
}

int messi_ctx_last_launches(messi_ctx* ctx, int64_t* launches)
{
    if (!ctx || !launches) return MESSI_EINVAL;
    *launches = ctx->launches;
    return MESSI_OK;
}

const char* messi_ctx_last_error(messi_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "no context"; }

int messi_dataset_create(messi_ctx* ctx, const messi_alignment* aln, int32_t maxbasepairdistance,
                         const uint8_t* pairmask, messi_dataset** out)
{
    int rc = begin(ctx);
    if (rc) return rc;
    if (!aln || !out) return fail(ctx, MESSI_EINVAL, "dataset: null argument");
    *out = nullptr;
    messi_dataset* ds = new (std::nothrow) messi_dataset();
    if (!ds) return fail(ctx, MESSI_ENOMEM, "dataset: host allocation");
    ds->ctx = ctx;
    std::string err;
    rc = build_plan(ds, aln, maxbasepairdistance, pairmask, &err);
    if (rc) {
        messi_dataset_destroy(ds);
        return fail(ctx, rc, err);
    }
    *out = ds;
    return MESSI_OK;
}

int messi_dataset_destroy(messi_dataset* ds)
{
    if (!ds) return MESSI_EINVAL;
    if (ds->ctx) {
        messi_ctx* ctx = ds->ctx;
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        // a captured graph holds this dataset's pointers, and a later dataset
        // may be allocated at the same address: drop it with the dataset
        if (ctx->lgraph.key.ds == ds || ctx->lgraph.seen.ds == ds) {
            if (ctx->lgraph.exec) cudaGraphExecDestroy(ctx->lgraph.exec);
            ctx->lgraph = LikelihoodGraph{};
        }
        tune_forget(ctx, ds);
    }
    void* bufs[] = {ds->d_bandidx, ds->d_lr, ds->d_leaf, ds->d_nodes, ds->d_tiles, ds->d_masks, ds->d_tree,
                    ds->d_post, ds->d_arena_f, ds->d_arena_e, ds->d_mix, ds->d_mixlam, ds->d_leafnode,
                    ds->d_leafmsg};
    for (void* b : bufs)
        if (b) cudaFree(b);
    delete ds;
    return MESSI_OK;
}

int messi_dataset_stats(messi_dataset* ds, int64_t* out, int32_t n)
{
    if (!ds || !out || n < 0) return MESSI_EINVAL;
    const int64_t v[7] = {ds->band_pairs, ds->nroot, ds->executed, ds->naive, ds->H, ds->arena_rows, ds->chunk};
    for (int k = 0; k < n && k < 7; k++) out[k] = v[k];
    return MESSI_OK;
}

int messi_felsenstein_pairs(messi_ctx* ctx, messi_dataset* ds, const messi_model* model, double* pairedlogprobs,
                            double* museconditionals)
{
    int rc = begin(ctx);
    if (rc) return rc;
    if (!ds || !model || !pairedlogprobs) return fail(ctx, MESSI_EINVAL, "felsenstein_pairs: null argument");
    ModelDev md;
    if ((rc = upload_model(ctx, ds, model, true, true, nullptr, &md, true))) return rc;
    if ((rc = prepare_arena(ctx, ds, md.cat.C))) return rc;
    void *p, *pu;
    const size_t LL = (size_t)ds->L * ds->L;
    if ((rc = ensure(ctx, kSlotDense, LL * sizeof(double), &p))) return rc;
    double* d_dense = (double*)p;
    double* d_u = nullptr;
    if (md.cat.lamF) {  // unpaired columns for the factorised lambda categories, under the pruning
        if ((rc = ensure(ctx, kSlotVec, (size_t)ds->L * sizeof(double), &pu))) return rc;
        d_u = (double*)pu;
        if ((rc = fork_side(ctx))) return rc;
        SideLaunches side(ctx);
        if ((rc = launch_unpaired(ctx, ds, md.P4, ds->numnodes, md.pi4, md.logw_site, md.cat.nsite, d_u, nullptr)))
            return rc;
    }
    if ((rc = run_pairs(ctx, ds, md.P16, md.pi16, md.logw, md.lam, md.cat.C, md.cat.nlam, museconditionals != nullptr)))
        return rc;
    if (md.cat.lamF && (rc = join_side(ctx))) return rc;
    if ((rc = launch_scatter_dense(ctx, ds, ds->d_mix, d_u, md.cat.logwF, d_dense))) return rc;
    if ((rc = d2h(ctx, pairedlogprobs, d_dense, LL * sizeof(double)))) return rc;
    if (museconditionals) {
        // one L x L matrix per lambda category; the copy of the previous one
        // must finish before the buffer is reused (same stream: ordered)
        for (int l = 0; l < md.cat.nlam; l++) {
            const bool fl = (md.cat.lamF >> l) & 1u;
            if ((rc = launch_scatter_dense(ctx, ds, fl ? nullptr : ds->d_mixlam + (size_t)l * ds->nroot, d_u,
                                           fl ? md.cat.logw_lam[l] : -INFINITY, d_dense)))
                return rc;
            if ((rc = d2h(ctx, museconditionals + (size_t)l * LL, d_dense, LL * sizeof(double)))) return rc;
        }
    }
    return finish(ctx);
}

int messi_siterate_conditionals(messi_ctx* ctx, messi_dataset* ds, const messi_model* model,
                                const double* singleprobs, const double* pairprobs, double* conditionals)
{
    int rc = begin(ctx);
    if (rc) return rc;
    if (!ds || !model || !singleprobs || !pairprobs || !conditionals)
        return fail(ctx, MESSI_EINVAL, "site-rate conditionals: null argument");
    ModelDev md;
    if ((rc = upload_model(ctx, ds, model, true, true, nullptr, &md))) return rc;
    if ((rc = prepare_arena(ctx, ds, md.cat.C))) return rc;
    const int L = ds->L, C = md.cat.C, ns = md.cat.nsite;
    void *pc, *pv;
    if ((rc = ensure(ctx, kSlotCatLL, (size_t)C * std::max<int64_t>(ds->nroot, 1) * sizeof(double), &pc))) return rc;
    if ((rc = ensure(ctx, kSlotCond, ((size_t)L * L + (size_t)L * (ns + 1)) * sizeof(double), &pv))) return rc;
    double* d_catll = (double*)pc;
    double* d_pair = (double*)pv;
    double* d_single = d_pair + (size_t)L * L;
    double* d_out = d_single + L;
    // the root descriptor writes per-category values for this call only
    double* on = d_catll;
    double* off = nullptr;
    const size_t field = offsetof(NodeDev, catll);
    cudaError_t e = cudaMemcpyAsync((char*)ds->d_nodes + field, &on, sizeof(double*), cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "root descriptor");
    rc = run_pairs(ctx, ds, md.P16, md.pi16, md.logw, md.lam, C, md.cat.nlam, false);
    e = cudaMemcpyAsync((char*)ds->d_nodes + field, &off, sizeof(double*), cudaMemcpyHostToDevice, ctx->stream);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "root descriptor");
    void* pu;
    if ((rc = ensure(ctx, kSlotVec, (size_t)L * sizeof(double), &pu))) return rc;
    if ((rc = launch_unpaired(ctx, ds, md.P4, ds->numnodes, md.pi4, md.logw_site, ns, (double*)pu, nullptr)))
        return rc;
    // per-site unpaired log-likelihoods: the last block of the unpaired scratch
    const size_t n = (size_t)ds->numnodes * L;
    const double* d_ull = (const double*)ctx->scratch[20].p + (size_t)ns * n * 5;
    if ((rc = h2d(ctx, d_pair, pairprobs, (size_t)L * L * sizeof(double)))) return rc;
    if ((rc = h2d(ctx, d_single, singleprobs, (size_t)L * sizeof(double)))) return rc;
    if ((rc = launch_siterate_conditionals(ctx, ds, d_catll, md.logw, ns, md.cat.nlam, d_single, d_pair, d_ull,
                                           md.logw_site, d_out)))
        return rc;
    if ((rc = d2h(ctx, conditionals, d_out, (size_t)L * ns * sizeof(double)))) return rc;
    return finish(ctx);
}

int messi_subcolumnrefs(messi_ctx* ctx, messi_dataset* ds, int32_t* subcolumnrefs)
{
    int rc = begin(ctx);
    if (rc) return rc;
    if (!ds || !subcolumnrefs) return fail(ctx, MESSI_EINVAL, "subcolumnrefs: null argument");
    const size_t n = (size_t)ds->numnodes * ds->L;
    const size_t work = subcolumnrefs_work_bytes(ds);
    void *pr, *pw;
    if ((rc = ensure(ctx, kSlotCond, 2 * n * sizeof(int32_t), &pr))) return rc;
    if ((rc = ensure(ctx, kSlotCatLL, work, &pw))) return rc;
    int* d_refs = (int*)pr;
    int* d_out = d_refs + n;
    if ((rc = run_subcolumnrefs(ctx, ds, d_refs, d_out, pw, work))) return rc;
    if ((rc = d2h(ctx, subcolumnrefs, d_out, n * sizeof(int32_t)))) return rc;
    return finish(ctx);
}

int messi_unpaired(messi_ctx* ctx, messi_dataset* ds, const messi_model* model, double* unpairedlogprobs)
{
    int rc = begin(ctx);
    if (rc) return rc;
    if (!ds || !model || !unpairedlogprobs) return fail(ctx, MESSI_EINVAL, "unpaired: null argument");
    ModelDev md;
    if ((rc = upload_model(ctx, ds, model, false, true, nullptr, &md))) return rc;
    void* p;
    if ((rc = ensure(ctx, kSlotVec, (size_t)ds->L * sizeof(double), &p))) return rc;
    if ((rc = launch_unpaired(ctx, ds, md.P4, ds->numnodes, md.pi4, md.logw_site, md.cat.nsite, (double*)p, nullptr))) return rc;
    if ((rc = d2h(ctx, unpairedlogprobs, p, (size_t)ds->L * sizeof(double)))) return rc;
    return finish(ctx);
}

int messi_likelihood(messi_ctx* ctx, messi_dataset* ds, const messi_model* model, const double* gapfrequency,
                     double gapcutoff, double* Z, double* unpaired)
{
    int rc = begin(ctx);
    if (rc) return rc;
    if (!ds || !model || !Z) return fail(ctx, MESSI_EINVAL, "likelihood: null argument");
    std::vector<uint8_t> gm;
    if (gapfrequency) {
        gm.resize(ds->L);
        for (int i = 0; i < ds->L; i++) gm[i] = (gapfrequency[i] >= gapcutoff) ? 1 : 0;
    }
    // host staging and every allocation first; the device steps are then one
    // replayable sequence (a CUDA graph from the second identical call on)
    ModelDev md;
    if ((rc = upload_model(ctx, ds, model, true, true, gapfrequency ? gm.data() : nullptr, &md, true, false)))
        return rc;
    if ((rc = prepare_arena(ctx, ds, md.cat.C))) return rc;
    Band t;
    const int Wb = std::max(0, std::min(ds->W, ds->L - 1));
    if ((rc = band_alloc(ctx, ds->L, Wb, false, &t))) return rc;
    tune_begin(ctx, ds, md.cat.C);
    LikelihoodKey key;
    key.ds = ds;
    key.C = md.cat.C;
    key.nsite = md.cat.nsite;
    key.nlam = md.cat.nlam;
    key.Wb = Wb;
    key.lamF = md.cat.lamF;
    key.gapmask = gapfrequency != nullptr;
    key.staged = md.stage_bytes;
    key.epoch = ctx->alloc_epoch;
    key.arena_gen = ds->arena_gen;
    key.wave_ctas = ctx->wave_ctas;
    key.wave_threads = ctx->wave_threads;
    key.prune_shape = ctx->prune_shape;
    const bool graphs = ctx->graphs && !ctx->profiling && !ctx->tune_timing;
    bool replay = graphs && ctx->lgraph.exec && ctx->lgraph.key == key;
    if (!replay && graphs && ctx->lgraph.seen == key) replay = capture_likelihood(ctx, ds, md, t, key);
    if (replay) {
        cudaError_t e = cudaGraphLaunch(ctx->lgraph.exec, ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "likelihood graph launch");
        ctx->launches += ctx->lgraph.launches;
        ctx->graph_replays++;
    } else {
        if ((rc = enqueue_likelihood(ctx, ds, md, t))) return rc;
        ctx->lgraph.seen = key;
    }
    if ((rc = d2h(ctx, Z, t.Zd, sizeof(double)))) return rc;
    if (unpaired && (rc = d2h(ctx, unpaired, t.u, (size_t)ds->L * sizeof(double)))) return rc;
    rc = finish(ctx);
    tune_end(ctx, ds, md.cat.C);
    return rc;
}

int messi_inside(messi_ctx* ctx, int32_t L, const double* unpaired, const double* paired, int32_t maxspan, double B,
                 double* Z, double* inside)
{
    int rc = begin(ctx);
    if (rc) return rc;
    if (L < 1 || !unpaired || !paired || !Z) return fail(ctx, MESSI_EINVAL, "inside: bad arguments");
    Band t;
    if ((rc = dense_pairs_to_band(ctx, L, unpaired, paired, maxspan, B, false, &t))) return rc;
    if ((rc = run_inside(ctx, t, B))) return rc;
    if ((rc = d2h(ctx, Z, t.Zd, sizeof(double)))) return rc;
    if (inside) {
        void* p;
        const size_t bytes = (size_t)3 * L * L * sizeof(double);
        if ((rc = ensure(ctx, kSlotTable, bytes, &p))) return rc;
        if ((rc = launch_dense_inside(ctx, t, (double*)p))) return rc;
        if ((rc = d2h(ctx, inside, p, bytes))) return rc;
    }
    return finish(ctx);
}

int messi_outside(messi_ctx* ctx, int32_t L, const double* inside, const double* unpaired, const double* paired,
                  int32_t maxspan, double* outside)
{
    int rc = begin(ctx);
    if (rc) return rc;
    if (L < 1 || !inside || !unpaired || !paired || !outside) return fail(ctx, MESSI_EINVAL, "outside: bad arguments");
    Band t;
    if ((rc = dense_pairs_to_band(ctx, L, unpaired, paired, maxspan, 1.0, true, &t))) return rc;
    void* p;
    const size_t bytes = (size_t)3 * L * L * sizeof(double);
    if ((rc = ensure(ctx, kSlotTable, bytes, &p))) return rc;
    if ((rc = h2d(ctx, p, inside, bytes))) return rc;
    if ((rc = launch_band_from_dense_inside(ctx, t, (const double*)p))) return rc;
    if ((rc = run_outside(ctx, t, 1.0))) return rc;
    if ((rc = launch_dense_outside(ctx, t, (double*)p))) return rc;
    if ((rc = d2h(ctx, outside, p, bytes))) return rc;
    return finish(ctx);
}

int messi_basepairprobs(messi_ctx* ctx, int32_t L, const double* inside, const double* outside,
                        const double* unpaired, const double* paired, int32_t maxspan, double* single,
                        double* pairprobs)
{
    int rc = begin(ctx);
    if (rc) return rc;
    if (L < 1 || !inside || !outside || !unpaired || !paired || !single || !pairprobs)
        return fail(ctx, MESSI_EINVAL, "basepairprobs: bad arguments");
    Band t;
    if ((rc = dense_pairs_to_band(ctx, L, unpaired, paired, maxspan, 1.0, true, &t))) return rc;
    void* p;
    const size_t bytes = (size_t)3 * L * L * sizeof(double);
    if ((rc = ensure(ctx, kSlotTable, bytes, &p))) return rc;
    if ((rc = h2d(ctx, p, inside, bytes))) return rc;
    if ((rc = launch_band_from_dense_inside(ctx, t, (const double*)p))) return rc;
    if ((rc = h2d(ctx, p, outside, bytes))) return rc;
    if ((rc = launch_band_from_dense_outside(ctx, t, (const double*)p))) return rc;
    void *ds_single, *ds_pair;
    if ((rc = ensure(ctx, kSlotVec, (size_t)L * sizeof(double), &ds_single))) return rc;
    if ((rc = ensure(ctx, kSlotDense, (size_t)L * L * sizeof(double), &ds_pair))) return rc;
    if ((rc = run_posteriors(ctx, t, 1.0, (double*)ds_single, (double*)ds_pair))) return rc;
    if ((rc = d2h(ctx, single, ds_single, (size_t)L * sizeof(double)))) return rc;
    if ((rc = d2h(ctx, pairprobs, ds_pair, (size_t)L * L * sizeof(double)))) return rc;
    return finish(ctx);
}

}  // extern "C"

namespace {

// Posterior decoding of device-resident posteriors; copies the requested
// outputs to the host buffers (queued on the context stream).
int decode_device(messi_ctx* ctx, int L, const double* d_single, const double* d_pair, double alpha,
                  double* ematrix, int32_t* smatrix, int32_t* paired)
{
    int rc;
    void *work, *ints;
    const size_t LL = (size_t)L * L;
    if ((rc = ensure(ctx, kSlotDecodeF, ((size_t)L + 3 * LL) * sizeof(float), &work))) return rc;
    if ((rc = ensure(ctx, kSlotDecodeI, (LL + 3 * (size_t)L + 16 + kSyncWords) * sizeof(int), &ints))) return rc;
    int* scol = (int*)ints;
    int* stack = scol + LL;
    int* d_paired = stack + 2 * ((size_t)L + 1);
    unsigned int* sync = (unsigned int*)(d_paired + L);
    double* eout = nullptr;
    if (ematrix) {
        void* q;
        if ((rc = ensure(ctx, kSlotTable, LL * sizeof(double), &q))) return rc;
        eout = (double*)q;
    }
    if ((rc = run_posterior_decoding(ctx, L, d_single, d_pair, alpha, (float*)work, scol, sync,
                                     paired ? d_paired : nullptr, stack, eout)))
        return rc;
    if (ematrix && (rc = d2h(ctx, ematrix, eout, LL * sizeof(double)))) return rc;
    if (smatrix && (rc = d2h(ctx, smatrix, scol, LL * sizeof(int32_t)))) return rc;
    if (paired && (rc = d2h(ctx, paired, d_paired, (size_t)L * sizeof(int32_t)))) return rc;
    return MESSI_OK;
}

}  // namespace

extern "C" {

int messi_posterior_decoding(messi_ctx* ctx, int32_t L, const double* singleprobs, const double* pairprobs,
                             double alpha, double* ematrix, int32_t* smatrix, int32_t* paired)
{
    int rc = begin(ctx);
    if (rc) return rc;
    if (L < 1 || !singleprobs || !pairprobs || !(std::isfinite(alpha)))
        return fail(ctx, MESSI_EINVAL, "posterior decoding: bad arguments");
    if ((size_t)L * L > (size_t)1 << 31) return fail(ctx, MESSI_ETOOBIG, "posterior decoding: L*L above 2^31");
    void *ds, *dp;
    if ((rc = ensure(ctx, kSlotVec, (size_t)L * sizeof(double), &ds))) return rc;
    if ((rc = ensure(ctx, kSlotDense, (size_t)L * L * sizeof(double), &dp))) return rc;
    if ((rc = h2d(ctx, ds, singleprobs, (size_t)L * sizeof(double)))) return rc;
    if ((rc = h2d(ctx, dp, pairprobs, (size_t)L * L * sizeof(double)))) return rc;
    if ((rc = decode_device(ctx, L, (const double*)ds, (const double*)dp, alpha, ematrix, smatrix, paired)))
        return rc;
    return finish(ctx);
}

int messi_consensus_structure(messi_ctx* ctx, int32_t L, const double* unpaired, const double* paired,
                              int32_t maxspan, double alpha, int32_t* structure)
{
    int rc = begin(ctx);
    if (rc) return rc;
    if (L < 1 || !unpaired || !paired || !structure || !std::isfinite(alpha))
        return fail(ctx, MESSI_EINVAL, "consensus structure: bad arguments");
    if ((size_t)L * L > (size_t)1 << 31) return fail(ctx, MESSI_ETOOBIG, "consensus structure: L*L above 2^31");
    Band t;
    if ((rc = dense_pairs_to_band(ctx, L, unpaired, paired, maxspan, 1.0, true, &t))) return rc;
    if ((rc = run_inside(ctx, t, 1.0))) return rc;
    if ((rc = run_outside(ctx, t, 1.0))) return rc;
    void *ds_single, *ds_pair;
    if ((rc = ensure(ctx, kSlotVec, (size_t)L * sizeof(double), &ds_single))) return rc;
    if ((rc = ensure(ctx, kSlotDense, (size_t)L * L * sizeof(double), &ds_pair))) return rc;
    if ((rc = run_posteriors(ctx, t, 1.0, (double*)ds_single, (double*)ds_pair))) return rc;
    if ((rc = decode_device(ctx, L, (const double*)ds_single, (const double*)ds_pair, alpha, nullptr, nullptr,
                            structure)))
        return rc;
    return finish(ctx);
}

int messi_sample_structures(messi_ctx* ctx, int32_t L, const double* unpaired, const double* paired,
                            int32_t maxspan, int32_t nstruct, uint64_t seed, int32_t* structures, double* logprior)
{
    int rc = begin(ctx);
    if (rc) return rc;
    if (L < 1 || !unpaired || !paired || nstruct < 1 || !structures)
        return fail(ctx, MESSI_EINVAL, "sample structures: bad arguments");
    Band t;
    if ((rc = dense_pairs_to_band(ctx, L, unpaired, paired, maxspan, 1.0, false, &t))) return rc;
    if ((rc = run_inside(ctx, t, 1.0))) return rc;
    void* ints;
    const size_t per = (size_t)L + 3 * ((size_t)L + 1);
    if ((rc = ensure(ctx, kSlotDecodeI, (per * nstruct + 16) * sizeof(int), &ints))) return rc;
    int* d_out = (int*)ints;
    int* d_stack = d_out + (size_t)L * nstruct;
    unsigned int* d_status = (unsigned int*)(d_stack + 3 * ((size_t)L + 1) * nstruct);
    double* d_prior = nullptr;
    if (logprior) {
        void* pp;
        if ((rc = ensure(ctx, kSlotCond, (size_t)nstruct * sizeof(double), &pp))) return rc;
        d_prior = (double*)pp;
    }
    if ((rc = run_sample_structures(ctx, t, 1.0, nstruct, (unsigned long long)seed, d_out, d_stack, d_prior,
                                    d_status)))
        return rc;
    unsigned int status = 0;
    if ((rc = d2h(ctx, structures, d_out, (size_t)L * nstruct * sizeof(int32_t)))) return rc;
    if (logprior && (rc = d2h(ctx, logprior, d_prior, (size_t)nstruct * sizeof(double)))) return rc;
    if ((rc = d2h(ctx, &status, d_status, sizeof(unsigned int)))) return rc;
    if ((rc = finish(ctx))) return rc;
    if (status != 0u) return fail(ctx, MESSI_ESTATE, "sample structures: a span had no derivation (check the inputs)");
    return MESSI_OK;
}

int messi_structure_likelihood(messi_ctx* ctx, messi_dataset* ds, const messi_model* model, const int32_t* paired,
                               double* total, double* pairll, double* unpaired)
{
    int rc = begin(ctx);
    if (rc) return rc;
    if (!ds || !model || !paired || !total) return fail(ctx, MESSI_EINVAL, "structure likelihood: null argument");
    const int L = ds->L;
    std::vector<int2> pairs;
    std::vector<int32_t> col_pair(L, -1);
    for (int i = 0; i < L; i++) {
        const int k = paired[i];
        if (k < 0 || k > L || k == i + 1 || (k > 0 && paired[k - 1] != i + 1))
            return fail(ctx, MESSI_EINVAL, "structure likelihood: paired must hold symmetric 1-based partners or 0");
        if (k > i + 1) {
            col_pair[i] = (int32_t)pairs.size();
            pairs.push_back(make_int2(i, k - 1));
        }
    }
    // plan of exactly the structure's pairs (subtree-pattern dedup as for the band)
    messi_dataset* sub = nullptr;
    std::vector<int32_t> pu;
    if (!pairs.empty()) {
        sub = new (std::nothrow) messi_dataset();
        if (!sub) return fail(ctx, MESSI_ENOMEM, "structure likelihood: host allocation");
        sub->ctx = ctx;
        messi_alignment aln{ds->N, ds->L, ds->numnodes, ds->masks.data(), ds->children.data(), ds->seqindex.data()};
        std::string err;
        if ((rc = build_plan(sub, &aln, L - 1, nullptr, &err, &pairs, &pu))) {
            messi_dataset_destroy(sub);
            return fail(ctx, rc, err);
        }
    }
    auto done = [&](int code) {
        if (sub) messi_dataset_destroy(sub);
        return code;
    };
    ModelDev md;
    if ((rc = upload_model(ctx, ds, model, !pairs.empty(), true, nullptr, &md, true))) return done(rc);
    if (sub) {
        if ((rc = prepare_arena(ctx, sub, md.cat.C))) return done(rc);
        if ((rc = run_pairs(ctx, sub, md.P16, md.pi16, md.logw, md.lam, md.cat.C, md.cat.nlam, false)))
            return done(rc);
    }
    void *dv, *di;
    if ((rc = ensure(ctx, kSlotVec, (2 * (size_t)L + 8) * sizeof(double), &dv))) return done(rc);
    if ((rc = ensure(ctx, kSlotDecodeI, (2 * (size_t)L + 8) * sizeof(int32_t), &di))) return done(rc);
    double* d_u = (double*)dv;
    double* d_pairll = d_u + L;
    double* d_total = d_pairll + L;
    int32_t* d_col = (int32_t*)di;
    std::vector<int32_t> colu(2 * (size_t)L, -1);  // root pair ids, then 0-based partners
    for (int i = 0; i < L; i++) {
        if (col_pair[i] >= 0) colu[i] = pu[col_pair[i]];
        else if (paired[i] > 0) colu[i] = -2;
        colu[(size_t)L + i] = paired[i] - 1;
    }
    if ((rc = launch_unpaired(ctx, ds, md.P4, ds->numnodes, md.pi4, md.logw_site, md.cat.nsite, d_u, nullptr)))
        return done(rc);
    if ((rc = h2d(ctx, d_col, colu.data(), 2 * (size_t)L * sizeof(int32_t)))) return done(rc);
    if ((rc = launch_structure_sum(ctx, L, d_u, d_col, d_col + L, sub ? sub->d_mix : nullptr, md.cat.logwF, d_total,
                                   d_pairll)))
        return done(rc);
    if ((rc = d2h(ctx, total, d_total, sizeof(double)))) return done(rc);
    if (pairll && (rc = d2h(ctx, pairll, d_pairll, (size_t)L * sizeof(double)))) return done(rc);
    if (unpaired && (rc = d2h(ctx, unpaired, d_u, (size_t)L * sizeof(double)))) return done(rc);
    return done(finish(ctx));
}

int messi_posteriors(messi_ctx* ctx, int32_t L, const double* unpaired, const double* paired, int32_t maxspan,
                     double* Z, double* single, double* pairprobs)
{
    int rc = begin(ctx);
    if (rc) return rc;
    if (L < 1 || !unpaired || !paired || !single || !pairprobs)
        return fail(ctx, MESSI_EINVAL, "posteriors: bad arguments");
    Band t;
    if ((rc = dense_pairs_to_band(ctx, L, unpaired, paired, maxspan, 1.0, true, &t))) return rc;
    if ((rc = run_inside(ctx, t, 1.0))) return rc;
    if ((rc = run_outside(ctx, t, 1.0))) return rc;
    void *ds_single, *ds_pair;
    if ((rc = ensure(ctx, kSlotVec, (size_t)L * sizeof(double), &ds_single))) return rc;
    if ((rc = ensure(ctx, kSlotDense, (size_t)L * L * sizeof(double), &ds_pair))) return rc;
    if ((rc = run_posteriors(ctx, t, 1.0, (double*)ds_single, (double*)ds_pair))) return rc;
    if (Z && (rc = d2h(ctx, Z, t.Zd, sizeof(double)))) return rc;
    if ((rc = d2h(ctx, single, ds_single, (size_t)L * sizeof(double)))) return rc;
    if ((rc = d2h(ctx, pairprobs, ds_pair, (size_t)L * L * sizeof(double)))) return rc;
    return finish(ctx);
}

}  // extern "C"
