"""Reference-named host API over the C ABI.

Each function keeps the name, argument meaning and return value of the Julia
function it replaces (see the citations); the work runs in libmessi_gb300.so
on the GPU.  There is no CPU fallback: ``usecuda=False`` raises.

Matrices come back as Fortran-ordered numpy arrays (Julia's layout), so
``inside[X, i, j]`` and ``pairedlogprobs[x, y]`` index them like the
reference's arrays (0-based).
"""
import collections
import ctypes
import hashlib
import threading

import numpy as np

from . import _lib
from .model import computeprior, getmusespecificparamsarray

_tls = threading.local()


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Context:
    """One CUDA device and stream (replaces CuContext(CuDevice(0)) per call,
    src/FelsensteinCUDA.jl:240-241, src/InsideCUDA.jl:96-97)."""

    def __init__(self, device=0):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(self.lib.messi_ctx_create(int(device), ctypes.byref(h)), "messi_ctx_create")
        self.handle = h
        self.device = device
        self._datasets = collections.OrderedDict()

    def close(self):
        for ds in list(self._datasets.values()):
            ds.close()
        self._datasets.clear()
        if self.handle:
            self.lib.messi_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def stream(self):
        s = ctypes.c_void_p()
        _lib.check(self.lib.messi_ctx_stream(self.handle, ctypes.byref(s)), "messi_ctx_stream")
        return s.value

    def last_launches(self):
        n = ctypes.c_int64()
        _lib.check(self.lib.messi_ctx_last_launches(self.handle, ctypes.byref(n)), "messi_ctx_last_launches")
        return n.value

    def launch_shapes(self):
        """Shapes of the last likelihood evaluation and the number of
        workloads whose autotuning has finished (messi_ctx_launch_shapes)."""
        p, w, t = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        self.check(self.lib.messi_ctx_launch_shapes(self.handle, ctypes.byref(p), ctypes.byref(w), ctypes.byref(t)),
                   "messi_ctx_launch_shapes")
        return {"prune_shape": p.value, "wave_threads": w.value, "tuned_workloads": t.value}

    def graph_replays(self):
        """messi_likelihood calls whose device work replayed a captured CUDA graph."""
        n = ctypes.c_int64()
        self.check(self.lib.messi_ctx_graph_replays(self.handle, ctypes.byref(n)), "messi_ctx_graph_replays")
        return n.value

    def selftest_bounded_wait(self):
        """Status produced by a device wait that cannot complete (a grid
        barrier one CTA never reaches): MESSI_ETIMEOUT when the bounded wait
        gives up as designed.  The context stays usable."""
        st = ctypes.c_int32()
        self.check(self.lib.messi_selftest_bounded_wait(self.handle, ctypes.byref(st)), "messi_selftest_bounded_wait")
        return st.value

    def profile(self, enable=True):
        """Enable (and reset) per-kernel CUDA-event timing."""
        self.check(self.lib.messi_ctx_profile(self.handle, 1 if enable else 0), "messi_ctx_profile")

    def profile_read(self, kernel):
        """(total_ms, launches, units) for kernel family 0 = pair node update,
        1 = inside diagonals, 2 = inside suffix, 3 = outside diagonals."""
        ms, n, units = ctypes.c_double(), ctypes.c_int64(), ctypes.c_double()
        self.check(self.lib.messi_ctx_profile_read(self.handle, int(kernel), ctypes.byref(ms), ctypes.byref(n),
                                                   ctypes.byref(units)), "messi_ctx_profile_read")
        return ms.value, n.value, units.value

    def check(self, status, what):
        _lib.check(status, what, self.handle)

    # dataset handles kept (each holds its pair plan and message arena on the device)
    MAX_CACHED_DATASETS = 4

    def dataset(self, dataset, maxbasepairdistance=1000000, pairmask=None):
        """Cached dataset handle (the reference caches the pair index of its
        last dataset in process globals, src/FelsensteinCUDA.jl:206-238; here
        the cache key is the dataset, the band and the pair mask, and the
        MAX_CACHED_DATASETS most recently used handles are kept: an evicted
        handle is destroyed, so a loop over many alignments does not hold
        every alignment's device arena)."""
        W = int(min(max(1, maxbasepairdistance), max(1, dataset.numcols - 1)))
        mkey = None if pairmask is None else hashlib.sha1(np.ascontiguousarray(pairmask, np.uint8)).hexdigest()
        key = (id(dataset), W, mkey)
        h = self._datasets.get(key)
        if h is None or h.dataset is not dataset:
            if h is not None:  # id() reused by a new dataset object
                h.close()
                del self._datasets[key]
            while len(self._datasets) >= self.MAX_CACHED_DATASETS:
                _, old = self._datasets.popitem(last=False)
                old.close()
            h = DatasetHandle(self, dataset, W, pairmask)
            self._datasets[key] = h
        else:
            self._datasets.move_to_end(key)
        return h


def get_context(device=0):
    ctxs = getattr(_tls, "ctxs", None)
    if ctxs is None:
        ctxs = _tls.ctxs = {}
    c = ctxs.get(device)
    if c is None:
        c = ctxs[device] = Context(device)
    return c


class DatasetHandle:
    def __init__(self, ctx, dataset, W, pairmask=None):
        self.ctx = ctx
        self.dataset = dataset
        self.W = W
        self._masks = np.ascontiguousarray(dataset.masks, np.uint8)
        self._children = np.ascontiguousarray(dataset.children, np.int32)
        self._seqindex = np.ascontiguousarray(dataset.seqindex, np.int32)
        aln = _lib.Alignment(dataset.numseqs, dataset.numcols, dataset.numnodes, _p(self._masks), _p(self._children),
                             _p(self._seqindex))
        pm = None if pairmask is None else np.asfortranarray(pairmask, np.uint8)
        h = ctypes.c_void_p()
        ctx.check(ctx.lib.messi_dataset_create(ctx.handle, ctypes.byref(aln), int(W), _p(pm), ctypes.byref(h)),
                  "messi_dataset_create")
        self.handle = h

    def stats(self):
        out = np.zeros(7, np.int64)
        self.ctx.check(self.ctx.lib.messi_dataset_stats(self.handle, _p(out), 7), "messi_dataset_stats")
        keys = ("band_pairs", "unique_root_pairs", "executed_updates_per_category", "naive_updates_per_category",
                "levels", "arena_rows", "categories_per_pass")
        return dict(zip(keys, (int(x) for x in out)))

    def close(self):
        if self.handle:
            self.ctx.lib.messi_dataset_destroy(self.handle)
            self.handle = None


class ModelArgs:
    """messi_model built from ModelParameters (+ museparams), arrays kept alive."""

    def __init__(self, params, museparams=None, branchlengths=None):
        if museparams is None:
            museparams = getmusespecificparamsarray(params)
        k = np.array([mp.lambdacat - 1 for mp in museparams], dtype=np.int64)
        self.lGC = np.ascontiguousarray(np.asarray(params.lambdaratesGC, np.float64)[k] + 1.0)
        self.lAT = np.ascontiguousarray(np.asarray(params.lambdaratesAT, np.float64)[k] + 1.0)
        self.lGT = np.ascontiguousarray(np.asarray(params.lambdaratesGT, np.float64)[k] + 1.0)
        self.lw = np.ascontiguousarray([mp.prob for mp in museparams], np.float64)
        self.sr = np.ascontiguousarray(params.siteRates, np.float64)
        self.sw = np.ascontiguousarray(params.siteWeights, np.float64)
        bl = params.branchlengths if branchlengths is None else branchlengths
        self.bl = np.ascontiguousarray(bl, np.float64)
        m = _lib.Model()
        for a in range(4):
            m.freqs[a] = float(params.freqs[a])
        for a, qv in enumerate(params.q):
            m.q[a] = float(qv)
        m.branchlengths = _p(self.bl)
        m.nsite = len(self.sr)
        m.siteRates = _p(self.sr)
        m.siteWeights = _p(self.sw)
        m.nlambda = len(self.lw)
        m.lambdaGC, m.lambdaAT, m.lambdaGT = _p(self.lGC), _p(self.lAT), _p(self.lGT)
        m.lambdaWeights = _p(self.lw)
        self.struct = m

    def pruned_categories(self):
        """Categories the library prunes with 16 states in a likelihood call:
        the lambda categories with all three lambdas equal to 1 are
        factorised into unpaired columns (src/FARCE.jl:1891-1901) unless
        every lambda category is such a one."""
        one = (self.lGC == 1.0) & (self.lAT == 1.0) & (self.lGT == 1.0)
        kept = len(self.lw) if one.all() else int((~one).sum())
        return len(self.sr) ** 2 * kept


def _need_cuda(flag):
    if not flag:
        raise NotImplementedError("messi_gb300 runs on the GPU only; there is no CPU path")


# ---------------------------------------------------------------------------
# HP1: pair pruning
# ---------------------------------------------------------------------------
def felsensteincuda(dataset, params, museparams=None, maxbasepairdistance=1000000, keepmuseconditionals=False,
                    pairmask=None, ctx=None):
    """src/FelsensteinCUDA.jl:214-516.  Returns (mat, ret): mat is the L x L
    mixed pair log-likelihood matrix (-Inf outside the band and mask), ret the
    per-lambda-category matrices when keepmuseconditionals."""
    ctx = ctx or get_context()
    h = ctx.dataset(dataset, maxbasepairdistance, pairmask)
    m = ModelArgs(params, museparams)
    L = dataset.numcols
    mat = np.empty((L, L), order="F")
    per = np.empty(len(m.lw) * L * L) if keepmuseconditionals else None
    ctx.check(ctx.lib.messi_felsenstein_pairs(ctx.handle, h.handle, ctypes.byref(m.struct), _p(mat), _p(per)),
              "messi_felsenstein_pairs")
    ret = []
    if keepmuseconditionals:
        ret = [per[k * L * L:(k + 1) * L * L].reshape((L, L), order="F") for k in range(len(m.lw))]
    return mat, ret


def subcolumnrefs(dataset, ctx=None):
    """Dataset.subcolumnrefs (src/Dataset.jl:180-196) on the device:
    numnodes x numcols, 1-based first column with the same subtree pattern."""
    ctx = ctx or get_context()
    h = ctx.dataset(dataset, 1)
    out = np.empty((dataset.numnodes, dataset.numcols), dtype=np.int32, order="F")
    ctx.check(ctx.lib.messi_subcolumnrefs(ctx.handle, h.handle, _p(out)), "messi_subcolumnrefs")
    return out.astype(np.int64)


def felsensteinposteriorsiterateconditionalscuda(singleprobs, pairprobs, dataset, params, museparams=None,
                                                  maxbasepairdistance=1000000, keepmuseconditionals=False, ctx=None):
    """src/FelsensteinCUDA.jl:518-717: siteCats x numcols log conditionals of
    each column's site-rate category given the structure posteriors."""
    ctx = ctx or get_context()
    h = ctx.dataset(dataset, maxbasepairdistance)
    m = ModelArgs(params, museparams)
    L = dataset.numcols
    out = np.empty((len(m.sr), L), order="F")
    ctx.check(ctx.lib.messi_siterate_conditionals(ctx.handle, h.handle, ctypes.byref(m.struct), _p(_f64c(singleprobs)),
                                                  _p(_f64f(pairprobs)), _p(out)), "messi_siterate_conditionals")
    return out


def coevolutionall(dataset, params, parallel=True, keepmatrices=False, integratesiterates=True,
                   maxbasepairdistance=1000000, usecuda=True):
    """src/FARCE.jl:1736-1741 (the GPU branch)."""
    _need_cuda(usecuda and integratesiterates)
    return felsensteincuda(dataset, params, getmusespecificparamsarray(params), maxbasepairdistance, keepmatrices)


def computeunpairedlikelihoods(dataset, params, museparams=None, states=None, paired=None, B=1.0,
                               conditionalRates=False, rng=None, likelihoodsOnly=True, ctx=None):
    """src/FARCE.jl:1198-1220 (site-rate categories integrated).  With
    `paired` (1-based partners, 0 = unpaired) the overload of
    src/FARCE.jl:1222-1250: 0 on paired columns."""
    ctx = ctx or get_context()
    if paired is not None:
        _need_cuda(not conditionalRates)
        _, _, u = _structure_call(dataset, params, paired, ctx)
        return u
    h = ctx.dataset(dataset, 1)  # the unpaired pass needs the tree only: smallest pair plan
    m = ModelArgs(params)
    u = np.empty(dataset.numcols)
    ctx.check(ctx.lib.messi_unpaired(ctx.handle, h.handle, ctypes.byref(m.struct), _p(u)), "messi_unpaired")
    return u


def _structure_call(dataset, params, paired, ctx):
    h = ctx.dataset(dataset, 1)
    m = ModelArgs(params)
    pr = np.ascontiguousarray(paired, np.int32)
    if pr.shape != (dataset.numcols,):
        raise ValueError("paired must have one entry per column")
    L = dataset.numcols
    total = ctypes.c_double()
    pairll = np.empty(L)
    u = np.empty(L)
    ctx.check(ctx.lib.messi_structure_likelihood(ctx.handle, h.handle, ctypes.byref(m.struct), _p(pr),
                                                 ctypes.byref(total), _p(pairll), _p(u)),
              "messi_structure_likelihood")
    return total.value, pairll, u


def felsensteincudapaired(dataset, paired, params, museparams=None, ctx=None):
    """src/FelsensteinCUDA.jl:721-912: sum over the pairs of a fixed structure
    (1-based partners, 0 = unpaired) of the pair log-likelihood mixed over
    all categories."""
    ctx = ctx or get_context()
    if not np.any(np.asarray(paired) > 0):
        return 0.0
    _, pairll, _ = _structure_call(dataset, params, paired, ctx)
    return float(pairll.sum())


def computemodellikelihood(rng, dataset, params, paired, samplebranchlengths=False, integratesiterates=True,
                           useprior=True, fixLambdaGT=False, usecuda=True, ctx=None):
    """src/FARCE.jl:2439-2520 (the integratesiterates / usecuda branch):
    prior + unpaired columns + pairs of the fixed structure."""
    _need_cuda(usecuda and integratesiterates)
    ctx = ctx or get_context()
    priorll = computeprior(params, samplebranchlengths, fixLambdaGT) if useprior else 0.0
    total, _, _ = _structure_call(dataset, params, paired, ctx)
    return priorll + total


def maskgapped(probs, gapfrequency, cutoff, v=0.0):
    """src/RNATools.jl:441-451 (in place, host matrix)."""
    g = np.asarray(gapfrequency) >= cutoff
    probs[g, :] = v
    probs[:, g] = v
    return probs


# ---------------------------------------------------------------------------
# HP2: inside / outside / posteriors
# ---------------------------------------------------------------------------
def _f64c(a):
    return np.ascontiguousarray(a, np.float64)


def _f64f(a):
    return np.asfortranarray(a, np.float64)


def computeinsideKH99(unpairedlogprobs, pairedlogprobs, B=1.0, zonly=True, usecudain=True, maxspan=-1, ctx=None):
    """src/InsideCUDA.jl:23-53.  Z when zonly, else the 3 x L x L table."""
    _need_cuda(usecudain)
    ctx = ctx or get_context()
    u = _f64c(unpairedlogprobs)
    p = _f64f(pairedlogprobs)
    L = len(u)
    Z = ctypes.c_double()
    ins = None if zonly else np.empty((3, L, L), order="F")
    ctx.check(ctx.lib.messi_inside(ctx.handle, L, _p(u), _p(p), int(maxspan), float(B), ctypes.byref(Z), _p(ins)),
              "messi_inside")
    return Z.value if zonly else ins


def computeoutsideKH99(inside, unpairedlogprobs, pairedlogprobs, usecuda=True, maxspan=-1, ctx=None):
    """src/InsideCUDA.jl:55-61."""
    _need_cuda(usecuda)
    ctx = ctx or get_context()
    u = _f64c(unpairedlogprobs)
    L = len(u)
    out = np.empty((3, L, L), order="F")
    ctx.check(ctx.lib.messi_outside(ctx.handle, L, _p(_f64f(inside)), _p(u), _p(_f64f(pairedlogprobs)),
                                    int(maxspan), _p(out)), "messi_outside")
    return out


def computebasepairprobs(inside, outside, unpairedlogprobs, pairedlogprobs, grammar=None, maxspan=-1, ctx=None):
    """src/InsideOutsideAlgorithm.jl:486-533: row-normalised posteriors."""
    ctx = ctx or get_context()
    u = _f64c(unpairedlogprobs)
    L = len(u)
    single = np.empty(L)
    pair = np.empty((L, L), order="F")
    ctx.check(ctx.lib.messi_basepairprobs(ctx.handle, L, _p(_f64f(inside)), _p(_f64f(outside)), _p(u),
                                          _p(_f64f(pairedlogprobs)), int(maxspan), _p(single), _p(pair)),
              "messi_basepairprobs")
    return single, pair


def computeposteriors(unpairedlogprobs, pairedlogprobs, maxspan=-1, ctx=None):
    """inside -> outside -> computebasepairprobs on the device
    (src/MESSI.jl:1101-1103).  Returns (Z, single, pair)."""
    ctx = ctx or get_context()
    u = _f64c(unpairedlogprobs)
    L = len(u)
    single = np.empty(L)
    pair = np.empty((L, L), order="F")
    Z = ctypes.c_double()
    ctx.check(ctx.lib.messi_posteriors(ctx.handle, L, _p(u), _p(_f64f(pairedlogprobs)), int(maxspan),
                                       ctypes.byref(Z), _p(single), _p(pair)), "messi_posteriors")
    return Z.value, single, pair


# ---------------------------------------------------------------------------
# structures: posterior decoding and sampling
# ---------------------------------------------------------------------------
def computeposteriordecodingcuda(singleprobs, pairprobs, alpha=2.0, ctx=None):
    """src/InsideCUDA.jl:183-215: (ematrix, smatrix) of the maximum expected
    accuracy recursion (FP32 on the device, as the reference)."""
    ctx = ctx or get_context()
    s = _f64c(singleprobs)
    L = len(s)
    e = np.empty((L, L), order="F")
    sm = np.empty((L, L), dtype=np.int32, order="F")
    ctx.check(ctx.lib.messi_posterior_decoding(ctx.handle, L, _p(s), _p(_f64f(pairprobs)), float(alpha), _p(e),
                                               _p(sm), None), "messi_posterior_decoding")
    return e, sm.astype(np.int64)


def getPosteriorDecodingConsensusStructure(pairedposteriorprobs, unpairedposteriorprobs, usecuda=True, alpha=2.0,
                                           ctx=None):
    """src/RNATools.jl:74-83 (GPU branch): consensus structure as 1-based
    partners, 0 when unpaired (decoding and traceback on the device)."""
    _need_cuda(usecuda)
    ctx = ctx or get_context()
    s = _f64c(unpairedposteriorprobs)
    L = len(s)
    paired = np.empty(L, np.int32)
    ctx.check(ctx.lib.messi_posterior_decoding(ctx.handle, L, _p(s), _p(_f64f(pairedposteriorprobs)), float(alpha),
                                               None, None, _p(paired)), "messi_posterior_decoding")
    return paired.astype(np.int64)


def consensusstructure(unpairedlogprobs, pairedlogprobs, maxspan=-1, alpha=2.0, ctx=None):
    """Scores -> inside -> outside -> posteriors -> posterior decoding ->
    traceback, device-resident (the --processmax chain, src/MESSI.jl:1101-1103
    and src/RNATools.jl:74-83).  1-based partners, 0 when unpaired."""
    ctx = ctx or get_context()
    u = _f64c(unpairedlogprobs)
    L = len(u)
    out = np.empty(L, np.int32)
    ctx.check(ctx.lib.messi_consensus_structure(ctx.handle, L, _p(u), _p(_f64f(pairedlogprobs)), int(maxspan),
                                                float(alpha), _p(out)), "messi_consensus_structure")
    return out.astype(np.int64)


def samplestructures(unpairedlogprobs, pairedlogprobs, count, seed=1, maxspan=-1, ctx=None):
    """samplestructure (src/InsideOutsideAlgorithm.jl:570-635), `count`
    independent draws on the device.  Returns (structures [count, L] as
    1-based partners / 0, log KH99 prior of each)."""
    ctx = ctx or get_context()
    u = _f64c(unpairedlogprobs)
    L = len(u)
    out = np.empty((int(count), L), np.int32)
    priors = np.empty(int(count))
    ctx.check(ctx.lib.messi_sample_structures(ctx.handle, L, _p(u), _p(_f64f(pairedlogprobs)), int(maxspan),
                                              int(count), int(seed) & 0xFFFFFFFFFFFFFFFF, _p(out), _p(priors)),
              "messi_sample_structures")
    return out.astype(np.int64), priors


# ---------------------------------------------------------------------------
# the likelihood evaluation of every NLopt / MCMC step
# ---------------------------------------------------------------------------
def computestructureintegratedlikelihood(dataset, params, maxbasepairdistance=1000000, samplebranchlengths=False,
                                         fixLambdaGT=False, integratesiterates=True, usecuda=True, gapcutoff=1.0,
                                         ctx=None, return_unpaired=False):
    """src/FARCE.jl:2322-2345 (+ maskgapped!, src/MESSI.jl:310): logprior + Z,
    with unpaired, pair and inside passes resident on the device."""
    _need_cuda(usecuda and integratesiterates)
    ctx = ctx or get_context()
    saved = params.lambdaGT
    if fixLambdaGT:
        params.lambdaGT = 1.0
    try:
        h = ctx.dataset(dataset, maxbasepairdistance)
        m = ModelArgs(params)
        Z = ctypes.c_double()
        gf = _f64c(dataset.gapfrequency)
        u = np.empty(dataset.numcols) if return_unpaired else None
        ctx.check(ctx.lib.messi_likelihood(ctx.handle, h.handle, ctypes.byref(m.struct), _p(gf), float(gapcutoff),
                                           ctypes.byref(Z), _p(u)), "messi_likelihood")
        params.logprior = computeprior(params, samplebranchlengths, fixLambdaGT)
    finally:
        params.lambdaGT = saved
    total = params.logprior + Z.value
    return (total, Z.value, u) if return_unpaired else total


# ---------------------------------------------------------------------------
# batches of alignments
# ---------------------------------------------------------------------------
class Batch:
    """Pair plans of many alignments evaluated together
    (include/messi_gb300.h, messi_batch_*): the batched form of
    computestructureintegratedlikelihood (src/FARCE.jl:2322-2345)."""

    def __init__(self, datasets, maxbasepairdistance=None, ctx=None):
        self.ctx = ctx or get_context()
        self.datasets = list(datasets)
        n = len(self.datasets)
        self._keep = []
        alns = (_lib.Alignment * n)()
        for k, d in enumerate(self.datasets):
            m = np.ascontiguousarray(d.masks, np.uint8)
            c = np.ascontiguousarray(d.children, np.int32)
            si = np.ascontiguousarray(d.seqindex, np.int32)
            self._keep += [m, c, si]
            alns[k] = _lib.Alignment(d.numseqs, d.numcols, d.numnodes, _p(m), _p(c), _p(si))
        W = None
        if maxbasepairdistance is not None:
            W = np.empty(n, np.int32)
            for k, d in enumerate(self.datasets):
                w = maxbasepairdistance[k] if np.ndim(maxbasepairdistance) else maxbasepairdistance
                W[k] = int(min(max(1, w), max(1, d.numcols - 1)))
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.messi_batch_create(self.ctx.handle, n, ctypes.cast(alns, ctypes.c_void_p),
                                                       _p(W), ctypes.byref(h)), "messi_batch_create")
        self.handle = h
        self.n = n
        self._gf = np.ascontiguousarray(np.concatenate([np.asarray(d.gapfrequency, np.float64)
                                                        for d in self.datasets]))

    def stats(self):
        out = np.zeros(8, np.int64)
        self.ctx.check(self.ctx.lib.messi_batch_stats(self.handle, _p(out), 8), "messi_batch_stats")
        keys = ("band_pairs", "unique_root_pairs", "executed_updates_per_category", "naive_updates_per_category",
                "levels", "arena_rows", "categories_per_pass", "nodes")
        return dict(zip(keys, (int(v) for v in out)))

    def likelihood(self, params_list, gapcutoff=1.0):
        """Z of every alignment (no prior).  params_list: one ModelParameters
        per alignment (its own branch lengths)."""
        if len(params_list) != self.n:
            raise ValueError("one parameter set per alignment")
        margs = [ModelArgs(p) for p in params_list]
        models = (_lib.Model * self.n)(*[m.struct for m in margs])
        Z = np.empty(self.n)
        self.ctx.check(self.ctx.lib.messi_batch_likelihood(self.ctx.handle, self.handle,
                                                           ctypes.cast(models, ctypes.c_void_p), _p(self._gf),
                                                           float(gapcutoff), _p(Z)), "messi_batch_likelihood")
        return Z

    def close(self):
        if getattr(self, "handle", None):
            self.ctx.lib.messi_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def computestructureintegratedlikelihoods(datasets, params_list, maxbasepairdistance=None, gapcutoff=1.0,
                                          batch=None, ctx=None):
    """computestructureintegratedlikelihood for every (dataset, params) pair
    in one batched evaluation: logprior + Z per alignment."""
    b = batch or Batch(datasets, maxbasepairdistance, ctx=ctx)
    Z = b.likelihood(params_list, gapcutoff)
    return np.array([computeprior(p) + z for p, z in zip(params_list, Z)])


# ---------------------------------------------------------------------------
# HP3: the learned-proposal network
# ---------------------------------------------------------------------------
class MLP:
    """BF16 MLP with a Gaussian-mixture head, trained and run by the
    library's kernels (include/messi_gb300.h, messi_mlp_*)."""

    def __init__(self, in_dim, width, ncomp, dim, seed=1, ctx=None):
        self.ctx = ctx or get_context()
        self.in_dim, self.width, self.ncomp, self.dim = in_dim, width, ncomp, dim
        self.out_dim = ncomp + 2 * ncomp * dim
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.messi_mlp_create(self.ctx.handle, in_dim, width, ncomp, dim, seed, ctypes.byref(h)),
                       "messi_mlp_create")
        self.handle = h
        n = ctypes.c_int32()
        self.ctx.check(self.ctx.lib.messi_mlp_nparams(h, ctypes.byref(n)), "messi_mlp_nparams")
        self.nparams = n.value

    def close(self):
        if self.handle:
            self.ctx.lib.messi_mlp_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self):
        out = np.empty(self.nparams, np.float32)
        self.ctx.check(self.ctx.lib.messi_mlp_get_params(self.ctx.handle, self.handle, _p(out)), "messi_mlp_get_params")
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        self.ctx.check(self.ctx.lib.messi_mlp_set_params(self.ctx.handle, self.handle, _p(p)), "messi_mlp_set_params")

    def forward(self, x):
        x = np.ascontiguousarray(np.atleast_2d(x), np.float32)
        y = np.empty((x.shape[0], self.out_dim), np.float32)
        self.ctx.check(self.ctx.lib.messi_mlp_forward(self.ctx.handle, self.handle, x.shape[0], _p(x), _p(y)),
                       "messi_mlp_forward")
        return y

    def gradients(self, x, target):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(target, np.float32)
        g = np.empty(self.nparams, np.float32)
        loss = ctypes.c_float()
        self.ctx.check(self.ctx.lib.messi_mlp_gradients(self.ctx.handle, self.handle, x.shape[0], _p(x), _p(t),
                                                        ctypes.byref(loss), _p(g)), "messi_mlp_gradients")
        return loss.value, g

    def train_step(self, x, target, lr=1e-3, max_grad_norm=10.0):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(target, np.float32)
        loss = ctypes.c_float()
        self.ctx.check(self.ctx.lib.messi_mlp_train_step(self.ctx.handle, self.handle, x.shape[0], _p(x), _p(t),
                                                         float(lr), float(max_grad_norm), ctypes.byref(loss)),
                       "messi_mlp_train_step")
        return loss.value

