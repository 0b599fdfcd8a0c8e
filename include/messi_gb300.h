/*
 * messi_gb300.h -- C ABI of the GB300 (sm_103a) implementation of MESSI's
 * likelihood hot path: 16-state site-pair pruning (HP1) and the KH99 SCFG
 * inside/outside passes with base-pairing posteriors (HP2).
 *
 * Every entry point returns MESSI_OK (0) or a negative status; there is no
 * CPU fallback.  Host buffers are caller-owned and copied in/out inside the
 * call.  Calls on one context are serialised on the context's CUDA stream and
 * are not re-entrant across threads.
 *
 * Conventions (those of the reference's Julia arrays):
 *   - matrices are column-major: element (i, j) of an L x L matrix is at
 *     i + j*L; element (X, i, j) of a 3 x L x L table is at X + 3*(i + L*j),
 *     X: 0 = S, 1 = F, 2 = L (src/InsideOutsideAlgorithm.jl:40-53);
 *   - impossible events are -Inf on input and output;
 *   - the tree is rooted and binary, nodes numbered in pre-order with the
 *     root = 0 (src/Tree.jl:190-208); branch length n is the branch above
 *     node n;
 *   - nucleotide masks: bit 0 = A, 1 = C, 2 = G, 3 = U/T; 15 = gap
 *     (src/Dataset.jl:13-96); the 16-state pair index is 4*first + second.
 */
#ifndef MESSI_GB300_H
#define MESSI_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MESSI_OK 0
#define MESSI_EINVAL -1   /* invalid argument */
#define MESSI_ENOMEM -2   /* device or host allocation failed */
#define MESSI_ECUDA -3    /* a CUDA call failed */
#define MESSI_ETIMEOUT -4 /* a bounded device-side wait gave up */
#define MESSI_ESTATE -5   /* object used in the wrong state */
#define MESSI_ETOOBIG -6  /* problem larger than a fixed-size buffer allows */

typedef struct messi_ctx messi_ctx;
typedef struct messi_dataset messi_dataset;

/* Alignment and rooted binary tree: the inputs of src/Dataset.jl:121-198. */
typedef struct {
    int32_t numseqs;
    int32_t numcols;
    int32_t numnodes;          /* 2*numseqs - 1 */
    const uint8_t* masks;      /* [numseqs][numcols] nucleotide masks, row-major */
    const int32_t* children;   /* [numnodes][2], -1 for leaves */
    const int32_t* seqindex;   /* [numnodes], row of `masks` for leaves, -1 otherwise */
} messi_alignment;

/* Substitution-model parameters after discretisation (the fields of
 * ModelParameters / MuseSpecificParameters, src/FARCE.jl:461-503, 699-727). */
typedef struct {
    double freqs[4];             /* nucleotide frequencies A, C, G, U */
    double q[6];                 /* GTR exchangeabilities q1..q6 */
    const double* branchlengths; /* [numnodes] */
    int32_t nsite;               /* site-rate categories */
    const double* siteRates;     /* [nsite] */
    const double* siteWeights;   /* [nsite] */
    int32_t nlambda;             /* coevolution categories */
    const double* lambdaGC;      /* [nlambda] multipliers (1 + lambdarate) */
    const double* lambdaAT;
    const double* lambdaGT;
    const double* lambdaWeights; /* [nlambda] */
} messi_model;

/* Human-readable text of a status code. */
const char* messi_strerror(int status);

/* Library version: major*10000 + minor*100 + patch. */
int messi_version(void);

/* Context: one CUDA device and one stream.  Replaces the per-call
 * CuContext(CuDevice(0)) / destroy! pairs of src/FelsensteinCUDA.jl:240-241,506
 * and src/InsideCUDA.jl:96-97,133. */
int messi_ctx_create(int device, messi_ctx** ctx);
int messi_ctx_destroy(messi_ctx* ctx);
/* The context's cudaStream_t (as void*), for event timing by callers. */
int messi_ctx_stream(messi_ctx* ctx, void** stream);
/* Number of kernel launches issued by the last call on this context. */
int messi_ctx_last_launches(messi_ctx* ctx, int64_t* launches);
/* Number of messi_likelihood calls on this context whose device work was a
 * replay of a captured CUDA graph (captured on the second call with the same
 * dataset, category layout and buffers; MESSI_GRAPHS=0 at context creation
 * turns graphs off). */
int messi_ctx_graph_replays(messi_ctx* ctx, int64_t* replays);
/* Launch shapes of the last likelihood evaluation (no counterpart in the
 * reference): the pruning pipeline shape (0 = 2 stages x 4 CTAs per SM,
 * 1 = 3 x 3, 2 = 2 x 3; 3 = the interior levels in the tcgen05 form, chosen
 * only by MESSI_PRUNE_SHAPE=3) and the wavefront CTA size (0 = chosen by band size),
 * and how many workloads have finished autotuning.  The first four
 * evaluations of a dataset (or batch) at a category count try candidate
 * shapes, timed with CUDA events, and later ones use the fastest
 * (MESSI_AUTOTUNE=0 at context creation turns this off; MESSI_PRUNE_SHAPE or
 * MESSI_WAVE_THREADS fix one knob).  Results do not depend on the shapes. */
int messi_ctx_launch_shapes(messi_ctx* ctx, int32_t* prune_shape, int32_t* wave_threads, int32_t* tuned);
/* Text of the last error recorded on this context. */
const char* messi_ctx_last_error(messi_ctx* ctx);
/* Self-test of the bounded device waits (no counterpart in the reference):
 * launches a two-CTA grid barrier that one CTA never reaches; the other
 * CTA's wait gives up after a few milliseconds and raises the error flag.
 * *status receives the status such a wait produces (MESSI_ETIMEOUT when the
 * mechanism works); the call itself returns MESSI_OK and leaves the context
 * usable. */
int messi_selftest_bounded_wait(messi_ctx* ctx, int32_t* status);
/* The host eigensystem behind P = exp(Qt) (no counterpart in the reference,
 * which diagonalises Q in Julia, src/FARCE.jl:410-433): Q (n x n row-major,
 * n <= 16) reversible with respect to pi > 0; on return w[n] are the
 * eigenvalues and U[n * n] (row-major, column p = eigenvector p) the
 * orthonormal eigenvectors of D^1/2 Q D^-1/2, D = diag(pi).  Host only: needs
 * no context and no GPU.  MESSI_EINVAL for n outside 1..16, a pi entry that is
 * not positive, a non-finite entry or no convergence. */
int messi_host_reversible_eig(int32_t n, const double* Q, const double* pi, double* w, double* U);

/* Per-kernel timing (instrumentation; no counterpart in the reference).
 * enable != 0 records a CUDA event pair around each launch of the timed
 * kernel families on the context's stream and resets the counters.
 * kernel: 0 = pair node update (every tree level), 1 = inside span diagonals,
 * 2 = inside suffix column, 3 = outside span diagonals.  units = node updates
 * (kernel 0) or cells (kernels 1-3) processed by the timed launches. */
int messi_ctx_profile(messi_ctx* ctx, int enable);
int messi_ctx_profile_read(messi_ctx* ctx, int kernel, double* total_ms, int64_t* launches, double* units);

/* Dataset handle: uploads the alignment and builds the per-node pair plan
 * (column-pattern compression and unique pair lists).  Replaces
 * getindexdict + its process-global cache, src/FelsensteinCUDA.jl:77-142,
 * 210-238, and Dataset.subcolumnrefs, src/Dataset.jl:180-196.
 *   maxbasepairdistance: pairs with y - x > W are not evaluated (-Inf).
 *   pairmask: optional L x L bytes, non-zero = evaluate (the
 *             dataset.maxbasepairprobs[x,y] > 0 test, src/FelsensteinCUDA.jl:91). */
int messi_dataset_create(messi_ctx* ctx, const messi_alignment* aln, int32_t maxbasepairdistance,
                         const uint8_t* pairmask, messi_dataset** ds);
int messi_dataset_destroy(messi_dataset* ds);
/* Dataset.subcolumnrefs (src/Dataset.jl:180-196) computed on the device:
 * for every tree node v and column x, the first column whose subtree
 * pattern at v equals x's.  Output: [numnodes x L] column-major with 1-based
 * values (the reference's Julia matrix). */
int messi_subcolumnrefs(messi_ctx* ctx, messi_dataset* ds, int32_t* subcolumnrefs);
/* Plan statistics: out[0] pairs in band, [1] unique root pairs, [2] node
 * updates per category executed (sum over internal nodes of unique pairs),
 * [3] naive node updates per category (pairs x internal nodes), [4] tree
 * levels, [5] partial-buffer rows per category, [6] categories per pass.
 * n = number of entries wanted (<= 7). */
int messi_dataset_stats(messi_dataset* ds, int64_t* out, int32_t n);

/* felsensteincuda (src/FelsensteinCUDA.jl:214-516): pair log-likelihoods
 * mixed over all nsite*nsite*nlambda categories.
 *   pairedlogprobs: [L x L] output, symmetric, -Inf outside band/mask and on
 *                   the diagonal.
 *   museconditionals: optional [nlambda][L x L] per-lambda-category mixtures
 *                   (keepmuseconditionals, src/FelsensteinCUDA.jl:387-398). */
int messi_felsenstein_pairs(messi_ctx* ctx, messi_dataset* ds, const messi_model* model,
                            double* pairedlogprobs, double* museconditionals);

/* felsensteinposteriorsiterateconditionalscuda (src/FelsensteinCUDA.jl:
 * 518-717): per column and site-rate category s, the log-sum-exp of
 * log w_s + log singleprobs[x] + (unpaired log-likelihood of x under s) and,
 * over the evaluated partners y of x, log pairprobs + log w_c + (pair
 * log-likelihood of category c) for the categories whose rate at x is s.
 *   singleprobs: [L], pairprobs: [L x L] posteriors;
 *   conditionals: [nsite x L] output (column-major, as the reference's
 *                 siteCats x numcols array). */
int messi_siterate_conditionals(messi_ctx* ctx, messi_dataset* ds, const messi_model* model,
                                const double* singleprobs, const double* pairprobs, double* conditionals);
/* computeunpairedlikelihoods(dataset, params) (src/FARCE.jl:1198-1220):
 * per-column log-likelihood mixed over site-rate categories.  [L] output. */
int messi_unpaired(messi_ctx* ctx, messi_dataset* ds, const messi_model* model, double* unpairedlogprobs);

/* computeinsideKH99 (src/InsideCUDA.jl:23-53): KH99 inside pass.
 *   maxspan: largest pair span to consider; < 0 infers it from `paired`
 *            (the largest j - i with a finite entry).  The result equals the
 *            unbanded pass whenever every pair beyond maxspan is -Inf.
 *   B:       exponent on rule and emission terms (1.0 in every caller).
 *   Z:       log marginal likelihood (scalar output).
 *   inside:  optional [3 x L x L] table.  Cells with span > maxspan are
 *            -Inf except S on the last column (the only ones Z uses). */
int messi_inside(messi_ctx* ctx, int32_t L, const double* unpaired, const double* paired, int32_t maxspan,
                 double B, double* Z, double* inside);

/* computeoutsideKH99 (src/InsideCUDA.jl:55-61): outside pass from a host
 * inside table.  [3 x L x L] output (same band convention as messi_inside). */
int messi_outside(messi_ctx* ctx, int32_t L, const double* inside, const double* unpaired,
                  const double* paired, int32_t maxspan, double* outside);

/* computebasepairprobs (src/InsideOutsideAlgorithm.jl:486-533) from host
 * inside/outside tables: row-normalised unpaired [L] and pair [L x L]
 * posteriors. */
int messi_basepairprobs(messi_ctx* ctx, int32_t L, const double* inside, const double* outside,
                        const double* unpaired, const double* paired, int32_t maxspan, double* single,
                        double* pairprobs);

/* Inside -> outside -> posteriors in one device-resident call (the
 * computeinsideKH99(zonly=false) / computeoutsideKH99 / computebasepairprobs
 * chain of src/MESSI.jl:1101-1103).  Z optional. */
int messi_posteriors(messi_ctx* ctx, int32_t L, const double* unpaired, const double* paired, int32_t maxspan,
                     double* Z, double* single, double* pairprobs);

/* Likelihood of one fixed structure, integrated over site rates: the
 * usecuda branch of computemodellikelihood (src/FARCE.jl:2480-2485) without
 * the prior, i.e. sum(computeunpairedlikelihoods(..., paired)) +
 * felsensteincudapaired(dataset, paired, params, museparams)
 * (src/FelsensteinCUDA.jl:721-912).  Only the structure's pairs are pruned
 * (subtree-pattern dedup as for the band); the reference's paired kernels
 * stride their child arrays incorrectly for more than one pair per unique
 * pattern (src/FelsensteinCUDA.jl:858-859), so this follows the CPU
 * computeuncachedlikelihood (src/FARCE.jl:1257-1456) instead.
 *   paired:   [L] 1-based partners, 0 when unpaired (symmetric);
 *   total:    sum of unpaired-column and pair log-likelihoods;
 *   pairll:   optional [L], the pair log-likelihood at the first column of
 *             each pair, 0 elsewhere;
 *   unpaired: optional [L], unpaired log-likelihoods, 0 on paired columns. */
int messi_structure_likelihood(messi_ctx* ctx, messi_dataset* ds, const messi_model* model, const int32_t* paired,
                               double* total, double* pairll, double* unpaired);
/* computeposteriordecodingcuda (src/InsideCUDA.jl:183-215) followed by
 * posteriordecodingtraceback (src/RNATools.jl:43-72): maximum expected
 * accuracy structure from posterior probabilities, in FP32 as the
 * reference's GPU path.  singleprobs [L], pairprobs [L x L] (symmetric).
 *   ematrix: optional [L x L] (e[i, j], zeros below the diagonal);
 *   smatrix: optional [L x L] traceback codes (-1: i unpaired, -2: i pairs j,
 *            k > 0: i pairs column k (1-based), bifurcation), 0 where unused;
 *   paired:  optional [L] 1-based partner of each column, 0 when unpaired
 *            (the reference's Julia vector). */
int messi_posterior_decoding(messi_ctx* ctx, int32_t L, const double* singleprobs, const double* pairprobs,
                             double alpha, double* ematrix, int32_t* smatrix, int32_t* paired);
/* getPosteriorDecodingConsensusStructure from scores (the --processmax chain
 * of src/MESSI.jl:1101-1103: inside, outside, basepairprobs, posterior
 * decoding, traceback), device-resident throughout.  structure: [L] 1-based
 * partners, 0 when unpaired. */
int messi_consensus_structure(messi_ctx* ctx, int32_t L, const double* unpaired, const double* paired,
                              int32_t maxspan, double alpha, int32_t* structure);
/* samplestructure (src/InsideOutsideAlgorithm.jl:570-635, B = 1 as every
 * caller uses it): nstruct structures drawn independently from the KH99
 * posterior given the scores.  structures: [nstruct][L] 1-based partners, 0
 * when unpaired.  logprior: optional [nstruct], the log KH99 prior of each
 * structure (calculateKH99prior, src/InsideOutsideAlgorithm.jl:86-144, which
 * samplestructure returns), summed over the sampled derivation.  Random
 * numbers: SplitMix64 streams keyed by (seed, index), so a seed always gives
 * the same structures. */
int messi_sample_structures(messi_ctx* ctx, int32_t L, const double* unpaired, const double* paired,
                            int32_t maxspan, int32_t nstruct, uint64_t seed, int32_t* structures, double* logprior);
/* computestructureintegratedlikelihood without the prior
 * (src/FARCE.jl:2322-2345, with maskgapped! as at src/MESSI.jl:310): unpaired
 * likelihoods, pair pruning, gap masking and the inside pass, all on the
 * device.  gapfrequency: [L]; columns with gapfrequency >= gapcutoff cannot
 * pair.  Z: log marginal likelihood.  unpaired: optional [L] output. */
int messi_likelihood(messi_ctx* ctx, messi_dataset* ds, const messi_model* model, const double* gapfrequency,
                     double gapcutoff, double* Z, double* unpaired);

/* ---- Batches of alignments (no single counterpart in the reference, which
 * evaluates one alignment per call; this is the batched form of the
 * felsensteincuda + computeinsideKH99 chain of src/FARCE.jl:2322-2345).
 * A batch holds the pair plans of n alignments.  messi_batch_likelihood
 * evaluates messi_likelihood for all of them in one pass: the tree levels of
 * all alignments are pruned together and all inside passes run in one
 * persistent launch.  Results equal n separate messi_likelihood calls. */
typedef struct messi_batch messi_batch;
/* maxbasepairdistance: [n] per-alignment band (nullable: numcols - 1 each). */
int messi_batch_create(messi_ctx* ctx, int32_t n, const messi_alignment* alns, const int32_t* maxbasepairdistance,
                       messi_batch** batch);
int messi_batch_destroy(messi_batch* batch);
/* out[0..7]: pairs in band, unique root pairs, executed and naive node
 * updates per category, deepest tree level, partial-buffer rows per
 * category, categories per pass, tree nodes (sums over the batch). */
int messi_batch_stats(messi_batch* batch, int64_t* out, int32_t n);
/* models: [n], one per alignment (its own branch lengths); models equal in
 * everything but their branch lengths share their category eigensystems,
 * and every model must have the same nsite and nlambda.
 * gapfrequency: nullable, the alignments' [numcols] vectors concatenated in
 * batch order.  Z: [n] log marginal likelihoods. */
int messi_batch_likelihood(messi_ctx* ctx, messi_batch* batch, const messi_model* models,
                           const double* gapfrequency, double gapcutoff, double* Z);

/* ---- Learned MCMC proposal network (HP3; no counterpart in the reference,
 * whose MCMC moves are all hand-tuned random walks, src/MCMC.jl:1307-1674).
 * A BF16 MLP (three linear layers in -> width -> width -> out, SiLU) whose
 * head is a diagonal Gaussian mixture of `ncomp` components over `dim`
 * values: [ncomp logits | ncomp*dim means | ncomp*dim log-sd].  Forward,
 * backward and Adam run in the library's own kernels. */
typedef struct messi_mlp messi_mlp;
int messi_mlp_create(messi_ctx* ctx, int32_t in_dim, int32_t width, int32_t ncomp, int32_t dim, uint64_t seed,
                     messi_mlp** mlp);
int messi_mlp_destroy(messi_mlp* mlp);
int messi_mlp_nparams(messi_mlp* mlp, int32_t* n);
/* FP32 master parameters in the layout W1[w][in] b1 W2[w][w] b2 W3[out][w] b3. */
int messi_mlp_get_params(messi_ctx* ctx, messi_mlp* mlp, float* params);
int messi_mlp_set_params(messi_ctx* ctx, messi_mlp* mlp, const float* params);
/* y[batch][out] = head(x[batch][in]). */
int messi_mlp_forward(messi_ctx* ctx, messi_mlp* mlp, int32_t batch, const float* x, float* y);
/* Mean mixture negative log-likelihood of target[batch][dim] and its
 * gradient w.r.t. the FP32 parameters (grads nullable). */
int messi_mlp_gradients(messi_ctx* ctx, messi_mlp* mlp, int32_t batch, const float* x, const float* target,
                        float* loss, float* grads);
/* One Adam step on that loss (gradient norm clipped to max_grad_norm if > 0). */
int messi_mlp_train_step(messi_ctx* ctx, messi_mlp* mlp, int32_t batch, const float* x, const float* target,
                         float lr, float max_grad_norm, float* loss);

/* KH99 inside pass that allocates nothing (no counterpart in the reference;
 * computeinsideKH99 always allocates its tables).  For callers that must not
 * call cudaMalloc -- code inside a framework that owns the device allocator,
 * or a loop that must not enter the driver's allocator (whose calls can
 * synchronise the device).  Inputs and output are DEVICE pointers; the work
 * is queued on `stream` (a cudaStream_t) of the current device:
 *   d_unpaired [L] doubles, d_paired [L x L] column-major doubles, d_Z one
 *   double.  maxspan as in messi_inside (< 0 infers it, which synchronises
 *   `stream` once to read the span back, and returns MESSI_EINVAL on a
 *   stream that is being captured).
 * Scratch lives in one fixed file-scope device array (about 25 MB per GPU
 * that loads the library, held until exit): each of its six band tables
 * holds L * RS <= 2^20 floats, RS = 32 * ceil((maxspan + 1) / 32), and
 * L <= 16384; larger problems return MESSI_ETOOBIG.  Every call shares that
 * array, so calls that overlap on the GPU race; serialise them.  The first
 * call on a device (and the first in a new CUDA context of that device)
 * resolves the array's address (set-up) and should come before any stream
 * capture.  The kernels run after the call returns: a bounded device wait
 * that gives up shows only as *d_Z == NaN (the return value is MESSI_OK), so
 * callers check Z. */
int messi_inside_noalloc(void* stream, int32_t L, const double* d_unpaired, const double* d_paired, int32_t maxspan,
                         double B, double* d_Z);

#ifdef __cplusplus
}
#endif

#endif /* MESSI_GB300_H */
