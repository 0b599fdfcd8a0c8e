/*
 * messi_oracle.c -- FP64 CPU restatement of MESSI's likelihood hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the only callers are the
 * tests under tests/, __graft_entry__.smoke() (as the checker) and bench.py's
 * cpu_baseline leg and `--impl reference` arm (as the timed CPU restatement of
 * the reference's CPU path).  The product library (messi_gb300/) never links or
 * calls it.
 *
 * Parity anchor.  The reference (michaelgoldendev/MESSI, Julia) ships no test
 * vectors, so this restatement is pinned by derived known-answer tests
 * (tests/test_oracle.py: P(0)=I, detailed balance, lambda=1 factorisation,
 * closed-form Z with all pairs forbidden, brute-force structure enumeration)
 * and by an independent numpy restatement (oracle/oracle_np.py).
 *
 * Each function names the reference file:line it restates.  Everything is
 * double precision and follows the reference CPU code's conventions:
 *   - -Inf for impossible events (src/CommonUtils.jl:145-156 logsumexp);
 *   - CPU pruning rescales a node only when its max partial is < 1e-20
 *     (src/FARCE.jl:2226-2238);
 *   - per-node subtree-pattern cache (src/FARCE.jl:20-55, 2182-2254), which
 *     changes work, never results.
 *
 * Layouts (0-based; matrices are column-major like Julia arrays):
 *   masks      [nseq][L]  uint8, bit a set <=> nucleotide a (A,C,G,U) allowed;
 *                         15 = gap (src/Dataset.jl:13-96 setnucleotides).
 *   children   [numnodes][2] int32, pre-order node numbering (root = 0),
 *              -1 for leaves (src/Tree.jl:202-208 getnodelist).
 *   seqindex   [numnodes] int32, row of `masks` for leaves, -1 otherwise.
 *   P          [ncat][numnodes][n][n] row-major (row = parent state).
 *   LxL        element (i,j) at i + j*L.
 *   3xLxL      element (X,i,j) at X + 3*(i + L*j), X: 0=S 1=F 2=L.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MO_OK 0
#define MO_EINVAL -1
#define MO_ENOMEM -2

/* ---------------------------------------------------------------------- */
/* log-sum-exp of two terms: src/CommonUtils.jl:145-156                   */
/* ---------------------------------------------------------------------- */
static double lse2(double a, double b)
{
    if (b == -INFINITY) return a;
    if (a == -INFINITY) return b;
    if (a < b) return b + log1p(exp(a - b));
    return a + log1p(exp(b - a));
}

double mo_logsumexp(double a, double b) { return lse2(a, b); }

/* log of a sum of n terms given as logs: max + log(sum exp(t - max)).  The
 * same value as folding lse2 over the terms, with one exp per term instead
 * of an exp and a log1p. */
static double mo_lse_terms(const double* t, int n)
{
    double m = -INFINITY;
    for (int k = 0; k < n; k++)
        if (t[k] > m) m = t[k];
    if (m == -INFINITY) return -INFINITY;
    double s = 0.0;
    for (int k = 0; k < n; k++) s += exp(t[k] - m);
    return m + log(s);
}


/* ---------------------------------------------------------------------- */
/* Substitution models: src/RateMatrices.jl                               */
/* ---------------------------------------------------------------------- */

/* gtr(q1..q6, piv): src/RateMatrices.jl:2-37.  Q row-major 4x4. */
void mo_gtr(const double* q, const double* piv, double* Q)
{
    double S[16];
    memset(S, 0, sizeof(S));
    S[0 * 4 + 1] = q[0]; S[0 * 4 + 2] = q[1]; S[0 * 4 + 3] = q[2];
    S[1 * 4 + 0] = q[0]; S[1 * 4 + 2] = q[3]; S[1 * 4 + 3] = q[4];
    S[2 * 4 + 0] = q[1]; S[2 * 4 + 1] = q[3]; S[2 * 4 + 3] = q[5];
    S[3 * 4 + 0] = q[2]; S[3 * 4 + 1] = q[4]; S[3 * 4 + 2] = q[5];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) S[i * 4 + j] *= piv[j];
    for (int i = 0; i < 4; i++) {
        double d = 0.0;
        for (int j = 0; j < 4; j++) {
            Q[i * 4 + j] = S[i * 4 + j];
            if (i != j) d -= S[i * 4 + j];
        }
        Q[i * 4 + i] = d;
    }
}

/* Pair class of a 16-state dinucleotide (first*4+second): 1=GC/CG,
 * 2=AU/UA, 3=GU/UG, 0=other.  src/RateMatrices.jl:49,71. */
static const int mo_basepairings[16] = {0, 0, 0, 2, 0, 0, 1, 0, 0, 1, 0, 3, 2, 0, 3, 0};

/* calculatemusefreqs: src/RateMatrices.jl:40-67. */
void mo_musefreqs(const double* pi4, double lGC, double lAT, double lGT, double* out16)
{
    double piGC = pi4[1] * pi4[2];
    double piAT = pi4[0] * pi4[3];
    double piGT = pi4[2] * pi4[3];
    double kappa = 1.0 / (1.0 + 2.0 * (piAT * (lAT * lAT - 1.0)) + 2.0 * (piGC * (lGC * lGC - 1.0)) +
                          2.0 * (piGT * (lGT * lGT - 1.0)));
    for (int h = 0; h < 4; h++)
        for (int v = 0; v < 4; v++) {
            int idx = h * 4 + v;
            double f = kappa * pi4[h] * pi4[v];
            if (mo_basepairings[idx] == 1) f *= lGC * lGC;
            else if (mo_basepairings[idx] == 2) f *= lAT * lAT;
            else if (mo_basepairings[idx] == 3) f *= lGT * lGT;
            out16[idx] = f;
        }
}

/* muse(...): src/RateMatrices.jl:69-148.  Q row-major 16x16. */
void mo_muse(double lGC, double lAT, double lGT, const double* q, const double* pi4, double sr1, double sr2,
             double* Q)
{
    double ones[4] = {1.0, 1.0, 1.0, 1.0};
    double g[16];
    mo_gtr(q, ones, g);
    memset(Q, 0, 256 * sizeof(double));
    const double lam[4] = {1.0, lGC, lAT, lGT};
    for (int h = 0; h < 16; h++)
        for (int v = h + 1; v < 16; v++) {
            int from = -1, to = -1;
            if (h / 4 == v / 4) { to = v % 4; from = h % 4; }
            else if (v % 4 == h % 4) { to = v / 4; from = h / 4; }
            if (from < 0) continue;
            double m1 = 1.0, m2 = 1.0;
            /* forming a pair multiplies the rate by lambda, breaking one divides */
            if (mo_basepairings[v]) { m1 *= lam[mo_basepairings[v]]; m2 /= lam[mo_basepairings[v]]; }
            if (mo_basepairings[h]) { m1 /= lam[mo_basepairings[h]]; m2 *= lam[mo_basepairings[h]]; }
            if (from != to) { m1 *= g[from * 4 + to]; m2 *= g[from * 4 + to]; }
            if (h / 4 == v / 4) { m1 *= sr2; m2 *= sr2; }
            else if (v % 4 == h % 4) { m1 *= sr1; m2 *= sr1; }
            Q[h * 16 + v] = m1 * pi4[to];
            Q[v * 16 + h] = m2 * pi4[from];
        }
    for (int i = 0; i < 16; i++) {
        double d = 0.0;
        for (int j = 0; j < 16; j++)
            if (i != j) d -= Q[i * 16 + j];
        Q[i * 16 + i] = d;
    }
}

/* ---------------------------------------------------------------------- */
/* exp(Qt) per branch: src/FARCE.jl:410-433 (gettransitionmatriceslist)   */
/* with absmat (entries <= 0 -> 1e-50, src/FARCE.jl:389-408).             */
/* The reference uses a general eigendecomposition; Q is reversible with  */
/* respect to pi, so the symmetric form diag(pi)^1/2 Q diag(pi)^-1/2 is   */
/* diagonalised by cyclic Jacobi instead (same matrix exponential).       */
/* ---------------------------------------------------------------------- */
static void jacobi_eig(int n, double* A, double* w, double* V)
{
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) V[i * n + j] = (i == j) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                tot += A[i * n + j] * A[i * n + j];
                if (i != j) off += A[i * n + j] * A[i * n + j];
            }
        if (off <= 1e-30 * tot) break;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) {
                double apq = A[p * n + q];
                if (fabs(apq) < 1e-300) continue;
                double app = A[p * n + p], aqq = A[q * n + q];
                double theta = (aqq - app) / (2.0 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; k++) {
                    double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {
                    double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; k++) {
                    double vkp = V[k * n + p], vkq = V[k * n + q];
                    V[k * n + p] = c * vkp - s * vkq;
                    V[k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < n; i++) w[i] = A[i * n + i];
}

/* Symmetric eigendecomposition of a reversible rate matrix:
 * Q = D^-1/2 U diag(w) U^T D^1/2 with D = diag(pi).  U column k = vector k. */
int mo_reversible_eig(int n, const double* Q, const double* pi, double* w, double* U)
{
    double A[256];
    if (n > 16) return MO_EINVAL;
    for (int i = 0; i < n; i++)
        if (!(pi[i] > 0.0)) return MO_EINVAL;
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) A[i * n + j] = sqrt(pi[i]) * Q[i * n + j] / sqrt(pi[j]);
    for (int i = 0; i < n; i++)
        for (int j = i + 1; j < n; j++) {
            double s = 0.5 * (A[i * n + j] + A[j * n + i]);
            A[i * n + j] = s;
            A[j * n + i] = s;
        }
    jacobi_eig(n, A, w, U);
    return MO_OK;
}

/* P[node] for all nodes; node 0 (root) is all zeros, zero branch -> identity. */
int mo_transition_matrices(int n, const double* Q, const double* pi, int numnodes, const double* bl, double* P)
{
    double w[16], U[256];
    int rc = mo_reversible_eig(n, Q, pi, w, U);
    if (rc) return rc;
    memset(P, 0, sizeof(double) * n * n);
    for (int v = 1; v < numnodes; v++) {
        double* Pv = P + (size_t)v * n * n;
        double t = bl[v];
        if (t == 0.0) {
            for (int i = 0; i < n; i++)
                for (int j = 0; j < n; j++) Pv[i * n + j] = (i == j) ? 1.0 : 0.0;
            continue;
        }
        double e[16];
        for (int k = 0; k < n; k++) e[k] = exp(w[k] * t);
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                double s = 0.0;
                for (int k = 0; k < n; k++) s += U[i * n + k] * e[k] * U[j * n + k];
                s *= sqrt(pi[j]) / sqrt(pi[i]);
                Pv[i * n + j] = (s <= 0.0) ? 1e-50 : s;
            }
    }
    return MO_OK;
}

/* ---------------------------------------------------------------------- */
/* Column patterns per node: src/Dataset.jl:180-196 (subcolumnrefs).       */
/* refs[v*L + x] = first column whose subtree pattern at v equals x's.     */
/* ---------------------------------------------------------------------- */
static int postorder(int numnodes, const int32_t* children, int* order)
{
    int* stack = (int*)malloc(sizeof(int) * 2 * numnodes + 2);
    int* state = (int*)calloc(numnodes, sizeof(int));
    int top = 0, k = 0;
    if (!stack || !state) { free(stack); free(state); return -1; }
    stack[top++] = 0;
    while (top > 0) {
        int v = stack[top - 1];
        if (children[2 * v] < 0 || state[v]) {
            order[k++] = v;
            top--;
        } else {
            state[v] = 1;
            stack[top++] = children[2 * v + 1];
            stack[top++] = children[2 * v];
        }
    }
    free(stack);
    free(state);
    return k;
}

int mo_subcolumnrefs(int numnodes, const int32_t* children, const int32_t* seqindex, const uint8_t* masks, int L,
                     int32_t* refs)
{
    int* order = (int*)malloc(sizeof(int) * numnodes);
    int64_t hsize = 1;
    while (hsize < 2 * (int64_t)L + 2) hsize <<= 1;
    int64_t* hkey = (int64_t*)malloc(sizeof(int64_t) * hsize);
    int32_t* hval = (int32_t*)malloc(sizeof(int32_t) * hsize);
    if (!order || !hkey || !hval) { free(order); free(hkey); free(hval); return MO_ENOMEM; }
    int k = postorder(numnodes, children, order);
    for (int t = 0; t < k; t++) {
        int v = order[t];
        int32_t* rv = refs + (size_t)v * L;
        if (children[2 * v] < 0) {
            int first[256];
            for (int i = 0; i < 256; i++) first[i] = -1;
            const uint8_t* row = masks + (size_t)seqindex[v] * L;
            for (int x = 0; x < L; x++) {
                if (first[row[x]] < 0) first[row[x]] = x;
                rv[x] = first[row[x]];
            }
        } else {
            const int32_t* r0 = refs + (size_t)children[2 * v] * L;
            const int32_t* r1 = refs + (size_t)children[2 * v + 1] * L;
            for (int64_t i = 0; i < hsize; i++) hkey[i] = -1;
            for (int x = 0; x < L; x++) {
                int64_t key = (int64_t)r0[x] * L + r1[x];
                uint64_t h = ((uint64_t)key * 0x9E3779B97F4A7C15ull) >> 17;
                int64_t s = (int64_t)(h & (uint64_t)(hsize - 1));
                while (hkey[s] >= 0 && hkey[s] != key) s = (s + 1) & (hsize - 1);
                if (hkey[s] < 0) { hkey[s] = key; hval[s] = x; }
                rv[x] = hval[s];
            }
        }
    }
    free(order);
    free(hkey);
    free(hval);
    return MO_OK;
}

/* ---------------------------------------------------------------------- */
/* Pair pruning: src/FARCE.jl:1992-2046 (felsensteinall) and 2182-2254     */
/* (felsensteinstack) with the FastCache of src/FARCE.jl:20-55.            */
/* ---------------------------------------------------------------------- */
typedef struct {
    int64_t size;
    int64_t* keys;
    double* vals; /* size x n */
    double* logm;
} mo_cache;

typedef struct {
    int n; /* alphabet: 4 or 16 */
    int L;
    const int32_t* children;
    const int32_t* seqindex;
    const uint8_t* masks;
    const int32_t* refs;
    const double* P; /* numnodes x n x n */
    mo_cache cache;
} mo_pruner;

static int cache_init(mo_cache* c, int64_t size, int n)
{
    c->size = size;
    c->keys = (int64_t*)malloc(sizeof(int64_t) * size);
    c->vals = (double*)malloc(sizeof(double) * size * n);
    c->logm = (double*)malloc(sizeof(double) * size);
    if (!c->keys || !c->vals || !c->logm) return MO_ENOMEM;
    for (int64_t i = 0; i < size; i++) c->keys[i] = -1;
    return MO_OK;
}

static void cache_free(mo_cache* c)
{
    free(c->keys);
    free(c->vals);
    free(c->logm);
}

static void cache_clear(mo_cache* c)
{
    for (int64_t i = 0; i < c->size; i++) c->keys[i] = -1;
}

/* Partial likelihood of node v for columns (x, y) (y < 0: single column).
 * Rescale rule of src/FARCE.jl:2226-2238: divide by max only below 1e-20. */
static void prune(mo_pruner* pr, int v, int x, int y, double* out, double* logm)
{
    const int n = pr->n;
    const int L = pr->L;
    int c0 = pr->children[2 * v];
    if (c0 < 0) {
        const uint8_t* row = pr->masks + (size_t)pr->seqindex[v] * L;
        if (n == 16) {
            uint8_t mx = row[x], my = row[y];
            for (int a = 0; a < 16; a++) out[a] = (double)(((mx >> (a / 4)) & 1) * ((my >> (a % 4)) & 1));
        } else {
            for (int a = 0; a < 4; a++) out[a] = (double)((row[x] >> a) & 1);
        }
        *logm = 0.0;
        return;
    }
    int c1 = pr->children[2 * v + 1];
    const int32_t* rv = pr->refs + (size_t)v * L;
    int64_t key = ((int64_t)v * L + rv[x]) * (int64_t)L + (y >= 0 ? rv[y] : 0);
    uint64_t h = ((uint64_t)key * 0x9E3779B97F4A7C15ull) >> 11;
    int64_t slot = (int64_t)(h % (uint64_t)pr->cache.size);
    if (pr->cache.keys[slot] == key) {
        memcpy(out, pr->cache.vals + slot * n, sizeof(double) * n);
        *logm = pr->cache.logm[slot];
        return;
    }
    double l[16], r[16], ml, mr;
    prune(pr, c0, x, y, l, &ml);
    prune(pr, c1, x, y, r, &mr);
    const double* Pl = pr->P + (size_t)c0 * n * n;
    const double* Pr = pr->P + (size_t)c1 * n * n;
    double m = -INFINITY;
    for (int a = 0; a < n; a++) {
        double sl = 0.0, sr = 0.0;
        for (int d = 0; d < n; d++) {
            sl += Pl[a * n + d] * l[d];
            sr += Pr[a * n + d] * r[d];
        }
        out[a] = sl * sr;
        if (out[a] > m) m = out[a];
    }
    if (m < 1e-20) {
        for (int a = 0; a < n; a++) out[a] /= m;
        *logm = log(m) + ml + mr;
    } else {
        *logm = ml + mr;
    }
    pr->cache.keys[slot] = key;
    memcpy(pr->cache.vals + slot * n, out, sizeof(double) * n);
    pr->cache.logm[slot] = *logm;
}

/* Number of (x<y) pairs evaluated for rows [x0, x1): y-x <= W and mask. */
static int64_t count_pairs(int L, int W, const uint8_t* pairmask, int x0, int x1)
{
    int64_t k = 0;
    for (int x = x0; x < x1; x++) {
        int yend = (x + W < L - 1) ? x + W : L - 1;
        for (int y = x + 1; y <= yend; y++)
            if (!pairmask || pairmask[x + (size_t)y * L]) k++;
    }
    return k;
}

/*
 * Full pair log-likelihood matrix, mixed over categories:
 * src/FARCE.jl:1736-1858 (coevolutionall, integratesiterates branch) and
 * src/FelsensteinCUDA.jl:277-419 (same mixture on the GPU path).
 *
 *   ncat categories, each with its own P (numnodes x 16 x 16), root
 *   frequencies pi16 and log weight logw.  lamidx[c] is the lambda category
 *   of c (for per-lambda conditionals, src/FelsensteinCUDA.jl:387-398).
 *   Rows x in [x0, x1) only (x1 <= 0 means all rows).
 *   out: LxL, -Inf outside the evaluated pairs; out_per_lambda: nlam x LxL.
 *   lambda1_unpaired: for categories whose lambda multipliers are all 1 the
 *   CPU reference uses the product of the two unpaired site likelihoods
 *   (src/FARCE.jl:1891-1901); when non-zero, `u_by_site` (nsite x L, the
 *   per-site-category unpaired log-likelihoods) and site1/site2 per category
 *   are used for those categories.
 */
int mo_pair_matrix(int numnodes, const int32_t* children, const int32_t* seqindex, const uint8_t* masks, int L,
                   int ncat, const double* P, const double* pi16, const double* logw, int W,
                   const uint8_t* pairmask, int x0, int x1, int nlam, const int32_t* lamidx, double* out,
                   double* out_per_lambda, int nthreads, const int32_t* lambda1_cat, const double* u_by_site,
                   const int32_t* site1, const int32_t* site2)
{
    if (L < 1 || numnodes < 1 || ncat < 1) return MO_EINVAL;
    if (x1 <= 0 || x1 > L) x1 = L;
    if (W < 0) W = 0;
    int32_t* refs = (int32_t*)malloc(sizeof(int32_t) * (size_t)numnodes * L);
    if (!refs) return MO_ENOMEM;
    int rc = mo_subcolumnrefs(numnodes, children, seqindex, masks, L, refs);
    if (rc) { free(refs); return rc; }
    int64_t npairs = count_pairs(L, W, pairmask, x0, x1);
    int32_t* px = (int32_t*)malloc(sizeof(int32_t) * (npairs + 1));
    int32_t* py = (int32_t*)malloc(sizeof(int32_t) * (npairs + 1));
    double* ll = (double*)malloc(sizeof(double) * (size_t)ncat * (npairs + 1));
    if (!px || !py || !ll) { free(refs); free(px); free(py); free(ll); return MO_ENOMEM; }
    {
        int64_t k = 0;
        for (int x = x0; x < x1; x++) {
            int yend = (x + W < L - 1) ? x + W : L - 1;
            for (int y = x + 1; y <= yend; y++)
                if (!pairmask || pairmask[x + (size_t)y * L]) { px[k] = x; py[k] = y; k++; }
        }
    }
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    int failed = 0;
#pragma omp parallel
    {
        mo_pruner pr;
        pr.n = 16;
        pr.L = L;
        pr.children = children;
        pr.seqindex = seqindex;
        pr.masks = masks;
        pr.refs = refs;
        int64_t csize = 1 << 18;
        if (cache_init(&pr.cache, csize, 16)) {
#pragma omp atomic write
            failed = 1;
        } else {
#pragma omp for schedule(dynamic, 1)
            for (int c = 0; c < ncat; c++) {
                double* llc = ll + (size_t)c * npairs;
                if (lambda1_cat && lambda1_cat[c]) {
                    const double* u1 = u_by_site + (size_t)site1[c] * L;
                    const double* u2 = u_by_site + (size_t)site2[c] * L;
                    for (int64_t k = 0; k < npairs; k++) llc[k] = u1[px[k]] + u2[py[k]];
                    continue;
                }
                pr.P = P + (size_t)c * numnodes * 256;
                cache_clear(&pr.cache);
                const double* pic = pi16 + (size_t)c * 16;
                for (int64_t k = 0; k < npairs; k++) {
                    double v[16], lm;
                    prune(&pr, 0, px[k], py[k], v, &lm);
                    double tot = 0.0;
                    for (int a = 0; a < 16; a++) tot += pic[a] * v[a];
                    llc[k] = log(tot) + lm;
                }
            }
        }
        cache_free(&pr.cache);
    }
    if (failed) { free(refs); free(px); free(py); free(ll); return MO_ENOMEM; }
    for (size_t i = 0; i < (size_t)L * L; i++) out[i] = -INFINITY;
    if (out_per_lambda)
        for (size_t i = 0; i < (size_t)nlam * L * L; i++) out_per_lambda[i] = -INFINITY;
    for (int64_t k = 0; k < npairs; k++) {
        double acc = -INFINITY;
        for (int c = 0; c < ncat; c++) acc = lse2(acc, logw[c] + ll[(size_t)c * npairs + k]);
        size_t x = px[k], y = py[k];
        out[x + y * L] = acc;
        out[y + x * L] = acc;
        if (out_per_lambda && lamidx) {
            for (int c = 0; c < ncat; c++) {
                double* o = out_per_lambda + (size_t)lamidx[c] * L * L;
                double t = lse2(o[x + y * L], logw[c] + ll[(size_t)c * npairs + k]);
                o[x + y * L] = t;
                o[y + x * L] = t;
            }
        }
    }
    free(refs);
    free(px);
    free(py);
    free(ll);
    return MO_OK;
}

/*
 * Unpaired column log-likelihoods, mixed over site-rate categories:
 * src/FARCE.jl:1198-1220 (computeunpairedlikelihoods(dataset, params)) and
 * src/FARCE.jl:742-773 (computeunpairedlikelihoodscat).
 *   P4: nsite x numnodes x 4 x 4 (exp(Q*rate*t)), pi4 root frequencies,
 *   logw: nsite log weights.  u_by_site (nullable): nsite x L unmixed values.
 */
int mo_unpaired(int numnodes, const int32_t* children, const int32_t* seqindex, const uint8_t* masks, int L,
                int nsite, const double* P4, const double* pi4, const double* logw, double* u, double* u_by_site)
{
    int32_t* refs = (int32_t*)malloc(sizeof(int32_t) * (size_t)numnodes * L);
    if (!refs) return MO_ENOMEM;
    int rc = mo_subcolumnrefs(numnodes, children, seqindex, masks, L, refs);
    if (rc) { free(refs); return rc; }
    mo_pruner pr;
    pr.n = 4;
    pr.L = L;
    pr.children = children;
    pr.seqindex = seqindex;
    pr.masks = masks;
    pr.refs = refs;
    if (cache_init(&pr.cache, 1 << 16, 4)) { cache_free(&pr.cache); free(refs); return MO_ENOMEM; }
    for (int s = 0; s < nsite; s++) {
        pr.P = P4 + (size_t)s * numnodes * 16;
        cache_clear(&pr.cache);
        for (int x = 0; x < L; x++) {
            double v[4], lm;
            prune(&pr, 0, x, -1, v, &lm);
            double tot = 0.0;
            for (int a = 0; a < 4; a++) tot += pi4[a] * v[a];
            double val = log(tot) + lm;
            if (u_by_site) u_by_site[(size_t)s * L + x] = val;
            u[x] = (s == 0) ? logw[0] + val : lse2(u[x], logw[s] + val);
        }
    }
    cache_free(&pr.cache);
    free(refs);
    return MO_OK;
}

/* maskgapped!: src/RNATools.jl:441-451. */
void mo_maskgapped(double* probs, const double* gapfreq, int L, double cutoff, double v)
{
    for (int i = 0; i < L; i++)
        for (int j = 0; j < L; j++)
            if (gapfreq[i] >= cutoff || gapfreq[j] >= cutoff) probs[i + (size_t)j * L] = v;
}

/* ---------------------------------------------------------------------- */
/* KH99 SCFG: src/InsideOutsideAlgorithm.jl:30-53                          */
/* S->LS (r1), S->s (r2), S->dFd (r3), F->dFd (r4), F->LS (r5), L->s (r6), */
/* L->dFd (r7).                                                             */
/* ---------------------------------------------------------------------- */
static const double mo_rule_prob[7] = {0.868534, 0.117609877998, 0.013856122002, 0.787640,
                                       0.21236,  0.894603,       0.105397};

void mo_kh99_logprobs(double* out7)
{
    for (int i = 0; i < 7; i++) out7[i] = log(mo_rule_prob[i]);
}

#define IDX3(X, i, j) ((size_t)(X) + 3 * ((size_t)(i) + (size_t)L * (size_t)(j)))

/*
 * Inside pass: src/InsideOutsideAlgorithm.jl:682-749 (computeinsideparallel,
 * the reference's CPU path) / :298-343 (computeinside); both evaluate the
 * same recurrences with pairwise logsumexp.  Cells of one span are
 * independent, so they are split across threads.
 */
int mo_inside(const double* u, const double* p, int L, double B, double* inside, int nthreads)
{
    double r[7];
    mo_kh99_logprobs(r);
    for (size_t i = 0; i < (size_t)3 * L * L; i++) inside[i] = -INFINITY;
    for (int i = 0; i < L; i++) {
        inside[IDX3(0, i, i)] = (u[i] + r[1]) * B;
        inside[IDX3(2, i, i)] = (u[i] + r[5]) * B;
    }
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    for (int d = 1; d < L; d++) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < L - d; i++) {
            int j = i + d;
            double tmp = -INFINITY;
            for (int h = i; h < j; h++) tmp = lse2(tmp, inside[IDX3(2, i, h)] + inside[IDX3(0, h + 1, j)]);
            /* type-3 rules: S->LS, F->LS */
            inside[IDX3(0, i, j)] = lse2(inside[IDX3(0, i, j)], r[0] * B + tmp);
            inside[IDX3(1, i, j)] = lse2(inside[IDX3(1, i, j)], r[4] * B + tmp);
            /* type-2 rules: S->dFd, F->dFd, L->dFd */
            double fin = (d >= 2) ? inside[IDX3(1, i + 1, j - 1)] : -INFINITY;
            double pij = p[i + (size_t)j * L];
            inside[IDX3(0, i, j)] = lse2(inside[IDX3(0, i, j)], (r[2] + pij) * B + fin);
            inside[IDX3(1, i, j)] = lse2(inside[IDX3(1, i, j)], (r[3] + pij) * B + fin);
            inside[IDX3(2, i, j)] = lse2(inside[IDX3(2, i, j)], (r[6] + pij) * B + fin);
        }
    }
    return MO_OK;
}

/* Outside pass: src/InsideOutsideAlgorithm.jl:447-483 (computeoutside). */
int mo_outside(const double* inside, const double* u, const double* p, int L, double* outside, int nthreads)
{
    (void)u;
    double r[7];
    mo_kh99_logprobs(r);
    for (size_t i = 0; i < (size_t)3 * L * L; i++) outside[i] = -INFINITY;
    outside[IDX3(0, 0, L - 1)] = 0.0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    /* type-3 rules are S->LS (parent S) and F->LS (parent F): parent index,
     * log prob */
    const int par[2] = {0, 1};
    const double rp[2] = {r[0], r[4]};
    for (int b = L - 2; b >= 0; b--) {
#pragma omp parallel for schedule(static)
        for (int j = 0; j <= L - b - 1; j++) {
            for (int t = 0; t < 2; t++) {
                double tmp = -INFINITY;
                for (int k = j + b + 1; k <= L - 1; k++)
                    tmp = lse2(tmp, outside[IDX3(par[t], j, k)] + inside[IDX3(0, j + b + 1, k)]);
                outside[IDX3(2, j, j + b)] = lse2(outside[IDX3(2, j, j + b)], tmp + rp[t]);
                tmp = -INFINITY;
                for (int k = 0; k <= j - 1; k++)
                    tmp = lse2(tmp, outside[IDX3(par[t], k, j + b)] + inside[IDX3(2, k, j - 1)]);
                outside[IDX3(0, j, j + b)] = lse2(outside[IDX3(0, j, j + b)], tmp + rp[t]);
            }
            if (j >= 1 && j + b + 1 < L) {
                double pij = p[(size_t)(j - 1) + (size_t)(j + b + 1) * L];
                /* S->dFd, F->dFd, L->dFd: the child is F */
                const int lhs[3] = {0, 1, 2};
                const double rr[3] = {r[2], r[3], r[6]};
                for (int t = 0; t < 3; t++)
                    outside[IDX3(1, j, j + b)] =
                        lse2(outside[IDX3(1, j, j + b)], rr[t] + pij + outside[IDX3(lhs[t], j - 1, j + b + 1)]);
            }
        }
    }
    return MO_OK;
}

/* Base-pairing posteriors: src/InsideOutsideAlgorithm.jl:486-533
 * (computebasepairprobs), including the per-row normalisation. */
int mo_basepairprobs(const double* inside, const double* outside, const double* u, const double* p, int L,
                     double* single, double* pairp)
{
    double r[7];
    mo_kh99_logprobs(r);
    double Z = inside[IDX3(0, 0, L - 1)];
    for (int j = 0; j < L; j++) {
        double tmp = -INFINITY;
        tmp = lse2(tmp, outside[IDX3(0, j, j)] + r[1]);
        tmp = lse2(tmp, outside[IDX3(2, j, j)] + r[5]);
        single[j] = tmp + u[j] - Z;
    }
    for (size_t i = 0; i < (size_t)L * L; i++) pairp[i] = -INFINITY;
    const int lhs[3] = {0, 1, 2};
    const double rr[3] = {r[2], r[3], r[6]};
    for (int j = 0; j < L; j++)
        for (int k = j + 1; k < L; k++) {
            double tmp = -INFINITY;
            double inres = (k - 1 >= j + 1) ? inside[IDX3(1, j + 1, k - 1)] : -INFINITY;
            for (int t = 0; t < 3; t++) tmp = lse2(tmp, outside[IDX3(lhs[t], j, k)] + rr[t] + inres);
            double v = tmp + p[j + (size_t)k * L] - Z;
            pairp[j + (size_t)k * L] = v;
            pairp[k + (size_t)j * L] = v;
        }
    double m = -INFINITY;
    for (int j = 0; j < L; j++) if (single[j] > m) m = single[j];
    for (size_t i = 0; i < (size_t)L * L; i++) if (pairp[i] > m) m = pairp[i];
    for (int j = 0; j < L; j++) single[j] = exp(single[j] - m);
    for (size_t i = 0; i < (size_t)L * L; i++) pairp[i] = exp(pairp[i] - m);
    for (int x = 0; x < L; x++) {
        double s = single[x];
        for (int y = 0; y < L; y++) s += pairp[x + (size_t)y * L];
        single[x] /= s;
        for (int y = 0; y < L; y++) pairp[x + (size_t)y * L] /= s;
    }
    return MO_OK;
}

/*
 * Banded inside pass (FP64): the same recurrences as mo_inside when every
 * pair of span > W is -Inf.  Only cells of span <= W and the S cells of the
 * last column reach Z (an S->LS chain ends at j = L-1; F and L need an
 * enclosing or own pair), so the band plus that column gives the dense Z
 * in O(L W^2).  Used to check Z at genome scale, where the dense O(L^3)
 * pass is out of reach; tests pin it to mo_inside at small sizes.
 */
int mo_inside_banded(const double* u, const double* p, int L, int W, double B, double* Zout, int nthreads)
{
    double r[7];
    mo_kh99_logprobs(r);
    if (L < 1) return MO_EINVAL;
    if (W > L - 1) W = L - 1;
    if (W < 0) W = 0;
    const size_t W1 = (size_t)W + 1;
    double* S = (double*)malloc(sizeof(double) * L * W1);
    double* F = (double*)malloc(sizeof(double) * L * W1);
    double* Lt = (double*)malloc(sizeof(double) * L * W1);
    double* suf = (double*)malloc(sizeof(double) * L);
    if (!S || !F || !Lt || !suf) { free(S); free(F); free(Lt); free(suf); return MO_ENOMEM; }
    for (size_t k = 0; k < (size_t)L * W1; k++) S[k] = F[k] = Lt[k] = -INFINITY;
    for (int i = 0; i < L; i++) {
        S[i * W1] = (u[i] + r[1]) * B;
        Lt[i * W1] = (u[i] + r[5]) * B;
        suf[i] = -INFINITY;
    }
    suf[L - 1] = S[(size_t)(L - 1) * W1];
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    for (int d = 1; d <= W; d++) {
#pragma omp parallel
        {
        double* terms = (double*)malloc(sizeof(double) * W1);
#pragma omp for schedule(static)
        for (int i = 0; i < L - d; i++) {
            int j = i + d;
            for (int k = 0; k < d; k++) terms[k] = Lt[i * W1 + k] + S[(size_t)(i + k + 1) * W1 + (d - 1 - k)];
            double tmp = mo_lse_terms(terms, d);
            double fin = (d >= 2) ? F[(size_t)(i + 1) * W1 + (d - 2)] : -INFINITY;
            double pij = p[i + (size_t)j * L];
            double s = lse2(-INFINITY, r[0] * B + tmp);
            double f = lse2(-INFINITY, r[4] * B + tmp);
            s = lse2(s, (r[2] + pij) * B + fin);
            f = lse2(f, (r[3] + pij) * B + fin);
            S[i * W1 + d] = s;
            F[i * W1 + d] = f;
            Lt[i * W1 + d] = lse2(-INFINITY, (r[6] + pij) * B + fin);
            if (j == L - 1) suf[i] = s;
        }
        free(terms);
        }
    }
    {
        double* terms = (double*)malloc(sizeof(double) * W1);
        for (int i = L - 2 - W; i >= 0; i--) {
            for (int k = 0; k <= W; k++) terms[k] = Lt[i * W1 + k] + suf[i + k + 1];
            suf[i] = r[0] * B + mo_lse_terms(terms, W + 1);
        }
        free(terms);
    }
    *Zout = suf[0];
    free(S);
    free(F);
    free(Lt);
    free(suf);
    return MO_OK;
}

/*
 * Banded inside -> outside -> base-pairing posteriors (FP64, B = 1): the
 * chain computeinside / computeoutside / computebasepairprobs
 * (src/InsideOutsideAlgorithm.jl:682-749, 447-483, 486-533) restricted to
 * pairs of span <= W, for genome-scale checks where the dense O(L^3) tables
 * are out of reach.  With every pair of span > W at -Inf, the only cells
 * beyond the band that carry probability are the S cells of the last column
 * (an S->LS chain ends at j = L-1), inside and outside; F and L need an
 * enclosing or own pair.  The outside recurrences are the adjoints of the
 * inside ones, written with A(i,j) = log(e^{OS(i,j)+r1} + e^{OF(i,j)+r5})
 * (the two LS parents):
 *   OS(k,j) = lse_{i<k} A(i,j) + L(i,k-1)
 *   OL(k,h) = lse_{j>h} A(k,j) + S(h+1,j)
 *   OF(k,j) = lse_{X in S,F,L} OX(k-1,j+1) + r_X(dFd) + p(k-1,j+1)
 * with OS(0,L-1) = 0.  Sums of many terms are taken as max + log(sum exp).
 * Outputs: Z; single[L]; up[x][d] = normalised posterior of the pair
 * (x, x+d) in row x and lo[x][d] that of (x-d, x) in row x (d = 1..W, rows
 * of W+1 entries, 0 outside the matrix), after the per-row normalisation of
 * computebasepairprobs.  tests/test_oracle.py pins it to the dense chain.
 */
int mo_posteriors_banded(const double* u, const double* p, int L, int W, double* Zout, double* single, double* up,
                         double* lo, int nthreads)
{
    double r[7];
    mo_kh99_logprobs(r);
    if (L < 1) return MO_EINVAL;
    if (W > L - 1) W = L - 1;
    if (W < 0) W = 0;
    const size_t W1 = (size_t)W + 1, n = (size_t)L * W1;
    double* buf = (double*)malloc(sizeof(double) * (7 * n + 2 * (size_t)L));
    if (!buf) return MO_ENOMEM;
    double *S = buf, *F = S + n, *Lt = F + n, *OS = Lt + n, *OF = OS + n, *OL = OF + n, *A = OL + n;
    double *Scol = A + n, *OScol = Scol + L;
    for (size_t k = 0; k < 7 * n + 2 * (size_t)L; k++) buf[k] = -INFINITY;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    /* inside, band */
    for (int i = 0; i < L; i++) {
        S[i * W1] = u[i] + r[1];
        Lt[i * W1] = u[i] + r[5];
    }
    for (int d = 1; d <= W; d++) {
#pragma omp parallel
        {
            double* t = (double*)malloc(sizeof(double) * (W1 + 1));
#pragma omp for schedule(static)
            for (int i = 0; i < L - d; i++) {
                const int j = i + d;
                for (int k = 0; k < d; k++) t[k] = Lt[i * W1 + k] + S[(size_t)(i + k + 1) * W1 + (d - 1 - k)];
                const double tmp = mo_lse_terms(t, d);
                const double fin = (d >= 2) ? F[(size_t)(i + 1) * W1 + (d - 2)] : -INFINITY;
                const double pij = p[i + (size_t)j * L];
                S[i * W1 + d] = lse2(r[0] + tmp, (r[2] + pij) + fin);
                F[i * W1 + d] = lse2(r[4] + tmp, (r[3] + pij) + fin);
                Lt[i * W1 + d] = (r[6] + pij) + fin;
            }
            free(t);
        }
    }
    /* inside, S cells of the last column (band, then the suffix beyond it) */
    for (int i = L - 1; i >= 0 && L - 1 - i <= W; i--) Scol[i] = S[i * W1 + (L - 1 - i)];
    {
        double* t = (double*)malloc(sizeof(double) * (W1 + 1));
        for (int i = L - 2 - W; i >= 0; i--) {
            for (int k = 0; k <= W; k++) t[k] = Lt[i * W1 + k] + Scol[i + k + 1];
            Scol[i] = r[0] + mo_lse_terms(t, W + 1);
        }
        free(t);
    }
    const double Z = Scol[0];
    *Zout = Z;
    /* outside: the last column beyond the band (increasing start) */
    OScol[0] = 0.0;
    {
        double* t = (double*)malloc(sizeof(double) * (W1 + 1));
        for (int k = 1; k < L - 1 - W; k++) {
            int m = 0;
            for (int i = (k - 1 - W > 0 ? k - 1 - W : 0); i <= k - 1; i++) t[m++] = OScol[i] + r[0] + Lt[i * W1 + (k - 1 - i)];
            OScol[k] = mo_lse_terms(t, m);
        }
        free(t);
    }
    /* outside, band, decreasing span */
    for (int d = W; d >= 0; d--) {
#pragma omp parallel
        {
            double* t = (double*)malloc(sizeof(double) * (W1 + 2));
#pragma omp for schedule(static)
            for (int k = 0; k <= L - 1 - d; k++) {
                const int j = k + d;
                double os;
                if (k == 0 && j == L - 1) {
                    os = 0.0;
                } else {
                    int m = 0;
                    for (int i = (k - 1 - W > 0 ? k - 1 - W : 0); i <= k - 1; i++) {
                        double a;
                        if (j - i <= W) a = A[i * W1 + (j - i)];
                        else if (j == L - 1) a = OScol[i] + r[0];
                        else a = -INFINITY;
                        t[m++] = a + Lt[i * W1 + (k - 1 - i)];
                    }
                    os = mo_lse_terms(t, m);
                }
                double of = -INFINITY;
                if (k >= 1 && j + 1 < L && d + 2 <= W) {
                    const size_t q = (size_t)(k - 1) * W1 + (d + 2);
                    const double pp = p[(size_t)(k - 1) + (size_t)(j + 1) * L];
                    double tt[3] = {OS[q] + r[2] + pp, OF[q] + r[3] + pp, OL[q] + r[6] + pp};
                    of = mo_lse_terms(tt, 3);
                }
                double ol;
                {
                    int m = 0;
                    const int jmax = (k + W < L - 1) ? k + W : L - 1;
                    for (int jj = j + 1; jj <= jmax; jj++) t[m++] = A[k * W1 + (jj - k)] + S[(size_t)(j + 1) * W1 + (jj - j - 1)];
                    if (L - 1 > k + W) t[m++] = OScol[k] + r[0] + Scol[j + 1];
                    ol = mo_lse_terms(t, m);
                }
                OS[k * W1 + d] = os;
                OF[k * W1 + d] = of;
                OL[k * W1 + d] = ol;
                A[k * W1 + d] = lse2(os + r[0], of + r[4]);
                if (j == L - 1) OScol[k] = os;
            }
            free(t);
        }
    }
    /* posteriors (log), then the global max shift and row normalisation */
    double m = -INFINITY;
    for (int j = 0; j < L; j++) {
        single[j] = lse2(OS[j * W1] + r[1], OL[j * W1] + r[5]) + u[j] - Z;
        if (single[j] > m) m = single[j];
    }
    for (size_t k = 0; k < n; k++) up[k] = lo[k] = -INFINITY;
    for (int j = 0; j < L; j++)
        for (int d = 1; d <= W && j + d < L; d++) {
            const size_t q = (size_t)j * W1 + d;
            const double fin = (d >= 2) ? F[(size_t)(j + 1) * W1 + (d - 2)] : -INFINITY;
            double tt[3] = {OS[q] + r[2], OF[q] + r[3], OL[q] + r[6]};
            const double v = mo_lse_terms(tt, 3) + fin + p[(size_t)j + (size_t)(j + d) * L] - Z;
            up[q] = v;
            lo[(size_t)(j + d) * W1 + d] = v;
            if (v > m) m = v;
        }
    for (int j = 0; j < L; j++) single[j] = exp(single[j] - m);
    for (size_t k = 0; k < n; k++) {
        up[k] = exp(up[k] - m);
        lo[k] = exp(lo[k] - m);
    }
    for (int x = 0; x < L; x++) {
        double s = single[x];
        for (int d = 1; d <= W; d++) s += up[(size_t)x * W1 + d] + lo[(size_t)x * W1 + d];
        single[x] /= s;
        for (int d = 0; d <= W; d++) {
            up[(size_t)x * W1 + d] /= s;
            lo[(size_t)x * W1 + d] /= s;
        }
    }
    free(buf);
    return MO_OK;
}

/*
 * Posterior decoding (maximum expected accuracy structure) as
 * computeposteriordecodingcuda runs it (src/InsideCUDA.jl:183-215 with the
 * kernel posteriordecoding of src/cuda/inside.cu:286-321): FP32 values,
 * e(i,i) = 0, diagonals in increasing span, and for cell (i,j)
 *   e1 = single[i] + e(i+1,j)
 *   e2 = alpha*pair(i,j) + e(i+1,j-1)
 *   e3 = max_{k=i+1..j-1} alpha*pair(i,k) + e(i+1,k-1) + e(k+1,j)
 * with ties going to e1, then e2, then the smallest k.  The alpha*x + y
 * products are single-rounding fused multiply-adds, as the CUDA compiler
 * contracts them.  e and s are L x L row-major (e[i*L+j]); s = -1 (i
 * unpaired), -2 (i pairs j) or k+1 (i pairs k, 0-based k).  pair is read as
 * pair[i*L+k], the reference kernel's indexing of the column-major matrix.
 */
int mo_posterior_decoding(const float* single, const float* pair, int L, float alpha, float* e, int* s)
{
    if (L < 1) return MO_EINVAL;
    memset(e, 0, sizeof(float) * (size_t)L * L);
    memset(s, 0, sizeof(int) * (size_t)L * L);
    for (int diag = 1; diag < L; diag++) {
        for (int i = 0; i < L - diag; i++) {
            const int j = i + diag;
            const float e1 = single[i] + e[(size_t)(i + 1) * L + j];
            const float e2 = fmaf(alpha, pair[(size_t)i * L + j], e[(size_t)(i + 1) * L + j - 1]);
            float maxe3 = -1e10f;
            int maxk = 0;
            for (int k = i + 1; k <= j - 1; k++) {
                const float v = fmaf(alpha, pair[(size_t)i * L + k], e[(size_t)(i + 1) * L + k - 1]) +
                                e[(size_t)(k + 1) * L + j];
                if (v > maxe3) {
                    maxe3 = v;
                    maxk = k;
                }
            }
            float maxval = e1;
            int sv = -1;
            if (e2 > maxval) {
                maxval = e2;
                sv = -2;
            }
            if (maxe3 > maxval) {
                maxval = maxe3;
                sv = maxk + 1;
            }
            s[(size_t)i * L + j] = sv;
            e[(size_t)i * L + j] = maxval;
        }
    }
    return MO_OK;
}

/* posteriordecodingtraceback (src/RNATools.jl:43-72) on the row-major s of
 * mo_posterior_decoding.  paired[i] = 1-based partner of column i (0-based
 * i), 0 when unpaired (the reference's Julia vector). */
int mo_posterior_traceback(const int* s, int L, int* paired)
{
    if (L < 1) return MO_EINVAL;
    memset(paired, 0, sizeof(int) * (size_t)L);
    int* stack = (int*)malloc(sizeof(int) * 2 * ((size_t)L + 2));
    if (!stack) return MO_ENOMEM;
    int top = 0;
    stack[top++] = 1;
    stack[top++] = L;  /* 1-based (i, j) as the reference */
    while (top > 0) {
        const int j = stack[--top];
        const int i = stack[--top];
        const int k = s[(size_t)(i - 1) * L + (j - 1)];
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
        } else if (k > 0) {
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
    free(stack);
    return MO_OK;
}
