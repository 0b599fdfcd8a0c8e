// host_model.cpp -- FP64 substitution models and their eigensystems (host side).
//
// Rate matrices restate src/RateMatrices.jl (gtr :2-37, calculatemusefreqs
// :40-67, muse :69-148).  exp(Qt) in the reference comes from a general
// eigendecomposition (src/FARCE.jl:410-433); every Q here is reversible with
// respect to its stationary frequencies, so the library diagonalises the
// symmetric matrix D^1/2 Q D^-1/2 (D = diag(pi); Householder reduction and
// symmetric QR steps, symmetric_eig) and the device assembles
// P = D^-1/2 U exp(W t) U^T D^1/2 per branch in FP64.
#include <cmath>
#include <cstring>

#include "internal.h"

namespace messi {

static const int kPairClass[16] = {0, 0, 0, 2, 0, 0, 1, 0, 0, 1, 0, 3, 2, 0, 3, 0};

void host_gtr(const double* q, const double* piv, double* Q)
{
    static const int ij[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
    double S[16] = {0};
    for (int k = 0; k < 6; k++) {
        S[ij[k][0] * 4 + ij[k][1]] = q[k];
        S[ij[k][1] * 4 + ij[k][0]] = q[k];
    }
    for (int i = 0; i < 4; i++) {
        double d = 0.0;
        for (int j = 0; j < 4; j++) {
            Q[i * 4 + j] = S[i * 4 + j] * piv[j];
            if (i != j) d -= Q[i * 4 + j];
        }
        Q[i * 4 + i] = d;
    }
}

void host_musefreqs(const double* pi4, double lGC, double lAT, double lGT, double* out16)
{
    const double lam[4] = {1.0, lGC, lAT, lGT};
    const double piGC = pi4[1] * pi4[2], piAT = pi4[0] * pi4[3], piGT = pi4[2] * pi4[3];
    const double kappa = 1.0 / (1.0 + 2.0 * (piAT * (lAT * lAT - 1.0)) + 2.0 * (piGC * (lGC * lGC - 1.0)) +
                                2.0 * (piGT * (lGT * lGT - 1.0)));
    for (int a = 0; a < 16; a++) {
        double l = lam[kPairClass[a]];
        out16[a] = kappa * l * l * pi4[a / 4] * pi4[a % 4];
    }
}

void host_muse(double lGC, double lAT, double lGT, const double* q, const double* pi4, double sr1, double sr2,
               double* Q)
{
    const double ones[4] = {1.0, 1.0, 1.0, 1.0};
    const double lam[4] = {1.0, lGC, lAT, lGT};
    double g[16];
    host_gtr(q, ones, g);
    for (int h = 0; h < 16; h++) {
        double d = 0.0;
        for (int v = 0; v < 16; v++) {
            double rate = 0.0;
            if (v != h) {
                int from = -1, to = -1;
                double sr = 1.0;
                if (h / 4 == v / 4) { from = h % 4; to = v % 4; sr = sr2; }
                else if (h % 4 == v % 4) { from = h / 4; to = v / 4; sr = sr1; }
                if (from >= 0) rate = g[from * 4 + to] * sr * pi4[to] * lam[kPairClass[v]] / lam[kPairClass[h]];
            }
            Q[h * 16 + v] = rate;
            d -= rate;
        }
        Q[h * 16 + h] = d;
    }
}

// Symmetric eigenproblem A = V diag(w) V^T (A row-major n x n, n <= 16, and
// destroyed; column p of V, V[k * n + p], is eigenvector p): Householder
// reduction to tridiagonal form with the reflections accumulated in V, then
// implicit symmetric QR steps with the Wilkinson shift, bulge chased by
// Givens rotations that are accumulated in V as well (Golub & Van Loan,
// Matrix Computations, algorithms 8.3.1-8.3.3).  About 18 us for a 16 x 16
// matrix on one host core, a third of cyclic Jacobi's time at the same
// accuracy (residual and orthogonality within 1e-14).  Returns nonzero if the
// iteration does not converge.
static int symmetric_eig(int n, double* A, double* w, double* V)
{
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) V[i * n + j] = (i == j) ? 1.0 : 0.0;
    for (int k = 0; k + 2 < n; k++) {
        // reflection H = I - beta v v^T mapping A[k+1.., k] onto alpha e1
        const int m = n - k - 1;
        double x[16], p[16];
        double tail = 0.0;
        for (int i = 0; i < m; i++) x[i] = A[(k + 1 + i) * n + k];
        for (int i = 1; i < m; i++) tail += x[i] * x[i];
        if (tail == 0.0) continue;
        const double nx = std::sqrt(x[0] * x[0] + tail);
        const double alpha = (x[0] >= 0.0) ? -nx : nx;
        x[0] -= alpha;
        const double beta = 2.0 / (x[0] * x[0] + tail);
        // trailing block: A <- H A H = A - v q^T - q v^T, q = p - (beta/2)(v.p) v, p = beta A v
        for (int i = 0; i < m; i++) {
            double acc = 0.0;
            for (int j = 0; j < m; j++) acc += A[(k + 1 + i) * n + (k + 1 + j)] * x[j];
            p[i] = beta * acc;
        }
        double vp = 0.0;
        for (int i = 0; i < m; i++) vp += x[i] * p[i];
        const double K = 0.5 * beta * vp;
        for (int i = 0; i < m; i++) p[i] -= K * x[i];
        for (int i = 0; i < m; i++)
            for (int j = 0; j < m; j++) A[(k + 1 + i) * n + (k + 1 + j)] -= x[i] * p[j] + p[i] * x[j];
        A[(k + 1) * n + k] = A[k * n + (k + 1)] = alpha;
        for (int i = 1; i < m; i++) A[(k + 1 + i) * n + k] = A[k * n + (k + 1 + i)] = 0.0;
        for (int r = 0; r < n; r++) {  // V <- V H
            double acc = 0.0;
            for (int j = 0; j < m; j++) acc += V[r * n + k + 1 + j] * x[j];
            acc *= beta;
            for (int j = 0; j < m; j++) V[r * n + k + 1 + j] -= acc * x[j];
        }
    }
    double d[16], e[16];  // diagonal; e[i] couples i and i + 1
    for (int i = 0; i < n; i++) d[i] = A[i * n + i];
    for (int i = 0; i + 1 < n; i++) e[i] = A[(i + 1) * n + i];
    e[n - 1] = 0.0;
    const double eps = 2.220446049250313e-16;
    int q = n - 1, steps = 0;
    while (q > 0) {
        for (int i = 0; i < q; i++)
            if (std::fabs(e[i]) <= eps * (std::fabs(d[i]) + std::fabs(d[i + 1]))) e[i] = 0.0;
        if (e[q - 1] == 0.0) {
            q--;
            continue;
        }
        int l = q - 1;  // unreduced block [l, q]
        while (l > 0 && e[l - 1] != 0.0) l--;
        if (++steps > 30 * n) return 1;
        // Wilkinson shift: the eigenvalue of the trailing 2 x 2 nearer d[q]
        const double half = 0.5 * (d[q - 1] - d[q]);
        const double b2 = e[q - 1] * e[q - 1];
        const double mu = d[q] - b2 / (half + std::copysign(std::sqrt(half * half + b2), half == 0.0 ? 1.0 : half));
        double xv = d[l] - mu, zv = e[l], bulge = 0.0;
        for (int k = l; k < q; k++) {
            // G in the plane (k, k+1) with G^T (xv, zv) = (r, 0); T <- G^T T G
            const double r = std::hypot(xv, zv);
            const double c = (r == 0.0) ? 1.0 : xv / r, s = (r == 0.0) ? 0.0 : -zv / r;
            if (k > l) e[k - 1] = c * e[k - 1] - s * bulge;
            const double dk = d[k], dk1 = d[k + 1], ek = e[k];
            d[k] = c * c * dk - 2.0 * c * s * ek + s * s * dk1;
            d[k + 1] = s * s * dk + 2.0 * c * s * ek + c * c * dk1;
            e[k] = c * s * (dk - dk1) + (c * c - s * s) * ek;
            if (k + 1 < q) {
                bulge = -s * e[k + 1];
                e[k + 1] *= c;
                xv = e[k];
                zv = bulge;
            }
            for (int r2 = 0; r2 < n; r2++) {
                const double a = V[r2 * n + k], b = V[r2 * n + k + 1];
                V[r2 * n + k] = c * a - s * b;
                V[r2 * n + k + 1] = s * a + c * b;
            }
        }
    }
    for (int i = 0; i < n; i++) w[i] = d[i];
    return 0;
}

int host_reversible_eig(int n, const double* Q, const double* pi, double* w, double* U)
{
    double A[256];
    if (n > 16) return MESSI_EINVAL;
    for (int i = 0; i < n; i++)
        if (!(pi[i] > 0.0) || !std::isfinite(pi[i])) return MESSI_EINVAL;
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) A[i * n + j] = std::sqrt(pi[i]) * Q[i * n + j] / std::sqrt(pi[j]);
    for (int i = 0; i < n; i++)
        for (int j = i + 1; j < n; j++) {
            double s = 0.5 * (A[i * n + j] + A[j * n + i]);
            A[i * n + j] = A[j * n + i] = s;
        }
    for (int i = 0; i < n * n; i++)
        if (!std::isfinite(A[i])) return MESSI_EINVAL;
    if (symmetric_eig(n, A, w, U)) return MESSI_EINVAL;
    return MESSI_OK;
}

static double safe_log(double x) { return x > 0.0 ? std::log(x) : -INFINITY; }

// Categories in the reference order: siteCat1 outer, siteCat2, lambda inner
// (src/FelsensteinCUDA.jl:277-279), weight log(w1) + log(w2) + log(w_lambda)
// (src/FelsensteinCUDA.jl:403-418).
//
// With factorise, the lambda categories whose three lambdas are exactly 1
// (the first category of getparams: rate 0, src/FARCE.jl:1566-1583) are left
// out, as long as another lambda category remains.  At lambda = 1 the paired
// rate matrix is the sum of two independent single-site GTR processes with
// rates r1 and r2 and pi16 = pi x pi, so the pair likelihood of category
// (s1, s2, l) is L4(x; r_s1) * L4(y; r_s2); summed over the site rates with
// their weights this is exp(u[x] + u[y]) times w_l, u being the unpaired
// log-likelihood.  The reference's CPU path takes the same shortcut
// (src/FARCE.jl:1891-1901).
int build_categories(const messi_model* m, int numnodes, Categories* out, std::string* err, bool pairs,
                     bool factorise, bool threads)
{
    if (!m || m->nsite < 1 || m->nlambda < 1 || !m->siteRates || !m->siteWeights || !m->lambdaGC ||
        !m->lambdaAT || !m->lambdaGT || !m->lambdaWeights || !m->branchlengths) {
        *err = "model: missing arrays or empty category sets";
        return MESSI_EINVAL;
    }
    if (m->nlambda > kMaxLambda) {
        *err = "model: at most 8 lambda categories are supported";
        return MESSI_EINVAL;
    }
    for (int a = 0; a < 4; a++)
        if (!(m->freqs[a] > 0.0)) { *err = "model: nucleotide frequencies must be positive"; return MESSI_EINVAL; }
    for (int k = 0; k < 6; k++)
        if (!(m->q[k] >= 0.0) || !std::isfinite(m->q[k])) { *err = "model: invalid exchangeability"; return MESSI_EINVAL; }
    for (int s = 0; s < m->nsite; s++)
        if (!(m->siteRates[s] >= 0.0) || !std::isfinite(m->siteRates[s]) || !(m->siteWeights[s] >= 0.0)) {
            *err = "model: invalid site rate or weight";
            return MESSI_EINVAL;
        }
    for (int l = 0; l < m->nlambda; l++)
        if (!(m->lambdaGC[l] > 0.0) || !(m->lambdaAT[l] > 0.0) || !(m->lambdaGT[l] > 0.0) ||
            !std::isfinite(m->lambdaGC[l] + m->lambdaAT[l] + m->lambdaGT[l]) || !(m->lambdaWeights[l] >= 0.0)) {
            *err = "model: invalid lambda category";
            return MESSI_EINVAL;
        }
    for (int v = 0; v < numnodes; v++)
        if (!(m->branchlengths[v] >= 0.0) || !std::isfinite(m->branchlengths[v])) {
            *err = "model: branch lengths must be finite and non-negative";
            return MESSI_EINVAL;
        }
    Categories& c = *out;
    c.nsite = m->nsite;
    c.nlam = m->nlambda;
    const int nl = m->nlambda, ns = m->nsite;
    c.lamF = 0;
    c.logwF = -INFINITY;
    c.logw_lam.assign(nl, 0.0);
    double wF = 0.0;
    for (int l = 0; l < nl; l++) {
        c.logw_lam[l] = safe_log(m->lambdaWeights[l]);
        if (factorise && m->lambdaGC[l] == 1.0 && m->lambdaAT[l] == 1.0 && m->lambdaGT[l] == 1.0) {
            c.lamF |= 1u << l;
            wF += m->lambdaWeights[l];
        }
    }
    if (c.lamF == (1u << nl) - 1u) c.lamF = 0;  // nothing left to prune: keep every category
    if (c.lamF) c.logwF = safe_log(wF);
    std::vector<int> kept;  // lambda categories pruned with 16 states
    for (int l = 0; l < nl; l++)
        if (!(c.lamF >> l & 1u)) kept.push_back(l);
    const int nk = (int)kept.size();
    c.C = ns * ns * nk;
    c.eig.assign(pairs ? (size_t)c.C * kEigStride : 0, 0.0);  // nothing to upload for unpaired-only calls
    c.pi16.assign(pairs ? (size_t)c.C * 16 : 0, 0.f);
    c.logw.assign(c.C, 0.0);
    c.lam.assign(c.C, 0);
    // the 16-state eigensystems are independent: one per host thread
    std::vector<int> bad(c.C, 0);
#pragma omp parallel for schedule(dynamic, 1) if (threads && pairs && c.C >= 4)
    for (int k = 0; k < c.C; k++) {
        const int s1 = k / (ns * nk), s2 = (k / nk) % ns, l = kept[k % nk];
        c.logw[k] = safe_log(m->siteWeights[s1]) + safe_log(m->siteWeights[s2]) + safe_log(m->lambdaWeights[l]);
        c.lam[k] = l;
        if (!pairs) continue;
        double Q[256], pi16[16];
        host_muse(m->lambdaGC[l], m->lambdaAT[l], m->lambdaGT[l], m->q, m->freqs, m->siteRates[s1],
                  m->siteRates[s2], Q);
        host_musefreqs(m->freqs, m->lambdaGC[l], m->lambdaAT[l], m->lambdaGT[l], pi16);
        double* e = &c.eig[(size_t)k * kEigStride];
        if (host_reversible_eig(16, Q, pi16, e, e + 16)) {
            bad[k] = 1;
            continue;
        }
        for (int a = 0; a < 16; a++) {
            e[16 + 256 + a] = std::sqrt(pi16[a]);
            c.pi16[(size_t)k * 16 + a] = (float)pi16[a];
        }
    }
    for (int k = 0; k < c.C; k++)
        if (bad[k]) {
            *err = "model: rate matrix is not diagonalisable";
            return MESSI_EINVAL;
        }
    // unpaired 4-state model per site rate: gtr(q, freqs) * rate (src/FARCE.jl:742-750)
    c.eig4.assign((size_t)m->nsite * kEig4Stride, 0.0);
    c.logw_site.assign(m->nsite, 0.0);
    double Q4[16];
    host_gtr(m->q, m->freqs, Q4);
    for (int s = 0; s < m->nsite; s++) {
        double Qr[16];
        for (int i = 0; i < 16; i++) Qr[i] = Q4[i] * m->siteRates[s];
        double* e = &c.eig4[(size_t)s * kEig4Stride];
        if (host_reversible_eig(4, Qr, m->freqs, e, e + 4)) {
            *err = "model: GTR matrix is not diagonalisable";
            return MESSI_EINVAL;
        }
        for (int a = 0; a < 4; a++) e[4 + 16 + a] = std::sqrt(m->freqs[a]);
        c.logw_site[s] = safe_log(m->siteWeights[s]);
    }
    for (int a = 0; a < 4; a++) c.pi4[a] = m->freqs[a];
    return MESSI_OK;
}

}  // namespace messi
