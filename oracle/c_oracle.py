"""ctypes binding of the FP64 C oracle (oracle/messi_oracle.c).

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py).  Array conventions follow
the C file: LxL matrices and 3xLxL tables are Fortran-ordered (Julia layout),
so ``a[X, i, j]`` indexes them directly.
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libmessi_oracle.so")
_lock = threading.Lock()
_lib = None

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_f64pF = np.ctypeslib.ndpointer(dtype=np.float64, flags="F_CONTIGUOUS")


def build(force=False):
    """Compile messi_oracle.c with the committed Makefile."""
    src = os.path.join(_HERE, "messi_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_LIB_PATH)
            c_int, c_double, c_void = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
            L.mo_logsumexp.restype = c_double
            L.mo_logsumexp.argtypes = [c_double, c_double]
            L.mo_gtr.argtypes = [_f64p, _f64p, _f64p]
            L.mo_musefreqs.argtypes = [_f64p, c_double, c_double, c_double, _f64p]
            L.mo_muse.argtypes = [c_double, c_double, c_double, _f64p, _f64p, c_double, c_double, _f64p]
            L.mo_reversible_eig.argtypes = [c_int, _f64p, _f64p, _f64p, _f64p]
            L.mo_transition_matrices.argtypes = [c_int, _f64p, _f64p, c_int, _f64p, _f64p]
            L.mo_subcolumnrefs.argtypes = [c_int, _i32p, _i32p, _u8p, c_int, _i32p]
            L.mo_pair_matrix.argtypes = [c_int, _i32p, _i32p, _u8p, c_int, c_int, _f64p, _f64p, _f64p, c_int,
                                         c_void, c_int, c_int, c_int, c_void, _f64pF, c_void, c_int, c_void,
                                         c_void, c_void, c_void]
            L.mo_unpaired.argtypes = [c_int, _i32p, _i32p, _u8p, c_int, c_int, _f64p, _f64p, _f64p, _f64p,
                                      c_void]
            L.mo_maskgapped.argtypes = [_f64pF, _f64p, c_int, c_double, c_double]
            L.mo_kh99_logprobs.argtypes = [_f64p]
            L.mo_inside.argtypes = [_f64p, _f64pF, c_int, c_double, _f64pF, c_int]
            L.mo_inside_banded.argtypes = [_f64p, _f64pF, c_int, c_int, c_double, ctypes.POINTER(c_double), c_int]
            L.mo_outside.argtypes = [_f64pF, _f64p, _f64pF, c_int, _f64pF, c_int]
            L.mo_posteriors_banded.argtypes = [_f64p, _f64pF, c_int, c_int, ctypes.POINTER(c_double), _f64p, _f64p,
                                               _f64p, c_int]
            _f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
            L.mo_posterior_decoding.argtypes = [_f32p, _f32p, c_int, ctypes.c_float, _f32p, _i32p]
            L.mo_posterior_traceback.argtypes = [_i32p, c_int, _i32p]
            L.mo_basepairprobs.argtypes = [_f64pF, _f64pF, _f64p, _f64pF, c_int, _f64p, _f64pF]
            for name in ("mo_reversible_eig", "mo_transition_matrices", "mo_subcolumnrefs", "mo_pair_matrix",
                         "mo_unpaired", "mo_inside", "mo_inside_banded", "mo_outside", "mo_basepairprobs",
                         "mo_posteriors_banded",
                         "mo_posterior_decoding", "mo_posterior_traceback"):
                getattr(L, name).restype = c_int
            _lib = L
    return _lib


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with status {rc}")


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def logsumexp(a, b):
    return lib().mo_logsumexp(float(a), float(b))


def kh99_logprobs():
    out = np.zeros(7)
    lib().mo_kh99_logprobs(out)
    return out


def gtr(q, piv):
    Q = np.zeros(16)
    lib().mo_gtr(np.ascontiguousarray(q, np.float64), np.ascontiguousarray(piv, np.float64), Q)
    return Q.reshape(4, 4)


def musefreqs(pi4, lGC, lAT, lGT):
    out = np.zeros(16)
    lib().mo_musefreqs(np.ascontiguousarray(pi4, np.float64), lGC, lAT, lGT, out)
    return out


def muse(lGC, lAT, lGT, q, pi4, sr1=1.0, sr2=1.0):
    Q = np.zeros(256)
    lib().mo_muse(lGC, lAT, lGT, np.ascontiguousarray(q, np.float64), np.ascontiguousarray(pi4, np.float64),
                  sr1, sr2, Q)
    return Q.reshape(16, 16)


def transition_matrices(Q, pi, branchlengths):
    Q = np.ascontiguousarray(Q, np.float64)
    n = Q.shape[0]
    bl = np.ascontiguousarray(branchlengths, np.float64)
    P = np.zeros(len(bl) * n * n)
    _check(lib().mo_transition_matrices(n, Q.ravel(), np.ascontiguousarray(pi, np.float64), len(bl), bl, P),
           "transition_matrices")
    return P.reshape(len(bl), n, n)


def subcolumnrefs(children, seqindex, masks):
    children = np.ascontiguousarray(children, np.int32)
    masks = np.ascontiguousarray(masks, np.uint8)
    numnodes = children.shape[0]
    L = masks.shape[1]
    refs = np.zeros(numnodes * L, np.int32)
    _check(lib().mo_subcolumnrefs(numnodes, children.ravel(), np.ascontiguousarray(seqindex, np.int32),
                                  masks.ravel(), L, refs), "subcolumnrefs")
    return refs.reshape(numnodes, L)


def pair_matrix(children, seqindex, masks, P, pi16, logw, W, pairmask=None, rows=None, lamidx=None, nlam=0,
                nthreads=0, lambda1_cat=None, u_by_site=None, site1=None, site2=None):
    """Mixed pair log-likelihood matrix (LxL, -Inf where not evaluated)."""
    children = np.ascontiguousarray(children, np.int32)
    seqindex = np.ascontiguousarray(seqindex, np.int32)
    masks = np.ascontiguousarray(masks, np.uint8)
    numnodes = children.shape[0]
    L = masks.shape[1]
    P = np.ascontiguousarray(P, np.float64)
    ncat = P.shape[0]
    out = np.zeros((L, L), order="F")
    outl = None
    if lamidx is not None:
        lamidx = np.ascontiguousarray(lamidx, np.int32)
        outl = np.zeros(nlam * L * L)
    pm = None
    if pairmask is not None:
        pm = np.asfortranarray(pairmask, np.uint8)
    x0, x1 = (0, 0) if rows is None else rows
    l1 = None if lambda1_cat is None else np.ascontiguousarray(lambda1_cat, np.int32)
    ubs = None if u_by_site is None else np.ascontiguousarray(u_by_site, np.float64)
    s1 = None if site1 is None else np.ascontiguousarray(site1, np.int32)
    s2 = None if site2 is None else np.ascontiguousarray(site2, np.int32)
    _check(lib().mo_pair_matrix(numnodes, children.ravel(), seqindex, masks.ravel(), L, ncat, P.ravel(),
                                np.ascontiguousarray(pi16, np.float64).ravel(),
                                np.ascontiguousarray(logw, np.float64), int(W), _ptr(pm), int(x0), int(x1),
                                int(nlam), _ptr(lamidx), out, _ptr(outl), int(nthreads), _ptr(l1), _ptr(ubs),
                                _ptr(s1), _ptr(s2)), "pair_matrix")
    if outl is not None:
        outl = outl.reshape(nlam, L, L).transpose(0, 2, 1)
    return out, outl


def unpaired(children, seqindex, masks, P4, pi4, logw):
    children = np.ascontiguousarray(children, np.int32)
    masks = np.ascontiguousarray(masks, np.uint8)
    numnodes = children.shape[0]
    L = masks.shape[1]
    P4 = np.ascontiguousarray(P4, np.float64)
    nsite = P4.shape[0]
    u = np.zeros(L)
    ubs = np.zeros(nsite * L)
    _check(lib().mo_unpaired(numnodes, children.ravel(), np.ascontiguousarray(seqindex, np.int32), masks.ravel(),
                             L, nsite, P4.ravel(), np.ascontiguousarray(pi4, np.float64),
                             np.ascontiguousarray(logw, np.float64), u, _ptr(ubs)), "unpaired")
    return u, ubs.reshape(nsite, L)


def maskgapped(p, gapfreq, cutoff, v=-np.inf):
    p = np.asfortranarray(p, np.float64).copy(order="F")
    lib().mo_maskgapped(p, np.ascontiguousarray(gapfreq, np.float64), p.shape[0], float(cutoff), float(v))
    return p


def inside(u, p, B=1.0, nthreads=0):
    u = np.ascontiguousarray(u, np.float64)
    L = len(u)
    p = np.asfortranarray(p, np.float64)
    ins = np.zeros((3, L, L), order="F")
    _check(lib().mo_inside(u, p, L, float(B), ins, int(nthreads)), "inside")
    return ins


def inside_banded_Z(u, p, W, B=1.0, nthreads=0):
    """Z of the banded inside pass (pairs of span > W must be -Inf in p)."""
    u = np.ascontiguousarray(u, np.float64)
    Z = ctypes.c_double()
    _check(lib().mo_inside_banded(u, np.asfortranarray(p, np.float64), len(u), int(W), float(B), ctypes.byref(Z),
                                  int(nthreads)), "inside_banded")
    return Z.value


def posteriors_banded(u, p, W, nthreads=0):
    """Banded inside -> outside -> posteriors (B = 1; pairs of span > W must
    be -Inf in p).  Returns (Z, single[L], up, lo): up[x, d] / lo[x, d] are
    the row-normalised posteriors of the pairs (x, x + d) / (x - d, x) in
    row x, d = 1..W (index 0 unused)."""
    u = np.ascontiguousarray(u, np.float64)
    L = len(u)
    W = max(0, min(int(W), L - 1))
    Z = ctypes.c_double()
    single = np.zeros(L)
    up = np.zeros(L * (W + 1))
    lo = np.zeros(L * (W + 1))
    _check(lib().mo_posteriors_banded(u, np.asfortranarray(p, np.float64), L, W, ctypes.byref(Z), single, up, lo,
                                      int(nthreads)), "posteriors_banded")
    return Z.value, single, up.reshape(L, W + 1), lo.reshape(L, W + 1)


def band_of(pair, W):
    """(up, lo) band views of a dense L x L posterior matrix, the layout of
    posteriors_banded."""
    pair = np.asarray(pair)
    L = pair.shape[0]
    W = max(0, min(int(W), L - 1))
    up = np.zeros((L, W + 1))
    lo = np.zeros((L, W + 1))
    x = np.arange(L)
    for d in range(1, W + 1):
        k = x[: L - d]
        up[k, d] = pair[k, k + d]
        lo[k + d, d] = pair[k + d, k]
    return up, lo


def outside(ins, u, p, nthreads=0):
    u = np.ascontiguousarray(u, np.float64)
    L = len(u)
    out = np.zeros((3, L, L), order="F")
    _check(lib().mo_outside(np.asfortranarray(ins, np.float64), u, np.asfortranarray(p, np.float64), L, out,
                            int(nthreads)), "outside")
    return out


def basepairprobs(ins, outs, u, p):
    u = np.ascontiguousarray(u, np.float64)
    L = len(u)
    single = np.zeros(L)
    pair = np.zeros((L, L), order="F")
    _check(lib().mo_basepairprobs(np.asfortranarray(ins, np.float64), np.asfortranarray(outs, np.float64), u,
                                  np.asfortranarray(p, np.float64), L, single, pair), "basepairprobs")
    return single, pair


def posterior_decoding(single, pair, alpha=2.0):
    """(e, s) L x L row-major, the GPU-path semantics of
    computeposteriordecodingcuda (FP32).  The reference kernel reads
    pair[i*L + k] of the column-major Julia matrix, i.e. element (k, i); the
    same element is passed here (row-normalised posteriors are symmetric only
    to rounding)."""
    L = len(single)
    e = np.zeros(L * L, np.float32)
    sm = np.zeros(L * L, np.int32)
    buf = np.ascontiguousarray(np.asarray(pair, np.float64).T.astype(np.float32))
    _check(lib().mo_posterior_decoding(np.ascontiguousarray(single, np.float32), buf, L, float(alpha), e, sm),
           "posterior_decoding")
    return e.reshape(L, L), sm.reshape(L, L)


def posterior_traceback(s):
    """1-based partner per column (0 = unpaired) from a row-major s."""
    s = np.ascontiguousarray(s, np.int32)
    L = s.shape[0]
    paired = np.zeros(L, np.int32)
    _check(lib().mo_posterior_traceback(s.ravel(), L, paired), "posterior_traceback")
    return paired
