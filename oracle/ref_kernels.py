"""Host harness for the reference's own CUDA kernels (TEST INFRASTRUCTURE).

The reference runs its kernels from Julia through CUDAdrv; Julia is not
available, so this harness loads the same kernels -- src/cuda/felsenstein.cu
and src/cuda/inside.cu compiled unmodified into oracle/_ref/*.cubin by
``make -C oracle ref`` -- through the CUDA driver API and replays the launch
sequences of the reference's host code:

* ``pair_matrix``: src/FelsensteinCUDA.jl:214-516 (index plan of getindexdict
  :77-142; per category: felsensteinleaves16 per leaf, felsensteinhelper16 per
  internal node in post-order, sumfinal at the root, storearr/logsumexparr for
  the category mixture, 1024-thread blocks);
* ``inside``: src/InsideCUDA.jl:63-181 (float sanitising :63-85,
  initialiseinside, insidealgorithm per span, insidez, 256-thread blocks);
* ``outside``: src/InsideCUDA.jl:301-389 (outsidealgorithm per span,
  descending, 1024-thread blocks);
* ``posterior_decoding``: src/InsideCUDA.jl:183-215 (posteriordecoding per
  span, 256-thread blocks, e and s zero-initialised).

It is used as a parity pin for the FP64 oracle (the reference's own outputs)
and to time the reference GPU path on the same GPU.  felsensteinhelper16 reads
its child-index arrays before its bounds check (src/cuda/felsenstein.cu:167-168),
so the index arrays are padded to a whole number of 1024-thread blocks; every
other access of these kernels is guarded.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")

# mangled names as bound by the reference (src/FelsensteinCUDA.jl:249-253,
# src/InsideCUDA.jl:107-111, 191, 360)
K_LEAVES = b"_Z19felsensteinleaves16iiPKiS0_PfS1_"
K_HELPER = b"_Z19felsensteinhelper16iiiiiiPKiS0_PKfS2_S2_Pf"
K_SUMFINAL = b"_Z8sumfinaliiPfS_S_"
K_STOREARR = b"_Z8storearrifPfS_"
K_LSEARR = b"_Z12logsumexparrifPffS_"
K_INIT = b"_Z16initialiseinsidePfS_S_PKfi"
K_INSIDE = b"_Z15insidealgorithmPfS_S_PKfS1_iif"
K_INSIDEZ = b"_Z7insidezPKfPfi"
K_OUTSIDE = b"_Z16outsidealgorithmPfPKfS1_S1_iif"
K_DECODE = b"_Z17posteriordecodingPfPiPKfS2_iif"


def available():
    return all(os.path.exists(os.path.join(REF_DIR, f)) for f in ("felsenstein.cubin", "inside.cubin"))


class _Driver:
    def __init__(self):
        import torch
        torch.zeros(1, device="cuda")  # primary context current on this thread
        self.torch = torch
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.cu.cuModuleLoad.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p]
        self.cu.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_char_p]
        self.cu.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 6 + [ctypes.c_uint, ctypes.c_void_p,
                                                                                     ctypes.c_void_p, ctypes.c_void_p]
        self.mods = {}
        self.fns = {}

    def fn(self, module, name):
        key = (module, name)
        if key not in self.fns:
            if module not in self.mods:
                m = ctypes.c_void_p()
                rc = self.cu.cuModuleLoad(ctypes.byref(m), os.path.join(REF_DIR, module).encode())
                if rc != 0:
                    raise RuntimeError(f"cuModuleLoad({module}) failed: {rc}")
                self.mods[module] = m
            f = ctypes.c_void_p()
            rc = self.cu.cuModuleGetFunction(ctypes.byref(f), self.mods[module], name)
            if rc != 0:
                raise RuntimeError(f"cuModuleGetFunction({name}) failed: {rc}")
            self.fns[key] = f
        return self.fns[key]

    def launch(self, module, name, blocks, threads, *args):
        """args: ('i', int) | ('f', float) | ('p', tensor)."""
        holders = []
        for kind, v in args:
            if kind == "i":
                holders.append(ctypes.c_int(int(v)))
            elif kind == "f":
                holders.append(ctypes.c_float(float(v)))
            else:
                holders.append(ctypes.c_void_p(v.data_ptr()))
        params = (ctypes.c_void_p * len(holders))(*[ctypes.cast(ctypes.pointer(h), ctypes.c_void_p) for h in holders])
        stream = self.torch.cuda.current_stream().cuda_stream
        rc = self.cu.cuLaunchKernel(self.fn(module, name), max(1, blocks), 1, 1, threads, 1, 1, 0,
                                    ctypes.c_void_p(stream), params, None)
        if rc != 0:
            raise RuntimeError(f"cuLaunchKernel({name}) failed: {rc}")


_drv = None


def driver():
    global _drv
    if _drv is None:
        _drv = _Driver()
    return _drv


def _first_occurrence(keys):
    """Dense ids of `keys` in order of first occurrence, and the position of
    each id's first occurrence."""
    uniq, first, inv = np.unique(keys, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")
    rank = np.empty_like(order)
    rank[order] = np.arange(len(order))
    return rank[inv], first[order]


def index_plan(children, seqindex, masks, W, pairmask=None):
    """getindexdict (src/FelsensteinCUDA.jl:77-142): per node the unique
    (pattern(x), pattern(y)) pairs in order of first occurrence, derived from
    the parent's list, and the child rows of every internal node's pairs."""
    from . import c_oracle as co
    refs = co.subcolumnrefs(children, seqindex, masks).astype(np.int64)
    nn, L = refs.shape
    bx, by = [], []
    for x in range(L):
        y = np.arange(x + 1, min(x + W, L - 1) + 1)
        if pairmask is not None:
            y = y[pairmask[x, y] != 0]
        bx.append(np.full(len(y), x))
        by.append(y)
    bx = np.concatenate(bx) if bx else np.zeros(0, np.int64)
    by = np.concatenate(by) if by else np.zeros(0, np.int64)
    xs, ys = [None] * nn, [None] * nn
    ids, first = _first_occurrence(refs[0, bx] * L + refs[0, by])
    xs[0], ys[0] = bx[first], by[first]
    root_map = (bx, by, ids)
    lr = {}
    for v in range(nn):  # pre-order: parents before children
        if children[v, 0] < 0:
            continue
        maps = []
        for c in children[v]:
            cid, cfirst = _first_occurrence(refs[c, xs[v]] * L + refs[c, ys[v]])
            xs[c], ys[c] = xs[v][cfirst], ys[v][cfirst]
            maps.append(cid)
        lr[v] = (maps[0], maps[1])
    return xs, ys, root_map, lr


def _postorder(children):
    out, stack, seen = [], [0], set()
    while stack:
        v = stack[-1]
        if children[v, 0] < 0 or v in seen:
            out.append(v)
            stack.pop()
        else:
            seen.add(v)
            stack.append(children[v, 1])
            stack.append(children[v, 0])
    return out


def pair_matrix(children, seqindex, masks, P, pi16, logw, W, plan=None, timing=None):
    """The reference GPU pair log-likelihood matrix (FP32 kernels), LxL FP64
    with -Inf outside the band.  P: [C][numnodes][16][16]."""
    drv = driver()
    torch = drv.torch
    children = np.asarray(children)
    L = masks.shape[1]
    nn = children.shape[0]
    if plan is None:
        plan = index_plan(children, seqindex, masks, W)
    xs, ys, root_map, lr = plan
    dev = "cuda"
    bs = 1024
    leafdata = {}
    for v in range(nn):
        if children[v, 0] < 0:
            m = masks[seqindex[v]]
            leafdata[v] = torch.tensor(np.array([[(mm >> a) & 1 for a in range(4)] for mm in m],
                                                dtype=np.float32).ravel(), device=dev)
    d_x = {v: torch.tensor(np.asarray(xs[v], np.int32), device=dev) for v in range(nn) if children[v, 0] < 0}
    d_y = {v: torch.tensor(np.asarray(ys[v], np.int32), device=dev) for v in range(nn) if children[v, 0] < 0}
    d_lr = {}
    for v, (li, ri) in lr.items():
        n = len(li)
        pad = ((n + bs - 1) // bs) * bs
        a = np.zeros(max(pad, bs), np.int32)
        b = np.zeros(max(pad, bs), np.int32)
        a[:n] = li
        b[:n] = ri
        d_lr[v] = (torch.tensor(a, device=dev), torch.tensor(b, device=dev))
    nroot = len(xs[0])
    store = {v: torch.zeros(max(1, len(xs[v])) * 17, dtype=torch.float32, device=dev) for v in range(nn)}
    final = torch.zeros(max(1, nroot), dtype=torch.float32, device=dev)
    logliks = torch.zeros(max(1, nroot), dtype=torch.float32, device=dev)
    post = _postorder(children)
    C = P.shape[0]
    if timing is not None:
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record()
    for c in range(C):
        d_trans = torch.tensor(np.asarray(P[c], np.float32).ravel(), device=dev)
        d_freqs = torch.tensor(np.asarray(pi16[c], np.float32), device=dev)
        for v in post:
            n = len(xs[v])
            if children[v, 0] < 0:
                drv.launch("felsenstein.cubin", K_LEAVES, (n + bs - 1) // bs, bs, ("i", L), ("i", n), ("p", d_x[v]),
                           ("p", d_y[v]), ("p", leafdata[v]), ("p", store[v]))
            else:
                c0, c1 = children[v]
                li, ri = d_lr[v]
                drv.launch("felsenstein.cubin", K_HELPER, (n + bs - 1) // bs, bs, ("i", L), ("i", n), ("i", nn),
                           ("i", v), ("i", c0), ("i", c1), ("p", li), ("p", ri), ("p", d_trans), ("p", store[c0]),
                           ("p", store[c1]), ("p", store[v]))
        drv.launch("felsenstein.cubin", K_SUMFINAL, (nroot + bs - 1) // bs, bs, ("i", 16), ("i", nroot),
                   ("p", d_freqs), ("p", store[0]), ("p", logliks))
        if c == 0:
            drv.launch("felsenstein.cubin", K_STOREARR, (nroot + bs - 1) // bs, bs, ("i", nroot), ("f", logw[c]),
                       ("p", final), ("p", logliks))
        else:
            drv.launch("felsenstein.cubin", K_LSEARR, (nroot + bs - 1) // bs, bs, ("i", nroot), ("f", 0.0),
                       ("p", final), ("f", logw[c]), ("p", logliks))
    if timing is not None:
        ev1.record()
        torch.cuda.synchronize()
        timing["ms"] = ev0.elapsed_time(ev1)
    fin = final.cpu().numpy().astype(np.float64)
    out = np.full((L, L), -np.inf)
    bx, by, ids = root_map
    out[bx, by] = fin[ids]
    out[by, bx] = fin[ids]
    return out


def _sanitise(u, p):
    """src/InsideCUDA.jl:63-85."""
    L = len(u)
    us = np.where(u < -1e20, -1e20, u).astype(np.float32)
    ps = np.full((L, L), np.float32(-1e20), dtype=np.float32)
    iu = np.triu_indices(L, 1)
    up = p[iu]
    ps[iu] = np.where(up < -1e20, -1e20, up).astype(np.float32)
    ps[(iu[1], iu[0])] = p[(iu[1], iu[0])].astype(np.float32)
    return us, ps


def inside(u, p, B=1.0, timing=None):
    """Z and the 3 x L x L table [S, F, L] from the reference inside kernels."""
    drv = driver()
    torch = drv.torch
    L = len(u)
    us, ps = _sanitise(np.asarray(u, np.float64), np.asarray(p, np.float64))
    d_u = torch.tensor(us, device="cuda")
    d_p = torch.tensor(np.ascontiguousarray(ps).ravel(), device="cuda")  # row-major = transposed upload
    S = torch.zeros(L * L, dtype=torch.float32, device="cuda")
    Lt = torch.zeros(L * L, dtype=torch.float32, device="cuda")
    F = torch.zeros(L * L, dtype=torch.float32, device="cuda")
    Z = torch.zeros(1, dtype=torch.float32, device="cuda")
    bs = 256
    g = (L + bs - 1) // bs
    if timing is not None:
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record()
    drv.launch("inside.cubin", K_INIT, g, bs, ("p", S), ("p", Lt), ("p", F), ("p", d_u), ("i", L))
    for a in range(1, L):
        drv.launch("inside.cubin", K_INSIDE, g, bs, ("p", S), ("p", Lt), ("p", F), ("p", d_p), ("p", d_u), ("i", a),
                   ("i", L), ("f", B))
    drv.launch("inside.cubin", K_INSIDEZ, g, bs, ("p", S), ("p", Z), ("i", L))
    if timing is not None:
        ev1.record()
        torch.cuda.synchronize()
        timing["ms"] = ev0.elapsed_time(ev1)
    tab = np.stack([S.cpu().numpy().reshape(L, L), F.cpu().numpy().reshape(L, L), Lt.cpu().numpy().reshape(L, L)])
    return float(Z.item()), tab.astype(np.float64)


def outside(inside_tab, u, p, B=1.0):
    """The 3 x L x L outside table [S, F, L] from the reference outside kernel
    (input: an inside table indexed [X, i, j])."""
    drv = driver()
    torch = drv.torch
    L = len(u)
    us, ps = _sanitise(np.asarray(u, np.float64), np.asarray(p, np.float64))
    ins = np.where(np.isfinite(inside_tab), inside_tab, -1e20).astype(np.float32)
    out = np.full((3, L, L), np.float32(-1e20), dtype=np.float32)
    out[0, 0, L - 1] = 0.0
    d_out = torch.tensor(out.ravel(), device="cuda")
    d_in = torch.tensor(np.ascontiguousarray(ins).ravel(), device="cuda")
    d_p = torch.tensor(np.ascontiguousarray(ps).ravel(), device="cuda")
    d_u = torch.tensor(us, device="cuda")
    bs = 1024
    g = (L + bs - 1) // bs
    for a in range(L - 2, -1, -1):
        drv.launch("inside.cubin", K_OUTSIDE, g, bs, ("p", d_out), ("p", d_in), ("p", d_p), ("p", d_u), ("i", a),
                   ("i", L), ("f", B))
    return d_out.cpu().numpy().reshape(3, L, L).astype(np.float64)


def posterior_decoding(single, pair, alpha=2.0):
    """(e, s) as L x L row-major arrays (device layout: e[i*L+j]) from the
    reference posteriordecoding kernel; single/pair are converted to FP32 as
    src/InsideCUDA.jl:184-185 does.  pair is uploaded in Julia column-major
    order (it is symmetric)."""
    drv = driver()
    torch = drv.torch
    L = len(single)
    d_s = torch.tensor(np.asarray(single, np.float32), device="cuda")
    d_p = torch.tensor(np.asarray(pair, np.float32).ravel(order="F"), device="cuda")
    e = torch.zeros(L * L, dtype=torch.float32, device="cuda")
    sm = torch.zeros(L * L, dtype=torch.int32, device="cuda")
    bs = 256
    g = (L + bs - 1) // bs
    for diag in range(1, L):
        drv.launch("inside.cubin", K_DECODE, g, bs, ("p", e), ("p", sm), ("p", d_p), ("p", d_s), ("i", L),
                   ("i", diag), ("f", alpha))
    return e.cpu().numpy().reshape(L, L), sm.cpu().numpy().reshape(L, L)
