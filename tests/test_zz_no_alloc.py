"""messi_inside_noalloc: the inside pass for callers that cannot allocate
device memory (a framework that owns the device allocator, loops that must
not enter the driver's allocator).  It runs on the caller's stream with device-pointer inputs and a
fixed file-scope scratch array; its Z must match messi_inside's within the
parity tolerance on consecutive calls, and oversize problems are refused.

Collected last on purpose so that a stop-at-first-failure run has already
run every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-6


def _scores(L, W, seed):
    rng = np.random.default_rng(seed)
    u = rng.uniform(-80.0, -20.0, L)
    p = np.full((L, L), -np.inf)
    for i in range(L):
        j = np.arange(i + 1, min(L, i + W + 1))
        p[i, j] = u[i] + u[j] + rng.normal(-3.0, 4.0, len(j)) + (rng.random(len(j)) < 0.05) * 25.0
    p = np.maximum(p, p.T)
    return u, p


def _noalloc_Z(lib, torch, u, p, maxspan=-1, B=1.0):
    du = torch.tensor(u, dtype=torch.float64, device="cuda")
    dp = torch.tensor(np.asfortranarray(p).ravel(order="F"), dtype=torch.float64, device="cuda")
    dZ = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.messi_inside_noalloc(ctypes.c_void_p(stream), len(u), ctypes.c_void_p(du.data_ptr()),
                                  ctypes.c_void_p(dp.data_ptr()), int(maxspan), float(B), ctypes.c_void_p(dZ.data_ptr()))
    torch.cuda.synchronize()
    return rc, float(dZ.item())


def test_inside_noalloc_matches_inside_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    from messi_gb300 import _lib, api
    lib = _lib.load()
    cases = [(300, 120, 1), (900, 500, 2), (300, 120, 1)]
    for L, W, seed in cases:
        u, p = _scores(L, W, seed)
        Zref = api.computeinsideKH99(u, p)
        rc, Z = _noalloc_Z(lib, torch, u, p)
        assert rc == _lib.MESSI_OK, lib.messi_strerror(rc)
        assert abs(Z - Zref) <= REL * abs(Zref), (L, W, Z, Zref)
        rc, Z2 = _noalloc_Z(lib, torch, u, p, maxspan=W)
        assert rc == _lib.MESSI_OK and abs(Z2 - Zref) <= REL * abs(Zref)


def test_inside_noalloc_with_exponent_B():
    torch = pytest.importorskip("torch")
    from messi_gb300 import _lib, api
    lib = _lib.load()
    u, p = _scores(400, 150, 5)
    for B in (0.5, 1.7):
        Zref = api.computeinsideKH99(u, p, B=B)
        for _ in range(2):
            rc, Z = _noalloc_Z(lib, torch, u, p, maxspan=150, B=B)
            assert rc == _lib.MESSI_OK, lib.messi_strerror(rc)
            assert abs(Z - Zref) <= REL * abs(Zref), (B, Z, Zref)


def test_inside_noalloc_refuses_oversize():
    torch = pytest.importorskip("torch")
    from messi_gb300 import _lib
    lib = _lib.load()
    u, p = _scores(1100, 1099, 3)   # 1100 * 1120 > 2^20 cells per band table
    rc, _ = _noalloc_Z(lib, torch, u, p)
    assert rc == _lib.MESSI_ETOOBIG
