"""ctypes binding of libmessi_gb300.so (the C ABI of include/messi_gb300.h).

There is no CPU fallback: loading fails loudly when the library is missing,
and every call raises ``MessiError`` on a non-zero status.
"""
import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmessi_gb300.so")

MESSI_OK = 0
MESSI_EINVAL = -1
MESSI_ENOMEM = -2
MESSI_ECUDA = -3
MESSI_ETIMEOUT = -4
MESSI_ESTATE = -5
MESSI_ETOOBIG = -6


class MessiError(RuntimeError):
    def __init__(self, status, what, detail=""):
        self.status = status
        super().__init__(f"{what}: {_strerror(status)} ({status}){': ' + detail if detail else ''}")


class Alignment(ctypes.Structure):
    _fields_ = [("numseqs", ctypes.c_int32), ("numcols", ctypes.c_int32), ("numnodes", ctypes.c_int32),
                ("masks", ctypes.c_void_p), ("children", ctypes.c_void_p), ("seqindex", ctypes.c_void_p)]


class Model(ctypes.Structure):
    _fields_ = [("freqs", ctypes.c_double * 4), ("q", ctypes.c_double * 6), ("branchlengths", ctypes.c_void_p),
                ("nsite", ctypes.c_int32), ("siteRates", ctypes.c_void_p), ("siteWeights", ctypes.c_void_p),
                ("nlambda", ctypes.c_int32), ("lambdaGC", ctypes.c_void_p), ("lambdaAT", ctypes.c_void_p),
                ("lambdaGT", ctypes.c_void_p), ("lambdaWeights", ctypes.c_void_p)]


_lock = threading.Lock()
_lib = None

# name -> (restype, argtypes)
_SIGS = {
    "messi_strerror": (ctypes.c_char_p, [ctypes.c_int]),
    "messi_version": (ctypes.c_int, []),
    "messi_ctx_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "messi_ctx_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "messi_ctx_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "messi_ctx_last_launches": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]),
    "messi_ctx_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "messi_selftest_bounded_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32)]),
    "messi_host_reversible_eig": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                 ctypes.c_void_p]),
    "messi_ctx_graph_replays": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]),
    "messi_ctx_launch_shapes": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32),
                                               ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]),
    "messi_ctx_profile": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "messi_ctx_profile_read": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                              ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double)]),
    "messi_dataset_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Alignment), ctypes.c_int32,
                                            ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "messi_dataset_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "messi_dataset_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]),
    "messi_felsenstein_pairs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Model),
                                               ctypes.c_void_p, ctypes.c_void_p]),
    "messi_unpaired": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Model), ctypes.c_void_p]),
    "messi_inside": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_int32, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]),
    "messi_outside": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]),
    "messi_basepairprobs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                           ctypes.c_void_p]),
    "messi_posteriors": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "messi_likelihood": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Model), ctypes.c_void_p,
                                        ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]),
    "messi_subcolumnrefs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "messi_siterate_conditionals": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Model),
                                                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "messi_structure_likelihood": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Model),
                                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "messi_posterior_decoding": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "messi_consensus_structure": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                                 ctypes.c_int32, ctypes.c_double, ctypes.c_void_p]),
    "messi_sample_structures": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64, ctypes.c_void_p,
                                               ctypes.c_void_p]),
    "messi_batch_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.POINTER(ctypes.c_void_p)]),
    "messi_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "messi_batch_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]),
    "messi_batch_likelihood": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_double, ctypes.c_void_p]),
    "messi_inside_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_int32, ctypes.c_double, ctypes.c_void_p]),
    "messi_mlp_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                        ctypes.c_int32, ctypes.c_uint64, ctypes.POINTER(ctypes.c_void_p)]),
    "messi_mlp_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "messi_mlp_nparams": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32)]),
    "messi_mlp_get_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "messi_mlp_set_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "messi_mlp_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                         ctypes.c_void_p]),
    "messi_mlp_gradients": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.c_void_p]),
    "messi_mlp_train_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_float, ctypes.c_float,
                                            ctypes.POINTER(ctypes.c_float)]),
}

EXPORTED = tuple(_SIGS)


def load(path=None):
    """Load the library (building it first when sources changed)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            try:
                from . import build as _build
                _build.build()
            except Exception as exc:  # toolkit missing, compile error
                raise ImportError(f"libmessi_gb300.so is not built and could not be built: {exc}") from exc
        lib = ctypes.CDLL(p)
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def _strerror(status):
    try:
        return load().messi_strerror(status).decode()
    except Exception:
        return "error"


def check(status, what, ctx=None):
    if status != MESSI_OK:
        detail = ""
        if ctx is not None:
            try:
                detail = load().messi_ctx_last_error(ctx).decode()
            except Exception:
                pass
        raise MessiError(status, what, detail)
