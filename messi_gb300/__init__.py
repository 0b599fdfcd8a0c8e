"""messi_gb300 -- GB300-native (sm_103a) implementation of MESSI's likelihood hot path.

* HP1: 16-state site-pair pruning over all column pairs of an alignment on a
  rooted tree (``felsensteincuda``), plus the unpaired column likelihoods.
* HP2: KH99 SCFG inside/outside passes and base-pairing posteriors
  (``computeinsideKH99``, ``computeoutsideKH99``, ``computebasepairprobs``).
* ``computestructureintegratedlikelihood``: the whole likelihood evaluation
  resident on the device.

The kernels live in libmessi_gb300.so (C ABI: include/messi_gb300.h); this
package is the host-side mirror of the reference's Julia interface.
"""
from .dataset import Dataset, parse_newick, roottree, getnodelist  # noqa: F401
from .model import (ModelParameters, MuseSpecificParameters, getparams, getparamsvector,  # noqa: F401
                    getmusespecificparamsarray, computeprior, DEFAULT_PARAMS15)

__version__ = "0.1.0"


_API_NAMES = ("felsensteincuda", "coevolutionall", "computeunpairedlikelihoods", "maskgapped", "computeinsideKH99",
              "computeoutsideKH99", "computebasepairprobs", "computeposteriors",
              "computestructureintegratedlikelihood", "computestructureintegratedlikelihoods", "Batch", "Context",
              "get_context", "computeposteriordecodingcuda", "getPosteriorDecodingConsensusStructure",
              "consensusstructure", "samplestructures", "felsensteincudapaired", "computemodellikelihood",
              "felsensteinposteriorsiterateconditionalscuda", "subcolumnrefs")


def __getattr__(name):
    # GPU entry points load the library lazily so CPU-only tooling can import
    # the package without a CUDA device.
    if name in _API_NAMES:
        import importlib
        return getattr(importlib.import_module(".api", __name__), name)
    raise AttributeError(name)
