"""FP64 CPU oracle for MESSI's likelihood hot path.

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
(as the checker) and by ``bench.py`` (CPU baseline and ``--impl reference``
arm).  The product package ``messi_gb300`` never imports it.

* ``oracle.c_oracle``  -- ctypes binding of ``messi_oracle.c`` (restates the
  reference's CPU code, src/FARCE.jl, src/RateMatrices.jl,
  src/InsideOutsideAlgorithm.jl; see the C file for line citations).
* ``oracle.oracle_np`` -- an independent numpy/pure-Python restatement for
  tiny cases, used to cross-check the C oracle.

Parity anchor: the reference ships no golden vectors and its host language
(Julia) is absent, but its CUDA kernels (src/cuda/felsenstein.cu, inside.cu)
compile unmodified (``make -C oracle ref``, replayed by
``oracle.ref_kernels``).  Their outputs on seeded inputs are committed as
fixtures (tests/golden/reference_outputs.npz, written by
tests/golden/make_reference_fixtures.py) and the CPU suite checks the oracle
against them (tests/test_reference_fixtures.py): pair matrices, inside Z and
tables, outside tables and the posterior decoding bit for bit.  Derived
known-answer tests (tests/test_oracle.py) and the agreement of the two
restatements cover what the kernels do not.
"""
