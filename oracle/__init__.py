"""FP64 CPU oracle for MESSI's likelihood hot path.

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
(as the checker) and by ``bench.py`` (CPU baseline and ``--impl reference``
arm).  The product package ``messi_gb300`` never imports it.

* ``oracle.c_oracle``  -- ctypes binding of ``messi_oracle.c`` (restates the
  reference's CPU code, src/FARCE.jl, src/RateMatrices.jl,
  src/InsideOutsideAlgorithm.jl; see the C file for line citations).
* ``oracle.oracle_np`` -- an independent numpy/pure-Python restatement for
  tiny cases, used to cross-check the C oracle.

Parity anchor: the reference ships no golden vectors and cannot run here (it is
Julia), so the oracle is pinned by derived known-answer tests
(tests/test_oracle.py) and by the agreement of the two restatements.
"""
