"""CPU oracle for the ugacc RHF coupled-cluster hot path.

TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg import this package, and only as the checker (or as the timed CPU
baseline); the GPU library never calls it.

Two parts:

* ``oracle.cc`` -- a numpy restatement of the reference's algorithm (ugacc
  ccwfn.cc, hbar.cc, cclambda.cc, ccdensity.cc, ccpert.cc, ccresp.cc and the
  response recipe of ugacc.cc), term by term, each function citing the reference
  lines it follows.  Pinned against the golden fixtures in tests/golden/, which were
  produced by the reference's own sources (see ``oracle/Makefile``).
* ``oracle/Makefile`` + ``oracle/ref_shim/`` -- builds the reference's own hot-path
  sources, read in place, against a small psi4 stand-in into ``oracle/_ref/``.  That
  binary exists only where the reference tree is present.
"""
