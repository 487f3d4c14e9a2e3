"""ORACLE -- test infrastructure, not the product.

A CPU restatement of pydyn's dynamic step (the reference's NumPy transcription of TM5):
scalar C for the per-line and per-column kernels (oracle/src/*.c, built by oracle/build.py
into oracle/_build/liboracle.so) and NumPy for the region-tree glue and the driver
(oracle/zoom.py).  Each function cites the reference file:line it follows.

It is pinned to the reference by the golden fixtures under tests/golden/ (made by
tests/golden/make_golden.py from pydyn itself) and is used only by tests/, by
__graft_entry__.smoke() and by bench.py's CPU-baseline leg, always as the checker or the
baseline, never as the thing measured or shipped.
"""
