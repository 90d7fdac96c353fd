"""CPU oracle of the sparse-mesh path (TEST INFRASTRUCTURE ONLY).

A restatement of the reference's algorithms, used as the checker by
``tests/``, by ``__graft_entry__.smoke()`` and as the timed CPU baseline of
``bench.py``; the product never imports it.  Every function cites the
reference file:line it follows.  Parity of the oracle itself is pinned by
``tests/test_oracle_golden.py`` against fixtures produced by running the
reference (``tests/golden/make_golden.py``).

Floating-point work is written with torch CPU ops, the same aten ops the
reference's CPU backend executes (index, scatter_reduce_, elementwise), in
the reference's order; integer work in numpy / plain Python.
"""
