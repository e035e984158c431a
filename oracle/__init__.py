"""Oracles for the bitstream hot path.

TEST INFRASTRUCTURE ONLY.  These modules are the checker: ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py``
may use them; the product (``bitgen_gb300``) never imports, links or executes anything here.

* ``pablo_ref``  – big-integer whole-stream Pablo interpreter and transpose restatement.
* ``nfa_ref``    – independent byte-level NFA simulator producing regex match-end streams.
* ``bg_cpu.c``   – multi-threaded C word-parallel evaluator (full-size parity and CPU baseline),
  loaded through ``cpu.py``.
"""
