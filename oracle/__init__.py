"""CPU oracle of the TensorSat contraction path -- test infrastructure only.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use this
package, as the checker (or as the timed CPU baseline). The product package
``tensorsat_gb300`` never imports it.
"""
