"""CPU oracle for the photara_drender hot path (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import this
package. The product package never does.
"""
