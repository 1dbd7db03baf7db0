"""Oracle for the astronomix MHD step -- TEST INFRASTRUCTURE ONLY.

A CPU restatement (NumPy, optionally torch for gradients) of the reference's
finite-volume and finite-difference MHD path, written operation for operation
from leo1200/astronomix 0.5.1 and pinned against the reference's own golden
data (tests/mhd_tests/final_state_orszag_tang.npz), the exact Sod solution and
conservation properties.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this package, and only as the checker or the timed CPU
baseline.  The product (``astronomix_gb300``) never imports it and has no CPU
fallback.
"""
