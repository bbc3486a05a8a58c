"""CPU oracle for the ExaMiniMD hot path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
arm use this package, and only as the checker or the timed CPU baseline.
The product library (examinimd_gb300) never imports it.
"""
