"""ORACLE — test infrastructure only.

Nothing under oracle/ is imported, linked or executed by the product path
(mdtraj_gb300/).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg use it, and only as the checker or as the timed CPU baseline.

* fp64.py     — FP64 Kabsch/SVD oracle (mdtraj/geometry/alignment.py:117-181)
* cpu.py      — ctypes access to the C restatement (qcp_port.c) and to the
                reference's own CPU kernels compiled by oracle/Makefile
"""
