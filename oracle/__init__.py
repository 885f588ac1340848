"""TEST INFRASTRUCTURE ONLY: the CPU oracle (C++ restatement of CosTaL 2.1.0's kNN-graph path).

Only tests/, __graft_entry__.smoke() (as the checker) and bench.py's CPU-baseline leg use it.
"""
