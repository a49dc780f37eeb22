"""CPU oracle for the DFPSR triangle path -- test infrastructure only.

`oracle.port` loads the plain-C restatement (oracle/dsr_oracle.c); `oracle.ref`
loads the reference itself, built out-of-tree by oracle/Makefile.ref into
oracle/_ref/ (present only where the reference sources were available).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package; the product never does.
"""
