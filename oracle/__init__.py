"""Oracle: CPU restatement of the reference's FP64 query path. TEST INFRASTRUCTURE ONLY —
only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use it."""
