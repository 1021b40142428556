"""Oracle package — test infrastructure only (CPU FP64 restatement of the
reference hot path and the reference's own compiled ba_interp2).  Only tests,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may use it."""
