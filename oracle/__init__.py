"""Oracle package: CPU restatement of the reference's path-tracing math.

Test infrastructure only. Product code never imports this package; tests,
`__graft_entry__.smoke()` and bench.py's CPU-baseline leg do.
"""
