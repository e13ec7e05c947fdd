"""Oracle package: a CPU restatement of the reference's grid-fluid path, used
only by the test-suite, __graft_entry__.smoke() and bench.py's CPU baseline
as the checker / timed CPU reference.  Product code never imports it."""
