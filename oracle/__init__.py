"""Oracle package: a CPU restatement of the reference's grid-fluid path, used
only by the test-suite, __graft_entry__.smoke() and bench.py's CPU baseline
as the reference results to compare against and the timed CPU
baseline.  Product code never imports it."""
