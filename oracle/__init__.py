"""Oracle package — test infrastructure only.

CPU restatements of LightNE's hot path that the tests, the smoke check and
the CPU leg of the benchmark use as the checker.  Product code never imports
this package.
"""
