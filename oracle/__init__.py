"""CPU checkers for the GPU path tracer -- test infrastructure only.

``oracle`` holds the project's CPU restatement of the reference path tracer
(xgb_cpu.cpp) and the recipe that builds the reference's own headers as a
second checker (build_ref.py, ref_harness.cpp). Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline legs import it; the product
library never does.
"""
