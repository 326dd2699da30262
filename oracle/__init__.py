"""Oracle for the Flash-SD-KDE hot path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import anything from this package, and only as the checker (or, for the
baseline, as the timed CPU implementation) -- never as part of the product.

* reference_numpy: a numpy restatement of the reference's own CPU path
  (flash_sd_kde/reference.py) in FP32, same algorithm step by step.
* fp64: the FP64 log-space density oracle (restating
  experiments/error_suite_16d/reference.py:32-82) used as ground truth.
* mlp: CPU restatement of the surrogate MLP forward/backward/Adam.
* cpu_baseline: the multi-threaded, blocked timing harness for the
  reference CPU path.

Parity pin: tests/golden/ holds fixtures generated by importing the actual
reference package (tests/golden/make_golden.py); tests/test_oracle.py checks
this restatement against them.
"""
