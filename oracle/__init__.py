"""CPU oracle (test infrastructure): a restatement of the reference hot path, used only by
tests/, __graft_entry__.smoke() and bench.py's CPU baseline to check against. Parity of the oracle is
pinned against fixtures generated by executing the reference (tests/golden/make_golden.py)."""
