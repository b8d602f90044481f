"""TEST INFRASTRUCTURE ONLY: the CPU oracle (restatement of the reference CPU
path) and its parity helpers.  Not part of the product; see tw_oracle.cpp."""
