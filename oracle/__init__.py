"""CPU FP64 restatement of binary2d's finite-volume step: test infrastructure
only (correctness oracle and timed CPU baseline).  Parity with the Rust
reference is unpinned; see oracle.h."""
