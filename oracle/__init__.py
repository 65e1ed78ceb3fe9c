"""CPU oracle for AMDAT's hot path: test infrastructure only (checker, CPU baseline)."""
