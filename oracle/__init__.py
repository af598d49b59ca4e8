"""CPU restatement of strobealign's mapping path (test infrastructure only): the
checker for the GPU library's parity tests and the timed CPU baseline."""
