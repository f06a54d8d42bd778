"""Oracle: CPU FP64 restatement of IDWarp's warping path (test infrastructure only)."""
