"""Oracle: CPU restatement of the reference's contraction path (test infrastructure only)."""
