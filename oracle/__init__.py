"""The oracle: a CPU restatement of lyon's tessellation algorithms (test infrastructure only)."""
