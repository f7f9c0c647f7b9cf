"""CPU oracle for the breseq read-evidence scoring path (test infrastructure only)."""
