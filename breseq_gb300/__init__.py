"""GB300-native replacement for breseq's read-evidence scoring path (error_count, identify_mutations,
per-position coverage), over the C ABI declared in include/breseq_gb300.h."""
