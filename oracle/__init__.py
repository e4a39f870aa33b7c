"""FP64 CPU oracle of the vibrational-level solver (test infrastructure only)."""
