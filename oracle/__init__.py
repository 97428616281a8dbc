"""CPU oracle for the GB300 decoder (test infrastructure only)."""
