"""CPU restatement of the reference shader: test infrastructure (the oracle)."""
