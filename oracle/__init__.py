"""CPU oracle for the Bio-CFD hot path -- test infrastructure only, never shipped."""
