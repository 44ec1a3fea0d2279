"""CPU oracle (test infrastructure only): see oracle/psim_oracle.h."""
