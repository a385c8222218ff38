"""CPU oracle for the GPU sweep: test infrastructure only (see sn_oracle.h)."""
