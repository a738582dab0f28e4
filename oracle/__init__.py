"""TEST INFRASTRUCTURE ONLY: the CPU oracle (see oracle/ocsl_oracle.h)."""
