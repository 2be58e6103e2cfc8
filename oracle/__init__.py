"""The CPU oracle (test infrastructure only; see vsmc_oracle.h)."""
