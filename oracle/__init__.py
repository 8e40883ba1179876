"""CPU oracle of the FDTD hot path (test infrastructure; see fdtd_oracle.cpp)."""
