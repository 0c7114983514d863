"""CPU oracle of the BGPQ hot path -- test infrastructure only (see bgpq_oracle.h)."""
