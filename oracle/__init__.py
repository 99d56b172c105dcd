"""CPU oracle for the BoR-MoM path -- TEST INFRASTRUCTURE ONLY (see bor_oracle)."""
