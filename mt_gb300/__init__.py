"""GB300-native engine for MADDY's Brownian/Langevin hot path (klyshko/MT)."""
