"""GB300-native stochastic myocyte simulator (drop-in for cuda_Cell_Detailed)."""
