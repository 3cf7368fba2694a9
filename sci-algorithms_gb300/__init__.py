"""GB300-native GAP-TV / ADMM-TV reconstruction for snapshot compressive imaging."""
