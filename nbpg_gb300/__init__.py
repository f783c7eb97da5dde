"""GB300-native NBPG search/build hot path (greedy beam search, RobustPrune build, brute-force kNN)."""
