"""GB300-native generalized-coordinates physics step (brax.generalized drop-in)."""
