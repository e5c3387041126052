"""GB300-native Levenberg-Marquardt back end for SymForce's sym::Optimizer hot path."""
