"""GB300-native backend for subby's eigensubstitution hot path (placeholder init)."""
