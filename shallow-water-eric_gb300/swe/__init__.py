"""GB300-native explicit P1 shallow-water step (host-side Python package)."""
