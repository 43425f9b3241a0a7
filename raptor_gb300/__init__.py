"""GB300-native engine for RAPTOR's per-pixel imaging hot path."""
