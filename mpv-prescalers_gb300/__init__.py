"""GB300-native RAVU / NNEDI3 prescalers (placeholder, filled in below)."""
