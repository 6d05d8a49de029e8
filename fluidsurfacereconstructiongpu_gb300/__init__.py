"""GB300-native particle-to-mesh fluid surface reconstruction."""
