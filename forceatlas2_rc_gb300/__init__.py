"""GB300-native ForceAtlas2 layout engine (placeholder; filled below)."""
