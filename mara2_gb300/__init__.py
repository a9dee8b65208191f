"""GB300-native finite-volume time step for Mara2 (placeholder; filled below)."""
