"""GB300-native node evolver for Galacticus (mergerTreeNodeEvolver drop-in)."""
