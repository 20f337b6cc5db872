"""GB300-native drop-in for sfmtory's sfm-ba bundle adjuster (placeholder, filled below)."""
