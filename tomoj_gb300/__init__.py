"""GB300-native projection/backprojection engine for TomoJ."""
