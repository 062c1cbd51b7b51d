"""GB300-native depth-fusion hot path of voxelhashmt."""
