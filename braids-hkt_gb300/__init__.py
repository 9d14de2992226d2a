"""GB300-native shallow-water solver step of BRAIDS-HKT (augmented f-wave river path)."""
