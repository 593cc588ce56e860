"""GB300-native step engine for the GENESIS hsolve chanmode 4/5 path."""
