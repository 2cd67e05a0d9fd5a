"""htr_gb300: GB300-native explicit RHS of the HTR solver (package root)."""
