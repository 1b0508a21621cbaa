"""mmsp_gb300: GB300-native explicit phase-field step for MMSP grids."""
