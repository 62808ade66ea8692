"""postmps_gb300 -- GB300-native particle-to-surface pipeline (see include/pms.h)."""
