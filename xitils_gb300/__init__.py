"""xitils_gb300 -- GB300-native drop-in for Xitils' path-tracer render call."""
