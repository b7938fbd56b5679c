"""GB300-native engine for Spinach's static powder-averaged FID path."""
