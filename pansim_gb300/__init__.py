"""pansim_gb300: GB300-native PanSim per-timestep agent loop."""
__version__ = "0.1.0"
