"""Python side of the GB300 Euler residual-and-update path (ctypes over libaero_gb300.so)."""
