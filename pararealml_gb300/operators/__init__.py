"""GPU operators mirroring ``pararealml.operators`` (fdm and parareal)."""
