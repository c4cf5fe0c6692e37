"""Minimal Triangulation stand-in (no trifinder: the reference then falls back
to its own KD-tree localizer, cylag/core/solver.pyx:261-268)."""
import numpy as np


class Triangulation:
    def __init__(self, x, y, triangles=None, *args, **kwargs):
        self.x = np.asarray(x)
        self.y = np.asarray(y)
        self.triangles = np.asarray(triangles)

    def get_trifinder(self):
        raise RuntimeError("trifinder not available in the oracle environment")
