"""Minimal Path stand-in (even-odd point-in-polygon test)."""
import numpy as np


class Path:
    def __init__(self, vertices, codes=None, *args, **kwargs):
        self.vertices = np.asarray(vertices, dtype=float)
        self.codes = codes

    def contains_point(self, point, *args, **kwargs):
        x, y = float(point[0]), float(point[1])
        v = self.vertices
        inside = False
        n = len(v)
        for i in range(n):
            x0, y0 = v[i]
            x1, y1 = v[(i + 1) % n]
            if (y0 > y) != (y1 > y):
                xc = x0 + (y - y0) * (x1 - x0) / (y1 - y0)
                if x < xc:
                    inside = not inside
        return inside

    def contains_points(self, points, *args, **kwargs):
        return np.array([self.contains_point(p) for p in points], dtype=bool)
