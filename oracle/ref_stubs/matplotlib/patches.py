"""Minimal Polygon stand-in built on the Path stand-in."""
from .path import Path


class Polygon:
    def __init__(self, xy, *args, **kwargs):
        self._path = Path(xy)

    def get_path(self):
        return self._path

    def contains_point(self, point, *args, **kwargs):
        return self._path.contains_point(point)
