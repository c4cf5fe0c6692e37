"""Triangular mesh: host-side connectivity and P1 basis, uploaded once.

Mirrors ``cylag.TriangularMesh`` (cylag/geom/triangular_mesh.pyx:28-629):
the same constructor arguments and public arrays, built with vectorized
numpy instead of per-edge Python loops (a 5e5-triangle mesh builds in about a
second instead of ~11 s).  Every array is identical to the reference's,
element for element, because the path walk visits a triangle's edges in
``triedge_map`` order and picks neighbours through ``edgetri_map``:

* ``edges``: unique (min, max) vertex pairs, lexicographically sorted
  (``np.unique(..., axis=0)``, triangular_mesh.pyx:288-309);
* ``triedge_map[k]``: the three edge ids of triangle k in increasing order
  (edges are visited in index order, triangular_mesh.pyx:427-488);
* ``edgetri_map[e]``: the triangles sharing edge e in increasing order, -1
  in the second slot on the boundary;
* ``edges_labels``: -1 inside, 0 on walls, the vertex label where both
  vertices of a boundary edge carry the same label (triangular_mesh.pyx:490-558);
* ``gradx``, ``grady``, ``det``: P1 basis with alpha = 0.5/signed_area
  (triangular_mesh.pyx:560-600), same expression order.

A uniform bucket grid of triangles (``locator_grid``) replaces the KD-tree as
the global point-location structure on the device.
"""
from __future__ import annotations

import numpy as np

EPSILON = 1.0e-16
INTERN_REF = -1
BND_WALL_REF = 0
MAX_VERTEX_ADJACENCY = 15


class TriangularMesh:
    """Host mirror of ``cylag.TriangularMesh`` (triangular_mesh.pyx:75-179)."""

    def __init__(self, x, y, triangles, edges=None, vertex_adjacency=None,
                 triangle_adjacency=None, triangle_neighbors=None,
                 edgetri_map=None, triedge_map=None, boundary_points=None,
                 boundary_edges=None, vertex_labels=None, edges_labels=None,
                 signed_area=None, gradx=None, grady=None, det=None,
                 triangle_centroids=None, nopen=0):
        self.x = np.ascontiguousarray(x, dtype=np.float64)
        self.y = np.ascontiguousarray(y, dtype=np.float64)
        self.triangles = np.ascontiguousarray(triangles, dtype=np.int32)
        if self.triangles.ndim != 2 or self.triangles.shape[1] != 3:
            raise ValueError("triangles must have shape (nt, 3)")
        self.nv = self.x.shape[0]
        self.nt = self.triangles.shape[0]
        if self.nt and (self.triangles.min() < 0 or self.triangles.max() >= self.nv):
            raise ValueError("triangle vertex index out of range")
        if not (np.all(np.isfinite(self.x)) and np.all(np.isfinite(self.y))):
            raise ValueError("mesh coordinates must be finite")

        self.edges = (self._init_edges() if edges is None
                      else np.ascontiguousarray(edges, dtype=np.int32))
        self.ne = self.edges.shape[0]

        if edgetri_map is None or triedge_map is None:
            self._check_vertex_adjacency()
            self._init_triangles_edges_connectivity()
        else:
            self.edgetri_map = np.ascontiguousarray(edgetri_map, dtype=np.int32)
            self.triedge_map = np.ascontiguousarray(triedge_map, dtype=np.int32)
        self.vertex_adjacency = (self._init_vertex_adjacency() if vertex_adjacency is None
                                 else np.ascontiguousarray(vertex_adjacency, dtype=np.int32))
        self.triangle_adjacency = triangle_adjacency
        self.triangle_neighbors = triangle_neighbors

        self.nopen = int(nopen)
        self.boundary_points = boundary_points
        self.boundary_edges = boundary_edges
        if vertex_labels is None or edges_labels is None:
            self._init_boundaries()
        else:
            self.vertex_labels = np.ascontiguousarray(vertex_labels, dtype=np.int32)
            self.edges_labels = np.ascontiguousarray(edges_labels, dtype=np.int32)
            self.nvb = 0 if boundary_points is None else len(boundary_points)

        if signed_area is None:
            self._init_mesh_properties()
        else:
            self.signed_area = np.asarray(signed_area, dtype=np.float64)
            self.gradx = np.ascontiguousarray(gradx, dtype=np.float64)
            self.grady = np.ascontiguousarray(grady, dtype=np.float64)
            self.det = np.ascontiguousarray(det, dtype=np.float64)
        if triangle_centroids is None:
            # triangular_mesh.pyx:605-628 (the KD-tree's points; the bucket
            # grid replaces the tree, the centroids are kept for the files)
            t = self.triangles
            triangle_centroids = np.stack(
                [(self.x[t[:, 0]] + self.x[t[:, 1]] + self.x[t[:, 2]]) / 3.0,
                 (self.y[t[:, 0]] + self.y[t[:, 1]] + self.y[t[:, 2]]) / 3.0], axis=1)
        self.triangle_centroids = np.ascontiguousarray(triangle_centroids, dtype=np.float64)
        self._grid = None

    # -- HDF5 files (triangular_mesh.pyx:204-290) ------------------------------
    _HDF5_ARRAYS = ("x", "y", "triangles", "edges", "vertex_adjacency", "edgetri_map",
                    "triedge_map", "boundary_points", "boundary_edges", "vertex_labels",
                    "edges_labels", "signed_area", "gradx", "grady", "det",
                    "triangle_centroids")

    @staticmethod
    def from_hdf5(file_name="cylag_mesh_file.h5"):
        """triangular_mesh.pyx:204-246: every array from a CyLag mesh file
        (written by the reference's ``save_mesh_hdf5`` or by this one), so the
        mesh keeps the file's edge numbering; read by ``cylag_gb300.hdf5``."""
        from . import hdf5
        f = hdf5.read(file_name)
        missing = [k for k in TriangularMesh._HDF5_ARRAYS + ("nopen",) if k not in f]
        if missing:
            raise KeyError(f"{file_name}: not a CyLag mesh file (no {', '.join(missing)})")
        return TriangularMesh(
            f["x"], f["y"], f["triangles"], f["edges"], f["vertex_adjacency"],
            f.get("triangle_adjacency"), f.get("triangle_neighbors"), f["edgetri_map"],
            f["triedge_map"], f["boundary_points"], f["boundary_edges"], f["vertex_labels"],
            f["edges_labels"], f["signed_area"], f["gradx"], f["grady"], f["det"],
            f["triangle_centroids"], int(np.asarray(f["nopen"]).reshape(-1)[0]))

    def save_mesh_hdf5(self, file_name="cylag_mesh_file.h5"):
        """triangular_mesh.pyx:248-286: the same datasets, names and dtypes."""
        from . import hdf5
        d = {k: np.asarray(getattr(self, k)) for k in self._HDF5_ARRAYS}
        for k in ("triangle_adjacency", "triangle_neighbors"):
            if getattr(self, k, None) is not None:
                d[k] = np.asarray(getattr(self, k))
        d["nopen"] = np.array([self.nopen], dtype=np.int64)
        hdf5.write(file_name, d)

    # -- edges (triangular_mesh.pyx:288-309) --------------------------------
    @staticmethod
    def from_matplotlib(tri, boundary_points=None, boundary_edges=None, nopen=0):
        """triangular_mesh.pyx:182-201: a mesh from a triangulation object
        with ``x``, ``y``, ``triangles`` and ``edges`` (a matplotlib
        Triangulation or anything shaped like one)."""
        return TriangularMesh(tri.x, tri.y, tri.triangles, edges=tri.edges,
                              boundary_points=boundary_points, boundary_edges=boundary_edges,
                              nopen=nopen)

    def _init_edges(self):
        t = self.triangles
        a = t.reshape(-1)
        b = t[:, [1, 2, 0]].reshape(-1)
        e = np.stack([np.minimum(a, b), np.maximum(a, b)], axis=1)
        return np.ascontiguousarray(np.unique(e, axis=0), dtype=np.int32)

    # -- triangular_mesh.pyx:311-367 (overflow check only) ---------------------
    # -- triangular_mesh.pyx:311-367 ------------------------------------------
    def _init_vertex_adjacency(self):
        """[nv, MAX_VERTEX_ADJACENCY] triangles around each vertex in
        increasing triangle index, -1 padded."""
        self._check_vertex_adjacency()
        va = -np.ones((self.nv, MAX_VERTEX_ADJACENCY), dtype=np.int32)
        if self.nt == 0:
            return va
        v = self.triangles.reshape(-1).astype(np.int64)
        k = np.repeat(np.arange(self.nt, dtype=np.int64), 3)
        order = np.lexsort((k, v))
        v, k = v[order], k[order]
        start = np.searchsorted(v, np.arange(self.nv))
        slot = np.arange(len(v)) - start[v]
        va[v, slot] = k
        return va

    def _check_vertex_adjacency(self):
        cnt = np.bincount(self.triangles.reshape(-1), minlength=self.nv)
        if self.nv and cnt.max() > MAX_VERTEX_ADJACENCY:
            bad = np.nonzero(cnt > MAX_VERTEX_ADJACENCY)[0]
            raise ValueError(
                f"MAX_VERTEX_ADJACENCY overflow: {len(bad)} vertices exceed limit "
                f"{MAX_VERTEX_ADJACENCY} (max {int(cnt.max())}); first: {bad[:5].tolist()}")

    # -- triangular_mesh.pyx:427-488 -------------------------------------------
    def _init_triangles_edges_connectivity(self):
        nt, ne = self.nt, self.ne
        t = self.triangles.astype(np.int64)
        a = t.reshape(-1)
        b = t[:, [1, 2, 0]].reshape(-1)
        lo, hi = np.minimum(a, b), np.maximum(a, b)
        key = lo * np.int64(self.nv) + hi
        ekey = self.edges[:, 0].astype(np.int64) * np.int64(self.nv) + self.edges[:, 1]
        eid = np.searchsorted(ekey, key)
        if np.any(eid >= ne) or np.any(ekey[np.minimum(eid, ne - 1)] != key):
            raise ValueError("edges do not cover the triangles' sides")
        eid = eid.reshape(nt, 3)
        self.triedge_map = np.ascontiguousarray(np.sort(eid, axis=1), dtype=np.int32)
        # edge -> triangles, increasing triangle id
        flat_e = eid.reshape(-1)
        flat_k = np.repeat(np.arange(nt, dtype=np.int64), 3)
        order = np.lexsort((flat_k, flat_e))
        se, sk = flat_e[order], flat_k[order]
        first = np.ones(len(se), dtype=bool)
        first[1:] = se[1:] != se[:-1]
        etm = -np.ones((ne, 2), dtype=np.int32)
        etm[se[first], 0] = sk[first]
        second = ~first
        if np.any(second):
            # a third triangle on one edge would be a non-manifold mesh
            third = np.zeros(len(se), dtype=bool)
            third[2:] = second[2:] & second[1:-1] & (se[2:] == se[:-2])
            if np.any(third):
                raise ValueError("non-manifold mesh: an edge is shared by 3+ triangles")
            etm[se[second], 1] = sk[second]
        self.edgetri_map = etm

    # -- triangular_mesh.pyx:490-558 -------------------------------------------
    def _init_boundaries(self):
        bnd_edge = self.edgetri_map[:, 1] == -1
        if self.boundary_points is None:
            be = self.edges[bnd_edge]
            pts = np.unique(be.reshape(-1))
            self.boundary_points = np.stack(
                [pts, np.full_like(pts, BND_WALL_REF)], axis=1).astype(np.int32)
            self.boundary_edges = np.concatenate(
                [be, np.full((len(be), 1), BND_WALL_REF, dtype=np.int32)], axis=1)
        else:
            bp = np.asarray(self.boundary_points, dtype=np.int32)
            self.boundary_points = bp
            nxt = np.roll(bp, -1, axis=0)
            lab = np.where(bp[:, 1] == nxt[:, 1], bp[:, 1], BND_WALL_REF)
            self.boundary_edges = np.stack([bp[:, 0], nxt[:, 0], lab], axis=1).astype(np.int32)
        self.nvb = self.boundary_points.shape[0]
        vl = np.full(self.nv, INTERN_REF, dtype=np.int32)
        vl[self.boundary_points[:, 0]] = self.boundary_points[:, 1]
        self.vertex_labels = vl
        el = np.full(self.ne, INTERN_REF, dtype=np.int32)
        i0 = self.edges[bnd_edge, 0]
        i1 = self.edges[bnd_edge, 1]
        el[bnd_edge] = np.where(vl[i0] == vl[i1], vl[i0], BND_WALL_REF)
        self.edges_labels = el

    # -- triangular_mesh.pyx:560-600 -------------------------------------------
    def _init_mesh_properties(self):
        t = self.triangles
        xa, ya = self.x[t[:, 0]], self.y[t[:, 0]]
        xb, yb = self.x[t[:, 1]], self.y[t[:, 1]]
        xc, yc = self.x[t[:, 2]], self.y[t[:, 2]]
        sa = 0.5 * ((xb - xa) * (yc - ya) - (yb - ya) * (xc - xa))
        bad = np.abs(sa) < EPSILON
        if np.any(bad):
            k = int(np.nonzero(bad)[0][0])
            raise ValueError(f"Degenerate triangle detected at index {k}: area = {sa[k]:.2e}")
        alpha = 0.5 / sa
        self.signed_area = sa
        self.gradx = np.ascontiguousarray(np.stack(
            [(yb - yc) * alpha, (yc - ya) * alpha, (ya - yb) * alpha], axis=1))
        self.grady = np.ascontiguousarray(np.stack(
            [(xc - xb) * alpha, (xa - xc) * alpha, (xb - xa) * alpha], axis=1))
        self.det = np.ascontiguousarray(np.stack(
            [(xb * yc - xc * yb) * alpha, (xc * ya - xa * yc) * alpha,
             (xa * yb - xb * ya) * alpha], axis=1))

    # -- global point-location structure (replaces the KD-tree) ---------------
    def locator_grid(self, target_per_cell: float = 2.0):
        """Uniform grid of triangle buckets: (x0, y0, inv_cell, nx, ny,
        cell_start[nx*ny+1], cell_tris[...]).  Each bucket lists, in increasing
        triangle id, every triangle whose bounding box touches the cell, so a
        first-hit scan returns the lowest-id triangle containing a point."""
        if self._grid is not None:
            return self._grid
        t = self.triangles
        tx, ty = self.x[t], self.y[t]
        x0, x1 = float(self.x.min()), float(self.x.max())
        y0, y1 = float(self.y.min()), float(self.y.max())
        area = max((x1 - x0) * (y1 - y0), 1e-300)
        cell = max(np.sqrt(area * target_per_cell / max(self.nt, 1)), 1e-12)
        # pad each box so that points a few ulps outside a triangle (which the
        # product-sign test can still accept) stay in its buckets
        pad = 1e-6 * cell
        bx0, bx1 = tx.min(axis=1) - pad, tx.max(axis=1) + pad
        by0, by1 = ty.min(axis=1) - pad, ty.max(axis=1) + pad
        nx = max(1, int(np.ceil((x1 - x0) / cell)))
        ny = max(1, int(np.ceil((y1 - y0) / cell)))
        inv = 1.0 / cell
        cx0 = np.clip(np.floor((bx0 - x0) * inv).astype(np.int64), 0, nx - 1)
        cx1 = np.clip(np.floor((bx1 - x0) * inv).astype(np.int64), 0, nx - 1)
        cy0 = np.clip(np.floor((by0 - y0) * inv).astype(np.int64), 0, ny - 1)
        cy1 = np.clip(np.floor((by1 - y0) * inv).astype(np.int64), 0, ny - 1)
        wx, wy = cx1 - cx0 + 1, cy1 - cy0 + 1
        cnt = wx * wy
        tid = np.repeat(np.arange(self.nt, dtype=np.int64), cnt)
        off = np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt)
        wxr = np.repeat(wx, cnt)
        cx = np.repeat(cx0, cnt) + off % wxr
        cy = np.repeat(cy0, cnt) + off // wxr
        cid = cy * nx + cx
        order = np.lexsort((tid, cid))
        cid, tid = cid[order], tid[order]
        start = np.zeros(nx * ny + 1, dtype=np.int64)
        np.add.at(start, cid + 1, 1)
        start = np.cumsum(start)
        if start[-1] > np.iinfo(np.int32).max:
            raise ValueError("locator grid too large")
        self._grid = (x0, y0, inv, nx, ny, start.astype(np.int32),
                      tid.astype(np.int32))
        return self._grid

    def find_triangle(self, x: float, y: float) -> int:
        """The lowest-id triangle containing (x, y) under the reference's
        point-in-triangle test (utils.pyx:332-385: for each vertex v with
        outgoing edge eo and incoming edge ei, the cross products of eo and
        ei with p - v have one sign or one of them is zero), searched in the
        point's bucket of ``locator_grid``; -1 when none contains it.  The
        host counterpart of the device's global fallback, for pre- and
        post-processing."""
        x0, y0, inv, nx, ny, start, tris = self.locator_grid()
        fx = np.floor((x - x0) * inv)
        fy = np.floor((y - y0) * inv)
        cx = 0 if not fx >= 0. else (nx - 1 if fx > nx - 1 else int(fx))
        cy = 0 if not fy >= 0. else (ny - 1 if fy > ny - 1 else int(fy))
        c = cy * nx + cx
        cand = tris[start[c]:start[c + 1]]
        if len(cand) == 0:
            return -1
        t = self.triangles[cand]
        ax, ay = self.x[t[:, 0]], self.y[t[:, 0]]
        bx, by = self.x[t[:, 1]], self.y[t[:, 1]]
        qx, qy = self.x[t[:, 2]], self.y[t[:, 2]]

        def rot(vx, vy, eox, eoy, eix, eiy):
            wx, wy = x - vx, y - vy
            t1 = eox * wy - wx * eoy
            t2 = eix * wy - wx * eiy
            ok = (t1 == 0.) | (t2 == 0.) | (np.signbit(t1) == np.signbit(t2))
            return ok & ~np.isnan(t1) & ~np.isnan(t2)

        abx, aby = bx - ax, by - ay
        bcx, bcy = qx - bx, qy - by
        cax, cay = ax - qx, ay - qy
        inside = (rot(ax, ay, abx, aby, cax, cay) & rot(bx, by, bcx, bcy, abx, aby) &
                  rot(qx, qy, cax, cay, bcx, bcy))
        hit = np.flatnonzero(inside)
        return int(cand[hit[0]]) if len(hit) else -1
