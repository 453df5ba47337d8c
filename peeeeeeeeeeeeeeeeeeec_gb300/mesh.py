"""Synthetic PEEC meshes (plates and closed boxes) as the C ABI structs.

Wraps libpeec_mesh.so: the mesh, its topology and its dual mesh are built in
C with the reference's numbering rules, and exposed both as ctypes structs
(to pass to the drop-in entry points) and as numpy views.
"""
import ctypes as C

import numpy as np

from . import abi


class SynthMesh:
    """A Mesh + DualMesh pair owned by the C mesher (freed on close())."""

    def __init__(self):
        self.mesh = abi.Mesh()
        self.dual = abi.DualMesh()
        self._lib = abi.load_mesh_lib()
        self._open = False

    # ---- constructors ------------------------------------------------
    @classmethod
    def plate(cls, lx, ly, nx, ny):
        m = cls()
        m._check(m._lib.peec_synth_plate(lx, ly, nx, ny, C.byref(m.mesh)), "plate")
        m._finish()
        return m

    @classmethod
    def box(cls, lx, ly, lz, nx, ny, nz):
        m = cls()
        m._check(m._lib.peec_synth_box(lx, ly, lz, nx, ny, nz, C.byref(m.mesh)), "box")
        m._finish()
        return m

    @classmethod
    def box_h(cls, lx, ly, lz, h):
        """Box with cells of edge ~h (counts rounded to the nearest integer)."""
        n = [max(1, int(round(v / h))) for v in (lx, ly, lz)]
        return cls.box(lx, ly, lz, *n)

    @classmethod
    def from_arrays(cls, xyz, quads):
        m = cls()
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        quads = np.ascontiguousarray(quads, dtype=np.int32).reshape(-1, 4)
        m._check(m._lib.peec_synth_from_arrays(
            xyz.ctypes.data_as(abi.c_double_p), xyz.shape[0],
            quads.ctypes.data_as(abi.c_int_p), quads.shape[0], C.byref(m.mesh)), "from_arrays")
        m._finish()
        return m

    def _check(self, status, what):
        if status != 0:
            raise RuntimeError("synthetic mesh step failed: %s" % what)

    def _finish(self):
        self._open = True
        self._check(self._lib.peec_synth_topology(C.byref(self.mesh)), "topology")
        self._check(self._lib.peec_synth_dual(C.byref(self.mesh), C.byref(self.dual)), "dual")

    def close(self):
        if self._open:
            self._lib.peec_synth_dual_free(C.byref(self.dual))
            self._lib.peec_synth_mesh_free(C.byref(self.mesh))
            self._open = False

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- sizes and views ---------------------------------------------
    @property
    def n_nodes(self):
        return self.mesh.n_nodes

    @property
    def n_edges(self):
        return self.mesh.n_edges

    @property
    def n_quads(self):
        return self.mesh.n_quads

    def array(self, name, shape, dtype=np.float64):
        ptr = getattr(self.mesh, name)
        n = int(np.prod(shape))
        ctype = C.c_double if dtype == np.float64 else C.c_int
        buf = C.cast(ptr, C.POINTER(ctype * n)).contents
        return np.frombuffer(buf, dtype=dtype).reshape(shape).copy()

    def edges(self):
        return self.array("edges", (self.n_edges, 2), np.int32)

    def edge_lengths(self):
        return self.array("edge_lengths", (self.n_edges,))

    def edge_directions(self):
        return self.array("edge_directions", (self.n_edges, 3))

    def cell_edges(self):
        return self.array("cell_edges", (self.n_quads, 4), np.int32)

    def cell_edge_signs(self):
        return self.array("cell_edge_signs", (self.n_quads, 4), np.int32)

    def patches(self, kind):
        """List (per region) of (count, 4, 3) corner arrays; kind 'edge' or 'node'."""
        lists = self.dual.edge_patches if kind == "edge" else self.dual.node_patches
        n = self.n_edges if kind == "edge" else self.n_nodes
        out = []
        for r in range(n):
            L = lists[r]
            pts = np.array([[L.patches[k].points[t] for t in range(12)] for k in range(L.count)])
            out.append(pts.reshape(-1, 4, 3))
        return out

    def region_areas(self, kind):
        n = self.n_edges if kind == "edge" else self.n_nodes
        ptr = self.dual.edge_region_areas if kind == "edge" else self.dual.node_region_areas
        return np.ctypeslib.as_array(ptr, shape=(n,)).copy()

    def incidence(self):
        """Dense Ne x Nv incidence, -1 at the tail and +1 at the head of each
        edge (the harmonic system's A block)."""
        e = self.edges()
        A = np.zeros((self.n_edges, self.n_nodes))
        A[np.arange(self.n_edges), e[:, 0]] = -1.0
        A[np.arange(self.n_edges), e[:, 1]] = 1.0
        return A
