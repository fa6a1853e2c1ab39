"""Incircle packing of a simplex mesh (pg_pack_incenters in include/perigrain.h): the grain
centres and radii of the reference's packing generator, get_incenter_mesh_loc
(exp_dict.py:1072-1313), computed on the GPU from a mesh. The mesher itself (gmsh through pygmsh,
genmesh.py:124-291) is the caller's: `PackMesh` holds what genmesh returns (node positions,
elements, boundary nodes and segments, nodal volumes), and `rect_mesh` / `cube_mesh` build
seeded structured meshes of a rectangle / box for tests and benchmarks.

`IncenterNodes` mirrors the reference's result class (exp_dict.py:897-1000): count, range, mean,
std, occupied volume, packing ratio and trim.
"""
import ctypes as C

import numpy as np

from . import _native as N


class PackMesh:
    """A simplex mesh as genmesh returns it (genmesh.py:160-291): pos [n, dim], T [m, dim + 1],
    bdry_nodes, bdry_edges (2D boundary segments [k, 2]; boundary triangles in 3D) and the nodal
    volume `vol` (each element's area / volume split evenly over its vertices)."""

    def __init__(self, pos, T, bdry_nodes=(), bdry_edges=None):
        self.pos = np.ascontiguousarray(pos, np.float64)
        self.T = np.ascontiguousarray(T, np.int64)
        self.bdry_nodes = np.asarray(sorted(set(int(v) for v in bdry_nodes)), np.int64)
        dim = self.pos.shape[1]
        self.bdry_edges = (np.zeros((0, dim), np.int64) if bdry_edges is None
                           else np.ascontiguousarray(bdry_edges, np.int64))
        self._vol = None

    @property
    def dim(self):
        return self.pos.shape[1]

    @property
    def vol(self):
        if self._vol is None:
            self._vol = nodal_volume(self.pos, self.T)
        return self._vol


def element_volume(pos, T):
    """Triangle areas 0.5 |u x v| (genmesh.py:196-206) or tetrahedron volumes |det| / 6
    (genmesh.py:212-237)."""
    p = [pos[T[:, k]] for k in range(T.shape[1])]
    if pos.shape[1] == 2:
        u, v = p[1] - p[0], p[2] - p[0]
        return 0.5 * np.abs(u[:, 0] * v[:, 1] - u[:, 1] * v[:, 0])
    a, b, c = p[1] - p[0], p[2] - p[0], p[3] - p[0]
    return np.abs(np.einsum("ij,ij->i", c, np.cross(a, b))) / 6.0


def nodal_volume(pos, T):
    vol = np.zeros(len(pos))
    ev = element_volume(pos, T) / T.shape[1]
    for k in range(T.shape[1]):
        np.add.at(vol, T[:, k], ev)
    return vol


def rect_mesh(nx, ny, width=1.0, height=1.0, jitter=0.2, seed=0):
    """Structured triangulation of [0, width] x [0, height]: (nx + 1) x (ny + 1) nodes, interior
    nodes jittered by U(-jitter, jitter) cell sizes, every cell cut along alternating diagonals;
    boundary segments run around the rectangle."""
    rng = np.random.default_rng(seed)
    hx, hy = width / nx, height / ny
    ii, jj = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), indexing="xy")
    x = ii * hx
    y = jj * hy
    inner = (ii > 0) & (ii < nx) & (jj > 0) & (jj < ny)
    x = np.where(inner, x + rng.uniform(-jitter, jitter, x.shape) * hx, x)
    y = np.where(inner, y + rng.uniform(-jitter, jitter, y.shape) * hy, y)
    pos = np.stack([x.ravel(), y.ravel()], axis=1)
    idx = lambda i, j: j * (nx + 1) + i
    T = []
    for j in range(ny):
        for i in range(nx):
            a, b, c, d = idx(i, j), idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1)
            if (i + j) % 2 == 0:
                T += [(a, b, c), (a, c, d)]
            else:
                T += [(a, b, d), (b, c, d)]
    ring = ([idx(i, 0) for i in range(nx)] + [idx(nx, j) for j in range(ny)] +
            [idx(i, ny) for i in range(nx, 0, -1)] + [idx(0, j) for j in range(ny, 0, -1)])
    edges = [(ring[k], ring[(k + 1) % len(ring)]) for k in range(len(ring))]
    return PackMesh(pos, np.array(T, np.int64), ring, np.array(edges, np.int64))


def cube_mesh(n, size=1.0, jitter=0.2, seed=0):
    """Structured tetrahedral mesh of [0, size]^3: (n + 1)^3 nodes, interior nodes jittered, every
    cube cut into the six tetrahedra around its main diagonal; boundary triangles are the halves of
    the boundary cube faces."""
    rng = np.random.default_rng(seed)
    h = size / n
    g = np.stack(np.meshgrid(np.arange(n + 1), np.arange(n + 1), np.arange(n + 1), indexing="ij"), -1)
    g = g.reshape(-1, 3)
    inner = np.all((g > 0) & (g < n), axis=1)
    pos = g * h + np.where(inner[:, None], rng.uniform(-jitter, jitter, g.shape) * h, 0.0)
    idx = lambda i, j, k: (i * (n + 1) + j) * (n + 1) + k
    perms = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    T = []
    for i in range(n):
        for j in range(n):
            for k in range(n):
                for p in perms:
                    v = [0, 0, 0]
                    path = [idx(i, j, k)]
                    for ax in p:
                        v[ax] += 1
                        path.append(idx(i + v[0], j + v[1], k + v[2]))
                    T.append(path)
    bn = np.nonzero(~inner)[0]
    tri = []
    for axis in range(3):
        for side in (0, n):
            for a in range(n):
                for b in range(n):
                    c = [0, 0, 0]
                    o = [ax for ax in range(3) if ax != axis]
                    def node(da, db):
                        c[axis], c[o[0]], c[o[1]] = side, a + da, b + db
                        return idx(*c)
                    q = [node(0, 0), node(1, 0), node(1, 1), node(0, 1)]
                    tri += [(q[0], q[1], q[2]), (q[0], q[2], q[3])]
    return PackMesh(pos, np.array(T, np.int64), bn, np.array(tri, np.int64))


class IncenterNodes:
    """Centres and radii of a packing (exp_dict.py:897-1000)."""

    def __init__(self, incenter, incircle_rad, mesh=None, unpolished=0):
        self.incenter = incenter
        self.incircle_rad = incircle_rad
        self.mesh = mesh
        self.unpolished = unpolished

    def dim(self):
        return len(self.incenter[0])

    def count(self):
        return len(self.incircle_rad)

    def range(self):
        return [np.amin(self.incircle_rad), np.amax(self.incircle_rad)]

    def mean(self):
        return np.mean(self.incircle_rad)

    def std(self):
        return np.std(self.incircle_rad)

    def total_volume(self):
        return np.sum(self.mesh.vol)

    def occupied_volume(self):
        if self.dim() == 2:
            return np.sum(np.pi * self.incircle_rad ** 2)
        return np.sum(4 * np.pi / 3 * self.incircle_rad ** 3)

    def packing_ratio(self):
        return self.occupied_volume() / self.total_volume()

    def info(self):
        print("Count: ", self.count())
        print("Range: ", self.range())
        print("Mean: ", self.mean())
        print("Standard deviation: ", self.std())
        print("Packing ratio: ", self.packing_ratio())

    def trim(self, min_rad=None, max_rad=None):
        """Drop circles with radius below min_rad, then above max_rad (exp_dict.py:959-981)."""
        if min_rad is not None:
            keep = ~(np.ravel(self.incircle_rad) < min_rad)
            self.incenter, self.incircle_rad = self.incenter[keep], self.incircle_rad[keep]
        if max_rad is not None:
            keep = ~(np.ravel(self.incircle_rad) > max_rad)
            self.incenter, self.incircle_rad = self.incenter[keep], self.incircle_rad[keep]


def _u32(a, cols=None):
    import torch

    a = np.ascontiguousarray(a, np.int64)
    if a.size and (a.min() < 0 or a.max() > 0xFFFFFFFF):
        raise ValueError("index out of the uint32 range")
    return torch.from_numpy(a.astype(np.uint32).view(np.int32)).cuda()


def get_incenter_mesh_loc(mesh, modify_nodal_circles=True, gen_bdry=True, stream=None):
    """Incircle packing of `mesh` on the GPU; returns an IncenterNodes whose incircle_rad has
    shape [count, 1] like the reference's. modify_nodal_circles needs a 2D mesh."""
    import torch

    dim = mesh.dim
    nn, ne = len(mesh.pos), len(mesh.T)
    d_pos = torch.from_numpy(mesh.pos).cuda()
    d_T = _u32(mesh.T)
    d_bn = _u32(mesh.bdry_nodes)
    be = mesh.bdry_edges if dim == 2 else np.zeros((0, 2), np.int64)
    d_be = _u32(be)
    total = ne + nn
    d_cen = torch.empty((max(total, 1), dim), dtype=torch.float64, device="cuda")
    d_rad = torch.empty(max(total, 1), dtype=torch.float64, device="cuda")
    m = N.PackMesh()
    m.dim, m.n_nodes, m.n_elems = dim, nn, ne
    m.pos = C.c_void_p(d_pos.data_ptr())
    m.elems = C.c_void_p(d_T.data_ptr())
    m.n_bdry_nodes = len(mesh.bdry_nodes)
    m.bdry_nodes = C.c_void_p(d_bn.data_ptr() if len(mesh.bdry_nodes) else 0)
    m.n_bdry_edges = len(be)
    m.bdry_edges = C.c_void_p(d_be.data_ptr() if len(be) else 0)
    n_out, unp = C.c_uint32(), C.c_uint32()
    torch.cuda.synchronize()
    rc = N.lib().pg_pack_incenters(C.byref(m), int(bool(modify_nodal_circles)), int(bool(gen_bdry)),
                                   C.c_void_p(d_cen.data_ptr()), C.c_void_p(d_rad.data_ptr()), C.byref(n_out),
                                   C.byref(unp), stream)
    if rc != N.PG_OK:
        raise N.PerigrainError(rc, N.lib().pg_pack_last_error().decode())
    k = n_out.value
    cen = d_cen[:k].cpu().numpy()
    rad = d_rad[:k].cpu().numpy()[:, None]
    return IncenterNodes(cen, rad, mesh, unp.value)
