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
    ci, cj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    ci, cj = ci.ravel(), cj.ravel()  # cells in row-major order (j outer, i inner)
    a = cj * (nx + 1) + ci
    b, c, d = a + 1, a + nx + 2, a + nx + 1
    even = (ci + cj) % 2 == 0
    t1 = np.where(even[:, None], np.stack([a, b, c], 1), np.stack([a, b, d], 1))
    t2 = np.where(even[:, None], np.stack([a, c, d], 1), np.stack([b, c, d], 1))
    T = np.stack([t1, t2], 1).reshape(-1, 3)
    idx = lambda i, j: j * (nx + 1) + i
    ring = np.concatenate([idx(np.arange(nx), 0), idx(nx, np.arange(ny)), idx(np.arange(nx, 0, -1), ny),
                           idx(0, np.arange(ny, 0, -1))])
    edges = np.stack([ring, np.roll(ring, -1)], 1)
    return PackMesh(pos, T, ring, edges)


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


def pack_device(d_pos, d_T, d_bdry_nodes, d_bdry_edges, modify_nodal_circles=True, gen_bdry=True, stream=None):
    """pg_pack_incenters on device tensors (float64 [n, dim]; int32 views of uint32 indices);
    returns (centres [k, dim], radii [k], unpolished) as device tensors."""
    import torch

    nn, dim = d_pos.shape
    ne = d_T.shape[0]
    total = ne + nn
    d_cen = torch.empty((max(total, 1), dim), dtype=torch.float64, device=d_pos.device)
    d_rad = torch.empty(max(total, 1), dtype=torch.float64, device=d_pos.device)
    m = N.PackMesh()
    m.dim, m.n_nodes, m.n_elems = dim, nn, ne
    m.pos = C.c_void_p(d_pos.data_ptr())
    m.elems = C.c_void_p(d_T.data_ptr())
    m.n_bdry_nodes = d_bdry_nodes.numel()
    m.bdry_nodes = C.c_void_p(d_bdry_nodes.data_ptr() if d_bdry_nodes.numel() else 0)
    m.n_bdry_edges = d_bdry_edges.shape[0] if d_bdry_edges.numel() else 0
    m.bdry_edges = C.c_void_p(d_bdry_edges.data_ptr() if d_bdry_edges.numel() else 0)
    n_out, unp = C.c_uint32(), C.c_uint32()
    rc = N.lib().pg_pack_incenters(C.byref(m), int(bool(modify_nodal_circles)), int(bool(gen_bdry)),
                                   C.c_void_p(d_cen.data_ptr()), C.c_void_p(d_rad.data_ptr()), C.byref(n_out),
                                   C.byref(unp), stream)
    if rc != N.PG_OK:
        raise N.PerigrainError(rc, N.lib().pg_pack_last_error().decode())
    k = n_out.value
    return d_cen[:k], d_rad[:k], unp.value


def get_incenter_mesh_loc(mesh, modify_nodal_circles=True, gen_bdry=True, stream=None):
    """Incircle packing of `mesh` on the GPU; returns an IncenterNodes whose incircle_rad has
    shape [count, 1] like the reference's. modify_nodal_circles needs a 2D mesh."""
    import torch

    be = mesh.bdry_edges if mesh.dim == 2 else np.zeros((0, 2), np.int64)
    d_pos = torch.from_numpy(mesh.pos).cuda()
    d_T, d_bn, d_be = _u32(mesh.T), _u32(mesh.bdry_nodes), _u32(be.reshape(-1, 2))
    torch.cuda.synchronize()
    d_cen, d_rad, unp = pack_device(d_pos, d_T, d_bn, d_be, modify_nodal_circles, gen_bdry, stream)
    return IncenterNodes(d_cen.cpu().numpy(), d_rad.cpu().numpy()[:, None], mesh, unp)
