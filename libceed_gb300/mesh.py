"""Structured box meshes and seeded inputs for the hexahedral operators (user-side helpers).

The pattern is that of examples/ceed/ex1-volume.c (BuildCartesianRestriction): an nx x ny x nz box of
hexahedra on [0,1]^3, lexicographic element and node numbering, a trilinear coordinate field on the
vertices, and an H1 field of degree P-1 on Gauss-Lobatto nodes.  Vertices interior to the box move by
noise*h*U[-1,1) per coordinate, so the box faces stay planar.

Random values come from a counter-based splitmix64 stream: value i of stream `seed` is uniform on [lo, hi)
and independent of how the stream is cut, so any slice of a large input can be regenerated.
"""
import numpy as np

_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_K1 = np.uint64(0xD1B54A32D192ED03)
_K2 = np.uint64(0x9E3779B97F4A7C15)


def uniform(seed, n, lo=-1.0, hi=1.0, start=0):
    """n values of the stream `seed`, starting at index `start`, uniform on [lo, hi)."""
    return _uniform_at(seed, np.arange(start, start + n, dtype=np.uint64), lo, hi)


def box_vertices(nx, ny, nz, noise, seed):
    """Vertex coordinates, component-major: coords[c * num_vertices + v] (comp_stride = num_vertices)."""
    nvx, nvy, nvz = nx + 1, ny + 1, nz + 1
    nv = nvx * nvy * nvz
    k, j, i = np.meshgrid(np.arange(nvz), np.arange(nvy), np.arange(nvx), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    v = i + nvx * (j + nvy * k)
    interior = (i > 0) & (i < nx) & (j > 0) & (j < ny) & (k > 0) & (k < nz)
    coords = np.empty(3 * nv)
    for c, (idx, n) in enumerate(((i, nx), (j, ny), (k, nz))):
        x = idx.astype(np.float64) / float(n)
        r = _uniform_at(seed, 3 * v.astype(np.uint64) + np.uint64(c))
        x = np.where(interior, x + noise * (1.0 / float(n)) * r, x)
        coords[c * nv + v] = x
    return coords


def _uniform_at(seed, counters, lo=-1.0, hi=1.0):
    with np.errstate(over="ignore"):
        z = np.uint64(seed) * _K1 + (counters.astype(np.uint64) + np.uint64(1)) * _K2
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    u = (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return lo + (hi - lo) * u


def box_offsets(nx, ny, nz, P, ncomp_interlaced=1):
    """int32 offsets [elem][P^3] of a degree P-1 field; scaled by ncomp_interlaced for interlaced components."""
    p = P - 1
    ndx, ndy = nx * p + 1, ny * p + 1
    ez, ey, ex = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    lz, ly, lx = np.meshgrid(np.arange(P), np.arange(P), np.arange(P), indexing="ij")
    ex, ey, ez = (a.reshape(-1, 1).astype(np.int64) for a in (ex, ey, ez))
    lx, ly, lz = (a.reshape(1, -1).astype(np.int64) for a in (lx, ly, lz))
    g = (ex * p + lx) + ndx * ((ey * p + ly) + ndy * (ez * p + lz))
    scale = ncomp_interlaced if ncomp_interlaced > 1 else 1
    g = g * scale
    if g.max() >= 2 ** 31:
        raise ValueError("offsets exceed int32 (CeedInt) range")
    return np.ascontiguousarray(g.astype(np.int32).ravel())


class Box:
    """A box-mesh problem: sizes, offsets, coordinates and a seeded input vector.

    n elements per direction, polynomial degree `degree` (P = degree + 1, Q = degree + 2 Gauss points).
    """

    def __init__(self, n, degree, ncomp=1, noise=0.05, seed=1):
        self.n, self.degree, self.ncomp = n, degree, ncomp
        self.P, self.Q = degree + 1, degree + 2
        self.num_elem = n ** 3
        nd = n * degree + 1
        self.num_nodes = nd ** 3
        self.l_size = self.num_nodes * ncomp
        self.comp_stride = self.num_nodes if ncomp == 1 else 1
        self.num_vertices = (n + 1) ** 3
        self.seed, self.noise = seed, noise

    def coords(self):
        return box_vertices(self.n, self.n, self.n, self.noise, self.seed)

    def vertex_offsets(self):
        return box_offsets(self.n, self.n, self.n, 2, 1)

    def offsets(self):
        return box_offsets(self.n, self.n, self.n, self.P, self.ncomp)

    def u(self, seed=None):
        return uniform(self.seed + 1 if seed is None else seed, self.l_size)

    def node_coords(self):
        """Physical (x, y, z) of every solution node, shape [num_nodes, 3] in L-vector node order: the trilinear map
        of each element's 8 vertices evaluated at its Gauss-Lobatto nodes (the coordinate field that Poisson3DBuild and
        Mass3DBuild see; neighbouring elements agree on shared nodes because the map is conforming)."""
        from .basis1d import lobatto_quadrature

        n, p = self.n, self.degree
        nd, nv1 = n * p + 1, n + 1
        gll, _ = lobatto_quadrature(p + 1)
        lat = np.arange(nd)
        elem = np.minimum(lat // p, n - 1)                     # element along one direction; the last node stays in n - 1
        t = 0.5 * (gll[lat - elem * p] + 1.0)                  # reference coordinate in [0, 1] inside that element
        X = self.coords().reshape(3, nv1, nv1, nv1)            # [c][k][j][i]
        out = np.zeros((3, nd, nd, nd))
        for dk in (0, 1):
            wz = (t if dk else 1.0 - t)[:, None, None]
            for dj in (0, 1):
                wy = (t if dj else 1.0 - t)[None, :, None]
                for di in (0, 1):
                    wx = (t if di else 1.0 - t)[None, None, :]
                    corner = X[:, (elem + dk)[:, None, None], (elem + dj)[None, :, None], (elem + di)[None, None, :]]
                    out += wz * wy * wx * corner
        return np.ascontiguousarray(out.reshape(3, -1).T)


def node_lattice(n, degree):
    """Reference (unperturbed) coordinates in [0,1] of the 1D node lattice: element k's Gauss-Lobatto nodes."""
    from .basis1d import lobatto_quadrature

    gll, _ = lobatto_quadrature(degree + 1)
    x = np.empty(n * degree + 1)
    for k in range(n):
        x[k * degree:(k + 1) * degree + 1] = (k + 0.5 * (gll + 1.0)) / n
    return x


def box_mask(n, degree, ncomp=1):
    """1 on nodes strictly inside the box, 0 on its faces (homogeneous Dirichlet), per L-vector entry."""
    nd = n * degree + 1
    inner = np.ones(nd)
    inner[0] = inner[-1] = 0.0
    m = (inner[None, None, :] * inner[None, :, None] * inner[:, None, None]).reshape(-1)
    return np.repeat(m, ncomp) if ncomp > 1 else m


def smooth_field(n, degree, seed, modes=8):
    """Sum of `modes` seeded low-frequency sines on the node lattice (the manufactured solution of the solve)."""
    x = node_lattice(n, degree)
    r = uniform(seed, 4 * modes, 0.0, 1.0)
    out = np.zeros((x.size, x.size, x.size))
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    for k in range(modes):
        fx, fy, fz = 1 + int(3 * r[4 * k]), 1 + int(3 * r[4 * k + 1]), 1 + int(3 * r[4 * k + 2])
        out += (0.5 + r[4 * k + 3]) * np.sin(np.pi * fx * X) * np.sin(np.pi * fy * Y) * np.sin(np.pi * fz * Z)
    return out.reshape(-1)
