"""Synthetic surface meshes in the reference VTK dialect.

The reference reads legacy ASCII VTK where the first integer of every CELLS
row is the body id (src/preprocess/mesh_data.rs:132-142).  These generators
produce the benchmark bodies (icosphere, cube-sphere, ellipsoid, harmonic
perturbed sphere) with outward normals, as the reference's test meshes have,
and write them in that dialect (one body, id 1).
"""
import math

import numpy as np


def write_vtk(path, nodes, cells, cell_type, body_id=1, title="synthetic mesh"):
    nodes = np.asarray(nodes, dtype=float)
    cells = np.asarray(cells, dtype=np.int64)
    with open(path, "w") as f:
        f.write("# vtk DataFile Version 2.0\n%s\nASCII\nDATASET UNSTRUCTURED_GRID\n" % title)
        f.write("POINTS %d double\n" % len(nodes))
        f.write("\n".join("%.17g %.17g %.17g" % tuple(p) for p in nodes))
        f.write("\n\nCELLS %d %d\n" % (len(cells), cells.size + len(cells)))
        f.write("\n".join(("%d " % body_id) + " ".join(str(v) for v in c) for c in cells))
        f.write("\n\nCELL_TYPES %d\n" % len(cells))
        f.write(("%d\n" % cell_type) * len(cells))


def _orient_outward(nodes, tris):
    """Flip triangles whose (e1-e0)x(e2-e0) normal points toward the origin."""
    p = nodes[tris]
    n = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    c = p.mean(axis=1)
    flip = (n * c).sum(axis=1) < 0
    tris = tris.copy()
    tris[flip] = tris[flip][:, [0, 2, 1]]
    return tris


def icosphere(subdivisions, radius=1.0):
    """Icosahedron subdivided `subdivisions` times: 20*4^s triangles
    (s=3: 1280 triangles, 642 nodes)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
             (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
             (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
             (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(v, dtype=float) / np.linalg.norm(v) for v in verts]
    for _ in range(subdivisions):
        cache = {}
        nf = []

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    nodes = np.array(verts) * radius
    return nodes, _orient_outward(nodes, np.array(faces, dtype=np.int64))


def cube_sphere(m, radius=1.0):
    """Equiangular cube-sphere: 6*m^2 bilinear quads, counter-clockwise seen
    from outside (m=32: 6144 quads)."""
    a = np.tan(np.linspace(-np.pi / 4, np.pi / 4, m + 1))
    index = {}
    nodes = []
    quads = []

    def node(p):
        key = tuple(np.round(p / np.linalg.norm(p), 12))
        if key not in index:
            index[key] = len(nodes)
            nodes.append(p / np.linalg.norm(p))
        return index[key]
    for axis in range(3):
        for sign in (1.0, -1.0):
            grid = np.empty((m + 1, m + 1), dtype=np.int64)
            for i in range(m + 1):
                for j in range(m + 1):
                    p = np.zeros(3)
                    p[axis] = sign
                    p[(axis + 1) % 3] = a[i]
                    p[(axis + 2) % 3] = a[j]
                    grid[i, j] = node(p)
            for i in range(m):
                for j in range(m):
                    q = [grid[i, j], grid[i + 1, j], grid[i + 1, j + 1], grid[i, j + 1]]
                    if sign < 0:
                        q = q[::-1]
                    quads.append(q)
    nodes = np.array(nodes) * radius
    quads = np.array(quads, dtype=np.int64)
    # orientation check on the bilinear normal at the centre
    p = nodes[quads]
    n = np.cross(p[:, 1] + p[:, 2] - p[:, 0] - p[:, 3], p[:, 2] + p[:, 3] - p[:, 0] - p[:, 1])
    flip = (n * p.mean(axis=1)).sum(axis=1) < 0
    quads[flip] = quads[flip][:, ::-1]
    return nodes, quads


def uv_ellipsoid(semi_axes, n_lon=256, n_bands=81):
    """UV-sphere with pole fans scaled to an ellipsoid:
    2*n_lon + 2*n_lon*(n_bands-2) triangles (256, 81 -> 40960)."""
    a, b, c = semi_axes
    theta = np.linspace(0.0, np.pi, n_bands + 1)[1:-1]
    phi = np.linspace(0.0, 2 * np.pi, n_lon, endpoint=False)
    nodes = [np.array([0.0, 0.0, c])]
    for th in theta:
        for ph in phi:
            nodes.append(np.array([a * np.sin(th) * np.cos(ph), b * np.sin(th) * np.sin(ph), c * np.cos(th)]))
    nodes.append(np.array([0.0, 0.0, -c]))
    nodes = np.array(nodes)
    south = len(nodes) - 1
    ring = lambda r, k: 1 + r * n_lon + (k % n_lon)
    tris = []
    for k in range(n_lon):
        tris.append((0, ring(0, k), ring(0, k + 1)))
    for r in range(len(theta) - 1):
        for k in range(n_lon):
            tris.append((ring(r, k), ring(r + 1, k), ring(r + 1, k + 1)))
            tris.append((ring(r, k), ring(r + 1, k + 1), ring(r, k + 1)))
    last = len(theta) - 1
    for k in range(n_lon):
        tris.append((south, ring(last, k + 1), ring(last, k)))
    return nodes, _orient_outward(nodes, np.array(tris, dtype=np.int64))


def _real_sph_harm(l, m, theta, phi):
    """Real spherical harmonic Y_lm (orthonormal), theta polar, phi azimuth."""
    from scipy.special import lpmv
    am = abs(m)
    norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
    p = lpmv(am, l, np.cos(theta))
    if m == 0:
        return norm * p
    if m > 0:
        return math.sqrt(2) * norm * p * np.cos(am * phi)
    return math.sqrt(2) * norm * p * np.sin(am * phi)


def perturbed_sphere(n_tri, seed, lmax=4, sigma=0.05):
    """r(theta,phi) = 1 + sum_{l<=lmax,m} a_lm Y_lm, a_lm ~ N(0, sigma^2) from
    `seed`; meshed as the hull of V = (T+4)/2 Fibonacci-sphere points mapped
    radially (hull triangle count 2V-4 = T)."""
    from scipy.spatial import ConvexHull
    if n_tri % 2:
        n_tri += 1
    v = (n_tri + 4) // 2
    rng = np.random.default_rng(seed)
    coeffs = {(l, m): rng.normal(0.0, sigma) for l in range(lmax + 1) for m in range(-l, l + 1)}
    i = np.arange(v) + 0.5
    theta = np.arccos(1 - 2 * i / v)
    phi = np.pi * (1 + 5 ** 0.5) * i
    unit = np.stack([np.sin(theta) * np.cos(phi), np.sin(theta) * np.sin(phi), np.cos(theta)], axis=1)
    tris = np.asarray(ConvexHull(unit).simplices, dtype=np.int64)
    r = np.ones(v)
    for (l, m), a in coeffs.items():
        r += a * _real_sph_harm(l, m, theta, phi % (2 * np.pi))
    nodes = unit * r[:, None]
    return nodes, _orient_outward(nodes, tris)


def fibonacci_points(n, radius):
    i = np.arange(n) + 0.5
    theta = np.arccos(1 - 2 * i / n)
    phi = np.pi * (1 + 5 ** 0.5) * i
    return radius * np.stack([np.sin(theta) * np.cos(phi), np.sin(theta) * np.sin(phi), np.cos(theta)], axis=1)
