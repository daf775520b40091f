"""The benchmark bodies and inputs as reference-format JSON (synthetic meshes,
seeded; there is no external dataset).

  pulsating_sphere   icosphere 1280 triangles r=1, classical, vn = 1, ka = 1,
                     Direct, 100 field points on r = 5 (analytic monopole check)
  rigid_sphere_bm    cube-sphere 6144 quads r=1, Burton-Miller, rigid, plane
                     wave +z, 16 frequencies ka = 1..10, GMRES 2500 (restart 50)
                     tol 1e-8, 100 field points on r = 5
  ellipsoid_bm       UV ellipsoid (2, 1, 0.5) with 40960 triangles, BM, plane
                     wave along a seeded direction + point source at (0,0,3),
                     ka (a = 2) = 2.5..20 at 8 frequencies, H-matrix leaf 64,
                     eta 1, ACA 1e-5, GMRES tol 1e-6
  perturbed_spheres  256 harmonic-perturbed spheres, 500-5000 triangles each,
                     impedance Z = rho c (1 + 0.2 i), BM, ka = 0.5..8 at 8
                     frequencies
"""
import math
import os

import numpy as np

from . import meshgen

C_AIR = 343.0
RHO_AIR = 1.21


def _freqs_for_ka(ka_values, radius=1.0, c=C_AIR):
    return [float(ka) * c / (2.0 * math.pi * radius) for ka in ka_values]


def base_input(mesh_file, freqs, method="BurtonMiller", solver=None, incident=None, bc=None, field_points=None,
               output_type="Scattered"):
    return {
        "mesh_file": mesh_file,
        "body_index": 1,
        "frequency": {"List": {"values": list(map(float, freqs))}},
        "sound_speed": C_AIR,
        "mass_density": RHO_AIR,
        "problem_type": "Exterior",
        "method_type": method,
        "solver": solver or {"Direct": {}},
        "incident_wave": incident or {"PlaneWave": {"direction": [0.0, 0.0, 1.0], "amplitude": [1.0, 0.0]}},
        "surface_bc": bc or {"bc_type": "NormalVelocity", "value": [0.0, 0.0]},
        "output": {"o_type": output_type, "field": "Pressure", "file": "",
                   "field_points": (field_points if field_points is not None
                                    else meshgen.fibonacci_points(100, 5.0)).tolist()},
    }


def pulsating_sphere(workdir):
    nodes, tris = meshgen.icosphere(3)
    path = os.path.join(workdir, "icosphere_1280.vtk")
    meshgen.write_vtk(path, nodes, tris, 5)
    return base_input(path, _freqs_for_ka([1.0]), method="Classical",
                      incident={"PlaneWave": {"direction": [0.0, 0.0, 1.0], "amplitude": [0.0, 0.0]}},
                      bc={"bc_type": "NormalVelocity", "value": [1.0, 0.0]})


def rigid_sphere_bm(workdir, m=32, nfreq=16, ka_lo=1.0, ka_hi=10.0):
    nodes, quads = meshgen.cube_sphere(m)
    path = os.path.join(workdir, "cube_sphere_%d.vtk" % (6 * m * m))
    meshgen.write_vtk(path, nodes, quads, 9)
    return base_input(path, _freqs_for_ka(np.linspace(ka_lo, ka_hi, nfreq)),
                      solver={"Iterative": {"tolerance": 1e-8, "max_iterations": 2500}})


def ellipsoid_bm(workdir, n_lon=256, n_bands=81, nfreq=8, seed=1):
    nodes, tris = meshgen.uv_ellipsoid((2.0, 1.0, 0.5), n_lon, n_bands)
    path = os.path.join(workdir, "ellipsoid_%d.vtk" % len(tris))
    meshgen.write_vtk(path, nodes, tris, 5)
    rng = np.random.default_rng(seed)
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    inp = base_input(path, _freqs_for_ka(np.linspace(2.5, 20.0, nfreq), radius=2.0),
                     solver={"Hierarchical": {"tolerance": 1e-6, "max_iterations": 1000, "leaf_size": 64,
                                              "eta": 1.0, "aca_tolerance": 1e-5}},
                     incident={"PlaneWave": {"direction": d.tolist(), "amplitude": [1.0, 0.0]}})
    point_source = dict(inp, incident_wave={"SphericalWave": {"origin": [0.0, 0.0, 3.0], "amplitude": [1.0, 0.0]}})
    return inp, point_source


def perturbed_sphere_input(workdir, body_seed, n_tri, ka_values, tol=1e-6):
    nodes, tris = meshgen.perturbed_sphere(n_tri, body_seed)
    path = os.path.join(workdir, "perturbed_%d_%d.vtk" % (body_seed, len(tris)))
    meshgen.write_vtk(path, nodes, tris, 5)
    z = [RHO_AIR * C_AIR, 0.2 * RHO_AIR * C_AIR]
    return base_input(path, _freqs_for_ka(ka_values),
                      solver={"Iterative": {"tolerance": tol, "max_iterations": 1000}},
                      bc={"bc_type": "Impedance", "value": z})


def perturbed_spheres(workdir, count=256, seed=0, nfreq=8, tri_lo=500, tri_hi=5000, tol=1e-6):
    rng = np.random.default_rng(seed)
    counts = rng.integers(tri_lo, tri_hi + 1, size=count)
    return [perturbed_sphere_input(workdir, 1000 * seed + b, int(t), np.linspace(0.5, 8.0, nfreq), tol=tol)
            for b, t in enumerate(counts)]
