import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def sphere_input(mesh="sphere.vtk", **kw):
    """The default_input() of src/tests/verification.rs:8-33 with the settings
    shared by its four enabled tests (water, 100 Hz, plane wave +x, field
    point (10,0,0))."""
    d = {"mesh_file": os.path.join(GOLDEN, mesh), "body_index": 3,
         "frequency": {"List": {"values": [100.0]}},
         "sound_speed": 1500.0, "mass_density": 1000.0, "problem_type": "Exterior",
         "method_type": "Classical", "solver": {"Direct": {}},
         "incident_wave": {"PlaneWave": {"direction": [1.0, 0.0, 0.0], "amplitude": [1.0, 0.0]}},
         "surface_bc": {"bc_type": "NormalVelocity", "value": [0.0, 0.0]},
         "output": {"o_type": "Scattered", "field": "Pressure", "file": "",
                    "field_points": [[10.0, 0.0, 0.0]]}}
    d.update(kw)
    return d


@pytest.fixture
def goldens():
    import json
    with open(os.path.join(GOLDEN, "reference_goldens.json")) as f:
        return json.load(f)
