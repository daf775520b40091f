"""Regenerates the committed fixtures of tests/golden/ from the cc_abstemious
source tree (run in a container that has it; the GPU machine does not).

* sphere.vtk, sphere_quad.vtk, refined_sphere.vtk: the reference's test meshes
  (src/tests/*.vtk) re-emitted in the reference VTK dialect (body id as the
  first integer of each CELLS row) by parsing them and writing them back.
* input_1.json: the reference's sample input (src/tests/input_1.json).
* reference_goldens.json: the published known answers with their citations.

Usage: python tests/golden/make_fixtures.py /path/to/cc_abstemious
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def parse_vtk(path):
    lines = open(path).read().split("\n")
    nodes, cells, types = [], [], []
    i = 0
    while i < len(lines):
        w = lines[i].split()
        if w and w[0] == "POINTS":
            n = int(w[1])
            nodes = [lines[i + 1 + j].split()[:3] for j in range(n)]
            i += n
        elif w and w[0] == "CELLS":
            n = int(w[1])
            cells = [lines[i + 1 + j].split() for j in range(n)]
            i += n
        elif w and w[0] == "CELL_TYPES":
            n = int(w[1])
            types = [lines[i + 1 + j].split()[0] for j in range(n)]
            i += n
        i += 1
    return nodes, cells, types


def write_vtk(path, nodes, cells, types, origin):
    with open(path, "w") as f:
        f.write("# vtk DataFile Version 2.0\n")
        f.write(f"fixture re-emitted from {origin}\nASCII\nDATASET UNSTRUCTURED_GRID\n")
        f.write(f"POINTS {len(nodes)} double\n")
        for p in nodes:
            f.write(" ".join(p) + "\n")
        f.write(f"\nCELLS {len(cells)} {sum(len(c) for c in cells)}\n")
        for c in cells:
            f.write(" ".join(c) + "\n")
        f.write(f"\nCELL_TYPES {len(types)}\n")
        for t in types:
            f.write(t + "\n")


GOLDENS = {
    "lu_100_seed10_x0": {"value": [0.0035386336544537098, 0.0017794290945383035], "abs_tol": 1e-10,
                          "source": "src/solve.rs:216-217"},
    "rigid_sphere_plane_wave": {"value": [-0.000039380091293979903, 0.00047605686656319906],
                                "norm": 0.0004776828778512934, "abs_tol": 1e-10,
                                "source": "src/tests/verification.rs:95-120"},
    "rigid_sphere_plane_wave_iterative": {"value": [-0.000039380091293979903, 0.00047605686656319906],
                                          "abs_tol": 1e-8, "source": "src/tests/verification.rs:122-148"},
    "rigid_sphere_plane_wave_hmatrix": {"value": [-3.9380308176032198e-05, 0.00047605563272935873],
                                        "abs_tol": 1e-10, "source": "src/tests/verification.rs:150-176"},
    "rigid_sphere_plane_wave_burton_miller": {"value": [0.00012125591274707629, 0.0004814465829556038],
                                              "norm": 0.0004964814282687255, "abs_tol": 1e-10,
                                              "source": "src/tests/verification.rs:178-204"},
    "vtk_reader_cells": {"value": 336, "source": "src/preprocess/mesh_data.rs:179-187"},
    "json_reader_body_index": {"value": 3, "source": "src/preprocess/input_data.rs:116-122"},
    "cluster_tree_diameter": {"value": 33.94, "abs_tol": 1e-2, "source": "src/solve/h_matrix/cluster.rs:120-138"},
    "block_tree_children_1_1_1_admissible": {"value": True, "source": "src/solve/h_matrix/block.rs:104-115"},
    "block_list_5_admissible": {"value": True, "source": "src/solve/h_matrix/block.rs:125-145"},
}


def main(ref):
    for name in ("sphere.vtk", "sphere_quad.vtk", "refined_sphere.vtk"):
        nodes, cells, types = parse_vtk(os.path.join(ref, "src", "tests", name))
        write_vtk(os.path.join(HERE, name), nodes, cells, types, "src/tests/" + name)
    with open(os.path.join(ref, "src", "tests", "input_1.json")) as f:
        inp = json.load(f)
    with open(os.path.join(HERE, "input_1.json"), "w") as f:
        json.dump(inp, f, indent=4)
    with open(os.path.join(HERE, "reference_goldens.json"), "w") as f:
        json.dump(GOLDENS, f, indent=1)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py <path of the cc_abstemious source tree>")
    main(sys.argv[1])
