"""Regenerate the committed golden fixtures from the reference checkout.

Run with the path of a reference checkout (argument, or the environment
variable EDGEFEM_REFERENCE):

    python tests/golden/make_golden.py <reference-root>

Writes
  * rect_waveguide_mesh.npz, cube_cavity_mesh.npz: the reference's committed
    Gmsh meshes (examples/*.msh) as arrays, parsed with this package's
    Gmsh v2 reader;
  * published.json: the numbers the reference publishes for this path
    (docs/validation.md:20-29 WR-90 table, :50-56 port-ABC scale table) and
    the three triangles of tests/test_triangle_mass_matrix.cpp:93-105.
The fixtures are data only; nothing reads the reference at test time.
"""
from __future__ import annotations

import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("EDGEFEM_REFERENCE", "")
if __name__ == "__main__" and not os.path.isdir(REF):
    raise SystemExit("usage: make_golden.py <reference-root> (or set EDGEFEM_REFERENCE)")
sys.path.insert(0, REPO)

from edgefem_gb300.mesh import read_gmsh_v2  # noqa: E402


def save_mesh(name: str, out: str) -> None:
    m = read_gmsh_v2(os.path.join(REF, "examples", name))
    np.savez_compressed(os.path.join(HERE, out), node_ids=m.node_ids, xyz=m.xyz, tets=m.tets,
                        tet_phys=m.tet_phys, tris=m.tris, tri_phys=m.tri_phys)


def parse_tables() -> dict:
    text = open(os.path.join(REF, "docs", "validation.md")).read().splitlines()
    wr90 = []
    for ln in text[19:29]:
        m = re.match(r"\|\s*([\d.]+)\s*\|\s*([\d.]+)\s*\|\s*([\d.]+)\s*\|\s*([-\d.]+)°", ln)
        if m:
            wr90.append({"freq_ghz": float(m.group(1)), "s11_mag": float(m.group(2)),
                         "s21_mag": float(m.group(3)), "s21_phase_deg": float(m.group(4))})
    abc = []
    for ln in text[45:60]:
        m = re.match(r"\|\s*\**([\d.]+)\**\s*\|\s*\**([\d.]+)\**\s*\|\s*\**([\d.]+)\**\s*\|", ln)
        if m:
            abc.append({"alpha": float(m.group(1)), "s11_mag": float(m.group(2)), "s21_mag": float(m.group(3))})
    return {"wr90_7_12ghz": wr90, "port_abc_scale_10ghz": abc,
            "source": "docs/validation.md:20-29 and :50-56 of jman4162/EdgeFEM"}


def triangles() -> list:
    src = open(os.path.join(REF, "tests", "test_triangle_mass_matrix.cpp")).read()
    body = src[src.index("int main()"):]
    tris = re.findall(r"check_triangle\(\{(.*?)\},\s*\"", body, re.S)
    out = []
    for t in tris:
        vecs = re.findall(r"Vector3d\(([^)]*)\)", t)
        out.append([[float(v) for v in vec.split(",")] for vec in vecs])
    return out


def main() -> None:
    save_mesh("rect_waveguide.msh", "rect_waveguide_mesh.npz")
    save_mesh("cube_cavity.msh", "cube_cavity_mesh.npz")
    pub = parse_tables()
    pub["triangle_mass_triangles"] = triangles()
    pub["triangle_mass_source"] = "tests/test_triangle_mass_matrix.cpp:93-105 of jman4162/EdgeFEM"
    with open(os.path.join(HERE, "published.json"), "w") as f:
        json.dump(pub, f, indent=1)
    print("wrote fixtures:", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
