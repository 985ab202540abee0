"""Generates tests/golden/reference_host.json from the reference's own host code (2D and 3D),
and tests/golden/reference_channel8x4.{mesh,particles}.vtu from its VTU writers.

Builds oracle/_ref/ref_host_dump with oracle/build_ref.sh (the reference's DAT reader,
CSR pattern builder, vertex-sharing neighbour search, particle-handler constructor and
quadrature factories, compiled from its sources and run on the CPU against a
host-memory stand-in for the CUDA runtime), runs it on the shipped meshes of the
reference and on meshes of the committed generator, and records for each mesh the
sizes and SHA-256 digests of the arrays it produced.  Sub-cell centroids and
quadrature tables are stored as exact hex floats.

Run from the repository root where the reference tree is available:
    python tests/golden/make_reference_fixtures.py [/path/to/reference]
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from gpupfem2_gb300 import meshgen as mg  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden", "reference_host.json")

GENERATED = {
    "square64": lambda: mg.unit_square(64),
    "channel256x64": lambda: mg.channel(),
    "channel64x16": lambda: mg.channel(64, 16, 4.0, 1.0),
    "cylinder_nx100": lambda: mg.cylinder_channel(nxh=100, nyh=100, nr=6),
}
SHIPPED = ["cases/Poisson2D/TestProblem2.dat",
           "cases/PoiseuilleFlow2D/ChannelMesh.dat", "cases/Cylinder2D/CylinderMesh.dat",
           "cases/Cylinder2D/CylinderMesh3.dat"]
ARRAYS = [("xy", "f64"), ("tri", "i32"), ("nboff", "i32"), ("nbidx", "i32"), ("rowptr", "i32"), ("col", "i32")]
GENERATED3D = {
    "box8x4x2": lambda: mg.box_tets(8, 4, 2),
    "box40x20x10": lambda: mg.box_tets(),
}
SHIPPED3D = ["cases/Poisson3D/BoxMesh.dat", "cases/Poisson3D/BoxMesh2.dat"]
ARRAYS3D = [("xyz", "f64"), ("tet", "i32"), ("rowptr", "i32"), ("col", "i32")]


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def run_dump(exe, dat, prefix):
    r = subprocess.run([exe, dat, prefix], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    out = {}
    for name, t in ARRAYS:
        out[name] = np.fromfile(prefix + "." + name + "." + t, dtype=np.float64 if t == "f64" else np.int32)
    return out


def run_dump3d(exe, dat, prefix):
    r = subprocess.run([exe, dat, prefix], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    out = {}
    for name, t in ARRAYS3D + [("quad", "f64")]:
        out[name] = np.fromfile(prefix + "." + name + "." + t, dtype=np.float64 if t == "f64" else np.int32)
    return out


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    env = dict(os.environ, REF=os.path.join(ref, "src"))
    subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True, env=env)
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_host_dump")
    fixtures = {"generator": "reference host code (mesh_2d.cu:36-139, sparse_matrix.cu:8-54, "
                             "particle_handler_2d.cu:238-294, quadrature_formula_{1d,2d}.cu) via oracle/build_ref.sh",
                "meshes": {}}
    with tempfile.TemporaryDirectory() as tmp:
        items = [(k, None) for k in GENERATED] + [(os.path.basename(s), os.path.join(ref, s)) for s in SHIPPED]
        for name, path in items:
            if path is None:
                xy, tri = GENERATED[name]()
                path = os.path.join(tmp, name + ".dat")
                mg.write_dat(path, xy, tri)
                kind = "generated"
            else:
                if not os.path.exists(path):
                    continue
                kind = "shipped"
            a = run_dump(exe, path, os.path.join(tmp, name))
            rec = {"kind": kind, "nv": int(a["xy"].size // 2), "nc": int(a["nboff"].size - 1),
                   "nnz": int(a["col"].size), "n_neighbor_entries": int(a["nbidx"].size)}
            rec.update({"sha256_" + k: digest(v) for k, v in a.items()})
            fixtures["meshes"][name] = rec
            print(name, rec["nv"], rec["nc"], rec["nnz"], rec["n_neighbor_entries"])
        pre = os.path.join(tmp, "square64")
        fixtures["subcell_centers"] = {str(L): [float(v).hex() for v in np.fromfile(pre + ".centers%d.f64" % L)]
                                       for L in range(1, 5)}
        q = np.fromfile(pre + ".quad.f64")
        fixtures["quadrature"] = {"face_index1_xyzw": [float(v).hex() for v in q[:12]],
                                  "edge_index1_cw": [float(v).hex() for v in q[12:]]}
    exe3 = os.path.join(ROOT, "oracle", "_ref", "ref_host_dump3d")
    fixtures["generator3d"] = ("reference host code (mesh_3d.cu:84-147, sparse_matrix.cu:56-97, "
                               "quadrature_formula_3d.cu) via oracle/build_ref.sh")
    fixtures["meshes3d"] = {}
    with tempfile.TemporaryDirectory() as tmp:
        items = [(k, None) for k in GENERATED3D] + [(os.path.basename(s), os.path.join(ref, s)) for s in SHIPPED3D]
        quad = None
        for name, path in items:
            if path is None:
                xyz, tet = GENERATED3D[name]()
                path = os.path.join(tmp, name + ".dat")
                mg.write_dat3(path, xyz, tet)
                kind = "generated"
            else:
                if not os.path.exists(path):
                    continue
                kind = "shipped"
            a = run_dump3d(exe3, path, os.path.join(tmp, name))
            quad = a.pop("quad")
            rec = {"kind": kind, "nv": int(a["xyz"].size // 3), "nc": int(a["tet"].size // 4),
                   "nnz": int(a["col"].size)}
            rec.update({"sha256_" + k: digest(v) for k, v in a.items()})
            fixtures["meshes3d"][name] = rec
            print(name, rec["nv"], rec["nc"], rec["nnz"])
        fixtures["quadrature3d"] = {"cell_index1_xyzw_weight": [float(v).hex() for v in quad]}
    with open(OUT, "w") as f:
        json.dump(fixtures, f, indent=1, sort_keys=True)
    print("wrote", OUT)
    # the reference's VTU writers on the 8 x 4 channel (oracle/refhost/dump_ref_vtu.cu
    # states the fields and particles it writes)
    exe_vtu = os.path.join(ROOT, "oracle", "_ref", "ref_vtu_dump")
    with tempfile.TemporaryDirectory() as tmp:
        xy, tri = mg.channel(8, 4, 4.0, 1.0)
        dat = os.path.join(tmp, "channel8x4.dat")
        mg.write_dat(dat, xy, tri)
        subprocess.run([exe_vtu, dat, os.path.join(tmp, "channel8x4")], check=True, capture_output=True)
        for part in ("mesh", "particles"):
            dst = os.path.join(ROOT, "tests", "golden", "reference_channel8x4.%s.vtu" % part)
            with open(os.path.join(tmp, "channel8x4.%s.vtu" % part)) as src, open(dst, "w") as f:
                f.write(src.read())
            print("wrote", dst)


if __name__ == "__main__":
    main()
