"""Writes tests/golden/reference_inputs.npz: input files that the reference
(limkjae/Quake-DFN) ships, carried into the tests so that they run where the
reference checkout is absent.

  bp5qd_text        Input_BulkFaultGeometry.txt, the reference's default
                    input (BP5QD-like: 18-column rectangle bulk file), verbatim
  ridgecrest_text   Tools/InputGeometryExamples/Input_BulkFaultGeometry_Ridgecrest.txt,
                    verbatim
  obj_vertices, obj_faces
                    Tools/TriangleMeshReader/NormalFaults.obj as read by
                    ObjReader.jl (vertices as in the file, faces 0-based)
  *_sha256          SHA-256 of each source file's bytes

Run from the repository root with the reference checkout at /root/reference:
    python tests/golden/make_reference_inputs.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "quake-dfn_gb300"))
REF = os.environ.get("QDFN_REFERENCE", "/root/reference")


def main():
    from qdfn import geometry
    out = {}
    for key, rel in (("bp5qd", "Input_BulkFaultGeometry.txt"),
                     ("ridgecrest", "Tools/InputGeometryExamples/Input_BulkFaultGeometry_Ridgecrest.txt")):
        raw = open(os.path.join(REF, rel), "rb").read()
        out[key + "_text"] = np.array(raw.decode())
        out[key + "_sha256"] = np.array(hashlib.sha256(raw).hexdigest())
    obj = os.path.join(REF, "Tools/TriangleMeshReader/NormalFaults.obj")
    V, F = geometry.read_obj_mesh(obj)
    out["obj_vertices"] = V
    out["obj_faces"] = F.astype(np.int32)
    out["obj_sha256"] = np.array(hashlib.sha256(open(obj, "rb").read()).hexdigest())
    path = os.path.join(HERE, "reference_inputs.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, {k: getattr(v, "shape", None) for k, v in out.items()})


if __name__ == "__main__":
    main()
