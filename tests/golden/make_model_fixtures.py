"""Generates tests/golden/models.npz from the sample meshes the reference ships (Data/Models/{cube,sphere,teapot}.obj).

Each file is read twice, by the library's OBJ reader (thea_gb300.read_mesh, host C++) and by the pure-Python restatement
of the reference's reader (oracle/mesh_oracle.py); the script stops unless both give identical arrays. The fixture holds,
per model, the triangle list the reference's MeshGroup<DisplayMesh>::load would index (vertices, triangles, source face
of each triangle, submesh offsets) and the SHA-256 of the source file, so GPU tests can run the queries on real meshes
without the reference present.

Run: python tests/golden/make_model_fixtures.py <path to the reference's Data/Models directory>
"""

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import mesh_oracle as MO  # noqa: E402

MODELS = ("cube", "sphere", "teapot")


def main():
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_model_fixtures.py <the reference's Data/Models directory>")
    src = sys.argv[1]
    from thea_gb300 import build as B
    B.build()
    import thea_gb300 as T
    out = {}
    for name in MODELS:
        path = os.path.join(src, name + ".obj")
        lib = T.read_mesh(path)
        ref = MO.read_mesh(path)
        for key in ("vertices", "vertex_source", "triangles", "triangle_face", "submesh_vertex_offsets",
                    "submesh_triangle_offsets"):
            if not np.array_equal(getattr(lib, key), ref[key]):
                raise SystemExit("%s: the library's reader and the restatement differ in %s" % (name, key))
        out[name + "_vertices"] = lib.vertices
        out[name + "_triangles"] = lib.triangles
        out[name + "_triangle_face"] = lib.triangle_face
        out[name + "_submesh_triangle_offsets"] = lib.submesh_triangle_offsets
        out[name + "_sha256"] = np.frombuffer(hashlib.sha256(open(path, "rb").read()).digest(), np.uint8)
        print("%s: %d vertices, %d triangles, %d submeshes" % (name, len(lib.vertices), len(lib.triangles),
                                                               len(lib.submesh_triangle_offsets) - 1))
    np.savez_compressed(os.path.join(HERE, "models.npz"), **out)


if __name__ == "__main__":
    main()
