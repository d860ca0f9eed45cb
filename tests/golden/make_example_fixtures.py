"""Generate the topology known-answer fixtures from the reference example scene.

Reads, from the reference checkout (read-only):
  example/ClothArmadillo/cloth{1,2}/cloth{1,2}.obj     the 75x75 Blender cloths
  example/ClothArmadillo/cloth{1,2}/fixed_points.txt   'c N' + N pinned ids
  example/ClothArmadillo/cloth{1,2}/boundary.dat       cached boundary lists
      (int count + ids; int count + (vi,vj); int count + (vi,vj,vk)),
      written by PdIpcModel::saveBoundaryInfo (Simulator/PD-IPC/PdIpcModel.h:219-251)
  example/ClothArmadillo/cloth{1,2}/patchInfo.dat      cached patch partition
      (4 ints: #points #edges #faces #patches; then per patch: count + face ids),
      written by PdIpcModel::saveCollisionPatchInfo (PdIpcModel.h:291-318)
and writes tests/golden/example_cloth_topology.npz holding the input mesh and
the expected edges / patch partition, for tests that run without the reference.
The config uses <patchDim> 50 for both cloths (example/ClothArmadillo/config.xml).

Usage: python tests/golden/make_example_fixtures.py [/path/to/reference]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_obj(path):
    V, F = [], []
    with open(path) as f:
        for line in f:
            if line.startswith("v "):
                V.append([float(t) for t in line.split()[1:4]])
            elif line.startswith("f "):
                F.append([int(t.split("/")[0]) - 1 for t in line.split()[1:4]])
    return np.asarray(V, np.float64), np.asarray(F, np.int32)


def read_ints(path):
    return np.fromfile(path, dtype="<i4")


def parse_boundary(a):
    p = 0
    n = a[p]; p += 1
    pts = a[p:p + n]; p += n
    n = a[p]; p += 1
    edges = a[p:p + 2 * n].reshape(n, 2); p += 2 * n
    n = a[p]; p += 1
    faces = a[p:p + 3 * n].reshape(n, 3); p += 3 * n
    assert p == a.size
    return pts, edges, faces


def parse_patches(a):
    bp, be, bf, npatch = a[:4]
    p = 4
    off = [0]
    faces = []
    for _ in range(npatch):
        n = a[p]; p += 1
        faces.extend(a[p:p + n].tolist()); p += n
        off.append(len(faces))
    assert p == a.size
    return (bp, be, bf), np.asarray(off, np.int32), np.asarray(faces, np.int32)


def main(ref):
    out = {}
    for name in ("cloth1", "cloth2"):
        d = os.path.join(ref, "example", "ClothArmadillo", name)
        X, F = read_obj(os.path.join(d, name + ".obj"))
        with open(os.path.join(d, "fixed_points.txt")) as f:
            tok = f.read().split()
        assert tok[0] == "c"
        fixed = np.asarray([int(t) for t in tok[2:2 + int(tok[1])]], np.int32)
        pts, edges, faces = parse_boundary(read_ints(os.path.join(d, "boundary.dat")))
        counts, poff, pfaces = parse_patches(read_ints(os.path.join(d, "patchInfo.dat")))
        assert np.array_equal(pts, np.arange(X.shape[0])), "cloth boundary points are the identity"
        assert np.array_equal(faces, F), "boundary faces are the OBJ faces in file order"
        assert counts == (X.shape[0], edges.shape[0], F.shape[0])
        out[f"{name}_X"] = X
        out[f"{name}_F"] = F
        out[f"{name}_fixed"] = fixed
        out[f"{name}_edges"] = edges.astype(np.int32)
        out[f"{name}_patch_off"] = poff
        out[f"{name}_patch_faces"] = pfaces
    out["patch_dim"] = np.asarray(50, np.int32)
    path = os.path.join(HERE, "example_cloth_topology.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    # the reference tree: the first argument, else $PDIPC_REFERENCE_DIR
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PDIPC_REFERENCE_DIR")
    if not ref:
        raise SystemExit("usage: make_example_fixtures.py <reference tree> (or set PDIPC_REFERENCE_DIR)")
    main(ref)
