"""Tet meshes from gmsh 4.1 ASCII files and the reference's mesh placement.

read_msh: MeshUtils::loadTetMeshFromGmshFile (src/utils/MeshUtils.cpp:92-220)
goes over the model's entities in (dimension, tag) order, appends each
entity's nodes, and keeps its tetrahedra (element type 4) and triangles
(type 2) with 1-based node tags turned into 0-based indices (tag - 1). This
reader parses the file itself in that order instead of calling the gmsh API.

place: MeshObject::loadAndConfigureMesh (include/simobject/MeshObject.hpp:35-62)
-- optional uniform resize to max-size, optional per-axis resize to size
(Mesh::resize, src/geometry/Mesh.cpp:224-262), then the surface's centre of
mass is moved to `position` (Mesh::massCenter, :366-399), then the mesh is
rotated about `position` by x, y, z angles in degrees, x first
(Mesh::rotateAbout, :285-312).
"""
from __future__ import annotations

import math

import numpy as np


def read_msh(path_or_text: str):
    """(X (V,3) float64, tets (T,4) int32, faces (F,3) int32)."""
    if "\n" in path_or_text or "$MeshFormat" in path_or_text:
        text = path_or_text
    else:
        with open(path_or_text) as f:
            text = f.read()
    tok = text.split()
    i = 0

    def section(name):
        nonlocal i
        while i < len(tok) and tok[i] != name:
            i += 1
        if i == len(tok):
            raise ValueError(f"{name} section missing")
        i += 1

    section("$MeshFormat")
    version = tok[i]
    if not version.startswith("4."):
        raise ValueError(f"gmsh format {version}: only 4.x ASCII is supported")
    if tok[i + 1] != "0":
        raise ValueError("binary gmsh files are not supported")
    section("$Nodes")
    n_blocks, n_nodes = int(tok[i]), int(tok[i + 1])
    i += 4
    node_blocks = []
    for _ in range(n_blocks):
        dim, etag, param, n = int(tok[i]), int(tok[i + 1]), int(tok[i + 2]), int(tok[i + 3])
        i += 4
        tags = np.array(tok[i:i + n], dtype=np.int64)
        i += n
        per = 3 + (dim if param else 0)
        xyz = np.array(tok[i:i + n * per], dtype=np.float64).reshape(n, per)[:, :3]
        i += n * per
        node_blocks.append(((dim, etag), tags, xyz))
    section("$Elements")
    n_blocks = int(tok[i])
    i += 4
    elem_blocks = {}
    nper = {1: 2, 2: 3, 3: 4, 4: 4, 5: 8, 6: 6, 7: 5, 8: 3, 9: 6, 10: 9, 11: 10, 15: 1}
    for _ in range(n_blocks):
        dim, etag, etype, n = int(tok[i]), int(tok[i + 1]), int(tok[i + 2]), int(tok[i + 3])
        i += 4
        if etype not in nper:
            raise ValueError(f"unsupported gmsh element type {etype}")
        k = nper[etype]
        rows = np.array(tok[i:i + n * (k + 1)], dtype=np.int64).reshape(n, k + 1)[:, 1:]
        i += n * (k + 1)
        elem_blocks.setdefault((dim, etag), []).append((etype, rows))
    # vertices: entity blocks in (dimension, tag) order, as gmsh::model::getEntities lists them
    order = sorted(range(len(node_blocks)), key=lambda b: node_blocks[b][0])
    X = np.concatenate([node_blocks[b][2] for b in order]) if node_blocks else np.zeros((0, 3))
    tets, tris = [], []
    for key in sorted(elem_blocks):
        for etype, rows in elem_blocks[key]:
            if etype == 4:
                tets.append(rows - 1)
            elif etype == 2:
                tris.append(rows - 1)
    tets = np.concatenate(tets).astype(np.int32) if tets else np.zeros((0, 4), np.int32)
    faces = np.concatenate(tris).astype(np.int32) if tris else np.zeros((0, 3), np.int32)
    if X.shape[0] != n_nodes:
        raise ValueError("node count mismatch")
    for a in (tets, faces):
        if a.size and (a.min() < 0 or a.max() >= X.shape[0]):
            raise ValueError("element references a node outside the node list")
    return X, tets, faces


def write_msh(path: str, X, tets, faces):
    """gmsh 4.1 ASCII: all nodes on one volume entity, the surface triangles
    on surface entity 1, the tetrahedra on volume entity 1 (1-based tags in
    vertex order), so read_msh returns the same arrays."""
    X = np.asarray(X, np.float64)
    tets = np.asarray(tets, np.int64)
    faces = np.asarray(faces, np.int64)
    V = X.shape[0]
    out = ["$MeshFormat", "4.1 0 8", "$EndMeshFormat", "$Nodes", f"1 {V} 1 {V}", f"3 1 0 {V}"]
    out += [str(k + 1) for k in range(V)]
    out += [f"{x!r} {y!r} {z!r}" for x, y, z in X.tolist()]
    out.append("$EndNodes")
    nb = (1 if len(faces) else 0) + (1 if len(tets) else 0)
    ne = len(faces) + len(tets)
    out += ["$Elements", f"{nb} {ne} 1 {ne}"]
    tag = 1
    if len(faces):
        out.append(f"2 1 2 {len(faces)}")
        for f in faces.tolist():
            out.append(f"{tag} {f[0] + 1} {f[1] + 1} {f[2] + 1}")
            tag += 1
    if len(tets):
        out.append(f"3 1 4 {len(tets)}")
        for t in tets.tolist():
            out.append(f"{tag} {t[0] + 1} {t[1] + 1} {t[2] + 1} {t[3] + 1}")
            tag += 1
    out.append("$EndElements")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


def mass_center(X, faces):
    """Centre of mass of the closed surface (sum of origin-apex tets)."""
    X = np.asarray(X, np.float64)
    f = np.asarray(faces)
    v1, v2, v3 = X[f[:, 0]], X[f[:, 1]], X[f[:, 2]]
    vol = np.einsum("ij,ij->i", v1, np.cross(v2, v3)) / 6.0
    cm = 0.25 * (v1 + v2 + v3)
    return (cm * vol[:, None]).sum(0) / vol.sum()


def rotation_xyz(deg):
    """The reference's "123" rotation matrix for x, y, z angles in degrees."""
    x, y, z = (a * math.pi / 180.0 for a in deg)
    cx, sx, cy, sy, cz, sz = math.cos(x), math.sin(x), math.cos(y), math.sin(y), math.cos(z), math.sin(z)
    return np.array([[cy * cz, sx * sy * cz - cx * sz, cx * sy * cz + sx * sz],
                     [cy * sz, sx * sy * sz + cx * cz, cx * sy * sz - sx * cz],
                     [-sy, sx * cy, cx * cy]])


def place(X, faces, position=(0, 0, 0), rotation=(0, 0, 0), max_size=None, size=None):
    """The reference's placement of a loaded mesh (see the module docstring)."""
    X = np.array(X, np.float64)
    if max_size is not None:
        ext = X.max(0) - X.min(0)
        X *= float(max_size) / ext.max()
    if size is not None:
        ext = X.max(0) - X.min(0)
        s = np.asarray(size, np.float64)
        X *= np.where(ext != 0, s / np.where(ext != 0, ext, 1), 1.0)
    p = np.asarray(position, np.float64)
    if len(faces):
        X += -mass_center(X, faces) + p
    else:
        X += p
    R = rotation_xyz(rotation)
    return (X - p) @ R.T + p
