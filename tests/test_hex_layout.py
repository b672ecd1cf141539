"""The patch layouts the versioned sweep's register path is specialised for.

The sweep keeps a patch's eight vertices in registers when the patch's local
layout (3 bits per tet corner, first-appearance numbering of the patch
builder, csrc/xpbd_build.cu build_patches) is kHexLocA; the build reorders two
tets' corners in every split-B hex of a grid mesh (kHexLocB) so that it has
that layout too. These tests replay the patch builder on the grid generator's
meshes (the oracle's copy of the generator, MeshUtils.cpp:424-660) and check
the constants in csrc/xpbd_kernels.cuh against it, on the CPU."""
import os
import re

import numpy as np

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(HERE, "..", "xpbd-tissue-sim_gb300", "csrc", "xpbd_kernels.cuh")


def _constant(name):
    m = re.search(rf"constexpr unsigned long long {name} = (0x[0-9a-fA-F]+)ull;", open(HEADER).read())
    assert m, name
    return int(m.group(1), 16)


def _patches(tets, cap=5, max_verts=8):
    """build_patches: runs of consecutive tets sharing a vertex with the run,
    at most `cap` tets on at most `max_verts` vertices; loc packs each tet
    corner's local vertex id at bit 12 i + 3 j."""
    out, cur = [], None
    for t, e in enumerate(tets.tolist()):
        fits = cur is not None and cur["n"] < cap
        if fits:
            fresh = sum(1 for v in e if v not in cur["v"])
            fits = any(v in cur["v"] for v in e) and len(cur["v"]) + fresh <= max_verts
        if not fits:
            if cur is not None:
                out.append(cur)
            cur = {"first": t, "n": 0, "v": [], "loc": 0}
        for j, v in enumerate(e):
            if v not in cur["v"]:
                cur["v"].append(v)
            cur["loc"] |= cur["v"].index(v) << (12 * cur["n"] + 3 * j)
        cur["n"] += 1
    out.append(cur)
    return out


def _canonical(tets):
    """The build's reordering: in a split-B hex, tet 0 (a,b,c,d) -> (c,a,b,d)
    and tet 2 (a,b,c,d) -> (a,c,b,d)."""
    B = _constant("kHexLocB")
    out = tets.copy()
    for p in _patches(tets):
        if p["n"] == 5 and len(p["v"]) == 8 and p["loc"] == B:
            a, b, c, d = out[p["first"]]
            out[p["first"]] = (c, a, b, d)
            a, b, c, d = out[p["first"] + 2]
            out[p["first"] + 2] = (a, c, b, d)
    return out


def _signed_volumes(X, tets):
    a, b, c, d = (X[tets[:, k]] for k in range(4))
    return np.einsum("ij,ij->i", a - d, np.cross(b - d, c - d))


def test_grid_hexes_have_the_two_layouts():
    A, B = _constant("kHexLocA"), _constant("kHexLocB")
    for dims in [(4, 4, 4), (5, 3, 7), (10, 2, 2)]:
        X, tets, _ = O.grid_mesh(*dims, 0.1)
        ps = _patches(tets)
        assert len(ps) == int(np.prod(dims))
        assert all(p["n"] == 5 and len(p["v"]) == 8 for p in ps)
        assert {p["loc"] for p in ps} == {A, B}
        X, tets, _ = O.grid_mesh(*dims, 0.1, split=1)  # the uniform split: A only
        assert {p["loc"] for p in _patches(tets)} == {A}


def test_canonical_corner_order_gives_one_layout_and_keeps_the_geometry():
    A = _constant("kHexLocA")
    for dims in [(4, 4, 4), (5, 3, 7), (3, 8, 2)]:
        X, tets, _ = O.grid_mesh(*dims, 0.1)
        can = _canonical(tets)
        assert {p["loc"] for p in _patches(can)} == {A}
        # same vertex set per tet, same |volume| (the reordering of tet 2 is odd,
        # so its signed volume flips; the element's F = Ds Dm^-1 does not)
        assert np.array_equal(np.sort(can, 1), np.sort(tets, 1))
        np.testing.assert_allclose(np.abs(_signed_volumes(X, can)), np.abs(_signed_volumes(X, tets)), rtol=1e-12)
        # the patches (and so the colouring and the slot order) are unchanged
        assert [(p["first"], p["n"]) for p in _patches(can)] == [(p["first"], p["n"]) for p in _patches(tets)]


def test_layout_a_is_the_documented_tet_list():
    A = _constant("kHexLocA")
    tets = [[(A >> (12 * i + 3 * j)) & 7 for j in range(4)] for i in range(5)]
    assert tets == [[0, 1, 2, 3], [0, 2, 4, 5], [0, 3, 6, 5], [2, 3, 7, 5], [0, 2, 3, 5]]
