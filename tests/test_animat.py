"""ANIMAT (create_visualization, visualization.f90:24-54): the sampling grid,
its point location, and the VTK writer, on the CPU."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from exfem import workloads
from exfem.model import write_vtu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
TOL = 1e-9


def length_words(text):
    """Start offsets of the 8-character block-length words of the appended
    data (field, points, connectivity, offsets, types)."""
    s = text.index("\n_") + 2
    starts = []
    for _ in range(4):
        starts.append(s)
        # the word's first 4 characters encode the block's base64 length
        import base64
        n = int.from_bytes(base64.b64decode(text[s:s + 4]), "little")
        s += 8 + n
    starts.append(s)   # types: the offsets' word again
    return starts


def masked(text):
    """io.cpp:657 encodes the fourth byte of a length word from past the end
    of the int; blank those two characters."""
    t = list(text)
    for w in length_words(text):
        t[w + 4] = t[w + 5] = "?"
    return "".join(t)


def test_vtu_matches_the_reference_writer_on_the_golden_case(tmp_path):
    c = json.load(open(os.path.join(GOLD, "vtu_small.json")))
    out = tmp_path / "x.vtu"
    write_vtu(out, c["eptr"], c["eind"], np.reshape(c["points"], (-1, 2)), np.reshape(c["field"], (-1, 2)), c["name"])
    ours = out.read_text()
    ref = open(os.path.join(GOLD, "vtu_small.vtu")).read()
    assert len(ours) == len(ref)
    assert masked(ours) == masked(ref)
    # our length words carry the int's own high byte (0 here)
    assert all(ours[w + 4:w + 8] == "AA==" for w in length_words(ours))


@pytest.mark.parametrize("ncells", [4, 5, 7])
def test_vtu_matches_the_live_reference_writer(tmp_path, ncells):
    """Live against the reference's write_vtk_unst_field (oracle/_ref), with
    cell counts that are not multiples of 3 (the types block's tail)."""
    from oracle import build
    lib_path = build.build_ref_io()
    if lib_path is None:
        pytest.skip("reference tree not present (its io.cpp is the pin)")
    lib = C.CDLL(lib_path)
    rng = np.random.default_rng(ncells)
    npts = 2 * ncells + 2
    pts = rng.normal(size=(npts, 2)) * 1e3
    fld = rng.normal(size=(npts, 2)) * 1e-3
    eptr = np.arange(ncells + 1, dtype=np.int32) * 4 + 1
    eind = (rng.integers(0, npts, size=4 * ncells) + 1).astype(np.int32)
    ours_p, ref_p = tmp_path / "ours.vtu", tmp_path / "ref.vtu"
    write_vtu(ours_p, eptr, eind, pts, fld, "displacements")
    fn = str(ref_p).encode()
    name = b"displacements"
    ip = lambda a: np.ascontiguousarray(a, np.int32).ctypes.data_as(C.POINTER(C.c_int))
    dp = lambda a: np.ascontiguousarray(a, np.float64).ctypes.data_as(C.POINTER(C.c_double))
    lib.write_vtk_unst_field(C.byref(C.c_int(len(fn))), C.c_char_p(fn), C.byref(C.c_int(ncells)), ip(eptr), ip(eind),
                             C.byref(C.c_int(npts)), dp(pts), C.byref(C.c_int(len(name))), C.c_char_p(name), dp(fld))
    ours, ref = ours_p.read_text(), ref_p.read_text()
    assert len(ours) == len(ref) and masked(ours) == masked(ref)


def test_grid_points_and_cells_follow_visu_points_and_create_struct_mesh():
    m = workloads.build("canyon", scale=0.15, steps=5)
    g = m.grid(12.0, 780.0, 3.0, 301.0, 25.0)
    nx, ny = int((780.0 - 12.0) / 25.0), int((301.0 - 3.0) / 25.0)
    assert (g["nx"], g["ny"]) == (nx, ny)
    i, j = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), indexing="ij")
    want = np.stack([12.0 + i.ravel() * 25.0, 3.0 + j.ravel() * 25.0], axis=1)
    assert np.array_equal(g["points"], want)
    assert np.array_equal(g["eptr"], 1 + 4 * np.arange(nx * ny + 1))
    cells = g["eind"].reshape(-1, 4)
    ii, jj = np.meshgrid(np.arange(1, nx + 1), np.arange(1, ny + 1), indexing="ij")
    ii, jj = ii.ravel(), jj.ravel()
    want_c = np.stack([(ii - 1) * (ny + 1) + jj, ii * (ny + 1) + jj, ii * (ny + 1) + jj + 1, (ii - 1) * (ny + 1) + jj + 1], 1)
    assert np.array_equal(cells, want_c)


@pytest.mark.parametrize("name", ["canyon", "valley"])
def test_points_are_located_as_search_quadtree_does(name):
    """Every found point lies in its element, and a point strictly inside an
    element finds that element.  A point is unfound only when no element
    holds it, or only elements that end at it (a cut void on its other
    side, which the quadtree's descent enters).  Points on shared edges may
    take either neighbour; the displacement is continuous across them."""
    m = workloads.build(name, scale=0.1, steps=5)
    xy = m.nodes().reshape(-1, 2)
    c = m.corners() - 1
    x0, y0, x1, y1 = xy[c[:, 0], 0], xy[c[:, 0], 1], xy[c[:, 2], 0], xy[c[:, 2], 1]
    h = (x1 - x0).min()
    W, H = xy[:, 0].max(), xy[:, 1].max()
    # spacing 4h puts points on element edges and corners of every size; 3.7h mostly off them
    for g in (m.grid(0.0, W, 0.0, H, 4 * h), m.grid(0.3 * h, W, 0.7 * h, H, 3.7 * h)):
        check_location(g, x0, y0, x1, y1)
    if name == "canyon":       # the cut canyon leaves points in its void
        assert g["nfound"] < len(g["elem"])
    mat = g["material"]
    found = g["elem"] > 0
    assert (mat[~found] == 0).all() and (mat[found, 0] >= 1).all() and (mat[found, 1] > 0).all()


def check_location(g, x0, y0, x1, y1):
    assert g["nfound"] > 0
    pts, elem = g["points"], g["elem"]
    for lo in range(0, len(pts), 512):
        px, py = pts[lo:lo + 512, :1], pts[lo:lo + 512, 1:]
        e = elem[lo:lo + 512]
        holds = (px >= x0 - TOL) & (px <= x1 + TOL) & (py >= y0 - TOL) & (py <= y1 + TOL)
        inner = (px > x0 + TOL) & (px < x1 - TOL) & (py > y0 + TOL) & (py < y1 - TOL)
        rows = np.arange(len(e))
        has_inner = inner.any(axis=1)
        assert np.array_equal(e[has_inner], inner.argmax(axis=1)[has_inner] + 1)
        f = e > 0
        assert holds[rows[f], e[f] - 1].all()
        on_edge = ((np.abs(x0 - px) < TOL) | (np.abs(x1 - px) < TOL) | (np.abs(y0 - py) < TOL) |
                   (np.abs(y1 - py) < TOL))
        assert not (holds & ~on_edge)[~f].any()
