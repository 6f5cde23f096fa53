"""Host side (the Fortran host's role): deck parsing, materials, mesher,
problem setup, receivers, and the reference file formats."""
import ctypes as C
import os

import numpy as np
import pytest

from exfem import decks, workloads
from exfem.abi import ExfemError
from exfem.model import Model, write_mass, write_sheet, write_step


def test_homogeneous_rectangle_sizes():
    m = workloads.build("homogeneous_rectangle")
    p = m.problem
    assert (m.nelems, m.nnodes) == (32768, 257 * 129)
    assert p.nhanging == 0 and p.nrecv == 64 and p.nrhs == 1
    assert p.deltat == 3.90625e-3 and p.nsteps == 4000 and p.io_interval == 1
    mc = m.matconst()[0]
    assert mc[0] == 2000 * 1000.0 ** 2 and mc[1] == 2000 * 2000.0 ** 2 - 2 * mc[0]
    xy, el = m.receivers()
    assert np.allclose(xy[:, 0], 62.5 * np.arange(1, 65)) and np.all(xy[:, 1] == 0)


def test_nu_material_form():
    # 's 1000 v 0.333333333333 1000' (rectan1..6 decks): vp = 2*vs
    d = decks._deck(1000, 500, 1, 0.01, 0.25, 10, 4, ["s 1000 v 0.333333333333 1000"], "WAVESV",
                    [500, 200, 500, 0, 1, 1, 0, 1, 1])
    m = Model(d)
    mc = m.matconst()[0]
    assert abs(mc[3] - 2000.0) < 1e-6 and mc[4] == 1000.0


def test_absorbing_tags_match_create_absorbingbc():
    m = workloads.build("canyon", scale=0.2, steps=10)
    xy = m.nodes()
    w, h = m.info["width"], (m.info["totrows"] - 1) * m.info["blength"]
    right = (m.info["totcols"] - 1) * m.info["blength"]
    want = np.zeros(m.nnodes, np.int32)
    side = (np.abs(xy[:, 0]) < 1e-9) | (np.abs(xy[:, 0] - right) < 1e-9)
    want[(np.abs(xy[:, 1] - h) < 1e-9) & ~side] = 1
    want[side] = 2
    assert np.array_equal(m.absorbing(), want)


def test_hanging_list_matches_ediv_and_is_unchained():
    m = workloads.build("canyon", scale=0.3, steps=10)
    eptr, eind, ediv = m.eptr(), m.eind(), m.ediv()
    want = []
    for e in range(m.nelems):
        b, t = eptr[e] - 1, eptr[e + 1] - 1
        for j in range(b, t):
            if ediv[j]:
                nxt = eind[j + 1] if j + 1 < t else eind[b]
                want.append((eind[j], eind[j - 1], nxt))
    hg = m.hanging()
    assert len(want) == len(hg) > 0 and np.array_equal(hg, np.array(want))
    assert not np.isin(hg[:, 1:], hg[:, 0]).any()          # 2:1 balance: no chains
    xy = m.nodes()
    mid = (xy[hg[:, 1] - 1] + xy[hg[:, 2] - 1]) / 2
    assert np.allclose(mid, xy[hg[:, 0] - 1])               # hanging nodes are edge midpoints


def test_quadtree_levels_and_balance():
    m = workloads.build("valley", scale=0.2, steps=10)
    assert m.info["nlevels"] == 4
    c = m.corners()
    xy = m.nodes()
    h = xy[c[:, 2] - 1, 1] - xy[c[:, 0] - 1, 1]
    lev = np.round(np.log2(h.max() / h)).astype(int)
    assert set(lev) == {0, 1, 2, 3}
    # neighbours across an edge differ by at most one level: every hanging
    # node's coarse element is exactly twice the size of the fine elements
    hg = m.hanging()
    seg = np.linalg.norm(xy[hg[:, 1] - 1] - xy[hg[:, 2] - 1], axis=1)
    assert np.all(np.isin(np.round(np.log2(h.max() / seg)), lev))


def test_seismic_layer_kinds():
    m = workloads.build("homogeneous_rectangle", scale=0.25, steps=10)
    s = m.seismic()
    kinds, counts = np.unique(s[:, 1], return_counts=True)
    assert set(kinds) == {1, 2, 4, 5, 6}
    assert counts[list(kinds).index(5)] == 1 and counts[list(kinds).index(6)] == 1


def test_canyon_cut_and_receivers_on_surface():
    m = workloads.build("canyon", scale=0.3, steps=10)
    full = m.info["totcols"] - 1
    assert m.nelems < 4 * full * (m.info["totrows"] - 1)
    xy, el = m.receivers()
    gp = (m.info["width"] / 2, 0.0, 500 * 0.3)
    inside = np.abs(xy[:, 0] - gp[0]) < gp[2] * 0.9
    assert (xy[inside, 1] > 0).all() and (xy[~inside & (np.abs(xy[:, 0] - gp[0]) > gp[2] * 1.2), 1] == 0).all()


def test_bad_decks_are_rejected():
    with pytest.raises(ExfemError):
        Model("NOT A DECK\n")
    with pytest.raises(ExfemError):   # more steps than the deck's TIME gives
        Model(decks.homogeneous_rectangle(scale=0.25, steps=10), nsteps=20)


REF = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "libref_io.so")


@pytest.fixture(scope="module")
def ref_io():
    from oracle import build
    if build.build_ref_io() is None:
        pytest.skip("reference tree not present (its io.cpp is the pin)")
    return C.CDLL(REF)


def test_mesh_bin_reads_back_with_reference_io(tmp_path, ref_io):
    m = workloads.build("canyon", scale=0.2, steps=10)
    path = str(tmp_path / "mesh.000.bin").encode()
    m.save_mesh(path.decode())
    ne, nn = C.c_int(), C.c_int()
    eptr, eind = C.POINTER(C.c_int)(), C.POINTER(C.c_int)()
    ediv, nodes = C.POINTER(C.c_ubyte)(), C.POINTER(C.c_double)()
    ref_io.load_binmesh(C.byref(C.c_int(len(path))), C.c_char_p(path), C.byref(ne), C.byref(eptr), C.byref(eind),
                        C.byref(ediv), C.byref(nn), C.byref(nodes))
    assert (ne.value, nn.value) == (m.nelems, m.nnodes)
    L = m.eptr()[-1] - 1   # the reference reads eptr[ne] = L + 1 entries; the last is padding
    assert np.array_equal(np.ctypeslib.as_array(eptr, (ne.value + 1,)), m.eptr())
    assert np.array_equal(np.ctypeslib.as_array(eind, (L,)), m.eind())
    assert np.array_equal(np.ctypeslib.as_array(ediv, (L,)), m.ediv())
    assert np.array_equal(np.ctypeslib.as_array(nodes, (2 * nn.value,)), m.nodes().ravel())


def test_problem_in_parse_matches_reference_parser(tmp_path, ref_io):
    deck = decks.canyon(scale=0.5, steps=100)
    f = tmp_path / "problem.in"
    f.write_text(deck)
    path = str(f).encode()
    dd = [C.c_double() for _ in range(7)]
    nmats, nppars, ngpars = C.c_int(), C.c_int(), C.c_int()
    cm, vm, vp, vg = C.POINTER(C.c_char)(), C.POINTER(C.c_double)(), C.POINTER(C.c_double)(), C.POINTER(C.c_double)()
    prob, geom = C.create_string_buffer(6), C.create_string_buffer(6)
    ref_io.load_problem_file(C.byref(C.c_int(len(path))), C.c_char_p(path), *[C.byref(x) for x in dd],
                             C.byref(nmats), C.byref(cm), C.byref(vm), prob, C.byref(nppars), C.byref(vp), geom,
                             C.byref(ngpars), C.byref(vg))
    height, width, time, inttime, chper, nperlen, sperlen = [x.value for x in dd]
    m = Model(deck)
    assert (width, height, chper, nperlen, sperlen) == (m.info["width"], m.info["height"], m.info["chper"],
                                                        m.info["nperlen"], m.info["sperlen"])
    assert prob.raw == b"WAVEP " and geom.raw == b"CANYON"
    pp = np.ctypeslib.as_array(vp, (nppars.value,))
    assert nppars.value == 9 and pp[0] > 0


def test_step_and_mass_files_read_back_with_reference_io(tmp_path, ref_io):
    u = np.arange(10, dtype=float) * 0.5
    p = str(tmp_path / "step.000.bin")
    write_step(p, 0, u, append=False)
    write_step(p, 1, 2 * u, append=True)
    step, nd, st = C.c_int(1), C.c_int(), C.c_int()
    out = C.POINTER(C.c_double)()
    b = p.encode()
    ref_io.load_binstep(C.byref(C.c_int(len(b))), C.c_char_p(b), C.byref(step), C.byref(nd), C.byref(out), C.byref(st))
    assert st.value == 0 and nd.value == 10
    assert np.array_equal(np.ctypeslib.as_array(out, (10,)), 2 * u)
    pm = str(tmp_path / "mass.000.bin")
    write_mass(pm, u)
    b = pm.encode()
    ref_io.load_binmass(C.byref(C.c_int(len(b))), C.c_char_p(b), C.byref(nd), C.byref(out))
    assert np.array_equal(np.ctypeslib.as_array(out, (10,)), u)


def test_sheet_txt_layout(tmp_path):
    pts = np.array([[1.0, 0.0], [2.0, 0.5]])
    fld = np.arange(12, dtype=float).reshape(3, 2, 2)
    p = tmp_path / "sheet.txt"
    write_sheet(str(p), pts, fld, 0.01)
    txt = p.read_text()
    assert txt.startswith("POINTS = [ 1.0000000000 0.0000000000 2.0000000000 0.5000000000  ];\nFIELD = [ ")
    rows = txt.split("FIELD = [ ")[1].split(" ];")[0].strip().split("\n")
    assert len(rows) == 3 and [float(v) for v in rows[1].split()] == list(range(4, 8))
    assert txt.rstrip().endswith("SAMP = 0.010000 ;")


MESH_SHA = {   # sha256 of eptr, eind, ediv, nodes, ematprop, hanging, seismic, absorbing
    "canyon": (17504, 17990, "39c7d8b3c0340a35c892167c986383769a2624065a2f1815e34d698753f27620"),
    "valley": (137724, 139151, "b63dc9a5f188b8a89b55990e2f9ae391c31f3d63efabfe0d054500b035e3587f"),
}


@pytest.mark.parametrize("name", sorted(MESH_SHA))
def test_mesher_output_is_pinned(name):
    """The mesh (element order, node numbering, hanging list) is pinned: the
    divide passes number new nodes in the reference's append order whatever
    the thread count."""
    import hashlib
    d = decks.canyon(scale=0.3, steps=10) if name == "canyon" else decks.valley(scale=0.3, steps=10)
    m = Model(d)
    h = hashlib.sha256()
    for a in (m.eptr(), m.eind(), m.ediv(), m.nodes(), m.ematprop(), m.hanging(), m.seismic(), m.absorbing()):
        h.update(np.ascontiguousarray(a).tobytes())
    assert (m.nelems, m.nnodes, h.hexdigest()) == MESH_SHA[name]
