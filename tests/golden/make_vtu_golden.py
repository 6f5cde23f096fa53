"""Writes tests/golden/vtu_small.{json,vtu}: a 3x2-cell structured grid with
fixed point values, written by the reference's own write_vtk_unst_field
(io.cpp:699-842, compiled from the reference tree into oracle/_ref by
oracle/build.py).  Run where the reference tree is present:

    python tests/golden/make_vtu_golden.py
"""
import ctypes as C
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def case():
    nx, ny = 3, 2
    pts, eptr, eind = [], [1], []
    for i in range(nx + 1):          # create_struct_mesh order
        for j in range(ny + 1):
            pts += [10.0 + 2.5 * i, -1.25 + 2.5 * j]
    for i in range(1, nx + 1):
        for j in range(1, ny + 1):
            eptr.append(eptr[-1] + 4)
            eind += [(i - 1) * (ny + 1) + j, i * (ny + 1) + j, i * (ny + 1) + j + 1, (i - 1) * (ny + 1) + j + 1]
    field = [0.001 * k * k - 0.5 * k + 1.0 / (k + 3) for k in range(2 * len(pts) // 2)]
    return {"eptr": eptr, "eind": eind, "points": pts, "field": field, "name": "displacements"}


def main():
    from oracle import build
    lib_path = build.build_ref_io()
    if lib_path is None:
        raise SystemExit("reference tree not present")
    lib = C.CDLL(lib_path)
    c = case()
    out = os.path.join(HERE, "vtu_small.vtu")
    fn = out.encode()
    eptr = (C.c_int * len(c["eptr"]))(*c["eptr"])
    eind = (C.c_int * len(c["eind"]))(*c["eind"])
    pts = (C.c_double * len(c["points"]))(*c["points"])
    fld = (C.c_double * len(c["field"]))(*c["field"])
    name = c["name"].encode()
    lib.write_vtk_unst_field(C.byref(C.c_int(len(fn))), C.c_char_p(fn), C.byref(C.c_int(len(c["eptr"]) - 1)),
                             eptr, eind, C.byref(C.c_int(len(c["points"]) // 2)), pts,
                             C.byref(C.c_int(len(name))), C.c_char_p(name), fld)
    with open(os.path.join(HERE, "vtu_small.json"), "w") as f:
        json.dump(c, f)
    print("wrote", out)


if __name__ == "__main__":
    main()
