"""Writes tests/golden/canyon_kawase.json from the reference tree: the two
canyon decks the reference ships for vertically incident SV and P waves
(canyon1/problem.in, canyon4/problem.in, copied as text, unchanged) and the
digitized surface-amplification curves its comparison scripts plot against
the solver's sheets (sheets/canyonsvx.m, canyonsvy.m, canyonpx.m,
canyonpy.m; consumed by sheets/comparison.m:1-42 through comparitrans.m:1-28).

Each curve is a list of (x/a, |U|) pairs: horizontal position over the
canyon radius a, and the amplitude of the surface displacement component
(x: horizontal, y: vertical) for a unit incident wave at one frequency.
The curve names carry the variable names of the .m files (SVX, SVY, PX, PY).

Run where the reference tree is present:

    python tests/golden/make_canyon_golden.py [reference-tree]
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "canyon_kawase.json")


def read_curve(path):
    text = open(path).read()
    name, rest = text.split("=", 1)
    body = rest.split("[", 1)[1].split("]", 1)[0]
    vals = [float(v) for v in re.findall(r"[-+]?[0-9]*\.?[0-9]+(?:[eE][-+]?[0-9]+)?", body)]
    if len(vals) % 2:
        raise ValueError("odd number of values in %s" % path)
    return name.strip(), [[vals[i], vals[i + 1]] for i in range(0, len(vals), 2)]


def main(tree):
    out = {"provenance": {
        "decks": {"canyon_sv": "canyon1/problem.in", "canyon_p": "canyon4/problem.in"},
        "curves": {"SVX": "sheets/canyonsvx.m", "SVY": "sheets/canyonsvy.m",
                   "PX": "sheets/canyonpx.m", "PY": "sheets/canyonpy.m"},
        "used_by": "sheets/comparison.m:1-42, sheets/comparitrans.m:1-28, sheets/transmex.m:1-10",
    }, "decks": {}, "curves": {}}
    for key, rel in out["provenance"]["decks"].items():
        out["decks"][key] = open(os.path.join(tree, rel)).read()
    for key, rel in out["provenance"]["curves"].items():
        name, pts = read_curve(os.path.join(tree, rel))
        if name != key:
            raise ValueError("%s holds %s, expected %s" % (rel, name, key))
        out["curves"][key] = pts
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote %s: %s" % (OUT, {k: len(v) for k, v in out["curves"].items()}))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("EXFEM_REFERENCE_TREE", "/root/reference"))
