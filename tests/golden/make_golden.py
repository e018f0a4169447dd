"""Writes the golden fixtures under tests/golden/ from the reference's source tree.

Usage: python tests/golden/make_golden.py REFERENCE_DIR (or set ORB_REFERENCE_DIR); the
directory is the andrinr/gpu-load-balance checkout. Without it the script stops and the
committed fixtures stay as they are.

doc_example.json: the reference thesis's worked 2-D partition example
  (andrinr/gpu-load-balance documentation/particles10.csv -> particles11.csv ->
  particles12.csv, documentation/notes.tex:386-418 and 696-732): seven particles are
  partitioned at x = 0.65, then the first four at y = 0.55. The expected orders are the
  thesis's own tables.

oracle_builds.json: SHA-256 digests of oracle builds on seeded inputs, so that any change
  of the oracle's results is caught. These pin the oracle against itself; the reference
  pins are the doc example and the arithmetic cases in tests/test_oracle.py.
"""
import csv
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def reference_dir():
    d = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ORB_REFERENCE_DIR")
    if not d or not os.path.isdir(os.path.join(d, "documentation")):
        sys.exit("make_golden.py: give the reference's checkout as an argument or in "
                 "ORB_REFERENCE_DIR (the committed fixtures are left unchanged)")
    return d


def read(name):
    with open(os.path.join(reference_dir(), "documentation", name)) as f:
        rows = [[c.strip() for c in r] for r in csv.reader(f) if r]
    head, body = rows[0], rows[1:]
    cols = {h: [r[i] for r in body] for i, h in enumerate(head)}
    return {"x": [float(v) for v in cols["x"]], "y": [float(v) for v in cols["y"]],
            "id": [int(v) for v in cols["id"]]}


def doc_example():
    return {
        "source": "documentation/particles10.csv, particles11.csv, particles12.csv; "
                  "documentation/notes.tex:386-418, 696-732",
        "initial": read("particles10.csv"),
        "after_x_cut": read("particles11.csv"),
        "after_y_cut": read("particles12.csv"),
        "x_cut": 0.65,   # notes.tex:696
        "y_cut": 0.55,   # notes.tex:710
        "y_cut_cell": [0, 4],
    }


def oracle_digests():
    sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
    import oracle as O
    out = []
    for seed, n, d, kind in [(1, 1 << 12, 1 << 4, "uniform"), (2, 1 << 16, 1 << 8, "uniform"),
                             (3, 1 << 16, 1 << 10, "plummer")]:
        gen = O.gen_uniform if kind == "uniform" else O.gen_plummer
        x, y, z = gen(seed, n)
        r = O.build_tree(x, y, z, d)
        h = hashlib.sha256()
        for a in (r.heap, r.ranges, r.perm, r.x, r.y, r.z):
            h.update(a.tobytes())
        hin = hashlib.sha256()
        for a in (x, y, z):
            hin.update(a.tobytes())
        out.append({"seed": seed, "n": n, "d": d, "kind": kind, "input_sha256": hin.hexdigest(),
                    "build_sha256": h.hexdigest(), "stats": {k: r.stats[k] for k in
                    ("iterations", "degenerate_cells", "unfound_cells")}})
    return out


if __name__ == "__main__":
    with open(os.path.join(HERE, "doc_example.json"), "w") as f:
        json.dump(doc_example(), f, indent=1)
    with open(os.path.join(HERE, "oracle_builds.json"), "w") as f:
        json.dump(oracle_digests(), f, indent=1)
    print("wrote doc_example.json, oracle_builds.json")
