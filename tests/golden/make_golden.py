"""Extract the reference's golden test vectors into a JSON fixture.

The reference (msiglreith/panopaea) pins its DEC grid operators with two unit
tests in ``panopaea/src/dec/grid.rs``:

* ``grid_2d_divergence`` (grid.rs:428-482): a 5x5 f32 grid, hand-set face
  velocities ``velocities_y`` (6x5) / ``velocities_x`` (5x6) and the expected
  divergence ``div_ref`` (grid.rs:459-465), eps 1e-3;
* ``grid_2d_laplacian`` (grid.rs:484-515): a 3x3 f64 cell field
  ``faces_primal`` (grid.rs:488-492) and the expected Laplacian
  ``laplacian_ref`` (grid.rs:504), eps 1e-3.

The reference is Rust and cannot be built in this environment, so its test
source is read as text and the array literals are copied out verbatim.  Run
once where the reference source tree is available:

    python tests/golden/make_golden.py <reference-root>

The fixture (grid_rs_vectors.json) is committed; tests never read the
reference tree.
"""

import json
import os
import re
import sys


def _array_after(src, name):
    """Return the nested float list of the array literal bound to `name`."""
    m = re.search(r"\b%s\b\s*=\s*(?:&|Simplex2\(arr2\(&)?\s*\[" % re.escape(name), src)
    if not m:
        raise KeyError(name)
    i = m.end() - 1  # at the opening '['
    depth = 0
    for j in range(i, len(src)):
        if src[j] == "[":
            depth += 1
        elif src[j] == "]":
            depth -= 1
            if depth == 0:
                body = src[i:j + 1]
                break
    else:
        raise ValueError("unbalanced array literal for " + name)
    body = re.sub(r",\s*\]", "]", body)  # trailing commas
    return json.loads(body)


def write_header(json_path=None):
    """The same vectors as a C/C++ header (grid_rs_vectors.h) for the
    compiled API tests, generated from the committed JSON fixture."""
    here = os.path.dirname(os.path.abspath(__file__))
    d = json.load(open(json_path or os.path.join(here, "grid_rs_vectors.json")))

    def arr(name, ctype, rows):
        flat = [v for row in rows for v in (row if isinstance(row, list) else [row])]
        return "static const %s %s[%d] = {%s};\n" % (ctype, name, len(flat), ", ".join(repr(float(v)) for v in flat))

    dv, lp = d["grid_2d_divergence"], d["grid_2d_laplacian"]
    out = ["/* Golden vectors of panopaea/src/dec/grid.rs (grid_2d_divergence :428-482,\n"
           " * grid_2d_laplacian :484-515), generated from grid_rs_vectors.json by\n"
           " * tests/golden/make_golden.py --header.  Do not edit. */\n",
           "#pragma once\n",
           arr("GOLDEN_DIV_VELOCITIES_Y", "float", dv["velocities_y"]),
           arr("GOLDEN_DIV_VELOCITIES_X", "float", dv["velocities_x"]),
           arr("GOLDEN_DIV_REF", "float", dv["div_ref"]),
           "static const double GOLDEN_DIV_EPS = %r;\n" % dv["eps"],
           arr("GOLDEN_LAP_FACES_PRIMAL", "double", lp["faces_primal"]),
           arr("GOLDEN_LAP_REF", "double", lp["laplacian_ref"]),
           "static const double GOLDEN_LAP_EPS = %r;\n" % lp["eps"]]
    dst = os.path.join(here, "grid_rs_vectors.h")
    with open(dst, "w") as f:
        f.write("".join(out))
    print("wrote", dst)


def main(ref_root):
    path = os.path.join(ref_root, "panopaea", "src", "dec", "grid.rs")
    src = open(path).read()
    div_start = src.index("fn grid_2d_divergence")
    lap_start = src.index("fn grid_2d_laplacian")
    div_src, lap_src = src[div_start:lap_start], src[lap_start:]
    out = {
        "source": "panopaea/src/dec/grid.rs",
        "grid_2d_divergence": {
            "lines": "428-482",
            "dim": [5, 5],
            "dtype": "f32",
            "eps": 1e-3,
            "velocities_y": _array_after(div_src, "velocities_y"),
            "velocities_x": _array_after(div_src, "velocities_x"),
            "div_ref": _array_after(div_src, "div_ref"),
        },
        "grid_2d_laplacian": {
            "lines": "484-515",
            "dim": [3, 3],
            "dtype": "f64",
            "eps": 1e-3,
            "faces_primal": _array_after(lap_src, "faces_primal"),
            "laplacian_ref": _array_after(lap_src, "laplacian_ref"),
        },
    }
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "grid_rs_vectors.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--header":
        write_header()
    elif len(sys.argv) == 2:
        main(sys.argv[1])
    else:
        sys.exit("usage: python tests/golden/make_golden.py <reference-root> | --header")
