"""Extracts the reference's own test fixtures into reference_fixtures.json.

Usage: ``python make_golden.py <reference checkout>`` (the directory that
holds the reference crate's src/ and data/); the GPU host never runs this.  It copies, as data:

* the SVG path strings of the reference's unit tests (SQUIRREL in
  src/path.rs, the star/boxes path of test_fill_rule and the 9x4 polygon of
  test_rasterizer in src/rasterize.rs);
* the small SVG path files of the reference's data/ directory;
* the input paths and expected outlines of test_stroke (src/path.rs).

Expected numbers of the known-answer tests are restated in
tests/test_oracle_kat.py next to the assertions that use them.
"""
import json
import os
import re
import sys

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_fixtures.json")


def raw_const(src, name):
    m = re.search(r'const %s: &str = r#"(.*?)"#;' % name, src, re.S)
    return " ".join(m.group(1).split())


def raw_in_fn(src, fn, idx=0):
    body = src[src.index("fn %s" % fn):]
    found = re.findall(r'r#"(.*?)"#', body, re.S)
    return " ".join(found[idx].split())


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <reference checkout>")
    global REF
    REF = sys.argv[1]
    path_rs = open(os.path.join(REF, "src/path.rs")).read()
    rast_rs = open(os.path.join(REF, "src/rasterize.rs")).read()
    fx = {
        "squirrel": raw_const(path_rs, "SQUIRREL"),
        "fill_rule_star_boxes": raw_in_fn(rast_rs, "test_fill_rule"),
        "square_on_pixel_edges": re.search(r'let path: Path = "(M1,1 v2 h1 v-2 Z)"', rast_rs).group(1),
        "data": {},
    }
    # test_stroke (src/path.rs): the input paths and the three expected outlines
    body = path_rs[path_rs.index("fn test_stroke"):]
    body = body[:body.index("#[test]")]
    fx["stroke_inputs"] = re.findall(r'let path: Path = "([^"]+)"\.parse', body)
    fx["stroke_expected"] = [" ".join(t.split()) for t in re.findall(r'r#"(.*?)"#', body, re.S)]
    for name in ("squirrel.path", "tv.path", "rust.path"):
        fx["data"][name] = open(os.path.join(REF, "data", name)).read().strip()
    with open(OUT, "w") as f:
        json.dump(fx, f, indent=1, sort_keys=True)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
