"""Extract the golden values of the reference's own tests into a fixture.

Reads, as text, the reference's known-answer tests for this path and writes
``reference_golden.json`` beside this script:

* every ``call Assert_Close(<expr>, <literal>, '<label>')`` with a literal
  expected value in src/mod_tests.F90 (the FN function values of
  Test_FN_Functions among them), keyed by its label, with the line number;
* the ``E_python`` probe field of Test_Acceleration_Without_Image_Charge;
* the sites, work functions, test points and expected answers of
  unit_test_voronoi in src/mod_work_function.F90;
* the record layouts (numpy dtypes) and the ramo_current.dt column names of
  the reference's output reader, scripts/python_package/rumdeed_io.py, which
  cannot be imported here (it needs pandas).

Nothing here runs the reference (it is Fortran and cannot be built here); the
values are the literals its tests compare against.  The fixture is committed,
so the tests need only it:

    python tests/golden/extract_reference_golden.py <reference checkout>
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
NUM = r"[-+]?\d+(?:\.\d*)?(?:[dDeE][-+]?\d+)?"


def fnum(s):
    return float(s.replace("d", "e").replace("D", "e"))


def joined_lines(path):
    """Fortran statements with '&' continuations joined, each with its first line number."""
    out, buf, start = [], "", 0
    with open(path) as f:
        for n, raw in enumerate(f, 1):
            line = raw.split("!")[0].rstrip() if "'" not in raw else raw.rstrip("\n")
            s = line.strip()
            if buf:
                s = s[1:].strip() if s.startswith("&") else s
                buf += " " + s
            else:
                buf, start = s, n
            if buf.endswith("&"):
                buf = buf[:-1].rstrip()
                continue
            out.append((start, buf))
            buf = ""
    return out


def assert_close_literals(path):
    pat = re.compile(r"call\s+Assert_Close\s*\((.*),\s*(" + NUM + r")\s*,\s*'([^']*)'\s*\)", re.I)
    found = {}
    for line, stmt in joined_lines(path):
        m = pat.search(stmt)
        if m:
            found[m.group(3)] = {"value": fnum(m.group(2)), "line": line, "expr": m.group(1).strip()}
    return found


def array_literal(path, name):
    pat = re.compile(name + r"\s*=\s*\(/(.*?)/\)", re.I)
    for line, stmt in joined_lines(path):
        m = pat.search(stmt)
        if m:
            return {"values": [fnum(v) for v in re.findall(NUM, m.group(1))], "line": line}
    raise SystemExit("%s not found in %s" % (name, path))


def voronoi_unit_test(path):
    text = open(path).read()
    body = text[text.index("function unit_test_voronoi"):]
    body = body[:body.index("end function unit_test_voronoi")]
    get = lambda name: [fnum(v) for v in re.findall(NUM, re.search(name + r"\s*=\s*\(/(.*?)/\)", body).group(1))]
    checks = re.findall(r"abs\(res\s*-\s*(" + NUM + r")\)\s*>\s*(" + NUM + r")\).*?sec\s*/=\s*(\d+)", body, re.S)
    points = []
    for m in re.finditer(r"pos\s*=\s*\(/(.*?)/\)", body):
        vals = []
        for term in m.group(1).split(","):
            parts = [fnum(v) for v in re.findall(NUM, term)]
            vals.append(parts[0] / parts[1] if "/" in term and len(parts) == 2 else parts[0])
        points.append(vals[:2])
    return {"sites_x": get("vor_sites_x"), "sites_y": get("vor_sites_y"), "w_theta": get("vor_w_theta"),
            "sec": [int(v) for v in get("vor_sec")], "points": points,
            "expect": [{"w_theta": fnum(a), "tol": fnum(t), "sec": int(s)} for a, t, s in checks]}


def reader_layouts(path):
    """The record layouts of the reference's output reader
    (scripts/python_package/rumdeed_io.py), read as text: every
    ``NAME = np.dtype([('field', np.type), ...])`` as a list of (field, numpy
    type string) pairs, every ``NAME = OTHER`` alias of one, and the column
    names of ramo_current.dt (RAMO_COLUMNS)."""
    with open(path) as f:
        text = f.read()
    out = {}
    for m in re.finditer(r"^(\w+)\s*=\s*np\.dtype\(\[(.*?)\]\)", text, re.S | re.M):
        fields = re.findall(r"\('(\w+)',\s*np\.(\w+)\)", m.group(2))
        out[m.group(1)] = [[name, "<" + {"float64": "f8", "int32": "i4", "int64": "i8",
                                          "float32": "f4"}[t]] for name, t in fields]
    for m in re.finditer(r"^(\w+)\s*=\s*(\w+_DTYPE)\s*$", text, re.M):
        if m.group(2) in out:
            out[m.group(1)] = out[m.group(2)]
    cols = re.search(r"^RAMO_COLUMNS\s*=\s*\[(.*?)\]", text, re.S | re.M)
    out["RAMO_COLUMNS"] = re.findall(r"'(\w+)'", cols.group(1))
    return out


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: extract_reference_golden.py <path of a RUMDEED checkout>")
    ref = sys.argv[1]
    tests = os.path.join(ref, "src", "mod_tests.F90")
    work = os.path.join(ref, "src", "mod_work_function.F90")
    reader = os.path.join(ref, "scripts", "python_package", "rumdeed_io.py")
    out = {
        "source": {"assert_close": "src/mod_tests.F90", "E_python": "src/mod_tests.F90",
                   "voronoi": "src/mod_work_function.F90 (unit_test_voronoi)",
                   "reader_layouts": "scripts/python_package/rumdeed_io.py"},
        "assert_close": assert_close_literals(tests),
        "E_python": array_literal(tests, "E_python"),
        "voronoi": voronoi_unit_test(work),
        "reader_layouts": reader_layouts(reader),
    }
    path = os.path.join(HERE, "reference_golden.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")
    print("wrote %s: %d Assert_Close literals" % (path, len(out["assert_close"])))


if __name__ == "__main__":
    main()
