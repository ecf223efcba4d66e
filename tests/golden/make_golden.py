"""Generates the committed golden fixtures from the mounted reference.

Run where the reference sources are readable, naming their root:
    python tests/golden/make_golden.py <reference root>
(or with the root in the environment variable PI_REFERENCE).
Writes tests/golden/dmc_table.json: a SHA-256 digest of the reference's
dual-marching-cubes canonicalisation table (include/visitorextract.h:35-293)
and of its per-case triangle lists (src/visitorextract.cpp:95-199), so tests
can check the generated tables without the reference present.  The digests
are computed over a canonical text form: for the table, per code
"trans0..trans7,flip,code;" and for the cases "code:e0,e1,e2,...;".
"""
import hashlib
import json
import os
import re
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PI_REFERENCE", "")
HERE = os.path.dirname(os.path.abspath(__file__))


def table_text(rows):
    return "".join("%s,%d,%d;" % (",".join(map(str, tr)), int(fl), code) for tr, fl, code in rows)


def cases_text(cases):
    return "".join("%d:%s;" % (code, ",".join(str(e) for t in tris for e in t)) for code, tris in sorted(cases.items()))


def parse_reference():
    src = open(os.path.join(REF, "include", "visitorextract.h")).read()
    rows = re.findall(r"/\*\s*([01]{8})\s*\*/\s*\{\{([^}]*)\},\s*(true|false),\s*0b([01]{8})\}", src)
    table = [None] * 256
    for idx, tr, fl, code in rows:
        table[int(idx, 2)] = ([int(x) for x in tr.split(",")], fl == "true", int(code, 2))
    cpp = open(os.path.join(REF, "src", "visitorextract.cpp")).read()
    body = cpp[cpp.index("switch (dual_grids[i].proc.code)"):cpp.index("void VisitorExtract::generate_mesh")]
    cases, cur = {}, None
    for line in body.splitlines():
        m = re.search(r"case 0b([01]{8}):", line)
        if m:
            cur = int(m.group(1), 2)
            cases[cur] = []
            continue
        m = re.search(r"append\((\d+), (\d+), (\d+)\)", line)
        if m and cur is not None:
            cases[cur].append(tuple(map(int, m.groups())))
    return table, cases


def main():
    if not REF or not os.path.isdir(REF):
        sys.exit("usage: make_golden.py <reference root> (or set PI_REFERENCE); got %r" % REF)
    table, cases = parse_reference()
    assert all(t is not None for t in table)
    out = {
        "table_sha256": hashlib.sha256(table_text(table).encode()).hexdigest(),
        "cases_sha256": hashlib.sha256(cases_text(cases).encode()).hexdigest(),
        "num_cases": len(cases),
        "source": "include/visitorextract.h:35-293, src/visitorextract.cpp:95-199",
    }
    with open(os.path.join(HERE, "dmc_table.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(out)


if __name__ == "__main__":
    main()
