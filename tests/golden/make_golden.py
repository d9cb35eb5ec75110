"""Extracts the reference's known-answer tests into tests/golden/reference_kats.json.

Reads the reference's GoogleTest sources as text (tests/BarnesHutTest.cpp,
tests/InputParserTest.cpp, tests/TimeConverterTest.cpp) and records, per TEST block, the input
vectors, configuration assignments and EXPECT_* known answers. Run it where the reference is
checked out:

    python tests/golden/make_golden.py /path/to/N-Body-Simulation

The JSON is committed so that the tests never need the reference at run time.
"""

from __future__ import annotations

import json
import os
import re
import sys

TEST_RE = re.compile(r"TEST\((\w+),\s*(\w+)\)\s*\{")
VEC_RE = re.compile(r"(?:std::vector<[^>]+>\s+)?(\w+?)(?:_vec)?\s*=\s*\{([^{}]*)\};")
EXPECT_RE = re.compile(r"EXPECT_(EQ|FLOAT_EQ)\(\s*([^,]+?)\s*,\s*(.+?)\s*\);")
THROW_RE = re.compile(r"EXPECT_THROW\(\s*(\w+)::(\w+)\((\w+)\)\s*,\s*([\w:]+)\s*\);")
CONF_RE = re.compile(r"configuration::([\w:]+)\s*=\s*([^;]+);")
INIT_RE = re.compile(r"configuration::initializeConfigValues\(([^)]*)\);")
STR_RE = re.compile(r'std::string\s+(\w+)\s*=\s*"([^"]*)";')
SPLIT_RE = re.compile(r'splitString\("([^"]*)"\)')
NODECOUNT_RE = re.compile(r"d_type::int_t\s+nodeCount\s*=\s*(\d+);")
BUILDER_RE = re.compile(r"^\s*(ParallelOctree\w+)\s+octree;", re.M)


def _num(tok: str):
    tok = tok.strip()
    try:
        return int(tok)
    except ValueError:
        pass
    try:
        return float(tok)
    except ValueError:
        pass
    m = re.fullmatch(r"([\d.]+)\s*/\s*([\d.]+)", tok)
    if m:
        return float(m.group(1)) / float(m.group(2))
    if tok.startswith('"') and tok.endswith('"'):
        return tok[1:-1]
    return tok


def _blocks(src: str):
    starts = [(m.start(), m.group(1), m.group(2), m.end()) for m in TEST_RE.finditer(src)]
    for k, (s, suite, name, body_start) in enumerate(starts):
        end = starts[k + 1][0] if k + 1 < len(starts) else len(src)
        yield suite, name, src[body_start:end]


def parse_file(path: str):
    src = open(path).read()
    out = []
    for suite, name, body in _blocks(src):
        rec = {"suite": suite, "name": name, "vectors": {}, "config": {}, "expects": [],
               "throws": [], "strings": {}, "split_inputs": []}
        for m in VEC_RE.finditer(body):
            rec["vectors"][m.group(1)] = [_num(t) for t in m.group(2).split(",") if t.strip()]
        for m in CONF_RE.finditer(body):
            rec["config"][m.group(1)] = _num(m.group(2))
        m = INIT_RE.search(body)
        if m:
            rec["config"]["initializeConfigValues"] = [_num(t) for t in m.group(1).split(",")]
        m = NODECOUNT_RE.search(body)
        if m:
            rec["config"]["nodeCount"] = int(m.group(1))
        m = BUILDER_RE.search(body)
        if m:
            rec["builder"] = m.group(1)
        for m in EXPECT_RE.finditer(body):
            lhs, rhs = m.group(2), m.group(3)
            am = re.fullmatch(r"(\w+)\[(\d+)\]", lhs)
            if am:
                rec["expects"].append({"kind": m.group(1), "array": am.group(1),
                                       "index": int(am.group(2)), "value": _num(rhs)})
            else:
                cm = re.fullmatch(r"result\.at\((\d+)\)", lhs)
                if cm:
                    rec["expects"].append({"kind": m.group(1), "array": "result",
                                           "index": int(cm.group(1)), "value": _num(rhs)})
                else:
                    rec["expects"].append({"kind": m.group(1), "expr": lhs, "value": _num(rhs)})
        for m in THROW_RE.finditer(body):
            rec["throws"].append({"cls": m.group(1), "fn": m.group(2), "arg": m.group(3),
                                  "exception": m.group(4)})
        for m in STR_RE.finditer(body):
            rec["strings"][m.group(1)] = m.group(2)
        rec["split_inputs"] = [m.group(1) for m in SPLIT_RE.finditer(body)]
        out.append(rec)
    return out


def main(ref_root: str, out_path: str):
    tests = {}
    for fname in ("BarnesHutTest.cpp", "InputParserTest.cpp", "TimeConverterTest.cpp"):
        tests[fname] = parse_file(os.path.join(ref_root, "tests", fname))
    doc = {"source": "reference tests/*.cpp (GoogleTest known answers), extracted by make_golden.py",
           "tests": tests}
    with open(out_path, "w") as f:
        json.dump(doc, f, indent=1, sort_keys=True)
    print(f"wrote {out_path}: " + ", ".join(f"{k}: {len(v)} tests" for k, v in tests.items()))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <root of the reference checkout>")
    main(sys.argv[1], os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                   "reference_kats.json"))
