"""Extracts the known-answer vectors of the reference's own tests into a fixture.

The reference (cg-tuwien/APBF) tests its parallel primitives and list edits in
source/test.cpp (run on the GPU through Vulkan in Debug builds only).  This
script reads that file as text, pulls the literal std::vector<uint32_t> inputs
and expected outputs of each known-answer test, and writes
tests/golden/reference_known_answers.json.  The tests only read the JSON (the
reference checkout is not available where the GPU tests run).

Usage: python tests/golden/make_golden.py path/to/reference
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent

# test.cpp function -> the vector literals it declares
TESTS = [
    "gpu_list_concatenation_1",
    "gpu_list_append_empty",
    "gpu_list_apply_edit",
    "indexed_list_write_increasing_sequence",
    "indexed_list_apply_hidden_edit_1",
    "indexed_list_apply_hidden_edit_2",
    "indexed_list_apply_hidden_edit_3",
    "prefix_sum",
    "short_prefix_sum_in_long_buffer",
    "sort",
    "sort_small_values",
    "sort_few_values_in_long_buffer",
    "delete_these_1",
    "delete_these_3",
    "duplicate_these",
    "duplicate_these_empty",
]

VEC = re.compile(r"auto\s+(\w+)\s*=\s*std::vector<uint32_t>\(\{([^}]*)\}\)")


def function_body(src: str, name: str) -> tuple[str, int]:
    m = re.search(r"bool\s+pbd::test::" + name + r"\s*\(\s*\)\s*\{", src)
    if not m:
        raise KeyError(name)
    depth, i = 1, m.end()
    while depth:
        depth += {"{": 1, "}": -1}.get(src[i], 0)
        i += 1
    line = src[: m.start()].count("\n") + 1
    return src[m.end(): i - 1], line


def parse_int(tok: str) -> int:
    return int(tok.strip().rstrip("u").rstrip("U"))


def main(ref: Path) -> None:
    src = (ref / "source" / "test.cpp").read_text()
    out = {"source": "source/test.cpp of cg-tuwien/APBF", "tests": {}}
    for name in TESTS:
        body, line = function_body(src, name)
        vecs = {}
        for m in VEC.finditer(body):
            toks = [t for t in m.group(2).split(",") if t.strip()]
            vecs[m.group(1)] = [parse_int(t) for t in toks]
        out["tests"][name] = {"line": line, "vectors": vecs}
    dst = HERE / "reference_known_answers.json"
    dst.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {dst} ({len(out['tests'])} tests)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the APBF reference checkout>")
    main(Path(sys.argv[1]))
