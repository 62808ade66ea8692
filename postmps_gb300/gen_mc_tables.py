"""Build step: extract the reference's marching-cubes tables.

Reads MarchingCubesHelper.cpp from the reference checkout named by
$PMS_REFERENCE_DIR (required for this step) and writes the git-ignored generated
header postmps_gb300/_build/gen/mc_tables.inc that mc_tables.cu includes, so
that triangle soups come out in the reference's exact order.  The tables are
not committed; without a reference checkout the build uses the tables derived
in mc_tables.cu instead.
"""
from __future__ import annotations

import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "gen", "mc_tables.inc")


def _block(src: str, name: str) -> list[int]:
    m = re.search(r"MarchingCubesHelper::" + name + r"\s*(\[[^=]*\])\s*=\s*\{", src)
    if not m:
        raise ValueError(f"table {name} not found")
    i = m.end() - 1
    depth = 0
    for j in range(i, len(src)):
        if src[j] == "{":
            depth += 1
        elif src[j] == "}":
            depth -= 1
            if depth == 0:
                body = src[i:j + 1]
                break
    body = re.sub(r"//[^\n]*", "", body)
    return [int(t, 0) for t in re.findall(r"-?0x[0-9a-fA-F]+|-?\d+", body)]


def extract(ref_dir: str) -> dict | None:
    path = os.path.join(ref_dir, "src", "inc", "marchingcube", "MarchingCubesHelper.cpp")
    if not os.path.exists(path):
        return None
    src = open(path).read()
    t = {
        "edge_flags": _block(src, "edgeFlags"),
        "tri": _block(src, "edgeIndexesOfTriangle"),
        "num_vertices": _block(src, "numVertices"),
        "edge_vertex": _block(src, "vertexIndexesOfEdge"),
    }
    assert len(t["edge_flags"]) == 256 and len(t["tri"]) == 256 * 16
    assert len(t["num_vertices"]) == 256 and len(t["edge_vertex"]) == 24
    return t


def write_inc(t: dict, path: str = OUT) -> None:
    os.makedirs(os.path.dirname(path), exist_ok=True)
    def arr(vals, per=16):
        rows = [", ".join(str(v) for v in vals[i:i + per]) for i in range(0, len(vals), per)]
        return ",\n    ".join(rows)
    tri_rows = ",\n    ".join("{" + ", ".join(str(v) for v in t["tri"][16 * c:16 * c + 16]) + "}" for c in range(256))
    ev_rows = ", ".join("{%d, %d}" % (t["edge_vertex"][2 * e], t["edge_vertex"][2 * e + 1]) for e in range(12))
    text = (
        "// GENERATED by postmps_gb300/gen_mc_tables.py from the reference's\n"
        "// MarchingCubesHelper.cpp -- build output, not committed.\n"
        "#pragma once\n#include <cstdint>\nnamespace pms {\n"
        f"static const uint32_t kRefEdgeFlags[256] = {{\n    {arr(t['edge_flags'])}\n}};\n"
        f"static const int32_t kRefTriangles[256][16] = {{\n    {tri_rows}\n}};\n"
        f"static const uint32_t kRefNumVertices[256] = {{\n    {arr(t['num_vertices'])}\n}};\n"
        f"static const uint32_t kRefEdgeVertices[12][2] = {{{ev_rows}}};\n"
        "}  // namespace pms\n"
    )
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        f.write(text)
    os.replace(tmp, path)


def main() -> int:
    ref = os.environ.get("PMS_REFERENCE_DIR")
    if not ref:
        have = "keeping existing " + OUT if os.path.exists(OUT) else "using the derived tables"
        print(f"gen_mc_tables: PMS_REFERENCE_DIR is not set (the reference checkout), {have}")
        return 0
    t = extract(ref)
    if t is None:
        if os.path.exists(OUT):
            print(f"gen_mc_tables: reference not found, keeping existing {OUT}")
        else:
            print("gen_mc_tables: reference not found, using the derived tables")
        return 0
    write_inc(t)
    print(f"gen_mc_tables: wrote {OUT}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
