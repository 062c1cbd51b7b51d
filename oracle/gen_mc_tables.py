"""Generate voxelhashmt_gb300/csrc/vh_mc_tables.h, the marching-cubes tables shared by the
CUDA product and the oracle.

* The edge table is computed here from the corner/edge numbering the reference uses
  (include/tsdfmc/marching_cubes.h:18-32): bit e of entry i is set when the two corners of
  edge e are on different sides of the iso level for case i.
* The triangle table is the 256x16 table the reference vendors from three.js (MIT licence,
  include/tsdfmc/marching_cubes_tables.h:7-8, :44).  Parity needs it entry-for-entry, so it is
  read from the reference header and re-emitted as int8 data with the upstream attribution.

Both tables are checked against the reference header when it is present
(tests/test_oracle_cpu.py repeats the check).

usage: python oracle/gen_mc_tables.py [path/to/marching_cubes_tables.h]
"""
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "..", "voxelhashmt_gb300", "csrc", "vh_mc_tables.h")
# the reference tree: VH_REFERENCE_ROOT, else the build container's mount point (as oracle/build.py)
DEFAULT_REF = os.path.join(os.environ.get("VH_REFERENCE_ROOT", "/root/reference"), "include", "tsdfmc",
                           "marching_cubes_tables.h")

EDGE_CORNERS = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4),
                (0, 4), (1, 5), (2, 6), (3, 7)]


def computed_edge_table():
    table = []
    for case in range(256):
        mask = 0
        for e, (c0, c1) in enumerate(EDGE_CORNERS):
            if ((case >> c0) & 1) != ((case >> c1) & 1):
                mask |= 1 << e
        table.append(mask)
    return table


def parse_reference(path):
    text = open(path).read()
    edge_src = text[text.index("kMarchingCubesEdgeTable"):text.index("kMarchingCubesTriTable")]
    tri_src = text[text.index("kMarchingCubesTriTable"):]
    edge = [int(x) for x in re.findall(r"-?\d+", edge_src.split("=", 1)[1].split("};", 1)[0])]
    tri = [int(x) for x in re.findall(r"-?\d+", tri_src.split("=", 1)[1].split("}};", 1)[0])]
    assert len(edge) == 256, len(edge)
    assert len(tri) == 256 * 16, len(tri)
    return edge, [tri[i * 16:(i + 1) * 16] for i in range(256)]


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else DEFAULT_REF
    if not os.path.exists(ref):
        sys.exit("reference not present: %s (set VH_REFERENCE_ROOT or pass the header's path)" % ref)
    edge = computed_edge_table()
    ref_edge, tri = parse_reference(ref)
    assert edge == ref_edge, "computed edge table differs from the reference table"
    for row in tri:
        n = next((i for i, v in enumerate(row) if v < 0), 16)
        assert n % 3 == 0 and all(v < 0 for v in row[n:]) and all(0 <= v < 12 for v in row[:n])
    lines = [
        "/* vh_mc_tables.h -- marching-cubes tables (generated by oracle/gen_mc_tables.py; do not edit).",
        " *",
        " * Edge table: computed from the cube corner/edge numbering (corner c = (c&1^(c>>1&1), c>>1&1, c>>2)",
        " * ordering of the reference, include/tsdfmc/marching_cubes.h:18-32).",
        " * Triangle table: the classic Lorensen-Cline case table as distributed with three.js",
        " * (examples/jsm/objects/MarchingCubes.js, MIT licence, (c) the three.js authors),",
        " * which the reference vendors in include/tsdfmc/marching_cubes_tables.h; kept entry-for-entry",
        " * identical because triangle counts and order within a cube are part of the parity contract.",
        " * Plain C so the CUDA product (copied into __constant__ memory) and the oracle share it. */",
        "#ifndef VH_MC_TABLES_H",
        "#define VH_MC_TABLES_H",
        "#include <stdint.h>",
        "",
        "/* storage class of the tables: plain static data by default, e.g. `static __constant__` in CUDA */",
        "#ifndef VH_MC_TABLE_QUALIFIER",
        "#define VH_MC_TABLE_QUALIFIER static",
        "#endif",
        "",
        "VH_MC_TABLE_QUALIFIER const uint16_t vh_mc_edge_table[256] = {",
    ]
    for i in range(0, 256, 8):
        lines.append("    " + ", ".join("%4d" % v for v in edge[i:i + 8]) + ",")
    lines.append("};")
    lines.append("")
    lines.append("VH_MC_TABLE_QUALIFIER const int8_t vh_mc_tri_table[256][16] = {")
    for row in tri:
        lines.append("    {" + ", ".join("%2d" % v for v in row) + "},")
    lines.append("};")
    lines.append("")
    lines.append("#endif")
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    with open(OUT, "w") as f:
        f.write("\n".join(lines) + "\n")
    print("wrote", os.path.normpath(OUT))


if __name__ == "__main__":
    main()
