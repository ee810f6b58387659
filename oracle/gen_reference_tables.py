"""Writes oracle/reference_tables.h: the reference's boundary-type tables
(include/system_files/{bnd_types,ifstream,icsr,xy_norm}.txt, loaded by
include/utils.hpp:728-793) as C arrays for the oracle, read straight from the
reference's files so that the oracle carries its own copy of that data.

The files hold one number per line, row-major by direction (9 rows, or 2 for
the normals) with one column per boundary type (52); icsr is 1-based in the file.

Test-infrastructure data; run once:
    python oracle/gen_reference_tables.py <reference>/include/system_files
    (or set MANTIIS_REF_DIR to the reference checkout)
"""
import os
import sys
from pathlib import Path


def load(path):
    with open(path) as fh:
        return [float(tok) for tok in fh.read().split()]


def main(src):
    codes = [int(v) for v in load(os.path.join(src, "bnd_types.txt"))]
    nt = len(codes)
    ifs = load(os.path.join(src, "ifstream.txt"))
    icsr = load(os.path.join(src, "icsr.txt"))
    xyn = load(os.path.join(src, "xy_norm.txt"))
    assert len(ifs) == 9 * nt and len(icsr) == 9 * nt and len(xyn) == 2 * nt
    out = ["/* The reference's boundary-type tables for the oracle (test infrastructure),",
           " * written by gen_reference_tables.py from the four text tables of the",
           " * reference's include/system_files folder.  Do not edit. */",
           "#ifndef ORACLE_REFERENCE_TABLES_H", "#define ORACLE_REFERENCE_TABLES_H", "",
           "#define ORACLE_N_BND_TYPES %d" % nt, "",
           "/* 9-bit 'neighbour is not a wall' code per type, MSB first over the directions {7,3,6,4,0,2,8,1,5} */",
           "static const int ORACLE_BND_CODES[%d] = {%s};" % (nt, ", ".join(str(c) for c in codes)), "",
           "/* per type and direction: 1 = the link streams, 0 = the link is a wall */",
           "static const unsigned char ORACLE_IFSTREAM[%d][9] = {" % nt]
    out += ["    {%s}," % ", ".join(str(int(ifs[q * nt + t])) for q in range(9)) for t in range(nt)]
    out += ["};", "", "/* per type and direction: specular target direction (0-based) */",
            "static const unsigned char ORACLE_ICSR[%d][9] = {" % nt]
    out += ["    {%s}," % ", ".join(str(int(icsr[q * nt + t]) - 1) for q in range(9)) for t in range(nt)]
    out += ["};", "", "/* per type: wall normal (x, y) */", "static const double ORACLE_XY_NORM[%d][2] = {" % nt]
    out += ["    {%.17g, %.17g}," % (xyn[t], xyn[nt + t]) for t in range(nt)]
    out += ["};", "", "#endif", ""]
    (Path(__file__).resolve().parent / "reference_tables.h").write_text("\n".join(out))


if __name__ == "__main__":
    if len(sys.argv) > 1:
        main(sys.argv[1])
    elif os.environ.get("MANTIIS_REF_DIR"):
        main(os.path.join(os.environ["MANTIIS_REF_DIR"], "include", "system_files"))
    else:
        sys.exit("usage: gen_reference_tables.py <reference>/include/system_files  (or set MANTIIS_REF_DIR)")
