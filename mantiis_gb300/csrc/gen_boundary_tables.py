"""Regenerate boundary_tables.h from the reference's boundary-type data files.

The reference reads four text tables at start-up (include/utils.hpp:728-793,
from include/system_files/{bnd_types,ifstream,icsr,xy_norm}.txt).  The solver
here compiles the same numbers in, so its wall links and specular targets are
exactly the reference's.  The text files hold one number per line, laid out
row-major by direction (9 rows, or 2 for the normals) with one column per
boundary type (52); icsr is 1-based in the file.

Usage: python gen_boundary_tables.py <system_files_dir> > boundary_tables.h
"""
import os
import sys


def load(path):
    with open(path) as fh:
        return [float(tok) for tok in fh.read().split()]


def main(src):
    codes = [int(v) for v in load(src + "/bnd_types.txt")]
    ntype = len(codes)
    ifs = load(src + "/ifstream.txt")
    icsr = load(src + "/icsr.txt")
    xyn = load(src + "/xy_norm.txt")
    assert ntype == 52 and len(ifs) == 9 * ntype and len(icsr) == 9 * ntype and len(xyn) == 2 * ntype
    out = []
    out.append("// Generated by gen_boundary_tables.py from the reference's boundary-type tables")
    out.append("// (include/system_files/*.txt, loaded by include/utils.hpp:728-793). Do not edit.")
    out.append("#pragma once")
    out.append("")
    out.append("#define MANTIIS_N_BND_TYPES %d" % ntype)
    out.append("")
    out.append("// 9-bit 'neighbour is not a wall' pattern of each boundary type, bit order")
    out.append("// (MSB first) over the D2Q9 directions {7,3,6,4,0,2,8,1,5}")
    out.append("static const int MANTIIS_BND_CODES[%d] = {%s};" % (ntype, ", ".join(str(c) for c in codes)))
    out.append("")
    out.append("// per type and direction: 1 = the link streams, 0 = the link is treated as a wall")
    out.append("static const unsigned char MANTIIS_IFSTREAM[%d][9] = {" % ntype)
    for t in range(ntype):
        out.append("    {%s}," % ", ".join(str(int(ifs[q * ntype + t])) for q in range(9)))
    out.append("};")
    out.append("")
    out.append("// per type and direction: specular-reflection target direction (0-based)")
    out.append("static const unsigned char MANTIIS_ICSR[%d][9] = {" % ntype)
    for t in range(ntype):
        out.append("    {%s}," % ", ".join(str(int(icsr[q * ntype + t]) - 1) for q in range(9)))
    out.append("};")
    out.append("")
    out.append("// per type: wall normal (x, y)")
    out.append("static const double MANTIIS_XY_NORM[%d][2] = {" % ntype)
    for t in range(ntype):
        out.append("    {%.17g, %.17g}," % (xyn[t], xyn[ntype + t]))
    out.append("};")
    print("\n".join(out))


if __name__ == "__main__":
    # the reference's include/system_files folder: first argument or $MANTIIS_REF_DIR/include/system_files
    if len(sys.argv) > 1:
        main(sys.argv[1])
    elif os.environ.get("MANTIIS_REF_DIR"):
        main(os.path.join(os.environ["MANTIIS_REF_DIR"], "include", "system_files"))
    else:
        sys.exit("usage: gen_boundary_tables.py <reference>/include/system_files  (or set MANTIIS_REF_DIR)")
