"""Generate ``nr_base_graphs.inc``: the 5G NR LDPC base graphs as C data.

The data are Tables 5.3.2-1 (lifting-size sets), 5.3.2-2 (base graph 1) and 5.3.2-3
(base graph 2) of 3GPP TS 38.212.  They are read from the reference's table module
(``crates/com-fec/src/nr/tables.rs``, which transcribes the standard) and written in this
project's own layout: one ``{row, col, V[0..7]}`` record per nonzero entry, row-major,
and the eight lifting sets.  The output is committed; this script only re-creates it.

Usage: ``python gen_nr_tables.py <reference root> > nr_base_graphs.inc``
"""

import os
import re
import sys


def entries(src: str, name: str):
    m = re.search(r"pub const %s: \[\(u8, u8, \[u16; 8\]\); (\d+)\] = \[(.*?)\n\];" % name, src, re.S)
    if not m:
        raise SystemExit(f"table {name} not found")
    out = []
    for i, j, v in re.findall(r"\((\d+), (\d+), \[([\d, ]+)\]\)", m.group(2)):
        out.append((int(i), int(j), [int(x) for x in v.split(",")]))
    if len(out) != int(m.group(1)):
        raise SystemExit(f"table {name}: {len(out)} entries, declared {m.group(1)}")
    return out


def lifting_sets(src: str):
    m = re.search(r"pub const LIFTING_SETS: \[&\[usize\]; 8\] = \[(.*?)\];", src, re.S)
    return [[int(x) for x in s.split(",") if x.strip()] for s in re.findall(r"&\[([\d, ]+)\]", m.group(1))]


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else "."
    src = open(os.path.join(root, "crates/com-fec/src/nr/tables.rs")).read()
    bg1, bg2 = entries(src, "BG1"), entries(src, "BG2")
    sets = lifting_sets(src)
    w = sys.stdout.write
    w("/* 5G NR LDPC base graphs and lifting sets (3GPP TS 38.212 Tables 5.3.2-1/2/3).\n")
    w("   Generated by gen_nr_tables.py; data only. Record = {row, col, V for iLS 0..7}. */\n")
    for name, t in (("NR_BG1", bg1), ("NR_BG2", bg2)):
        w(f"#define {name}_ENTRIES {len(t)}\n")
        w(f"static const unsigned short {name}[{len(t)}][10] = {{\n")
        for i, j, v in t:
            w("  {%d, %d, %s},\n" % (i, j, ", ".join(str(x) for x in v)))
        w("};\n")
    w("static const unsigned short NR_LIFTING_SETS[8][8] = {\n")
    for s in sets:
        w("  {%s},\n" % ", ".join(str(x) for x in s + [0] * (8 - len(s))))
    w("};\n")
    w("static const unsigned char NR_LIFTING_SET_SIZES[8] = {%s};\n" % ", ".join(str(len(s)) for s in sets))


if __name__ == "__main__":
    main()
