"""Writes ``dvbs2_tables.py``: the parity-accumulator address tables of the DVB-S2 LDPC
codes (ETSI EN 302 307-1, Annex B for the normal FECFRAME, Annex C for the short one).

The numbers are data of the standard and must be identical; they are read from the
transcription in com-rs (``crates/com-systems/src/dvbs2/tables.rs``) and written here as
one tuple of addresses per group of 360 information bits.

Usage: ``python gen_dvbs2_tables.py <com-rs root> > dvbs2_tables.py``
"""

import os
import re
import sys


def parse(text):
    tables = {}
    for name, body in re.findall(r"const (N\d+_P\d+): &\[u16\] = &\[(.*?)\];", text, re.S):
        nums = [int(x) for x in re.findall(r"\d+", body)]
        groups, i = [], 0
        while i < len(nums):
            cnt = nums[i]
            groups.append(tuple(nums[i + 1:i + 1 + cnt]))
            i += 1 + cnt
        tables[name] = groups
    return tables


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else "."
    text = open(os.path.join(root, "crates/com-systems/src/dvbs2/tables.rs")).read()
    tables = parse(text)
    w = sys.stdout.write
    w('"""DVB-S2 LDPC parity-accumulator addresses (ETSI EN 302 307-1, Annexes B and C): for\n')
    w("every table N<n>_P<n - k>, one tuple per group of 360 information bits holding the\n")
    w('addresses of the group\'s first bit.  Generated by gen_dvbs2_tables.py; data only."""\n\n')
    w("TABLES = {\n")
    for name in sorted(tables, key=lambda s: tuple(int(x) for x in re.findall(r"\d+", s))):
        w(f"    {name!r}: (\n")
        for g in tables[name]:
            w("        (" + ", ".join(str(x) for x in g) + ("," if len(g) == 1 else "") + "),\n")
        w("    ),\n")
    w("}\n")


if __name__ == "__main__":
    main()
