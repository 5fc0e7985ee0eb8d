"""Generate ``nr_bg_schedule.inc``: the structure of the 5G NR base graphs as compile-time
data for the graph-specialised layered decoder (``layered_nr.cuh``).

Reads this project's ``nr_base_graphs.inc`` (TS 38.212 Tables 5.3.2-2/3) and writes, per
base graph: the entries of each row (row-major, as the tables list them), their columns,
and the level schedule of the rows.  A row's level is one more than the highest level of
an earlier row sharing a column with it; rows of one level share no column, so their
lifted rows can run between the same two barriers with the sequential layered order's
results.  The rule is the one ``fill_dev_code`` (dev_code.h) applies at run time.

Usage: ``python gen_nr_schedule.py > nr_bg_schedule.inc`` (run from this directory).
"""

import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def base_graph(src, bg):
    m = re.search(r"NR_BG%d\[\d+\]\[10\] = \{(.*?)\};" % bg, src, re.S)
    return [(int(r), int(c)) for r, c in re.findall(r"\{(\d+), (\d+),", m.group(1))]


def schedule(entries):
    rows = max(r for r, _ in entries) + 1
    start = [0] * (rows + 1)
    for r, _ in entries:
        start[r + 1] += 1
    for i in range(rows):
        start[i + 1] += start[i]
    cols = [c for _, c in entries]
    last, level = {}, []
    for row in range(rows):
        lv = max([last.get(cols[t], -1) + 1 for t in range(start[row], start[row + 1])] + [0])
        level.append(lv)
        for t in range(start[row], start[row + 1]):
            last[cols[t]] = lv
    order, level_end = [], []
    for lv in range(max(level) + 1):
        members = [row for row in range(rows) if level[row] == lv]
        order += members
        level_end += [0] * (len(members) - 1) + [1]
    return rows, start, cols, order, level_end


def main():
    src = open(os.path.join(HERE, "nr_base_graphs.inc")).read()
    w = sys.stdout.write
    w("/* Compile-time structure of the 5G NR base graphs: entries per row, their columns and\n"
      "   the level schedule of the rows.  Generated by gen_nr_schedule.py from\n"
      "   nr_base_graphs.inc; data only. */\n")
    for bg in (1, 2):
        rows, start, cols, order, level_end = schedule(base_graph(src, bg))
        w(f"struct BaseGraph{bg} {{\n")
        w(f"  static constexpr int rows = {rows}, entries = {len(cols)}, levels = {sum(level_end)};\n")
        w(f"  static constexpr int start[{rows + 1}] = {{{', '.join(map(str, start))}}};\n")
        w(f"  static constexpr int col[{len(cols)}] = {{{', '.join(map(str, cols))}}};\n")
        w(f"  static constexpr int order[{rows}] = {{{', '.join(map(str, order))}}};\n")
        w(f"  static constexpr int level_end[{rows}] = {{{', '.join(map(str, level_end))}}};\n")
        w("};\n")


if __name__ == "__main__":
    main()
