"""The reference's command-line tools, restated on libgas:

* ``mtx2gr IN OUT`` -- any readable graph (.mtx, .edge, .gr) to a Lonestar
  ``.gr`` file (mtx2gr.cpp:22-53: load, CSR by source, edge data permuted
  along);
* ``gr2mtx IN OUT`` -- a graph to MatrixMarket (gr2mtx.cpp:22-43);
* ``check-dist TEST GOLD`` -- the BFS / SSSP distance comparator
  (regressions/checkDist.py:31-62);
* ``check-pagerank TEST GOLD`` -- the PageRank comparator
  (regressions/checkPageRank.py:38-83).

Result files are text, one ``vertex value`` pair per line, as the reference
apps write them.  Each command exits 0 on success ("No differences found" for
the distance check), 1 otherwise.

    python -m graphreduce_gb300.tools mtx2gr graph.mtx graph.gr
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path
from typing import Iterable

import numpy as np

from .graph import EdgeList

# unreachable distances: the gold programs write 10000000, the GPU apps
# INT_MAX - 100000 (checkDist.py:44)
GOLD_UNREACHED = 10000000
TEST_UNREACHED = 2147383647

# checkPageRank.py:76-83: |test - gold| decades and the fraction of vertices
# allowed in each ([0,1e-4), [1e-4,1e-3), ..., [10, inf))
PR_TOL_VALS = (1e-4, 1e-3, 1e-2, 0.1, 1.0, 10.0)
PR_ALLOWED = (1.0, 1e-2, 5e-3, 5e-4, 5e-5, 5e-6, 0.0)


def mtx2gr(src: str | Path, dst: str | Path) -> EdgeList:
    el = EdgeList.read(str(src))
    el.write_gr(str(dst))
    return el


def gr2mtx(src: str | Path, dst: str | Path) -> EdgeList:
    el = EdgeList.read(str(src))
    el.write_mtx(str(dst))
    return el


def _pairs(lines: Iterable[str], conv):
    for line in lines:
        parts = line.split()
        if len(parts) >= 2:
            yield int(parts[0]), conv(parts[1])


def check_dist(test_lines: Iterable[str], gold_lines: Iterable[str],
               log=print) -> bool:
    """Both inputs sorted by vertex id.  Every gold vertex must appear in the
    test output with the same value; a gold 10000000 matches a test
    2147383647 (the two apps' 'unreached').  Extra test vertices are fine."""
    test = iter(_pairs(test_lines, int))
    cur = next(test, None)
    for gv, gval in _pairs(gold_lines, int):
        while cur is not None and cur[0] < gv:
            cur = next(test, None)
        if cur is None or cur[0] != gv:
            log(f"vertex {gv} is in gold but not in test")
            return False
        if cur[1] != gval and not (gval == GOLD_UNREACHED and cur[1] == TEST_UNREACHED):
            log(f"{gv} gold={gval} ref={cur[1]}")
            return False
        cur = next(test, None)
    return True


def pagerank_histogram(test: dict[int, float], gold: dict[int, float]) -> np.ndarray:
    """Fraction of the test vertices per |difference| decade; vertices
    missing from gold are skipped but still count in the total."""
    counts = np.zeros(len(PR_TOL_VALS) + 1)
    for vid, val in test.items():
        if vid not in gold:
            continue
        diff = abs(gold[vid] - val)
        pos = len(PR_TOL_VALS) - 1
        while pos >= 0 and diff < PR_TOL_VALS[pos]:
            pos -= 1
        counts[pos + 1] += 1
    return counts / max(1, len(test))


def check_pagerank(test_lines: Iterable[str], gold_lines: Iterable[str],
                   log=print) -> bool:
    test = dict(_pairs(test_lines, float))
    gold = dict(_pairs(gold_lines, float))
    frac = pagerank_histogram(test, gold)
    for f, a in zip(frac, PR_ALLOWED):
        if f > a:
            log(f"Percentage too high: {a} {f}")
            return False
    return True


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m graphreduce_gb300.tools")
    sub = ap.add_subparsers(dest="cmd", required=True)
    for name in ("mtx2gr", "gr2mtx"):
        p = sub.add_parser(name)
        p.add_argument("input")
        p.add_argument("output")
    for name in ("check-dist", "check-pagerank"):
        p = sub.add_parser(name)
        p.add_argument("test")
        p.add_argument("gold")
    a = ap.parse_args(argv)
    if a.cmd in ("mtx2gr", "gr2mtx"):
        el = (mtx2gr if a.cmd == "mtx2gr" else gr2mtx)(a.input, a.output)
        print(f"Read input file with {el.nV} vertices and {el.nE} edges")
        return 0
    with open(a.test) as t, open(a.gold) as g:
        ok = (check_dist if a.cmd == "check-dist" else check_pagerank)(t, g)
    if ok and a.cmd == "check-dist":
        print("No differences found")
    return 0 if ok else 1


if __name__ == "__main__":
    sys.exit(main())
