"""Repository rules that keep the oracle a checker only: nothing in the
product package refers to it, and outside tests/ only bench.py's CPU legs and
__graft_entry__ import it."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ALLOWED = {"bench.py", "__graft_entry__.py"}


def _files(top, exts):
    for d, _, fs in os.walk(top):
        if "__pycache__" in d or "/_" in d.replace(ROOT, ""):
            continue
        for f in fs:
            if f.endswith(exts):
                yield os.path.join(d, f)


def test_product_package_never_refers_to_the_oracle():
    bad = [p for p in _files(os.path.join(ROOT, "pmmc_gb300"), (".py", ".cu", ".h", ".cuh", ".cpp"))
           if re.search(r"\boracle\b", open(p, errors="replace").read())]
    assert bad == []


def test_oracle_imported_only_by_tests_bench_and_entry():
    pat = re.compile(r"^\s*(from\s+oracle\b|import\s+oracle\b)", re.M)
    bad = []
    for p in _files(ROOT, (".py",)):
        rel = os.path.relpath(p, ROOT)
        if rel.startswith(("tests" + os.sep, "oracle" + os.sep, "_work" + os.sep)):
            continue
        if pat.search(open(p).read()) and rel not in ALLOWED:
            bad.append(rel)
    assert bad == []
