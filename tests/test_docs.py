"""The documentation's references to files of this repository resolve: every
backticked path under profiles/, tests/, oracle/, include/ or the package
(optionally with a ::test suffix) names a file or folder that exists."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# named on purpose as absent: the reference has no compiled parts to build there
ABSENT_ON_PURPOSE = {"oracle/_ref"}
PATH = re.compile(r"`((?:profiles|tests|hydrothermal3d_gb300|oracle|include|csrc)/[A-Za-z0-9_./]+?)(?:::[A-Za-z0-9_]+)?`")


def _docs():
    yield from ("DESIGN.md", "README.md", "INTEGRATION.md")
    for f in sorted(os.listdir(os.path.join(ROOT, "profiles"))):
        yield os.path.join("profiles", f)


def test_documented_paths_exist():
    missing = []
    for doc in _docs():
        with open(os.path.join(ROOT, doc), encoding="utf-8") as fh:
            text = fh.read()
        for m in PATH.finditer(text):
            path = m.group(1)
            if path in ABSENT_ON_PURPOSE:
                continue
            if not any(os.path.exists(os.path.join(ROOT, c)) for c in (path, os.path.join("hydrothermal3d_gb300", path))):
                missing.append((doc, path))
    assert not missing, missing


def test_test_references_name_existing_tests():
    """`tests/x.py::test_y` references name a test function defined in that file."""
    missing = []
    for doc in _docs():
        with open(os.path.join(ROOT, doc), encoding="utf-8") as fh:
            text = fh.read()
        for m in re.finditer(r"`(tests/[A-Za-z0-9_]+\.py)::([A-Za-z0-9_]+)`", text):
            with open(os.path.join(ROOT, m.group(1)), encoding="utf-8") as fh:
                if f"def {m.group(2)}(" not in fh.read():
                    missing.append((doc, m.group(0)))
    assert not missing, missing
