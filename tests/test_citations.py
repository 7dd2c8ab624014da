"""Every reference citation (path:line or path:first-last) in the product, the oracle and
the design notes names lines that exist in the reference tree, in exactly one file.
Skipped where the reference tree is absent (its root: HC_REFERENCE_ROOT)."""
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("HC_REFERENCE_ROOT", "/root/reference")
CITE = re.compile(r"([A-Za-z0-9_./]+\.(?:h|hpp|ipp|cpp)):(\d+)(?:-(\d+))?")


def sources():
    pats = ["include/*.h", "hyperboliconvergence_gb300/*.py", "hyperboliconvergence_gb300/csrc/*",
            "hyperboliconvergence_gb300/cpp/inc/hcgpu/*", "oracle/*.py", "oracle/*.hpp", "oracle/*.cpp",
            "oracle/ref/*", "tests/*.py", "tests/cpp/*", "tests/golden/*.py", "bench.py", "__graft_entry__.py",
            "DESIGN.md", "INTEGRATION.md", "README.md"]
    out = []
    for p in pats:
        out += [f for f in glob.glob(os.path.join(ROOT, p)) if os.path.isfile(f)]
    return sorted(set(out))


@pytest.fixture(scope="module")
def tree():
    if not os.path.isdir(os.path.join(REF, "cpp", "inc")):
        pytest.skip("reference tree absent")
    by_name = {}
    for dp, _dn, fn in os.walk(REF):
        for f in fn:
            by_name.setdefault(f, []).append(os.path.join(dp, f))
    return by_name


def test_every_citation_names_existing_lines(tree):
    lines, bad, checked = {}, [], 0
    for src in sources():
        with open(src, errors="replace") as fh:
            for ln, text in enumerate(fh, 1):
                for m in CITE.finditer(text):
                    path, a = m.group(1), int(m.group(2))
                    b = int(m.group(3) or a)
                    base = os.path.basename(path)
                    if base not in tree:
                        continue  # a file of this repository, not a reference citation
                    cands = [p for p in tree[base] if p.endswith("/" + path.lstrip("./")) or "/" not in path]
                    where = f"{os.path.relpath(src, ROOT)}:{ln} {m.group(0)}"
                    if len(cands) != 1:
                        bad.append(f"{where}: {len(cands)} reference files match")
                        continue
                    p = cands[0]
                    if p not in lines:
                        with open(p, errors="replace") as r:
                            lines[p] = sum(1 for _ in r)
                    if not (1 <= a <= b <= lines[p]):
                        bad.append(f"{where}: the file has {lines[p]} lines")
                    checked += 1
    assert checked > 200
    assert not bad, "\n".join(bad)
