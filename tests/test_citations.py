"""Every citation of a reference file (``fpie/<path>:<lines>``) resolves.

Source comments, docstrings and the design documents cite the reference's
files by path and line range.  This test parses every such citation in the
repository's text files and checks that the file exists in the reference
tree and that each cited range lies inside it.  A citation may list several
ranges (``fpie/process.py:113-122, 192-271``) or continue with ``:a-b``.
Short forms naming a file that exists only in the reference (for example
``np_solver.py:33-41`` or ``cuda/grid.cu:54-71``) are checked too.

The reference tree is read from the ``FPIE_REFERENCE`` environment variable;
without it the test is skipped.
"""

from __future__ import annotations

import os
import pathlib
import re

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
SKIP_DIRS = {".git", "_work", "gpurun_out", "_build", "_lib", "_ref", "baseline", "__pycache__",
             ".pytest_cache", "golden"}
# Written by the survey and the reviews, not by this repository's authors.
SKIP_FILES = {"SURVEY.md", "VERDICT.md", "ADVICE.md"}
SUFFIXES = {".py", ".md", ".h", ".cu", ".cuh", ".c", ".sh", ".txt"}
REF_SUFFIX = r"(?:py|cc|cu|h|md|rst)"
CITE = re.compile(r"((?:[A-Za-z0-9_]+/)*[A-Za-z0-9_]+\." + REF_SUFFIX + r"):"
                  r"(\d+(?:-\d+)?(?:\s*,\s*:?\d+(?:-\d+)?)*)")


def _reference_root():
    env = os.environ.get("FPIE_REFERENCE")
    if not env:
        return None
    p = pathlib.Path(env)
    return p if (p / "fpie").is_dir() else None


def _text_files():
    for p in sorted(ROOT.rglob("*")):
        rel = p.relative_to(ROOT)
        if any(part in SKIP_DIRS for part in rel.parts[:-1]) or not p.is_file():
            continue
        if p.name in SKIP_FILES or p.suffix not in SUFFIXES:
            continue
        yield rel, p


def _ranges(spec: str):
    for part in spec.split(","):
        part = part.strip().lstrip(":")
        a, _, b = part.partition("-")
        yield int(a), int(b or a)


def _resolve(name: str, ref: pathlib.Path, ref_files: list[str], ours: set[str]):
    """The reference file a cited name means, or None when it is not a
    reference citation (one of this repository's own files, or unknown)."""
    if name.startswith(("fpie/", "docs/", "tests/")) and (ref / name).is_file():
        return name
    if name.startswith("fpie/"):
        return name  # a reference path that does not exist: reported
    hits = [f for f in ref_files if f.endswith("/" + name)]
    mine = any(o == name or o.endswith("/" + name) for o in ours)
    if len(hits) == 1 and not mine:
        return hits[0]
    return None


def test_reference_citations_resolve():
    ref = _reference_root()
    if ref is None:
        pytest.skip("FPIE_REFERENCE is not set to a reference source tree")
    ref_files = sorted(str(p.relative_to(ref)) for p in ref.rglob("*")
                       if p.is_file() and p.suffix in {".py", ".cc", ".cu", ".h", ".md", ".rst"})
    files = list(_text_files())
    ours = {str(rel) for rel, _ in files}
    lengths: dict[str, int] = {}
    bad, seen = [], 0
    for rel, path in files:
        for ln, line in enumerate(path.read_text(errors="replace").splitlines(), 1):
            for m in CITE.finditer(line):
                target = _resolve(m.group(1), ref, ref_files, ours)
                if target is None:
                    continue
                seen += 1
                f = ref / target
                if not f.is_file():
                    bad.append(f"{rel}:{ln}: {m.group(0)} (no such reference file)")
                    continue
                n = lengths.setdefault(target, len(f.read_text(errors="replace").splitlines()))
                for a, b in _ranges(m.group(2)):
                    if not 1 <= a <= b <= n:
                        bad.append(f"{rel}:{ln}: {m.group(0)} ({target} has {n} lines)")
    assert seen > 50, f"only {seen} citations found: the parser missed them"
    assert not bad, "citations outside their files:\n" + "\n".join(bad)


def test_range_parser():
    assert list(_ranges("113-122, 192-271")) == [(113, 122), (192, 271)]
    assert list(_ranges("149-178, :286-319")) == [(149, 178), (286, 319)]
    assert list(_ranges("61")) == [(61, 61)]
    m = CITE.search("see (fpie/process.py:149-178, :286-319) here")
    assert m.group(1) == "fpie/process.py" and m.group(2) == "149-178, :286-319"
